"""Drop-in import path of the reference package (``from ARBInterp import ARBInterp``)."""
