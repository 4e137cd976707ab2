"""``from ARBInterp import ARBInterp`` / ``ARBInterp.tricubic(...)`` as in the reference
(src/ARBInterp/ARBInterp.py); the classes are the GB300 implementation."""
from arbinterp_gb300.interp import __version__, quadcubic, tricubic  # noqa: F401
