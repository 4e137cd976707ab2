"""Wheel-era import path of the reference (``from ARBTools.ARBInterp import tricubic``)."""
