"""GB300-native (sm_103a) Lekien-Marsden tricubic / quadcubic interpolation.

``arbinterp_gb300.tricubic`` and ``arbinterp_gb300.quadcubic`` are drop-in
replacements for the classes of DurhamDecLab/ARBInterp v1.8; the compute runs
in the CUDA library ``libarbinterp.so`` (C ABI in ``include/arbinterp.h``).
``arbinterp_gb300.genfromtxt`` reads the reference's CSV field files on the
GPU, as ``np.genfromtxt(path, delimiter=',')`` does.
"""
from .fieldfile import genfromtxt  # noqa: F401
from .interp import __version__, quadcubic, tricubic  # noqa: F401
