"""mara3p_gb300: GB300-native (sm_103a) Godunov finite-volume update of Mara3p.

The compute path is libmara_gb300.so (hand-written CUDA behind the C ABI of
include/mara_gb300.h). The modules that compute (minidisk, srhd, mhd) load it
on import and raise if it is missing: there is no CPU fallback. The build
module imports without it.
"""
__version__ = "0.1.0"
