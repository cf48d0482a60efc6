"""GB300-native CATHY subsurface (FLOW3D) solver.

Hand-written CUDA kernels for sm_103a behind a C ABI (include/cathy_gb300.h)
that replaces the reference's FLOW3D / SYMSLV / NSYSLV / ASSPIC calls, with a
Python layer mirroring pyCATHY's ``run_processor`` and ensemble runner.
"""
from .inputs import BC, Case, Dem, Parm, Soil  # noqa: F401
