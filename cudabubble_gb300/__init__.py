"""GB300-native (sm_103a) pseudo-spectral Allen-Cahn stepper for CudaBubble's
phase-field elastic bending energy.  The compute path is libcbstep.so
(``include/cbstep.h``); this package is its Python face."""
from . import capi, shapes  # noqa: F401

__all__ = ["capi", "shapes"]
