"""elsim_gb300 -- GB300-native (sm_103a) SBM electrochemistry hot path.

The CUDA library ``libsbm_gb300.so`` (built from ``csrc/`` by
``elsim_gb300.build``) carries every kernel behind the C-ABI declared in
``include/sbm_capi.h``; ``elsim_gb300.sbm`` binds it with ctypes.
"""
from . import sbm, synth  # noqa: F401
from .sbm import Context, Params, SbmError, load_library, reference_params  # noqa: F401

__all__ = ["sbm", "synth", "Context", "Params", "SbmError", "load_library", "reference_params"]
