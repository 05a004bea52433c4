"""GB300 (sm_103a) FP64 engine for CTSM's column biogeophysics step.

The compute path is libctsm_gpu.so (hand-written CUDA, C-ABI in
include/ctsm_gpu.h); the Python modules here are the host-side mirror of the
reference interface and the input/engine plumbing around it."""
from . import abi  # noqa: F401
