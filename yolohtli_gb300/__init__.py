"""yolohtli_gb300 — GB300 (sm_103a) implementation of Yolohtli's 2D monodomain
hot path: explicit reaction-diffusion step, spiral-tip tracker and the
symmetry-reduction step (BFECC comoving advection, FP64 phase integrals,
FP64 3x3 drift/rotation solve), behind the C ABI of include/yolohtli.h.

The CUDA library libyolohtli_gb300.so is required: there is no CPU path.
`load()` raises if it is missing or cannot be loaded.
"""
from . import _abi  # noqa: F401  (pure ctypes types)
from ._loader import load, lib_path  # noqa: F401

__version__ = "0.1.0"
