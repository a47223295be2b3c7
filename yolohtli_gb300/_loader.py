"""Locates and loads libyolohtli_gb300.so (built in-tree by build.py).

There is no fallback: if the library is missing or fails to load, `load()`
raises, so no caller can silently run without the CUDA kernels."""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def lib_path():
    return os.environ.get("YOLOHTLI_GB300_LIB",
                          os.path.join(_HERE, "_build", "libyolohtli_gb300.so"))


def load():
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                "libyolohtli_gb300.so not found at %s: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback)" % path)
        _LIB = C.CDLL(path, mode=C.RTLD_GLOBAL)
        from . import _bind
        _bind.declare(_LIB)
    return _LIB
