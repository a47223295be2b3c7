"""This library's binary checkpoint file (include/yolohtli.h, layer 4): a
64-byte header (grid, model, fields, mask flag, step, payload size,
FNV-1a 64-bit hash), then the parameters, the FK3V parameters, the mask and
the FP32 fields. Host code: reading and writing need no GPU. A file that
fails a check raises YolohtliError with status YH_ECORRUPT.

The reference keeps its state only as raw_data.dat, with six decimals per
value (printFunctions.cu:58-78), and its reload path is dead. refio writes
and reads that format; this one restores a run bit for bit."""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from ._loader import load
from .ops import check


@dataclass
class Checkpoint:
    p: A.ParamVar
    model: int
    fk: A.FKParams
    mask: object          # uint8 array of nx*ny, or None
    step: int
    fields: list          # nfields float32 arrays of nx*ny (u, v[, w])


def _path(path):
    return str(path).encode()


def _f32(x, n):
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    if x.size != n:
        raise ValueError("expected %d values, got %d" % (n, x.size))
    return x


def write(path, p, model, fk, step, u, v, w=None, mask=None):
    n = p.nx * p.ny
    arrs = [_f32(u, n), _f32(v, n), None if w is None else _f32(w, n)]
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8).ravel()
    if m is not None and m.size != n:
        raise ValueError("expected %d mask values, got %d" % (n, m.size))
    check("yh_write_checkpoint", load().yh_write_checkpoint(
        _path(path), C.byref(p), int(model),
        None if fk is None else C.byref(fk),
        None if m is None else m.ctypes.data, int(step),
        *[None if a is None else a.ctypes.data for a in arrs]))


def header(path):
    h = A.CheckpointHeader()
    check("yh_read_checkpoint_header",
          load().yh_read_checkpoint_header(_path(path), C.byref(h)))
    return h


def read(path):
    h = header(path)
    n = h.nx * h.ny
    p, fk = A.ParamVar(), A.FKParams()
    model, step = C.c_int(), C.c_longlong()
    mask = np.empty(n, np.uint8) if h.has_mask else None
    fields = [np.empty(n, np.float32) for _ in range(h.nfields)]
    ptrs = [f.ctypes.data for f in fields] + [None] * (3 - h.nfields)
    check("yh_read_checkpoint", load().yh_read_checkpoint(
        _path(path), C.byref(p), C.byref(model), C.byref(fk),
        None if mask is None else mask.ctypes.data, C.byref(step), *ptrs))
    return Checkpoint(p, model.value, fk, mask, step.value, fields)


# The parameters the step's coefficients are made of: the fields that
# yh_load_checkpoint compares (make_step_coeffs in csrc/yh_api.cu).
def same_problem(ckpt, p, model, fk, mask):
    """True when checkpoint `ckpt` belongs to the problem (p, model, fk,
    mask): yh_checkpoint_same_problem (the rule of yh_load_checkpoint) and
    the same tissue cells, for callers that keep the parameters on the host
    (the batched solver)."""
    fk = fk if fk is not None else A.FKParams()
    if not load().yh_checkpoint_same_problem(
            C.byref(ckpt.p), int(ckpt.model), C.byref(ckpt.fk), C.byref(p),
            int(model), C.byref(fk)):
        return False
    if (ckpt.mask is None) != (mask is None):
        return False
    return mask is None or np.array_equal(ckpt.mask != 0,
                                          np.asarray(mask).ravel() != 0)
