"""The reference's interchange files (layer 4 of include/yolohtli.h):
dataparamcsv.csv, raw_data.dat, dataTip.dat / dataTipSize.dat and
c_phi_list_sym.dat, written line for line as the reference writes them so
that its MATLAB post-processing reads them unchanged."""
import ctypes as C

import numpy as np

from . import _abi as A
from ._loader import load
from .ops import check


def _b(path):
    return None if path is None else str(path).encode()


def write_param_csv(path, p, ic_path=None, results_path=None):
    check("yh_write_param_csv", load().yh_write_param_csv(
        _b(path), C.byref(p), _b(ic_path), _b(results_path)))


def read_param_csv(path, p=None):
    """Parameters read as the reference's loadParamValues reads them, into a
    copy of p (default: the reference's defaults for a 4x4 grid, then
    overwritten by the file)."""
    q = (p.copy() if p is not None else A.param_defaults(4, 4))
    check("yh_read_param_csv", load().yh_read_param_csv(_b(path), C.byref(q)))
    return q


def _f32(x, n):
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    if x.size != n:
        raise ValueError("expected %d values, got %d" % (n, x.size))
    return x


def write_raw_data(path, p, u, v):
    n = p.nx * p.ny
    u, v = _f32(u, n), _f32(v, n)
    check("yh_write_raw_data", load().yh_write_raw_data(
        _b(path), C.byref(p), u.ctypes.data, v.ctypes.data))


def read_raw_data(path, p):
    n = p.nx * p.ny
    u, v = np.empty(n, np.float32), np.empty(n, np.float32)
    check("yh_read_raw_data", load().yh_read_raw_data(
        _b(path), C.byref(p), u.ctypes.data, v.ctypes.data))
    return u, v


def write_raw_window(path, p, u, v):
    n = p.nx * p.ny
    u, v = _f32(u, n), _f32(v, n)
    check("yh_write_raw_window", load().yh_write_raw_window(
        _b(path), C.byref(p), u.ctypes.data, v.ctypes.data))


def write_tips(tip_path, size_path, tips, append=True):
    """tips: a sequence of Tip (or an (n, 5) array x, y, vx, vy, t)."""
    tips = list(tips) if not isinstance(tips, np.ndarray) else tips
    n = len(tips)
    arr = (A.Tip * max(1, n))()
    for k in range(n):
        t = tips[k]
        if isinstance(t, A.Tip):
            arr[k] = t
        else:
            arr[k].x, arr[k].y, arr[k].vx, arr[k].vy, arr[k].t = [float(z) for z in t]
    check("yh_write_tips", load().yh_write_tips(
        _b(tip_path), _b(size_path), arr, n, 1 if append else 0))


def write_sym_list(path, c, phi):
    """c, phi: (n, 3) arrays (cx, cy, ctheta) and (phix, phiy, phitheta)."""
    c = np.ascontiguousarray(c, dtype=np.float64).reshape(-1, 3)
    phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(-1, 3)
    if c.shape != phi.shape:
        raise ValueError("c and phi differ in length")
    check("yh_write_sym_list", load().yh_write_sym_list(
        _b(path), c.ctypes.data, phi.ctypes.data, c.shape[0]))
