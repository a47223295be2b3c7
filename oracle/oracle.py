"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of oracle/_build/liboracle.so, the CPU restatement of the
reference's monodomain hot path (see yh_oracle_impl.h for what it follows
and how it is pinned). Only tests/, __graft_entry__.smoke() and the CPU legs
of bench.py import this module, always as the checker or the timed CPU
baseline, never as a product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from yolohtli_gb300 import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_D = C.POINTER(C.c_double)
_Fp = C.POINTER(C.c_float)
_U8 = C.POINTER(C.c_uint8)
_PP = C.c_void_p * 3


def build():
    subprocess.check_call([os.path.join(_HERE, "build_oracle.sh")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.orc_tips.restype = C.c_int
        _lib.orc_sr_create.restype = C.c_void_p
        for f in ("orc_sr_step", "orc_sr_destroy", "orc_sr_get",
                  "orc_sr_get_tangent"):
            getattr(_lib, f).argtypes = None
    return _lib


def _sfx(dtype):
    return "_f64" if np.dtype(dtype) == np.float64 else "_f32"


def _ptrs(arrs):
    a = _PP()
    for k, x in enumerate(arrs):
        a[k] = None if x is None else x.ctypes.data
    return a


def _solid_ptr(solid):
    return None if solid is None else solid.ctypes.data_as(_U8)


def _as(x, dtype):
    return np.ascontiguousarray(x, dtype=dtype)


def nfields(model):
    return A.NFIELDS[model]


def rd_step(p, model, fk, fields, solid=None, tangent=False, dtype=np.float64):
    """One Euler reaction-diffusion step; returns (out_fields, tan_fields|None)."""
    nf = nfields(model)
    ins = [_as(f, dtype) for f in fields[:nf]]
    outs = [np.empty_like(ins[0]) for _ in range(nf)]
    tans = [np.empty_like(ins[0]) for _ in range(nf)] if tangent else None
    if solid is not None:
        solid = _as(solid, np.uint8)
    getattr(lib(), "orc_rd_step" + _sfx(dtype))(
        C.byref(p), model, C.byref(fk) if fk is not None else None,
        _ptrs(ins), _ptrs(outs), _ptrs(tans) if tangent else None,
        _solid_ptr(solid))
    return outs, tans


def run(p, model, fk, fields, nsteps, stims=(), solid=None, step0=0,
        dtype=np.float64):
    """nsteps plain Euler steps with stimulus events; returns the fields."""
    nf = nfields(model)
    st = [_as(f, dtype).copy() for f in fields[:nf]]
    scratch = [np.empty_like(st[0]) for _ in range(nf)]
    while len(st) < 3:
        st.append(None)
        scratch.append(None)
    arr = (A.Stim * max(1, len(stims)))()
    for k, s in enumerate(stims):
        arr[k] = s
    if solid is not None:
        solid = _as(solid, np.uint8)
    getattr(lib(), "orc_run" + _sfx(dtype))(
        C.byref(p), model, C.byref(fk) if fk is not None else None,
        _ptrs(st), _ptrs(scratch), _solid_ptr(solid), int(nsteps), arr,
        len(stims), int(step0))
    return st[:nf]


def stimulate_box(p, u, solid, i0, j0, i1, j1, value):
    u = np.ascontiguousarray(u)
    getattr(lib(), "orc_stimulate_box" + _sfx(u.dtype))(
        C.byref(p), C.c_void_p(u.ctypes.data), _solid_ptr(solid), i0, j0, i1, j1,
        C.c_double(value) if u.dtype == np.float64 else C.c_float(value))
    return u


def comoving(p, c, phi):
    """Separable comoving field: adv_x per row (ny), adv_y per column (nx)."""
    ax = np.zeros(p.ny)
    ay = np.zeros(p.nx)
    cc = (C.c_double * 3)(*c)
    pp = (C.c_double * 3)(*phi)
    lib().orc_comoving_f64(C.byref(p), cc, pp, ax.ctypes.data_as(_D),
                           ay.ctypes.data_as(_D))
    return ax, ay


def bfecc(p, fields, c, phi, solid=None, dtype=np.float64):
    """BFECC advection of all fields by the comoving field of (c, phi)."""
    ins = [_as(f, dtype) for f in fields]
    outs = [np.empty_like(ins[0]) for _ in ins]
    uf = np.empty_like(ins[0])
    ue = np.empty_like(ins[0])
    ax, ay = comoving(p, c, phi)
    if solid is not None:
        solid = _as(solid, np.uint8)
    getattr(lib(), "orc_bfecc" + _sfx(dtype))(
        C.byref(p), len(ins), _ptrs(ins), _ptrs(outs), ax.ctypes.data_as(_D),
        ay.ctypes.data_as(_D), _solid_ptr(solid), C.c_void_p(uf.ctypes.data),
        C.c_void_p(ue.ctypes.data))
    return outs


def slices(p, fields, c_adv, phi_adv, centre, solid=None, template=True):
    """Current (upwinded) and template derivative slices of a state:
    returns dict with keys cx, cy, ct, tx, ty, tt (lists per field)."""
    ins = [_as(f, np.float64) for f in fields]
    nf = len(ins)
    mk = lambda: [np.zeros_like(ins[0]) for _ in range(nf)]
    out = {k: mk() for k in ("cx", "cy", "ct")}
    if template:
        out.update({k: mk() for k in ("tx", "ty", "tt")})
    ax, ay = comoving(p, c_adv, phi_adv)
    cen = (C.c_float * 2)(*centre)
    if solid is not None:
        solid = _as(solid, np.uint8)
    lib().orc_slices_f64(
        C.byref(p), nf, _ptrs(ins), ax.ctypes.data_as(_D), ay.ctypes.data_as(_D),
        _solid_ptr(solid), cen, _ptrs(out["cx"]), _ptrs(out["cy"]),
        _ptrs(out["ct"]),
        _ptrs(out["tx"]) if template else None,
        _ptrs(out["ty"]) if template else None,
        _ptrs(out["tt"]) if template else None)
    return out


def integrals(p, sl, tangent, centre):
    """The 12 FP64 phase integrals from slice dict `sl` and the tangent."""
    nf = len(tangent)
    I = np.zeros(12)
    tan = [_as(t, np.float64) for t in tangent]
    cen = (C.c_float * 2)(*centre)
    lib().orc_integrals_f64(
        C.byref(p), nf, _ptrs(sl["tx"]), _ptrs(sl["ty"]), _ptrs(sl["tt"]),
        _ptrs(sl["cx"]), _ptrs(sl["cy"]), _ptrs(sl["ct"]), _ptrs(tan), cen,
        I.ctypes.data_as(_D))
    return I


def solve(I, phi):
    """The reference's unpivoted 3x3 elimination (symmetryReduction.cu:386-412)."""
    c = np.zeros(3)
    Ia = np.ascontiguousarray(I, dtype=np.float64)
    pp = (C.c_double * 3)(*phi)
    lib().orc_solve_ref(Ia.ctypes.data_as(_D), pp, c.ctypes.data_as(_D))
    return c


def tips(p, past, present, solid=None, ptime=0.0, cap=1 << 16):
    """Tips between two u levels: array (n, 5) of x, y, vx, vy, t."""
    buf = (A.Tip * cap)()
    pa = _as(past, np.float64)
    pr = _as(present, np.float64)
    if solid is not None:
        solid = _as(solid, np.uint8)
    n = lib().orc_tips(C.byref(p), pa.ctypes.data_as(_D), pr.ctypes.data_as(_D),
                       _solid_ptr(solid), C.c_double(ptime), buf, cap)
    m = min(n, cap)
    arr = np.array([[buf[k].x, buf[k].y, buf[k].vx, buf[k].vy, buf[k].t]
                    for k in range(m)], dtype=np.float32).reshape(m, 5)
    return arr


def pick_centre(tip_arr, centre):
    n = len(tip_arr)
    buf = (A.Tip * max(1, n))()
    for k in range(n):
        buf[k].x, buf[k].y = float(tip_arr[k, 0]), float(tip_arr[k, 1])
    cen = (C.c_float * 2)(*centre)
    lib().orc_pick_centre(buf, n, cen)
    return (cen[0], cen[1])


class SR:
    """The symmetry-reduced step sequence of main.cu:894-954 in FP64."""

    def __init__(self, p, model, fk, fields, solid=None,
                 template_mode=A.YH_TEMPLATE_CURRENT, template=None):
        self.p = p.copy()
        self.model = model
        self.nf = nfields(model)
        self._keep = [_as(f, np.float64) for f in fields[:self.nf]]
        self._solid = None if solid is None else _as(solid, np.uint8)
        tmpl = None
        if template is not None:
            self._tkeep = [_as(f, np.float64) for f in template[:self.nf]]
            tmpl = _ptrs(self._tkeep)
        self._fk = fk if fk is not None else A.FKParams()
        self.h = lib().orc_sr_create(
            C.byref(self.p), model, C.byref(self._fk), _solid_ptr(self._solid),
            _ptrs(self._keep), template_mode, tmpl)

    def step(self, n=1):
        for _ in range(n):
            lib().orc_sr_step(C.c_void_p(self.h))

    def get(self):
        st = [np.zeros(self.p.nx * self.p.ny) for _ in range(self.nf)]
        c = np.zeros(3)
        phi = np.zeros(3)
        I = np.zeros(12)
        cen = (C.c_float * 2)()
        step = C.c_int()
        ntips = C.c_int()
        lib().orc_sr_get(C.c_void_p(self.h), _ptrs(st), c.ctypes.data_as(_D),
                         phi.ctypes.data_as(_D), I.ctypes.data_as(_D), cen,
                         C.byref(step), C.byref(ntips))
        return dict(state=st, c=c, phi=phi, integrals=I,
                    centre=(cen[0], cen[1]), step=step.value, ntips=ntips.value)

    def tangent(self):
        t = [np.zeros(self.p.nx * self.p.ny) for _ in range(self.nf)]
        lib().orc_sr_get_tangent(C.c_void_p(self.h), _ptrs(t))
        return t

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sr_destroy(C.c_void_p(self.h))
            self.h = None


def adj_tlm(p, fk, dfk, eps, nsteps, frame, sp, D, dD, state0, target):
    """FP64 tangent-linear model of the adjoint solver's forward map
    (yh_oracle_tlm.c): (loss, directional derivative) along (dD, dfk)."""
    f32 = [np.ascontiguousarray(x, np.float32) for x in
           (D, dD, state0[0], state0[1], state0[2], target)]
    L, dL = C.c_double(), C.c_double()
    P = C.POINTER(C.c_float)
    rc = lib().orc_adj_tlm(C.byref(p), C.byref(fk), C.byref(dfk),
                           C.c_double(eps), int(nsteps), int(frame), int(sp),
                           *[a.ctypes.data_as(P) for a in f32],
                           C.byref(L), C.byref(dL))
    if rc != 0:
        raise MemoryError("orc_adj_tlm")
    return L.value, dL.value
