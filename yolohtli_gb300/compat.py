"""The reference's own host entry points as this library exports them
(include/yolohtli_compat.h): ctypes bindings with their C++ signatures
(hostPrototypes.h:22-51), for Python programs written against the
reference's API and for the tests and the benchmark that call them. FP64
(REAL = double) device buffers; call set_params once with the program's
paramVar, as yh_compat_set_params is called after the reference's
cudaMemcpyToSymbol block (main.cu:309-402)."""
import ctypes as C

from . import _abi as A
from ._loader import load

class Dim3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class StateVar(C.Structure):
    _fields_ = [("u", C.c_void_p), ("v", C.c_void_p)]


class AdvVar(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p)]


class SliceVar(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("ux", "uy", "ut", "vx", "vy", "vt")]


class Real3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("t", C.c_double)]


class Int2(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int)]


SYMBOLS = {
    "rd": "_Z25reactionDiffusion_wrapperm4dim3S_8stateVarS0_S0_S0_bPbbPdb4int2",
    "tip": "_Z11tip_wrapperm4dim3S_8stateVarS0_S0_dibPbPiP7vec5dyn",
    "slice": "_Z13slice_wrapperm4dim3S_8stateVar8sliceVarS1_bb6advVariPbPiP7vec5dyni",
    "cxy": "_Z17Cxy_field_wrapperm4dim3S_6advVar5REAL3S1_Pb",
    "bfecc": "_Z18advFDBFECC_wrapperm4dim3S_8stateVarS0_6advVarS0_S0_S0_Pb",
    "solve": "_Z12solve_matrix5REAL3S_Pd",
    "trapz": "_Z13trapz_wrapper4dim3S_8sliceVarS0_8stateVarPdS2_PiP7vec5dyni",
    "contour": "_Z16countour_wrapperm4dim3S_PdS0_PbS1_PiP6float3fi",
    "sapd": "_Z12sAPD_wrapperm4dim3S_iPdS0_S0_S0_S0_S0_S0_S0_PbS1_b",
}

_v, _b, _z = C.c_void_p, C.c_bool, C.c_size_t


class Compat:
    """The wrappers by short name: rd, tip, slice, cxy, bfecc, solve,
    trapz (hostPrototypes.h:22-42), contour, sapd (hostPrototypes.h:46-51)."""

    def __init__(self):
        lib = load()
        f = {k: getattr(lib, v) for k, v in SYMBOLS.items()}
        f["rd"].argtypes = [_z, Dim3, Dim3, StateVar, StateVar, StateVar, StateVar,
                            _b, _v, _b, _v, _b, Int2]
        f["tip"].argtypes = [_z, Dim3, Dim3, StateVar, StateVar, StateVar,
                             C.c_double, C.c_int, _b, _v, _v, _v]
        f["slice"].argtypes = [_z, Dim3, Dim3, StateVar, SliceVar, SliceVar, _b, _b,
                               AdvVar, C.c_int, _v, _v, _v, C.c_int]
        f["cxy"].argtypes = [_z, Dim3, Dim3, AdvVar, Real3, Real3, _v]
        f["bfecc"].argtypes = [_z, Dim3, Dim3, StateVar, StateVar, AdvVar, StateVar,
                               StateVar, StateVar, _v]
        f["solve"].argtypes = [Real3, Real3, C.POINTER(C.c_double)]
        f["solve"].restype = Real3
        f["trapz"].argtypes = [Dim3, Dim3, SliceVar, SliceVar, StateVar,
                               C.POINTER(C.c_double), _v, _v, _v, C.c_int]
        f["contour"].argtypes = [_z, Dim3, Dim3] + [_v] * 6 + [C.c_float, C.c_int]
        f["sapd"].argtypes = [_z, Dim3, Dim3, C.c_int] + [_v] * 10 + [_b]
        for k in f:
            if k != "solve":
                f[k].restype = None
        self.f = f
        self.lib = lib
        lib.yh_compat_set_params.argtypes = [C.POINTER(A.ParamVar)]
        lib.yh_compat_last_error.restype = C.c_int

    def set_params(self, p):
        rc = self.lib.yh_compat_set_params(C.byref(p))
        if rc != 0:
            raise RuntimeError("yh_compat_set_params: %d" % rc)

    def err(self):
        return self.lib.yh_compat_last_error()


def sv(a, b):
    return StateVar(a.data_ptr(), b.data_ptr())


def slv(ts):
    return SliceVar(*[t.data_ptr() for t in ts])


G2, B2 = Dim3(1, 1, 1), Dim3(16, 16, 1)


def sr_driver(cp, p, gin, nsteps, count0=0, c=None, phi=None):
    """The reference's symmetry-reduced steps (main.cu:894-954) through
    the drop-in symbols, as its driver calls them: per step RD (with
    velTan), tips, slices, the 12 integrals (trapz_wrapper), the host
    3x3 solve, the comoving field, BFECC and phi += dt c. gin: the FP64
    (u, v) device tensors, advanced in place. Returns (c, phi)."""
    import torch
    n = p.nx * p.ny

    def z(k):
        return [torch.zeros(n, dtype=torch.float64, device=gin[0].device)
                for _ in range(k)]

    gout, J, vt = z(2), z(2), z(2)
    s, s0, adv = z(6), z(6), z(2)
    uf, ub, ue = z(2), z(2), z(2)
    cnt = torch.zeros(1, dtype=torch.int32, device=gin[0].device)
    vec = torch.zeros(5 * 500000, dtype=torch.float32, device=gin[0].device)
    plot = torch.zeros(n, dtype=torch.uint8, device=gin[0].device)
    intgl = torch.zeros(n, dtype=torch.uint8, device=gin[0].device)
    c = list(c or (0.0, 0.0, 0.0))
    phi = list(phi or (0.0, 0.0, 0.0))
    AV = AdvVar(adv[0].data_ptr(), adv[1].data_ptr())
    f = cp.f
    for count in range(count0, count0 + nsteps):
        f["rd"](0, G2, B2, sv(*gout), sv(*gin), sv(*J), sv(*vt), True, None,
                False, None, False, Int2(0, 0))
        f["tip"](0, G2, B2, sv(*gin), sv(*gout), sv(*vt), p.dt * count, 1, False,
                 plot.data_ptr(), cnt.data_ptr(), vec.data_ptr())
        for _ in range(2 if count == 0 else 1):
            f["slice"](0, G2, B2, sv(*gin), slv(s), slv(s0), True, True, AV, 2,
                       intgl.data_ptr(), cnt.data_ptr(), vec.data_ptr(), count)
            I = (C.c_double * 12)()
            f["trapz"](Dim3(256, 1, 1), Dim3(64, 1, 1), slv(s), slv(s0), sv(*vt),
                       I, None, cnt.data_ptr(), vec.data_ptr(), count)
            r = f["solve"](Real3(*c), Real3(*phi), C.cast(I, C.POINTER(C.c_double)))
            c = [r.x, r.y, r.t]
            f["cxy"](0, G2, B2, AV, Real3(*c), Real3(*phi), None)
        f["bfecc"](0, G2, B2, sv(*gin), sv(*gout), AV, sv(*uf), sv(*ub), sv(*ue),
                   None)
        phi = [phi[k] + c[k] * p.dt for k in range(3)]
    return c, phi
