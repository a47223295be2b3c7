"""ORACLE — TEST INFRASTRUCTURE ONLY.

Runs the reference's own CUDA kernels headless on the GPU (cubin built from
the reference sources by oracle/ref_build.sh, launched by
oracle/ref_harness.cpp) on FP64 torch tensors. Only GPU parity tests and the
golden-fixture generator use this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from yolohtli_gb300 import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(_HERE, "_ref", "yolohtli_ref.cubin")
_LIB = os.path.join(_HERE, "_build", "libref_harness.so")
_lib = None

BLOCK2D = (16, 16)     # BLOCK_DIM_X/Y (typeDefinition.cuh:140-141)
GRID1D, BLOCK1D = 256, 64  # GRIDSIZE_1D, BLOCKSIZE_1D (typeDefinition.cuh:142-143)


def available():
    return os.path.exists(CUBIN)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            subprocess.check_call([os.path.join(_HERE, "build_harness.sh")])
        _lib = C.CDLL(_LIB)
        _lib.refh_error.restype = C.c_char_p
        if _lib.refh_open(CUBIN.encode()) != 0:
            raise RuntimeError("ref harness: " + _lib.refh_error().decode())
    return _lib


def _ck(rc):
    if rc != 0:
        raise RuntimeError("ref harness: " + lib().refh_error().decode())


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def set_params(p):
    _ck(lib().refh_set_params(C.byref(p)))


def sync():
    _ck(lib().refh_sync())


def grid2d(p):
    bx, by = BLOCK2D
    return ((p.nx + bx - 1) // bx, (p.ny + by - 1) // by, bx, by)


def rd(p, out, inp, J, vt, solid=None, reduce_sym=False):
    """reactionDiffusion_kernel on (u, v) FP64 tensors; vt written when gateDiff."""
    gx, gy, bx, by = grid2d(p)
    _ck(lib().refh_rd(gx, gy, bx, by, _ptr(out[0]), _ptr(out[1]), _ptr(inp[0]),
                      _ptr(inp[1]), _ptr(J[0]), _ptr(J[1]), _ptr(vt[0]),
                      _ptr(vt[1]), int(reduce_sym), _ptr(solid), 0, None, 0,
                      p.nx // 2, p.ny // 2))


def tip(p, past_u, present_u, tip_plot, tip_count, tip_vec, ptime):
    """spiralTip_kernel(g_past, g_present); zero tip_count first."""
    gx, gy, bx, by = grid2d(p)
    _ck(lib().refh_tip(gx, gy, bx, by, _ptr(past_u), _ptr(present_u),
                       _ptr(tip_plot), _ptr(tip_count), _ptr(tip_vec),
                       C.c_double(ptime)))


def slice_(p, g, slc, slc0, advx, advy, intgl, tip_count, tip_vec, count,
           reduce_sym_start=True, scheme=2):
    gx, gy, bx, by = grid2d(p)
    s = (C.c_void_p * 6)(*[t.data_ptr() for t in slc])
    s0 = (C.c_void_p * 6)(*[t.data_ptr() for t in slc0])
    _ck(lib().refh_slice(gx, gy, bx, by, _ptr(g[0]), _ptr(g[1]), s, s0, 1,
                         int(reduce_sym_start), _ptr(advx), _ptr(advy), scheme,
                         _ptr(intgl), _ptr(tip_count), _ptr(tip_vec),
                         int(count)))


def trapz(f, g, h, w, dot, coeff, tip_count, tip_vec, count):
    _ck(lib().refh_trapz(GRID1D, BLOCK1D, _ptr(f), _ptr(g), _ptr(h), _ptr(w),
                         _ptr(dot), _ptr(coeff), _ptr(tip_count),
                         _ptr(tip_vec), int(count)))


def cxy(p, advx, advy, c, phi, solid=None):
    gx, gy, bx, by = grid2d(p)
    cc = (C.c_double * 3)(*c)
    pp = (C.c_double * 3)(*phi)
    _ck(lib().refh_cxy(gx, gy, bx, by, _ptr(advx), _ptr(advy), cc, pp,
                       _ptr(solid)))


def bfecc(p, out, inp, advx, advy, uf, ub, ue, solid=None):
    gx, gy, bx, by = grid2d(p)
    _ck(lib().refh_bfecc(gx, gy, bx, by, _ptr(out[0]), _ptr(out[1]),
                         _ptr(inp[0]), _ptr(inp[1]), _ptr(advx), _ptr(advy),
                         _ptr(uf[0]), _ptr(uf[1]), _ptr(ub[0]), _ptr(ub[1]),
                         _ptr(ue[0]), _ptr(ue[1]), _ptr(solid)))


# Pairings of trapz_wrapper (integralTrapz.cu:97-179): (template, current)
# slice indices into (ux, uy, ut, vx, vy, vt); 'tan' = velTan.
PAIRS = [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2), (2, 0), (2, 1),
         (2, 2), (0, "tan"), (1, "tan"), (2, "tan")]


def integrals(p, slc, slc0, vt, tip_count, tip_vec, count):
    """The 12 integrals as trapz_wrapper computes them (12 launches)."""
    import torch
    dot = torch.zeros(1, dtype=torch.float64, device="cuda")
    coeff = torch.zeros(p.nx * p.ny, dtype=torch.float64, device="cuda")
    out = np.zeros(12)
    for k, (a, b) in enumerate(PAIRS):
        dot.zero_()
        f, h = slc0[a], slc0[a + 3]
        if b == "tan":
            g, w = vt[0], vt[1]
        else:
            g, w = slc[b], slc[b + 3]
        trapz(f, g, h, w, dot, coeff, tip_count, tip_vec, count)
        sync()
        out[k] = float(dot.item())
    return out


def tips_to_array(tip_vec_tensor, n):
    """(n, 5) float32 array from a device vec5dyn buffer (int32 view)."""
    raw = tip_vec_tensor[: 5 * n].cpu().numpy()
    return raw.view(np.float32).reshape(n, 5) if raw.dtype != np.float32 else raw.reshape(n, 5)


def tip_alg(alg, p, past_u, present_u, tip_plot, tip_count, tip_vec, ptime):
    """spiralTipNewton_kernel (alg 2) or abouzarTip_kernel (alg 3), the
    arguments of spiralTip_kernel; zero tip_count first for alg 2."""
    gx, gy, bx, by = grid2d(p)
    _ck(lib().refh_tip_alg(int(alg), gx, gy, bx, by, _ptr(past_u),
                           _ptr(present_u), _ptr(tip_plot), _ptr(tip_count),
                           _ptr(tip_vec), C.c_double(ptime)))


def contour(p, field1, field2, plot, stim_area, count, vec, ptime, mode):
    """countour_kernel (spaceAPD.cu:18); zero count and plot first."""
    gx, gy, bx, by = grid2d(p)
    _ck(lib().refh_contour(gx, gy, bx, by, _ptr(field1), _ptr(field2),
                           _ptr(plot), _ptr(stim_area), _ptr(count), _ptr(vec),
                           C.c_float(ptime), int(mode)))


def sapd(count, uold, unew, apd1, apd2, sapd_, dapd, back, front, first,
         stim_area, stimulate):
    """sAPD_kernel (spaceAPD.cu:278) with GRIDSIZE_1D x BLOCKSIZE_1D."""
    _ck(lib().refh_sapd(GRID1D, BLOCK1D, int(count), _ptr(uold), _ptr(unew),
                        _ptr(apd1), _ptr(apd2), _ptr(sapd_), _ptr(dapd),
                        _ptr(back), _ptr(front), _ptr(first), _ptr(stim_area),
                        1 if stimulate else 0))


def sr_driver(p, gin, nsteps, solve, count0=0):
    """The reference's symmetry-reduced steps (main.cu:894-954) on its own
    kernels: RD, tips, slices, the 12 integrals (12 launches, each read
    back), the host 3x3 solve (`solve(I, phi)`, the oracle's restatement
    of solve_matrix), the comoving field, one BFECC launch and phi += dt c.
    gin: FP64 (u, v) device tensors, advanced in place. Returns (c, phi)."""
    import torch
    n = p.nx * p.ny

    def z(k):
        return [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(k)]

    gout, J, vt = z(2), z(2), z(2)
    s, s0, adv = z(6), z(6), z(2)
    uf, ub, ue = z(2), z(2), z(2)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 500000, dtype=torch.float32, device="cuda")
    plot = torch.zeros(n, dtype=torch.uint8, device="cuda")
    intgl = torch.zeros(n, dtype=torch.uint8, device="cuda")
    c, phi = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    set_params(p)
    for count in range(count0, count0 + nsteps):
        rd(p, gout, gin, J, vt, reduce_sym=True)
        cnt.zero_()
        tip(p, gin[0], gout[0], plot, cnt, vec, p.dt * count)
        for _ in range(2 if count == 0 else 1):
            slice_(p, gin, s, s0, adv[0], adv[1], intgl, cnt, vec, count)
            I = integrals(p, s, s0, vt, cnt, vec, count)
            c = list(solve(I, phi))
            cxy(p, adv[0], adv[1], c, phi)
        bfecc(p, gin, gout, adv[0], adv[1], uf, ub, ue)
        phi = [phi[k] + c[k] * p.dt for k in range(3)]
    sync()
    return c, phi
