"""The FP64 drop-in (include/yolohtli_compat.h): the reference's seven host
entry points, called by their C++ symbols exactly as the reference's driver
calls them, against the reference's own kernels on identical FP64 inputs."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refgpu as R
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import load
from yolohtli_gb300 import workloads as W

from gpu_util import dev, host, smooth_state

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.available(),
                                 reason="reference cubin not built (oracle/ref_build.sh)")]


from yolohtli_gb300.compat import (  # noqa: E402,F401
    B2, G2, AdvVar, Compat, Dim3, Int2, Real3, SliceVar, StateVar, slv, sv)


def zeros(n, k, dtype=None):
    import torch
    return [torch.zeros(n, dtype=dtype or torch.float64, device="cuda") for _ in range(k)]


def test_compat_rd_equals_reference_kernel():
    import torch
    cp = Compat()
    n = 96
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = 2.25
    p.hx = p.hy = 2.25 / (n - 1)
    A.param_derive(p)
    for holes in (False, True):
        q = p.copy()
        solid = None
        if holes:
            q.solidSwitch = True
            solid = dev(W.hole_mask(n, n, 8, 2, 4, np.random.default_rng(1)), torch.uint8)
        cp.set_params(q)
        R.set_params(q)
        u, v = W.ref2v_cross(n, n)
        a, b = [dev(u, torch.float64), dev(v, torch.float64)], zeros(n * n, 2)
        ra, rb = [t.clone() for t in a], zeros(n * n, 2)
        J, vt, rJ, rvt = zeros(n * n, 2), zeros(n * n, 2), zeros(n * n, 2), zeros(n * n, 2)
        for _ in range(100):
            cp.f["rd"](0, G2, B2, sv(*b), sv(*a), sv(*J), sv(*vt), False,
                       None if solid is None else solid.data_ptr(), False, None,
                       False, Int2(0, 0))
            R.rd(q, rb, ra, rJ, rvt, solid)
            a, b = b, a
            ra, rb = rb, ra
        torch.cuda.synchronize()
        assert cp.err() == 0
        d = max(float((a[k] - ra[k]).abs().max()) for k in range(2))
        dt = max(float((vt[k] - rvt[k]).abs().max()) for k in range(2))
        print("compat RD vs reference kernel, 100 steps, holes=%s: max |du| %.1e, "
              "max |dtan| %.1e" % (holes, d, dt))
        assert d <= 1e-13 and dt <= 1e-10


def test_compat_tips_cxy_slices_trapz_bfecc_equal_reference():
    import torch
    cp = Compat()
    nx, ny = 96, 80
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 25
    p.tipx, p.tipy = 40.2, 37.7
    cp.set_params(p)
    R.set_params(p)
    # tips
    jj, ii = np.mgrid[0:ny, 0:nx]
    x, y = ii - nx / 2 + 0.3, jj - ny / 2 - 0.2
    fld = lambda t: (0.5 + 0.5 * np.cos(np.arctan2(y, x) - 0.35 * np.hypot(x, y) - t)).ravel()
    past, present = dev(fld(0.0), torch.float64), dev(fld(0.3), torch.float64)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 500000, dtype=torch.float32, device="cuda")
    cnt2 = torch.zeros_like(cnt)
    vec2 = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    plot = torch.zeros(nx * ny, dtype=torch.uint8, device="cuda")
    # tip_wrapper(gOut_d, gIn_d): the kernel gets g_past = gIn_d.u, g_present = gOut_d.u
    cp.f["tip"](0, G2, B2, sv(present, present), sv(past, past), sv(past, past), 1.5,
                1, False, plot.data_ptr(), cnt.data_ptr(), vec.data_ptr())
    R.tip(p, past, present, plot, cnt2, vec2, 1.5)
    R.sync()
    n1, n2 = int(cnt.item()), int(cnt2.item())
    a = host(vec)[: 5 * n1].reshape(n1, 5)
    b = host(vec2)[: 5 * n2].reshape(n2, 5)
    a = a[np.lexsort((a[:, 0], a[:, 1]))]
    b = b[np.lexsort((b[:, 0], b[:, 1]))]
    assert n1 == n2 >= 1 and np.array_equal(a, b)
    # comoving field
    c, phi = Real3(0.011, -0.02, 0.004), Real3(0.0, 0.0, 0.6)
    adv, radv = zeros(nx * ny, 2), zeros(nx * ny, 2)
    cp.f["cxy"](0, G2, B2, AdvVar(adv[0].data_ptr(), adv[1].data_ptr()), c, phi, None)
    R.cxy(p, radv[0], radv[1], (c.x, c.y, c.t), (phi.x, phi.y, phi.t))
    R.sync()
    assert max(float((adv[k] - radv[k]).abs().max()) for k in range(2)) <= 1e-17
    # slices + 12 integrals around tip_vector[count - 1]
    st = [dev(z, torch.float64) for z in smooth_state(nx, ny, 3, 2)]
    vt = [dev(z, torch.float64) for z in smooth_state(nx, ny, 4, 2)]
    tipv = torch.tensor([41.3, 37.8, 0, 0, 0], dtype=torch.float32, device="cuda")
    one = torch.ones(1, dtype=torch.int32, device="cuda")
    intgl = torch.zeros(nx * ny, dtype=torch.uint8, device="cuda")
    for count in (0, 3):
        s, s0, rs, rs0 = zeros(nx * ny, 6), zeros(nx * ny, 6), zeros(nx * ny, 6), zeros(nx * ny, 6)
        cp.f["slice"](0, G2, B2, sv(*st), slv(s), slv(s0), True, True,
                      AdvVar(adv[0].data_ptr(), adv[1].data_ptr()), 2,
                      intgl.data_ptr(), one.data_ptr(), tipv.data_ptr(), count)
        R.slice_(p, st, rs, rs0, radv[0], radv[1], intgl, one, tipv, count)
        R.sync()
        for k in range(6):
            assert float((s[k] - rs[k]).abs().max()) <= 1e-12 * float(rs[k].abs().max() + 1e-300)
            assert float((s0[k] - rs0[k]).abs().max()) <= 1e-12 * float(rs0[k].abs().max() + 1e-300)
        I = (C.c_double * 12)()
        cp.f["trapz"](Dim3(256, 1, 1), Dim3(64, 1, 1), slv(s), slv(s0), sv(*vt), I,
                      None, one.data_ptr(), tipv.data_ptr(), count)
        assert cp.err() == 0
        Iref = R.integrals(p, rs, rs0, vt, one, tipv, count)
        assert np.allclose(np.array(I[:]), Iref, rtol=1e-12, atol=1e-14 * np.abs(Iref).max())
    # BFECC against the reference kernel's race-free fixed point
    pb = p.copy()
    pb.dt = 0.01
    A.param_derive(pb)
    cp.set_params(pb)
    R.set_params(pb)
    cb, phib = Real3(1.3, -0.7, 0.02), Real3(0, 0, 0.4)
    cp.f["cxy"](0, G2, B2, AdvVar(adv[0].data_ptr(), adv[1].data_ptr()), cb, phib, None)
    out, uf, ub, ue = zeros(nx * ny, 2), zeros(nx * ny, 2), zeros(nx * ny, 2), zeros(nx * ny, 2)
    cp.f["bfecc"](0, G2, B2, sv(*out), sv(*st), AdvVar(adv[0].data_ptr(), adv[1].data_ptr()),
                  sv(*uf), sv(*ub), sv(*ue), None)
    rout, ruf, rub, rue = zeros(nx * ny, 2), zeros(nx * ny, 2), zeros(nx * ny, 2), zeros(nx * ny, 2)
    for _ in range(3):
        R.bfecc(pb, rout, st, adv[0], adv[1], ruf, rub, rue)
    R.sync()
    assert max(float((out[k] - rout[k]).abs().max()) for k in range(2)) <= 1e-14


def test_compat_solve_matrix_matches_the_reference_solve():
    cp = Compat()
    rng = np.random.default_rng(5)
    for _ in range(20):
        I = rng.standard_normal(12)
        phi = rng.uniform(-3, 3)
        r = cp.f["solve"](Real3(0, 0, 0), Real3(0, 0, phi),
                          I.ctypes.data_as(C.POINTER(C.c_double)))
        want = O.solve(I, [0, 0, phi])
        assert np.allclose([r.x, r.y, r.t], want, rtol=1e-10, atol=1e-12)


def test_reference_driver_sequence_through_compat_symbols():
    """main.cu:894-954 (symmetry-reduced steps) driven through the seven
    compat symbols and, separately, through the reference's kernels: the
    states agree to FP64 rounding after several steps."""
    import torch
    cp = Compat()
    n = 64
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = 1.5
    p.hx = p.hy = 1.5 / (n - 1)
    p.dt *= 0.5  # main.cu:148
    A.param_derive(p)
    p.tipOffsetX = p.tipOffsetY = 4 * n  # the disc covers the grid
    cp.set_params(p)
    R.set_params(p)
    u, v = smooth_state(n, n, 6, 2)

    def run(use_compat):
        gin = [dev(u, torch.float64), dev(v, torch.float64)]
        gout, J, vt = zeros(n * n, 2), zeros(n * n, 2), zeros(n * n, 2)
        s, s0 = zeros(n * n, 6), zeros(n * n, 6)
        adv = zeros(n * n, 2)
        uf, ub, ue = zeros(n * n, 2), zeros(n * n, 2), zeros(n * n, 2)
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        vec = torch.zeros(5 * 500000, dtype=torch.float32, device="cuda")
        plot = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
        intgl = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
        c, phi = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
        AV = AdvVar(adv[0].data_ptr(), adv[1].data_ptr())
        for count in range(6):
            if use_compat:
                cp.f["rd"](0, G2, B2, sv(*gout), sv(*gin), sv(*J), sv(*vt), True,
                           None, False, None, False, Int2(0, 0))
                cp.f["tip"](0, G2, B2, sv(*gin), sv(*gout), sv(*vt), p.dt * count, 1,
                            False, plot.data_ptr(), cnt.data_ptr(), vec.data_ptr())
            else:
                R.rd(p, gout, gin, J, vt)
                cnt.zero_()
                R.tip(p, gout[0], gin[0], plot, cnt, vec, p.dt * count)
            reps = 2 if count == 0 else 1
            for r in range(reps):
                if use_compat:
                    cp.f["slice"](0, G2, B2, sv(*gin), slv(s), slv(s0), True, True, AV, 2,
                                  intgl.data_ptr(), cnt.data_ptr(), vec.data_ptr(), count)
                    I = (C.c_double * 12)()
                    cp.f["trapz"](Dim3(256, 1, 1), Dim3(64, 1, 1), slv(s), slv(s0),
                                  sv(*vt), I, None, cnt.data_ptr(), vec.data_ptr(), count)
                    rc = cp.f["solve"](Real3(*c), Real3(*phi),
                                       C.cast(I, C.POINTER(C.c_double)))
                    c = [rc.x, rc.y, rc.t]
                    cp.f["cxy"](0, G2, B2, AV, Real3(*c), Real3(*phi), None)
                else:
                    R.slice_(p, gin, s, s0, adv[0], adv[1], intgl, cnt, vec, count)
                    I = R.integrals(p, s, s0, vt, cnt, vec, count)
                    c = list(O.solve(I, phi))
                    R.cxy(p, adv[0], adv[1], c, phi)
            if use_compat:
                cp.f["bfecc"](0, G2, B2, sv(*gin), sv(*gout), AV, sv(*uf), sv(*ub),
                              sv(*ue), None)
            else:
                for _ in range(3):  # the race-free fixed point of the reference kernel
                    R.bfecc(p, gin, gout, adv[0], adv[1], uf, ub, ue)
            phi = [phi[k] + c[k] * p.dt for k in range(3)]
        torch.cuda.synchronize()
        return [host(t) for t in gin], c, phi

    a, ca, pa = run(True)
    assert cp.err() == 0
    b, cb, pb = run(False)
    print("compat SR driver vs reference kernels: c %s vs %s" % (ca, cb))
    assert np.allclose(ca, cb, rtol=1e-9, atol=1e-12)
    assert np.abs(a[0] - b[0]).max() <= 1e-11
