"""The CPU oracle (test infrastructure) against analytic results and against
the reference's own code (golden fixtures from its host functions and its
CUDA kernels run headless)."""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as O
from yolohtli_gb300 import _abi as A


def grid(nx, ny):
    j, i = np.mgrid[0:ny, 0:nx]
    return i.astype(float), j.astype(float)


def pure_diffusion_params(nx, ny):
    p = A.param_defaults(nx, ny)
    p.mu = 0.0  # REF2V reaction off with v = 0: I_sum = 0
    p.eps = 0.0
    p.gateDiff = False
    return p


# ---------------------------------------------------------------- RD step

def test_laplacian_exact_on_quadratics_interior():
    p = pure_diffusion_params(32, 24)
    i, j = grid(32, 24)
    u = (0.3 * i ** 2 + 0.7 * j ** 2 + 0.1 * i * j) * 1e-3
    (out, _), = [O.rd_step(p, A.YH_MODEL_REF2V, None, [u.ravel(), 0 * u.ravel()])]
    lap = (out[0].reshape(24, 32) - u)[1:-1, 1:-1]
    assert np.abs(lap - (2 * 0.3 * p.rx + 2 * 0.7 * p.ry) * 1e-3).max() < 1e-15


def test_mirror_ghost_at_the_boundary():
    # coord_i(-1) = 1, coord_i(nx) = nx-2 (helper_functions.cu:69-79)
    p = pure_diffusion_params(16, 12)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((12, 16))
    out, _ = O.rd_step(p, A.YH_MODEL_REF2V, None, [u.ravel(), 0 * u.ravel()])
    o = out[0].reshape(12, 16)
    exp00 = u[0, 0] + (u[0, 1] - 2 * u[0, 0] + u[0, 1]) * p.rx + \
        (u[1, 0] - 2 * u[0, 0] + u[1, 0]) * p.ry
    assert o[0, 0] == pytest.approx(exp00, rel=1e-14)
    expN = u[-1, 5] + (u[-1, 4] - 2 * u[-1, 5] + u[-1, 6]) * p.rx + \
        (u[-2, 5] - 2 * u[-1, 5] + u[-2, 5]) * p.ry
    assert o[-1, 5] == pytest.approx(expN, rel=1e-14)


def test_neumann_diffusion_conserves_trapezoid_weighted_sum():
    p = pure_diffusion_params(40, 30)
    rng = np.random.default_rng(1)
    u = rng.random((30, 40))
    wx = np.ones(40); wx[[0, -1]] = 0.5
    wy = np.ones(30); wy[[0, -1]] = 0.5
    wt = np.outer(wy, wx)
    st = O.run(p, A.YH_MODEL_REF2V, None, [u.ravel(), 0 * u.ravel()], 50)
    assert (wt * st[0].reshape(30, 40)).sum() == pytest.approx((wt * u).sum(), rel=1e-13)


@pytest.mark.parametrize("sw,sc,se,exp", [
    (1, 1, 1, (1, 2, 1)), (1, 1, 0, (2, 2, 0)), (0, 1, 1, (0, 2, 2)),
    (0, 1, 0, (0, 0, 0)), (1, 0, 1, (0, 0, 0))])
def test_hole_coefficients(sw, sc, se, exp):
    # reactionDiffusion.cu:162-169 on a 3-cell row embedded in a 5x5 grid
    p = pure_diffusion_params(5, 5)
    p.ry = 0.0
    p.solidSwitch = True
    solid = np.ones((5, 5), np.uint8)
    solid[2, 1], solid[2, 2], solid[2, 3] = sw, sc, se
    u = np.zeros((5, 5))
    u[2, 1], u[2, 2], u[2, 3] = 3.0, 5.0, 11.0
    out, _ = O.rd_step(p, A.YH_MODEL_REF2V, None, [u.ravel(), 0 * u.ravel()],
                       solid=solid.ravel())
    lap = (exp[0] * 3.0 - exp[1] * 5.0 + exp[2] * 11.0) * p.rx
    want = 5.0 + lap if sc else 0.0
    assert out[0].reshape(5, 5)[2, 2] == pytest.approx(want, rel=1e-14, abs=1e-300)


def fk_python(fk, u, v, w):
    """Fenton & Karma (1998) eqs. (2)-(6), written out directly."""
    p = 1.0 if u >= fk.u_c else 0.0
    q = 1.0 if u >= fk.u_v else 0.0
    jfi = -v * p * (1 - u) * (u - fk.u_c) / fk.tau_d
    jso = u * (1 - p) / fk.tau_0 + p / fk.tau_r
    jsi = -w * (1 + math.tanh(fk.k * (u - fk.u_csi))) / (2 * fk.tau_si)
    tvm = q * fk.tau_v1_minus + (1 - q) * fk.tau_v2_minus
    dv = (1 - p) * (1 - v) / tvm - p * v / fk.tau_v_plus
    dw = (1 - p) * (1 - w) / fk.tau_w_minus - p * w / fk.tau_w_plus
    return jfi + jso + jsi, dv, dw


@pytest.mark.parametrize("u,v,w", [(0.0, 1.0, 1.0), (0.05, 0.9, 0.95),
                                   (0.1, 0.5, 0.8), (0.5, 0.8, 0.9),
                                   (0.95, 0.1, 0.3), (1.0, 0.0, 0.5)])
def test_fk3v_reaction_matches_the_published_equations(u, v, w):
    fk = A.fk_defaults()
    p = A.fk_tissue_params(8, 8)
    f = [np.full(64, u), np.full(64, v), np.full(64, w)]
    out, tan = O.rd_step(p, A.YH_MODEL_FK3V, fk, f, tangent=True)
    J, dv, dw = fk_python(fk, u, v, w)
    assert out[0][27] == pytest.approx(u - p.dt * J, rel=1e-14, abs=1e-16)
    assert out[1][27] == pytest.approx(v + p.dt * dv, rel=1e-14, abs=1e-16)
    assert out[2][27] == pytest.approx(w + p.dt * dw, rel=1e-14, abs=1e-16)
    assert tan[0][27] == pytest.approx(-J, rel=1e-12, abs=1e-14)


def test_fp32_transcription_tracks_fp64():
    fk = A.fk_defaults()
    p = A.fk_tissue_params(48, 40)
    rng = np.random.default_rng(2)
    u = rng.uniform(0, 1, 48 * 40)
    v = rng.uniform(0, 1, 48 * 40)
    w = rng.uniform(0, 1, 48 * 40)
    a = O.run(p, A.YH_MODEL_FK3V, fk, [u, v, w], 20, dtype=np.float64)
    b = O.run(p, A.YH_MODEL_FK3V, fk, [u, v, w], 20, dtype=np.float32)
    assert np.abs(a[0] - b[0]).max() < 1e-5


def test_fk3v_switch_sensitivity():
    """The FK3V discrete map amplifies a tiny change of the state once
    fronts move: H(u - u_c) and H(u - u_v) switch the gate rates (v by
    dt/tau_v+ = 0.015 in one step), so a cell whose u lands on the other
    side of u_c a step earlier shifts its front. In FP64 a 1e-10 change of
    the spiral protocol's initial u (256^2) stays ~1e-10 for hundreds of
    steps and exceeds 1e-6 relative L2 by step 2000: the growth that FP32
    rounding (~1e-7 per step) meets far sooner. A tolerance of 1e-5 after
    N steps therefore holds only for N of a few hundred with FP32 fields."""
    from yolohtli_gb300 import workloads as W
    wl = W.fk_spiral_256(nsteps=2000)
    s0 = [x.astype(np.float64) for x in wl.state0()]
    s1 = [x.copy() for x in s0]
    s1[0] = s1[0] + 1e-10 * np.random.default_rng(5).standard_normal(wl.cells)
    a = O.run(wl.p, wl.model, wl.fk, s0, 300, wl.stims)
    b = O.run(wl.p, wl.model, wl.fk, s1, 300, wl.stims)
    early = np.linalg.norm(b[0] - a[0]) / np.linalg.norm(a[0])
    a = O.run(wl.p, wl.model, wl.fk, a, 1700, wl.stims, step0=300)
    b = O.run(wl.p, wl.model, wl.fk, b, 1700, wl.stims, step0=300)
    late = np.linalg.norm(b[0] - a[0]) / np.linalg.norm(a[0])
    assert early < 1e-9
    assert late > 1e-6


# ---------------------------------------------------------------- SR pieces

def test_bfecc_translates_a_gaussian_at_second_order():
    errs = []
    for n in (64, 128):
        p = A.param_defaults(n, n)
        p.Lx = p.Ly = 1.0
        p.hx = p.hy = 1.0 / (n - 1)
        p.dt = 0.2 * p.hx
        A.param_derive(p)
        x, y = grid(n, n)
        x *= p.hx
        y *= p.hy
        g = lambda x0, y0: np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / 0.01)
        # c = (cx, cy, 0), phi = 0: adv = (-cx, -cy); BFECC transports with
        # velocity -adv = (cx, cy) (advFDBFECC.cu:30-34 upwinds on -adv)
        c = [0.4, 0.3, 0.0]
        T = 0.25
        steps = int(round(T / p.dt))
        f = g(0.4, 0.4).ravel()
        for _ in range(steps):
            f = O.bfecc(p, [f], c, [0, 0, 0])[0]
        exact = g(0.4 + 0.4 * steps * p.dt, 0.4 + 0.3 * steps * p.dt).ravel()
        errs.append(np.abs(f - exact).max())
    assert errs[1] < errs[0] / 3.0, errs


def test_comoving_field_is_separable_and_matches_the_formula():
    p = A.param_defaults(24, 20)
    c = [0.3, -0.2, 0.05]
    phi = [0.0, 0.0, 0.9]
    ax, ay = O.comoving(p, c, phi)
    j = np.arange(20)
    i = np.arange(24)
    assert np.allclose(ax, p.hy * j * c[2] - c[0] * math.cos(0.9) + c[1] * math.sin(0.9), rtol=1e-15, atol=1e-17)
    assert np.allclose(ay, -p.hx * i * c[2] - c[0] * math.sin(0.9) - c[1] * math.cos(0.9), rtol=1e-15, atol=1e-17)


def test_slices_exact_on_polynomials():
    p = A.param_defaults(40, 40)
    p.tipOffsetX = p.tipOffsetY = 10
    x, y = grid(40, 40)
    hx, hy = p.hx, p.hy
    f = (0.2 * (x * hx) ** 2 - 0.1 * (y * hy) ** 2 + 0.05 * (x * hx) * (y * hy))
    f3 = (x * hx) ** 3 + 2 * (y * hy) ** 3
    for adv_sign in (+1, -1):
        c = [-adv_sign * 0.1, adv_sign * 0.1, 0.0]  # adv.x = -cx, adv.y = -cy
        s = O.slices(p, [f.ravel(), f3.ravel()], c, [0, 0, 0], (20.0, 20.0))
        disc = s["cx"][0].reshape(40, 40) != 0
        dfx = (0.4 * x * hx + 0.05 * y * hy)
        dfy = (-0.2 * y * hy + 0.05 * x * hx)
        cx = s["cx"][0].reshape(40, 40)
        cy = s["cy"][0].reshape(40, 40)
        assert np.abs(cx[disc] - dfx[disc]).max() < 1e-12
        assert np.abs(cy[disc] - dfy[disc]).max() < 1e-12
        # template: the NEGATED 4th-order central derivative, exact on cubics
        tx = s["tx"][1].reshape(40, 40)
        assert np.abs(tx[disc] + 3 * (x[disc] * hx) ** 2).max() < 1e-10
        tt = s["tt"][0].reshape(40, 40)
        want = hx * x * s["ty"][0].reshape(40, 40) - hy * y * s["tx"][0].reshape(40, 40)
        assert np.abs(tt - want).max() < 1e-14


def test_disc_integrals_of_constant_fields():
    p = A.param_defaults(50, 50)
    p.tipOffsetX = p.tipOffsetY = 7
    n = 2500
    sl = {k: [np.full(n, a), np.full(n, b)] for k, a, b in
          [("tx", 1.0, 2.0), ("ty", 3.0, 0.5), ("tt", -1.0, 1.0),
           ("cx", 2.0, 1.0), ("cy", 1.0, -1.0), ("ct", 0.5, 0.5)]}
    tan = [np.full(n, 4.0), np.full(n, 1.0)]
    centre = (20.0, 30.0)
    I = O.integrals(p, sl, tan, centre)
    ndisc = sum(1 for i in range(50) for j in range(50)
                if (i - 25 - (20 - 25)) ** 2 + (j - 25 - (30 - 25)) ** 2 < 49)
    dA = p.hx * p.hy
    assert I[0] == pytest.approx(dA * ndisc * (1 * 2 + 2 * 1))
    assert I[4] == pytest.approx(dA * ndisc * (3 * 1 + 0.5 * -1))
    assert I[11] == pytest.approx(dA * ndisc * (-1 * 4 + 1 * 1))


def test_solve_agrees_with_numpy_on_the_rotated_system():
    rng = np.random.default_rng(3)
    for _ in range(20):
        I = rng.standard_normal(12)
        pt = rng.uniform(-4, 4)
        cs, sn = math.cos(pt), math.sin(pt)
        M = np.array([[I[3 * r] * cs + I[3 * r + 1] * sn,
                       I[3 * r + 1] * cs - I[3 * r] * sn, I[3 * r + 2]]
                      for r in range(3)])
        c = O.solve(I, [0, 0, pt])
        assert np.allclose(c, np.linalg.solve(M, I[9:]), rtol=1e-9, atol=1e-12)


def test_tip_on_a_synthetic_bilinear_pair():
    # two bilinear fields whose Uth isolines cross at (10.3, 7.6); bilinear
    # interpolation is exact for them, so the closed form must find that
    # point (purely linear fields make the quadratic degenerate: den = 0)
    p = A.param_defaults(24, 20)
    x, y = grid(24, 20)
    dx, dy = x - 10.3, y - 7.6
    a = p.Uth + 0.05 * dx + 0.02 * dx * dy
    b = p.Uth + 0.05 * dy - 0.03 * dx * dy
    # roots: dx*(0.05 + 0.02 dy) = 0 and dy*(0.05 - 0.03 dx) = 0, i.e.
    # (dx, dy) = (0, 0) and (5/3, -2.5)
    tips = O.tips(p, b.ravel(), a.ravel(), ptime=3.0)
    tips = tips[np.argsort(tips[:, 0])]
    assert len(tips) == 2
    assert np.allclose(tips[0, :2], [10.3, 7.6], atol=1e-5)
    assert np.allclose(tips[1, :2], [10.3 + 5 / 3, 7.6 - 2.5], atol=1e-5)
    assert np.all(tips[:, 4] == np.float32(3.0))


def test_pick_centre_is_order_independent():
    t = np.array([[5, 5, 0, 0, 0], [1, 1, 0, 0, 0], [9, 2, 0, 0, 0]], np.float32)
    a = O.pick_centre(t, (2.0, 2.0))
    b = O.pick_centre(t[::-1].copy(), (2.0, 2.0))
    assert a == b == (1.0, 1.0)
    assert O.pick_centre(t[:0], (2.0, 3.0)) == (2.0, 3.0)


# ---------------------------------------------------------------- golden: reference

def test_oracle_solve_matches_reference_solve_matrix(golden_host):
    for I, phi, c in zip(golden_host["solve_I"], golden_host["solve_phi"],
                         golden_host["solve_c"]):
        assert np.array_equal(O.solve(I, phi), c) or \
            np.allclose(O.solve(I, phi), c, rtol=1e-14, atol=0)


def _p(raw):
    p = A.ParamVar()
    C.memmove(C.byref(p), raw.tobytes(), C.sizeof(p))
    return p


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("case", ["rd_sq", "rd_holes"])
@pytest.mark.parametrize("steps", [1, 20])
def test_oracle_rd_matches_reference_kernel(golden_gpu, case, steps):
    g = golden_gpu
    p = _p(g[case + "_p"])
    solid = g["rd_holes_solid"] if case == "rd_holes" else None
    st = [g["rd_sq_u0"], g["rd_sq_v0"]]
    if solid is not None:
        tan = None
    for _ in range(steps):
        st, tan = O.rd_step(p, A.YH_MODEL_REF2V, None, st, solid=solid, tangent=True)
    tol = 1e-14 if steps == 1 else 1e-13
    assert rel(st[0], g["%s_%d_u" % (case, steps)]) < tol
    assert rel(st[1], g["%s_%d_v" % (case, steps)]) < tol
    assert rel(tan[0], g["%s_%d_tu" % (case, steps)]) < 1e-11
    assert rel(tan[1], g["%s_%d_tv" % (case, steps)]) < 1e-11


def test_oracle_tips_match_reference_kernel(golden_gpu):
    g = golden_gpu
    p = A.param_defaults(48, 40)
    tips = O.tips(p, g["tip_past"], g["tip_present"], ptime=1.5)
    ref = g["tip_tips"]
    assert len(ref) >= 1 and len(tips) == len(ref)
    tips = tips[np.lexsort((tips[:, 0], tips[:, 1]))]
    assert np.abs(tips - ref).max() < 1e-5


def test_oracle_comoving_matches_reference_cxy(golden_gpu):
    g = golden_gpu
    p = A.param_defaults(48, 40)
    ax, ay = O.comoving(p, g["cxy_c"], g["cxy_phi"])
    X = np.broadcast_to(ax[:, None], (40, 48)).ravel()
    Y = np.broadcast_to(ay[None, :], (40, 48)).ravel()
    assert rel(X, g["cxy_x"]) < 1e-15
    assert rel(Y, g["cxy_y"]) < 1e-15


@pytest.mark.parametrize("count", [0, 7])
def test_oracle_slices_and_integrals_match_reference(golden_gpu, count):
    g = golden_gpu
    p = _p(g["slice_p"])
    centre = (p.tipx, p.tipy) if count == 0 else tuple(g["slice_tip"])
    s = O.slices(p, [g["slice_u"], g["slice_v"]], g["cxy_c"], g["cxy_phi"], centre)
    cur = g["slice_%d_cur" % count]
    tm = g["slice_%d_tmpl" % count]
    for k, key in enumerate(("cx", "cy", "ct")):
        assert rel(s[key][0], cur[k]) < 1e-13, key
        assert rel(s[key][1], cur[k + 3]) < 1e-13, key
    for k, key in enumerate(("tx", "ty", "tt")):
        assert rel(s[key][0], tm[k]) < 1e-13, key
        assert rel(s[key][1], tm[k + 3]) < 1e-13, key
    I = O.integrals(p, s, [g["slice_tu"], g["slice_tv"]], centre)
    ref = g["trapz_%d" % count]
    assert np.allclose(I, ref, rtol=1e-11, atol=1e-13 * np.abs(ref).max())


def test_oracle_bfecc_matches_reference_fixed_point(golden_gpu):
    g = golden_gpu
    p = _p(g["bfecc_p"])
    out = O.bfecc(p, [g["bfecc_u0"], g["bfecc_v0"]], g["bfecc_c"], g["bfecc_phi"])
    assert rel(out[0], g["bfecc_u"]) < 1e-13
    assert rel(out[1], g["bfecc_v"]) < 1e-13


def test_tangent_linear_model_matches_its_own_central_differences():
    # the FP64 tangent-linear oracle of the adjoint solver's forward map:
    # its directional derivative against central differences of its loss
    from yolohtli_gb300.adjoint import fk_array, fk_struct
    n, nsteps, frame, sp = 24, 80, 10, 4
    p = A.fk_tissue_params(n, n)
    rng = np.random.default_rng(3)
    D = rng.uniform(5e-4, 1.5e-3, n * n).astype(np.float32)
    u = np.zeros((n, n), np.float32)
    u[:, :4] = 1.0
    st = [u.ravel(), np.ones(n * n, np.float32), np.ones(n * n, np.float32)]
    tgt = rng.uniform(0, 0.5, (nsteps // frame) * (n // sp) ** 2).astype(np.float32)
    base = fk_array(A.fk_defaults())
    dth = rng.standard_normal(13) * base * 0.1
    dD = (rng.standard_normal(n * n) * 1e-4).astype(np.float32)
    h = 1e-4
    # D +- h dD is rounded to FP32: the direction is the step actually taken
    Dp = (D + h * dD).astype(np.float32)
    Dm = (D - h * dD).astype(np.float32)
    dD = ((Dp.astype(np.float64) - Dm) / (2 * h)).astype(np.float32)
    for eps in (0.0, 0.02):
        L, dL = O.adj_tlm(p, fk_struct(base), fk_struct(dth), eps, nsteps, frame,
                          sp, D, dD, st, tgt)
        Lp, _ = O.adj_tlm(p, fk_struct(base + h * dth), fk_struct(0 * dth), eps,
                          nsteps, frame, sp, Dp, 0 * dD, st, tgt)
        Lm, _ = O.adj_tlm(p, fk_struct(base - h * dth), fk_struct(0 * dth), eps,
                          nsteps, frame, sp, Dm, 0 * dD, st, tgt)
        assert L > 0
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd - dL) <= 1e-5 * abs(dL), (eps, fd, dL)


def _cable(tau_d, dx, dt, L_cm=8.0, t_ms=260.0):
    """Planar wave along a cable of FK3V tissue (the oracle, FP64): speed
    between 30 % and 60 % of the cable and the time u stays above 0.5 at
    30 %."""
    nx, ny = int(round(L_cm / dx)), 5
    p = A.fk_tissue_params(nx, ny)
    p.hx = p.hy = dx
    p.dt = dt
    p = A.param_derive(p)
    fk = A.fk_defaults()
    fk.tau_d = tau_d
    u = np.zeros((ny, nx))
    u[:, : int(round(0.25 / dx))] = 1.0
    st = [u.ravel(), np.ones(nx * ny), np.ones(nx * ny)]
    x1, x2 = int(nx * 0.3), int(nx * 0.6)
    up, down = {}, None
    every = max(1, int(round(0.5 / dt)))
    step = 0
    while step * dt < t_ms:
        st = O.run(p, A.YH_MODEL_FK3V, fk, st, every, step0=step)
        step += every
        row = st[0].reshape(ny, nx)[2]
        for x in (x1, x2):
            if x not in up and row[x] > 0.5:
                up[x] = step * dt
        if x1 in up and down is None and row[x1] < 0.5 and step * dt > up[x1] + 5:
            down = step * dt
    cv = (x2 - x1) * dx / (up[x2] - up[x1]) * 10.0  # m/s
    return cv, down - up[x1]


def test_fk3v_planar_wave_speed_and_duration():
    """Macroscopic observables of the BR-fit parameter set with tau_d =
    0.25 at the benchmark's dx = 0.025 cm, dt = 0.05 ms, D = 0.001 cm^2/ms
    (measured: 0.435 m/s, 135 ms above u = 0.5), converged within 5 % against
    dx = 0.0125 cm, dt = 0.0125 ms (0.455 m/s, 135.5 ms)."""
    cv, apd = _cable(0.25, 0.025, 0.05)
    cv2, apd2 = _cable(0.25, 0.0125, 0.0125)
    assert 0.40 < cv < 0.47 and 125.0 < apd < 145.0
    assert abs(cv2 / cv - 1) < 0.06 and abs(apd2 / apd - 1) < 0.03
