"""The adjoint (yh_adjoint_*): dLoss/dD of a probe loss against central
finite differences of the loss itself (FP64), the FP32 gradient against the
FP64 one, checkpointing that leaves the gradient's bits unchanged, and the
torch.autograd wrapper."""
import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300.adjoint import Adjoint, probe_loss

from gpu_util import dev, host, rel_l2

pytestmark = pytest.mark.gpu


def d_map(n, seed, bumps=8):
    """D(x, y): seeded Gaussian bumps mapped into [5e-4, 1.5e-3] cm^2/ms."""
    rng = np.random.default_rng(seed)
    jj, ii = np.mgrid[0:n, 0:n] / n
    z = np.zeros((n, n))
    for _ in range(bumps):
        cx, cy = rng.uniform(0, 1, 2)
        s = rng.uniform(0.05, 0.2)
        z += rng.uniform(-1, 1) * np.exp(-((ii - cx) ** 2 + (jj - cy) ** 2) / (2 * s * s))
    z = (z - z.min()) / max(z.max() - z.min(), 1e-12)
    return (5e-4 + 1e-3 * z).astype(np.float32).ravel()


def start(n):
    u = np.zeros((n, n), np.float32)
    u[:, :6] = 1.0          # a plane wave from the left edge
    u[: n // 3, : n // 2] = np.maximum(u[: n // 3, : n // 2], 0.0)
    v = np.ones((n, n), np.float32)
    w = np.ones((n, n), np.float32)
    return [u.ravel(), v.ravel(), w.ravel()]


def problem(n, nsteps, frame, spacing, ck, fp64, seed=5, smooth=0.0):
    import torch
    p = A.fk_tissue_params(n, n)
    adj = Adjoint(p, A.fk_defaults(), nsteps, frame, spacing, ck, fp64=fp64,
                  smooth=smooth)
    st = [dev(x) for x in start(n)]
    D_true = dev(d_map(n, seed))
    tgt = torch.empty(adj.target_shape, dtype=torch.float32, device="cuda")
    adj.record(D_true, st, tgt)
    adj.set_target(tgt)
    D = D_true * 1.1  # the estimate: 10 % off
    return adj, st, D


def test_fp64_gradient_matches_central_differences():
    import torch
    n, nsteps = 64, 240
    adj, st, D = problem(n, nsteps, 20, 8, 15, fp64=True)
    g = torch.empty_like(D)
    L0 = adj.run(D, st, g)
    assert L0 > 0
    rng = np.random.default_rng(1)
    for k in range(5):
        d = dev(rng.standard_normal(n * n).astype(np.float32))
        h = 1e-6 * float(D.abs().max())  # D is stored in FP32: h >> its ulp
        # the same FP32 perturbation both ways, so D +- h d is exact to
        # the extent FP32 allows; measure the step actually taken
        Dp, Dm = D + h * d, D - h * d
        step = (Dp.double() - Dm.double()) / 2
        Lp, Lm = adj.run(Dp, st), adj.run(Dm, st)
        fd = (Lp - Lm)
        ad = 2 * float((g.double() * step).sum())
        assert abs(fd - ad) <= 1e-5 * abs(ad) + 1e-12 * L0, (k, fd, ad)


@pytest.mark.parametrize("fp64", [True, False])
def test_smoothed_switches_give_a_gradient_central_differences_confirm(fp64):
    # with FK3V's switches as tanh ramps (width 0.01) the derivative stays
    # bounded over long horizons and central differences with h = 1e-3
    # (relative) agree with it; with steps they stop agreeing after a few
    # hundred steps (the derivative leaves out the threshold crossings)
    import torch
    n, nsteps = 96, 1500
    adj, st, D = problem(n, nsteps, 20, 8, 39, fp64=fp64, smooth=0.01)
    g = torch.empty_like(D)
    adj.run(D, st, g)
    rng = np.random.default_rng(4)
    for k in range(3):
        d = dev(rng.standard_normal(n * n).astype(np.float32)) * D
        Dp, Dm = D + 1e-3 * d, D - 1e-3 * d
        step = (Dp.double() - Dm.double()) / 2
        fd = adj.run(Dp, st) - adj.run(Dm, st)
        ad = 2 * float((g.double() * step).sum())
        tol = 1e-5 if fp64 else 1e-3
        assert abs(fd - ad) <= tol * abs(ad), (k, fd, ad)


def test_fp32_gradient_against_fp64():
    import torch
    n, nsteps = 96, 300
    a32, st, D = problem(n, nsteps, 20, 8, 17, fp64=False)
    a64, _, _ = problem(n, nsteps, 20, 8, 17, fp64=True)
    g32, g64 = torch.empty_like(D), torch.empty_like(D)
    L32, L64 = a32.run(D, st, g32), a64.run(D, st, g64)
    assert abs(L32 - L64) <= 1e-4 * abs(L64)
    err = rel_l2(host(g32), host(g64))
    print("FP32 gradient vs FP64: relative L2 %.2e" % err)
    assert err <= 1e-4


def test_checkpoint_interval_leaves_the_gradient_unchanged():
    import torch
    n, nsteps = 64, 200
    outs = []
    for ck in (7, 64, 200, 1):  # 1: every state kept, no recompute
        adj, st, D = problem(n, nsteps, 25, 8, ck, fp64=False)
        g = torch.empty_like(D)
        L = adj.run(D, st, g)
        outs.append((L, host(g)))
    for L, g in outs[1:]:
        assert L == outs[0][0]
        assert np.array_equal(g, outs[0][1])


def test_autograd_function():
    import torch
    n = 48
    adj, st, D = problem(n, 120, 20, 6, 11, fp64=False)
    g = torch.empty_like(D)
    adj.run(D, st, g)
    Dv = D.clone().requires_grad_(True)
    loss = probe_loss(Dv, adj, st)
    (3.0 * loss).backward()
    assert torch.allclose(Dv.grad, 3.0 * g)


def test_fk_parameter_gradient_matches_central_differences():
    # all 13 FK3V parameters, FP64, smoothed switches (so u_c and u_v act
    # through a differentiable ramp): the adjoint's dLoss/dtheta against
    # central differences with a relative step of 1e-5
    import torch
    from yolohtli_gb300.adjoint import fk_array, fk_struct
    n, nsteps = 48, 200
    adj, st, D = problem(n, nsteps, 20, 6, 14, fp64=True, smooth=0.02)
    g = torch.empty_like(D)
    gfk = A.FKParams()
    adj.run(D, st, g, gfk)
    ad = fk_array(gfk)
    base = fk_array(adj.fk)
    assert np.all(np.isfinite(ad)) and np.abs(ad).max() > 0
    fd = np.zeros(13)
    for q in range(13):
        h = 1e-5 * abs(base[q])
        for sgn in (1, -1):
            x = base.copy()
            x[q] += sgn * h
            adj.set_fk(fk_struct(x))
            fd[q] += sgn * adj.run(D, st)
        fd[q] /= 2 * h
    adj.set_fk(fk_struct(base))
    print("dL/dtheta adjoint", ad)
    print("dL/dtheta central", fd)
    for q in range(13):
        assert abs(fd[q] - ad[q]) <= 1e-5 * abs(ad[q]) + 1e-9 * np.abs(ad).max(), \
            (A.FK_NAMES[q], fd[q], ad[q])


def test_fk_parameter_gradient_fp32_against_fp64_and_steps():
    import torch
    from yolohtli_gb300.adjoint import fk_array
    n, nsteps = 64, 240
    out = []
    for fp64 in (True, False):
        adj, st, D = problem(n, nsteps, 20, 8, 15, fp64=fp64)
        g = torch.empty_like(D)
        gfk = A.FKParams()
        L = adj.run(D, st, g, gfk)
        g0 = torch.empty_like(D)
        assert adj.run(D, st, g0) == L      # the same forward pass
        assert torch.equal(g, g0)           # and the same dLoss/dD
        out.append(fk_array(gfk))
    a64, a32 = out
    err = np.abs(a32 - a64) / np.abs(a64).max()
    print("FK gradient FP32 vs FP64 (relative to the largest):", err.max())
    assert err.max() <= 1e-3


def test_autograd_with_fk_parameters():
    import torch
    from yolohtli_gb300.adjoint import fk_array
    n = 48
    adj, st, D = problem(n, 120, 20, 6, 11, fp64=False)
    g = torch.empty_like(D)
    gfk = A.FKParams()
    adj.run(D, st, g, gfk)
    Dv = D.clone().requires_grad_(True)
    fk = torch.tensor(fk_array(adj.fk), dtype=torch.float64, requires_grad=True)
    loss = probe_loss(Dv, adj, st, fk)
    (2.0 * loss).backward()
    assert torch.allclose(Dv.grad, 2.0 * g)
    assert np.allclose(fk.grad.numpy(), 2.0 * fk_array(gfk))
    # a different fk switches the handle and changes the loss
    fk2 = fk.detach().clone()
    fk2[0] *= 1.2
    assert float(probe_loss(D, adj, st, fk2)) != float(loss)


@pytest.mark.parametrize("smooth", [0.0, 0.02])
def test_gradients_match_the_fp64_tangent_linear_oracle(smooth):
    # 64x64 downscale: the adjoint's <dL/dD, dD> + <dL/dtheta, dtheta> against
    # the directional derivative of the oracle's tangent-linear model (dual
    # numbers through the same discrete map, no shared derivation)
    import torch
    from oracle import oracle as O
    from yolohtli_gb300.adjoint import fk_array, fk_struct
    n, nsteps, frame, sp = 64, 240, 20, 8
    adj, st, D = problem(n, nsteps, frame, sp, 15, fp64=True, smooth=smooth)
    tgt = torch.empty(adj.target_shape, dtype=torch.float32, device="cuda")
    adj.record(D / 1.1, st, tgt)  # a target: the run with D / 1.1
    adj.set_target(tgt)
    g = torch.empty_like(D)
    gfk = A.FKParams()
    L = adj.run(D, st, g, gfk)
    rng = np.random.default_rng(8)
    dD = (rng.standard_normal(n * n) * 1e-4).astype(np.float32)
    dth = rng.standard_normal(13) * fk_array(adj.fk) * 0.05
    Lo, dLo = O.adj_tlm(adj.p, adj.fk, fk_struct(dth), smooth, nsteps, frame, sp,
                        host(D), dD, [host(x) for x in st], host(tgt))
    ad = float(np.dot(host(g).astype(np.float64), dD.astype(np.float64))) + \
        float(np.dot(fk_array(gfk), dth))
    print("loss GPU %.12e oracle %.12e; dL adjoint %.10e tangent-linear %.10e"
          % (L, Lo, ad, dLo))
    assert abs(L - Lo) <= 1e-9 * abs(Lo)
    assert abs(ad - dLo) <= 1e-6 * abs(dLo)


@pytest.mark.parametrize("ck", [9, 1])
def test_batched_instances_equal_single_handles(ck):
    # three instances (own D, initial state, target) in one handle: each
    # instance's loss, dLoss/dD and dLoss/dtheta equal to the bit those of a
    # handle of its own
    import torch
    n, nsteps, frame, sp, B = 40, 90, 15, 5, 3
    p = A.fk_tissue_params(n, n)
    fk = A.fk_defaults()
    Ds, sts, tgts, trues = [], [], [], []
    for b in range(B):
        D_true = dev(d_map(n, 20 + b))
        trues.append(D_true)
        st = [dev(x) for x in start(n)]
        st[0] = st[0].roll(3 * b)  # a different start per instance
        one = Adjoint(p, fk, nsteps, frame, sp, ck)
        t = torch.empty(one.target_shape, dtype=torch.float32, device="cuda")
        one.record(D_true, st, t)
        Ds.append(D_true * (1.05 + 0.05 * b))
        sts.append(st)
        tgts.append(t)
    bat = Adjoint(p, fk, nsteps, frame, sp, ck, batch=B)
    tb = torch.empty(bat.target_shape, dtype=torch.float32, device="cuda")
    bat.record(torch.cat(trues), [torch.cat([s[q] for s in sts]) for q in range(3)], tb)
    for b in range(B):  # the batched forward records the same targets
        assert torch.equal(tb[b], tgts[b])
    bat.set_target(tb)
    Dcat = torch.cat(Ds)
    gb = torch.empty_like(Dcat)
    gfk = (A.FKParams * B)()
    Lb = bat.run(Dcat, [torch.cat([s[q] for s in sts]) for q in range(3)], gb, gfk)
    from yolohtli_gb300.adjoint import fk_array
    for b in range(B):
        one = Adjoint(p, fk, nsteps, frame, sp, ck)
        one.set_target(tgts[b])
        g = torch.empty_like(Ds[b])
        f1 = A.FKParams()
        L1 = one.run(Ds[b], sts[b], g, f1)
        assert L1 == Lb[b]
        assert torch.equal(g, gb[b * n * n:(b + 1) * n * n])
        assert np.array_equal(fk_array(f1), fk_array(gfk[b]))


def test_batched_fit_lowers_the_loss():
    """Parameter estimation over 4 instances in one batched handle (each its
    own true D; the 13 FK3V parameters shared): Adam on log D and log
    parameters from the true values + 10 %, 12 iterations; every
    instance's loss falls at least fourfold (measured 6.8-8.2x). (Recovering
    D itself is ill-posed from
    1024 probes: the errors of D and of the parameters are printed.)"""
    import torch
    from yolohtli_gb300.adjoint import fit, fk_array
    n, nsteps, B = 64, 400, 4
    p = A.fk_tissue_params(n, n)
    fk0 = A.fk_defaults()
    adj = Adjoint(p, fk0, nsteps, 20, 8, 20, smooth=0.01, batch=B)
    st = [dev(x).repeat(B) for x in start(n)]
    D_true = torch.cat([dev(d_map(n, 5 + k)) for k in range(B)])
    tgt = torch.empty(adj.target_shape, dtype=torch.float32, device="cuda")
    adj.record(D_true, st, tgt)
    adj.set_target(tgt)
    D = D_true * 1.1
    err0 = float((D - D_true).norm() / D_true.norm())
    th, losses = fit(adj, D, st, fk_array(fk0) * 1.1, iters=12, lr=0.02)
    err1 = float((D - D_true).norm() / D_true.norm())
    eth = float(np.abs(th / fk_array(fk0) - 1).max())
    print("batched fit: loss per instance", losses[0], "->", losses[-1],
          "; D error %.3f -> %.3f; FK parameters max error 0.100 -> %.3f" % (
              err0, err1, eth))
    assert losses.shape == (13, B)
    assert np.all(losses[-1] < 0.25 * losses[0])
    assert np.all(np.isfinite(th))
