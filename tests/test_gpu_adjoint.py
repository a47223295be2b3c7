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
    for ck in (7, 64, 200):
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
