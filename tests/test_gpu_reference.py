"""The reference's own CUDA kernels, run headless on the GPU (oracle/refgpu),
against the oracle (pinning it) and against the FP32 product kernels.

The reference computes in FP64, the product in FP32: the FP32 error against
the reference is reported as a function of the number of steps and bounded
by the tolerance stated in each test."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import refgpu as R
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import ops
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.solver import Monodomain

from gpu_util import dev, host, max_abs, rel_l2, smooth_state, tips_match

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.available(),
                                 reason="reference cubin not built (oracle/ref_build.sh)")]


def ref_run(p, st, steps, solid=None):
    import torch
    a = [dev(x, torch.float64) for x in st]
    b = [torch.zeros_like(a[0]) for _ in range(2)]
    J = [torch.zeros_like(a[0]) for _ in range(2)]
    vt = [torch.zeros_like(a[0]) for _ in range(2)]
    sol = None if solid is None else dev(solid, torch.uint8)
    R.set_params(p)
    for _ in range(steps):
        R.rd(p, b, a, J, vt, sol)
        a, b = b, a
    R.sync()
    return [host(t) for t in a], [host(t) for t in vt]


def cross_params(n, L=3.0):
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = L
    p.hx = p.hy = L / (n - 1)
    return A.param_derive(p)


@pytest.mark.parametrize("holes", [False, True])
def test_reference_rd_pins_oracle(holes):
    n = 96
    p = cross_params(n)
    st = list(W.ref2v_cross(n, n))
    solid = None
    if holes:
        p.solidSwitch = True
        solid = W.hole_mask(n, n, 8, 2.0, 4.0, np.random.default_rng(7))
    ref, rt = ref_run(p, st, 300, solid)
    orc = st
    for _ in range(300):
        orc, ot = O.rd_step(p, A.YH_MODEL_REF2V, None, orc, solid=solid, tangent=True)
    assert rel_l2(orc[0], ref[0]) < 1e-12
    assert rel_l2(orc[1], ref[1]) < 1e-12
    assert rel_l2(ot[0], rt[0]) < 1e-10


def test_product_fp32_against_reference_fp64_error_vs_steps():
    """REF2V from the reference's own initial condition: relative L2 error of
    u (FP32 product vs FP64 reference) after N steps."""
    n = 128
    p = cross_params(n)
    st = list(W.ref2v_cross(n, n))
    errs = {}
    for N in (1, 10, 100, 1000):
        ref, _ = ref_run(p, st, N)
        m = Monodomain(p, A.YH_MODEL_REF2V, None)
        m.set_state(*st)
        m.run(N)
        got = m.get_state()
        m.close()
        errs[N] = rel_l2(got[0], ref[0])
    print("REF2V 128^2 rel L2(u) FP32 vs reference FP64:",
          {k: "%.2e" % v for k, v in errs.items()})
    assert errs[1] < 1e-7
    assert errs[100] < 1e-6
    assert errs[1000] < 1e-5


def test_reference_tips_match_product():
    import torch
    nx, ny = 96, 80
    p = A.param_defaults(nx, ny)
    jj, ii = np.mgrid[0:ny, 0:nx]
    x, y = ii - nx / 2 + 0.3, jj - ny / 2 - 0.2
    f = lambda t: (0.5 + 0.5 * np.cos(np.arctan2(y, x) - 0.35 * np.hypot(x, y) - t)).ravel()
    past = f(0.0).astype(np.float32).astype(np.float64)
    present = f(0.3).astype(np.float32).astype(np.float64)
    R.set_params(p)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    plot = torch.zeros(nx * ny, dtype=torch.uint8, device="cuda")
    R.tip(p, dev(past, torch.float64), dev(present, torch.float64), plot, cnt, vec, 1.0)
    R.sync()
    nr = int(cnt.item())
    ref = host(vec)[: 5 * nr].reshape(nr, 5)
    cnt2 = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec2 = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    ops.spiral_tip(p, dev(past), dev(present), cnt2, vec2, 4096, 1.0)
    torch.cuda.synchronize()
    ng = int(cnt2.item())
    got = host(vec2)[: 5 * ng].reshape(ng, 5)
    assert nr >= 1
    assert tips_match(got, ref, 1e-4)


def test_reference_slices_and_trapz_match_product_phase_integrals():
    import torch
    nx, ny = 96, 80
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 25
    st = [x.astype(np.float32).astype(np.float64) for x in smooth_state(nx, ny, 3, 2)]
    tan = [x.astype(np.float32).astype(np.float64) for x in smooth_state(nx, ny, 4, 2)]
    c_adv, phi_adv = (0.011, -0.02, 0.004), (0.0, 0.0, 0.6)
    tip = (41.3, 37.8)
    # reference: Cxy -> slice -> 12 x trapz around tip_vector[count-1]
    R.set_params(p)
    ax = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    ay = torch.zeros_like(ax)
    R.cxy(p, ax, ay, c_adv, phi_adv)
    slc = [torch.zeros_like(ax) for _ in range(6)]
    slc0 = [torch.zeros_like(ax) for _ in range(6)]
    tipv = torch.tensor([tip[0], tip[1], 0, 0, 0], dtype=torch.float32, device="cuda")
    cnt = torch.ones(1, dtype=torch.int32, device="cuda")
    intgl = torch.zeros(nx * ny, dtype=torch.uint8, device="cuda")
    g = [dev(x, torch.float64) for x in st]
    R.slice_(p, g, slc, slc0, ax, ay, intgl, cnt, tipv, 5)
    R.sync()
    Iref = R.integrals(p, slc, slc0, [dev(x, torch.float64) for x in tan], cnt, tipv, 5)
    # product: one fused launch
    s = A.SymState()
    for k in range(3):
        s.c_adv[k], s.phi_adv[k] = c_adv[k], phi_adv[k]
    s.centre[0], s.centre[1] = tip
    s.step = 5
    sym = ops.sym_to_tensor(s)
    ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
    ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
    ops.comoving_field(p, sym, ar, ac)
    ws = torch.zeros(ops.phase_workspace_bytes(nx, ny), dtype=torch.uint8, device="cuda")
    ops.phase_integrals(p, A.YH_MODEL_REF2V, [dev(x) for x in st],
                        [dev(x) for x in tan], ar, ac, sym, ws)
    torch.cuda.synchronize()
    got = np.array(ops.sym_from_bytes(sym).integrals[:])
    assert np.abs(got - Iref).max() <= 2e-6 * np.abs(Iref).max()


def test_reference_bfecc_fixed_point_matches_product():
    import torch
    nx, ny = 64, 52
    p = A.param_defaults(nx, ny)
    p.dt = 0.01
    A.param_derive(p)
    st = [x.astype(np.float32).astype(np.float64) for x in smooth_state(nx, ny, 5, 2)]
    c, phi = (1.3, -0.7, 0.02), (0.0, 0.0, 0.4)
    R.set_params(p)
    ax = torch.zeros(nx * ny, dtype=torch.float64, device="cuda")
    ay = torch.zeros_like(ax)
    R.cxy(p, ax, ay, c, phi)
    gin = [dev(x, torch.float64) for x in st]
    gout = [torch.zeros_like(ax) for _ in range(2)]
    uf = [torch.zeros_like(ax) for _ in range(2)]
    ub = [torch.zeros_like(ax) for _ in range(2)]
    ue = [torch.zeros_like(ax) for _ in range(2)]
    outs = []
    for _ in range(4):
        R.bfecc(p, gout, gin, ax, ay, uf, ub, ue)
        R.sync()
        outs.append(host(gout[0]).copy())
    race = max_abs(outs[0], outs[2])
    print("reference BFECC: single-launch deviation from its fixed point %.2e" % race)
    assert np.array_equal(outs[2], outs[3])  # fixed point reached
    s = A.SymState()
    for k in range(3):
        s.c_adv[k], s.phi_adv[k] = c[k], phi[k]
    sym = ops.sym_to_tensor(s)
    ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
    ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
    arf = torch.zeros(ny, device="cuda")
    acf = torch.zeros(nx, device="cuda")
    ops.comoving_field(p, sym, ar, ac, arf, acf)
    inp = [dev(x) for x in st]
    out = [torch.zeros_like(inp[0]) for _ in range(2)]
    sf = [torch.zeros_like(inp[0]) for _ in range(2)]
    se = [torch.zeros_like(inp[0]) for _ in range(2)]
    ops.advect_bfecc(p, A.YH_MODEL_REF2V, out, inp, arf, acf, sf, se)
    torch.cuda.synchronize()
    assert max_abs(host(out[0]), outs[3]) < 2e-6
    assert max_abs(host(out[1]), host(gout[1])) < 2e-6


def test_reference_long_run_and_tip_trajectory():
    """REF2V, the reference's model, from its own cross-field initial
    condition (main.cu:604-618) on 256^2 for 20,000 steps: the FP32 product
    (solver handle) against the reference's own FP64 kernels run headless,
    rel L2(u) after N steps, and the plain-mode tip sets every sampleIt =
    40 steps (main.cu:156,961-964; the reference's spiralTip_kernel on its
    own two u levels) within 0.1 cell. The reference kernel is also run on
    the product's own two u levels (FP32 values, widened exactly): there
    the tip sets must be equal, so any difference of the trajectories
    comes from the states, not from the tip detection."""
    import torch
    from scipy.optimize import linear_sum_assignment
    n, nsteps, every = 256, 20000, 40
    marks = (1000, 5000, 10000, 20000)
    p = cross_params(n)
    st = list(W.ref2v_cross(n, n))
    a = [dev(x, torch.float64) for x in st]
    b = [torch.zeros_like(a[0]) for _ in range(2)]
    J = [torch.zeros_like(a[0]) for _ in range(2)]
    vt = [torch.zeros_like(a[0]) for _ in range(2)]
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    plot = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    R.set_params(p)
    errs, tip_d, ntips, samples_ok, nsamples, matched, extra = {}, 0.0, 0, 0, 0, 0, 0
    same_in, same_tips, same_d = 0, 0, 0.0
    shown = 0

    def match(x, y):
        if not len(x) or not len(y):
            return 0, 0.0
        d = np.hypot(x[:, None, 0] - y[None, :, 0], x[:, None, 1] - y[None, :, 1])
        r, c = linear_sum_assignment(d)
        ok = d[r, c] <= 0.1
        return int(ok.sum()), float(d[r, c][ok].max(initial=0.0))
    for step in range(every, nsteps + 1, every):
        for _ in range(every):
            R.rd(p, b, a, J, vt)
            a, b = b, a
        cnt.zero_()
        R.tip(p, b[0], a[0], plot, cnt, vec, p.dt * step)
        R.sync()
        nr = int(cnt.item())
        ref = host(vec)[: 5 * nr].reshape(nr, 5)
        m.run(every - 1)
        prev = m.get_state()[0]
        m.run(1)
        m.track_tips()
        got = m.get_tips()
        # the reference's tip kernel on the product's own levels
        cnt.zero_()
        R.tip(p, dev(prev, torch.float64), dev(m.get_state()[0], torch.float64),
              plot, cnt, vec, p.dt * step)
        R.sync()
        ns = int(cnt.item())
        same = host(vec)[: 5 * ns].reshape(ns, 5)
        ms_, ds_ = match(got, same)
        same_in += ms_ == ns == len(got)
        same_tips += ns
        same_d = max(same_d, ds_)
        nsamples += 1
        ntips += nr
        mk, dd = match(got, ref)
        tip_d = max(tip_d, dd)
        matched += mk
        extra += len(got) - mk
        if mk == nr == len(got):
            samples_ok += 1
        elif shown < 4:
            shown += 1
            print("  N=%d product %s | reference %s" % (
                step, np.round(got[:, :2], 3).tolist(),
                np.round(ref[:, :2], 3).tolist()))
        if step in marks:
            errs[step] = rel_l2(m.get_state()[0], host(a[0]))
    m.close()
    print("REF2V 256^2 FP32 product vs the reference's FP64 kernels: rel L2(u)",
          {k: "%.2e" % v for k, v in errs.items()},
          "; tips: %d of %d samples with equal sets, %d of %d reference tips "
          "matched within 0.1 cell (largest distance %.2e), %d extra; the "
          "reference's tip kernel on the product's levels: %d of %d samples "
          "equal (%d tips, largest distance %.2e)" % (
              samples_ok, nsamples, matched, ntips, tip_d, extra, same_in,
              nsamples, same_tips, same_d))
    assert ntips > 0
    # 1e-5 through 10,000 steps (measured 2e-7 .. 1.2e-6); 2.5e-5 at 20,000
    for k in marks[:3]:
        assert errs[k] < 1e-5, (k, errs[k])
    assert errs[20000] < 1e-4
    # every product tip is one of the reference's, and on the same levels
    # the two tip kernels agree
    assert extra == 0
    assert same_in >= 0.99 * nsamples
