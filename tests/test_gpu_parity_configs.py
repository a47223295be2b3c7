"""Parity at the benchmark configurations, over whole runs.

Config 0: FK3V spiral protocol on 256^2, 10,000 steps (S1 columns 0-9 at
t = 0, S2 on the lower-left quadrant at 320 ms). Config 1: 1024^2 with 300
holes and 12 S2 patches, 20,000 steps. Each run is compared with the FP64
oracle at several step counts N (relative L2 of u over tissue cells, and
max |du|), and the plain-mode tip sets are compared at the reference's
sampling period (param.sample = 2 ms, saveFiles.cu:201; every sampleIt =
40 steps, main.cu:156,961-964) within 0.1 cell.

Two runs per config:
  fp64 - this library's step and tip kernels instantiated in FP64
         (yh_reaction_diffusion_f64, yh_spiral_tip_f64). Against the FP64
         oracle this isolates the discrete map: 1e-17 .. 1e-14 relative
         for the first 1,000 steps.
  fp32 - the product (the solver handle, autotuned engine): 6e-8 .. 9e-8
         for the first 100 steps.
Past that the FK3V map amplifies any difference of the state by orders of
magnitude per thousand steps while fronts move (a 1e-10 change of the FP64
initial state exceeds 1e-6 by step 2,000:
tests/test_oracle.py::test_fk3v_switch_sensitivity), so FP32 rounding
reaches 1e-4 .. 1e-3 and even two FP64 evaluation orders part by 1e-4 in
the fibrillation-like config 1 at N = 10,000. The tests assert the
measured curves with a margin and print the tables.
"""
import numpy as np
import pytest

from oracle import oracle as O
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import ops
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.solver import Monodomain

pytestmark = pytest.mark.gpu

SAMPLE_IT = 40  # round(param.sample / dt) = round(2 ms / 0.05 ms)


def tissue(wl):
    return np.ones(wl.cells, bool) if wl.solid is None else wl.solid != 0


def errs(got, want, mask):
    d = np.asarray(got, np.float64)[mask] - np.asarray(want, np.float64)[mask]
    w = np.asarray(want, np.float64)[mask]
    return float(np.linalg.norm(d) / max(np.linalg.norm(w), 1e-300)), \
        float(np.abs(d).max())


def tip_distance(a, b):
    """Largest distance between matched tips of two sets (inf when the
    counts differ; 0 for two empty sets)."""
    if len(a) != len(b):
        return np.inf
    if len(a) == 0:
        return 0.0
    from scipy.optimize import linear_sum_assignment
    d = np.hypot(a[:, None, 0] - b[None, :, 0], a[:, None, 1] - b[None, :, 1])
    r, c = linear_sum_assignment(d)
    return float(d[r, c].max())


def run_oracle(wl, marks, tips_until):
    """FP64 oracle: u at each mark, tip sets every SAMPLE_IT steps up to
    tips_until."""
    st = [x.astype(np.float64) for x in wl.state0()]
    step, us, tips = 0, {}, {}
    stops = sorted(set(marks) | set(range(SAMPLE_IT, tips_until + 1, SAMPLE_IT)))
    for m in stops:
        if m % SAMPLE_IT == 0 and m <= tips_until:
            st = O.run(wl.p, wl.model, wl.fk, st, m - 1 - step, wl.stims,
                       solid=wl.solid, step0=step)
            past = st[0].copy()
            st = O.run(wl.p, wl.model, wl.fk, st, 1, wl.stims, solid=wl.solid,
                       step0=m - 1)
            tips[m] = O.tips(wl.p, past, st[0], solid=wl.solid)
        else:
            st = O.run(wl.p, wl.model, wl.fk, st, m - step, wl.stims,
                       solid=wl.solid, step0=step)
        step = m
        if m in marks:
            us[m] = st[0].copy()
    return us, tips


def run_fp64(wl, marks, tips_until):
    """The FP64 instances of the step, stimulus and tip kernels."""
    import torch
    dev = lambda x: torch.tensor(np.asarray(x, np.float64), device="cuda")
    cur = [dev(x) for x in wl.state0()]
    nxt = [torch.zeros_like(cur[0]) for _ in range(3)]
    solid = None if wl.solid is None else torch.tensor(wl.solid, device="cuda")
    cap = 1 << 14
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * cap, dtype=torch.float32, device="cuda")
    ev = sorted(wl.stims, key=lambda s: s.step)
    us, tips = {}, {}
    k = 0
    for step in range(max(marks)):
        while k < len(ev) and ev[k].step == step:
            s = ev[k]
            ops.stimulate_box_f64(wl.p, cur[0], s.i0, s.j0, s.i1, s.j1, s.value,
                                  solid)
            k += 1
        ops.reaction_diffusion_f64(wl.p, wl.model, wl.fk, nxt, cur,
                                   solid=solid)
        cur, nxt = nxt, cur
        n = step + 1
        if n % SAMPLE_IT == 0 and n <= tips_until:
            ops.spiral_tip_f64(wl.p, nxt[0], cur[0], cnt, vec, cap,
                               wl.p.dt * n, solid)
            m = int(cnt.item())
            assert m <= cap
            tips[n] = vec[:5 * m].cpu().numpy().reshape(m, 5)
        if n in marks:
            us[n] = cur[0].cpu().numpy()
    return us, tips


def run_fp32(wl, marks, tips_until):
    """The product: the solver handle, autotuned engine, tips between the
    last two u levels (yh_track_tips) every SAMPLE_IT steps."""
    m = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid)
    m.set_state(*wl.state0())
    engine = m.autotune(256)
    us, tips = {}, {}
    stops = sorted(set(marks) | set(range(SAMPLE_IT, tips_until + 1, SAMPLE_IT)))
    for s in stops:
        m.run(s - m.step_count(), wl.stims)
        if s % SAMPLE_IT == 0 and s <= tips_until:
            m.track_tips()
            tips[s] = m.get_tips()
        if s in marks:
            us[s] = m.get_state()[0]
    m.close()
    return us, tips, engine


def tip_match(a, b, tol=0.1):
    """Tips of set a within tol of a distinct tip of set b (an optimal
    one-to-one assignment): (matched, len(a), len(b))."""
    if len(a) == 0 or len(b) == 0:
        return 0, len(a), len(b)
    from scipy.optimize import linear_sum_assignment
    d = np.hypot(a[:, None, 0] - b[None, :, 0], a[:, None, 1] - b[None, :, 1])
    r, c = linear_sum_assignment(d)
    return int((d[r, c] <= tol).sum()), len(a), len(b)


def table(name, wl, marks, ref, runs):
    """Prints and returns, per run: rel L2(u) / max |du| at the marks, and
    the tip comparison with the oracle's tip sets: samples whose sets match
    within 0.1 cell, and oracle tips with a partner within 0.1 cell."""
    mask = tissue(wl)
    rows = {}
    print("\n%s: rel L2(u) over tissue / max |du| against the FP64 oracle" % name)
    for label, (us, _) in runs.items():
        rows[label] = [errs(us[n], ref[0][n], mask) for n in marks]
        print("  %-5s " % label + "  ".join(
            "N=%d %.2e/%.2e" % (n, r, a) for n, (r, a) in zip(marks, rows[label])))
    samples = sorted(ref[1])
    for label, (_, tips) in runs.items():
        d = np.array([tip_distance(tips[n], ref[1][n]) for n in samples])
        ok = d <= 0.1
        m = np.array([tip_match(ref[1][n], tips[n]) for n in samples])
        matched, ntips = int(m[:, 0].sum()), int(m[:, 1].sum())
        first_bad = next((n for n, g in zip(samples, ok) if not g), None)
        print("  %-5s tips: %d of %d samples with the same set within 0.1 "
              "cell (first other at N=%s); %d of %d oracle tips matched "
              "within 0.1 cell, %d extra tips" % (
                  label, int(ok.sum()), len(d), first_bad, matched, ntips,
                  int(m[:, 2].sum()) - matched))
        for n, g in list(zip(samples, ok))[:]:
            if not g:
                print("    N=%d %s: %s | oracle: %s" % (
                    n, label, np.round(tips[n][:, :2], 4).tolist(),
                    np.round(ref[1][n][:, :2], 4).tolist()))
        rows[label + "_tips"] = dict(samples_ok=int(ok.sum()), samples=len(d),
                                     matched=matched, oracle_tips=ntips,
                                     first_other=first_bad)
    return rows


def test_config0_spiral_256_error_vs_steps():
    wl = W.fk_spiral_256()
    marks = [10, 100, 1000, 5000, 10000]
    ref = run_oracle(wl, marks, wl.nsteps)
    f64 = run_fp64(wl, marks, wl.nsteps)
    f32 = run_fp32(wl, marks, wl.nsteps)
    rows = table("config 0 (FK3V 256^2, 10,000 steps)", wl, marks, ref,
                 {"fp64": f64, "fp32": f32[:2]})
    # the discrete map: the FP64 kernels stay on the FP64 oracle (measured
    # 1e-17 .. 1.2e-8); every tip set but the ones at the S2 onset, where
    # the two u levels' isolines are nearly parallel and a tip's position
    # is ill-conditioned, matches within 0.1 cell
    r64 = [r for r, _ in rows["fp64"]]
    assert max(r64[:3]) <= 1e-12 and max(r64) <= 1e-6
    t64 = rows["fp64_tips"]
    assert t64["samples_ok"] >= 0.99 * t64["samples"]
    # FP32: 6e-8 .. 9e-8 for the first 100 steps; 2e-4 .. 2e-3 once fronts
    # have crossed the tissue (the measured curve, with a margin)
    r32 = [r for r, _ in rows["fp32"]]
    assert r32[0] <= 2e-7 and r32[1] <= 2e-7
    assert max(r32) <= 1e-2
    t32 = rows["fp32_tips"]
    assert t32["samples_ok"] >= 0.98 * t32["samples"]


def test_config1_holes_1024_error_vs_steps():
    wl = W.fk_holes_1024()
    marks = [10, 100, 1000, 10000, 20000]
    tips_until = wl.nsteps
    ref = run_oracle(wl, marks, tips_until)
    f64 = run_fp64(wl, marks, tips_until)
    f32 = run_fp32(wl, marks, tips_until)
    rows = table("config 1 (FK3V 1024^2, 300 holes, 12 patches, 20,000 steps)",
                 wl, marks, ref, {"fp64": f64, "fp32": f32[:2]})
    # FP64 kernels: 1e-17 .. 1e-14 to N = 1000; in the fibrillation-like
    # state at N = 10,000 the map's sensitivity has grown the rounding
    # difference of two FP64 evaluation orders (the device contracts
    # products into FMAs, the oracle does not) to ~1.5e-4, as it grows a
    # 1e-15 perturbation of the oracle's own initial state; the final,
    # quiescent state agrees again (3.7e-10)
    r64 = [r for r, _ in rows["fp64"]]
    assert max(r64[:3]) <= 1e-12
    assert r64[3] <= 1e-3 and r64[4] <= 1e-6
    t64 = rows["fp64_tips"]
    assert t64["matched"] >= 0.99 * t64["oracle_tips"]
    r32 = [r for r, _ in rows["fp32"]]
    assert r32[0] <= 2e-7 and r32[1] <= 2e-7
    assert r32[2] <= 1e-3 and r32[3] <= 2e-3 and r32[4] <= 1e-4
    t32 = rows["fp32_tips"]
    assert t32["matched"] >= 0.9 * t32["oracle_tips"]
