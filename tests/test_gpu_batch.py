"""The batched solver (yh_batch_*): many independent FK3V grids, each with
its own size, parameters, hole mask and stimulus events, one launch per
step for the whole batch. Every instance must come out bit for bit as the
single-grid solver leaves the same grid (the cell update is the same code),
and within the FP32 budget of the FP64 oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.batch import Batch
from yolohtli_gb300.ops import YolohtliError
from yolohtli_gb300.solver import Monodomain

from gpu_util import rel_l2

pytestmark = pytest.mark.gpu


def _instances(seed=3):
    """Five grids of different shapes, D, time constants, holes and events."""
    rng = np.random.default_rng(seed)
    shapes = [(64, 48), (96, 96), (128, 80), (32, 32), (160, 64)]
    out = []
    for k, (nx, ny) in enumerate(shapes):
        D = float(rng.uniform(5e-4, 1.5e-3))
        p = A.fk_tissue_params(nx, ny, D=D)
        fk = A.fk_defaults()
        for name in W.TAU_NAMES:
            setattr(fk, name, getattr(fk, name) * float(rng.uniform(0.8, 1.2)))
        u, v, w = W._ic(nx, ny, rng)
        solid = None
        if k % 2 == 0:
            solid = W.hole_mask(nx, ny, 3 + k, 2.0, 5.0, rng)
            p.solidSwitch = True
            for f in (u, v, w):
                f[solid == 0] = 0.0
        stims = [W.stim(40 + 37 * k, 0, 0, nx // 2, ny // 2),
                 W.stim(120 + 11 * k, nx // 3, ny // 3, nx // 3 + 9, ny // 3 + 7, 0.8)]
        if k == 1:  # two events on one step: the later one wins where both apply
            stims.append(W.stim(200, 5, 5, 40, 40, 1.0))
            stims.append(W.stim(200, 20, 20, 60, 60, 0.3))
        out.append(W.Workload("b%d" % k, p, fk, A.YH_MODEL_FK3V, u, v, w,
                              solid, stims, 0))
    return out


def _single(wl, runs):
    m = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid)
    m.set_engine(A.YH_ENGINE_STEP, 1)
    m.set_state(*wl.state0())
    for n in runs:
        m.run(n, wl.stims)
    out = m.get_state()
    m.close()
    return out


def _batch(insts, runs):
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    for k, w in enumerate(insts):
        b.set_state(k, *w.state0())
    ev = [(k, s) for k, w in enumerate(insts) for s in w.stims]
    for n in runs:
        b.run(n, ev)
    b.synchronize()
    return b


def test_batch_equals_the_single_grid_solver_bitwise():
    insts = _instances()
    runs = [130, 170]  # a graph of 64 steps, direct launches, events in both
    b = _batch(insts, runs)
    assert b.step_count() == sum(runs)
    assert b.launch_count() == sum(runs)
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = _single(wl, runs)
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (k, f)
    b.close()


@pytest.mark.parametrize("depth", [1, 2])
@pytest.mark.parametrize("schedule", [(1 << 12, 3), (1, 4), (1 << 30, 1),
                                      (0, 3), (0, 8)])
def test_every_schedule_gives_the_same_bits(schedule, depth):
    # groups of one instance up to one group for all, on 1-4 streams, one or
    # two steps per launch (depth 2: TMA-staged 64 x 16 tiles; runs of odd
    # length and events on either step of a launch, including two events
    # on one step); group_cells 0: every instance its own sequence of
    # single-grid step launches (events by the stimulus kernel)
    insts = _instances()
    runs = [130, 170]
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    b.set_schedule(*schedule)
    b.set_depth(depth)
    for k, w in enumerate(insts):
        b.set_state(k, *w.state0())
    ev = [(k, st) for k, w in enumerate(insts) for st in w.stims]
    for n in runs:
        b.run(n, ev)
    b.synchronize()
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = _single(wl, runs)
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (schedule, k, f)
    b.close()


def _ragged_instances(seed=7, shapes=((36, 40), (100, 52), (44, 70), (52, 5),
                                      (100, 130))):
    """Widths that split unevenly into bands of quads (nx / 4 = 9, 25, 11,
    13) and are no multiple of 16, heights from 5 rows up, holes in two,
    events on both runs (one on the first step of a run, two on one step)."""
    rng = np.random.default_rng(seed)
    out = []
    for k, (nx, ny) in enumerate(shapes):
        p = A.fk_tissue_params(nx, ny, D=float(rng.uniform(5e-4, 1.5e-3)))
        fk = A.fk_defaults()
        u, v, w = W._ic(nx, ny, rng)
        solid = None
        if k in (1, 4):
            solid = W.hole_mask(nx, ny, 4 + k, 2.0, 5.0, rng)
            p.solidSwitch = True
            for f in (u, v, w):
                f[solid == 0] = 0.0
        stims = [W.stim(13 + 29 * k, 0, 0, nx // 2, max(ny // 2, 1)),
                 W.stim(130, nx // 3, 0, nx // 3 + 9, ny, 0.7)]
        if k == 2:
            stims.append(W.stim(211, 2, 2, 30, 30, 1.0))
            stims.append(W.stim(211, 10, 10, 40, 60, 0.4))
        out.append(W.Workload("r%d" % k, p, fk, A.YH_MODEL_FK3V, u, v, w,
                              solid, stims, 0))
    return out


@pytest.mark.parametrize("cluster,levels", [(1, 0), (2, 0), (4, 0), (1, 1),
                                            (2, 2), (4, 3), (2, 5), (1, 7)])
@pytest.mark.parametrize("which", ["mixed", "ragged"])
def test_wavefront_engine_gives_the_same_bits(cluster, levels, which):
    # one persistent launch per run: 1, 2 or 4 CTAs per instance (bands of
    # unequal width, neighbour columns through distributed shared memory),
    # passes of 1-7 steps or as many as the rings allow (a short last pass),
    # events on any level of a pass, mirror edges and holes
    insts = _instances() if which == "mixed" else _ragged_instances()
    runs = [130, 170]
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    b.set_wave(cluster, levels)
    cl, kcap, nclusters = b.wave()
    assert cl == cluster and kcap == levels and nclusters >= 1
    for k, w in enumerate(insts):
        b.set_state(k, *w.state0())
    ev = [(k, st) for k, w in enumerate(insts) for st in w.stims]
    for n in runs:
        b.run(n, ev)
    b.synchronize()
    assert b.launch_count() == len(runs)  # one launch per run
    assert b.step_count() == sum(runs)
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = _single(wl, runs)
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (cluster, levels, k, f)
    b.close()


@pytest.mark.parametrize("depth", [1, 2])
def test_per_instance_schedule_on_ragged_grids(depth):
    # every instance its own launch sequence (depth 2: the two-step
    # kernel; widths with and without 16-byte rows of hole codes), events
    # cutting the runs at odd and even steps: the same bits as single grids
    # (depth 2 needs 16-byte rows of hole codes: the grids with holes are
    # 96 and 112 wide there)
    insts = _ragged_instances() if depth == 1 else _ragged_instances(
        shapes=((36, 40), (96, 52), (44, 70), (52, 5), (112, 130)))
    runs = [131, 70, 99]
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    b.set_schedule(0, 3)
    b.set_depth(depth)
    for k, w in enumerate(insts):
        b.set_state(k, *w.state0())
    ev = [(k, st) for k, w in enumerate(insts) for st in w.stims]
    for n in runs:
        b.run(n, ev)
    b.synchronize()
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = _single(wl, runs)
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (depth, k, f)
    b.close()


@pytest.mark.parametrize("schedule", ["instance", "grouped", "wave"])
def test_run_host_copies_in_and_out(schedule):
    # states from host memory in, results out, one call: under every
    # schedule the same bits as set_state + run + get_state; five events of
    # one instance inside the run make two segments (copies in before the
    # first, out after the last)
    insts = _instances()
    insts[3].stims = [W.stim(10 + 9 * q, q, q, q + 10, q + 12, 1.0 - 0.1 * q)
                      for q in range(7)]
    ev = [(k, st) for k, w in enumerate(insts) for st in w.stims]
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    if schedule == "instance":
        b.set_schedule(0, 3)
        b.set_depth(2)
    elif schedule == "wave":
        b.set_wave(2, 5)
    b.run(20, ev)  # some other state in the batch first
    states = [tuple(np.ascontiguousarray(x) for x in w.state0()) for w in insts]
    outs = [tuple(np.empty(w.cells, np.float32) for _ in range(3)) for w in insts]
    outs[2] = (outs[2][0], None, outs[2][2])  # a field not copied out
    step0 = b.step_count()
    b.run_host(101, states, outs, ev)
    assert b.step_count() == step0 + 101
    for k, wl in enumerate(insts):
        m = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid)
        m.set_engine(A.YH_ENGINE_STEP, 1)
        m.set_state(*wl.state0())
        m.set_step(step0)
        m.run(101, wl.stims)
        ref = m.get_state()
        m.close()
        got = b.get_state(k)
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (schedule, k, f)
            if outs[k][f] is not None:
                assert np.array_equal(outs[k][f], ref[f]), (schedule, k, f)
    b.close()


def test_wavefront_engine_segments_and_switches_back():
    # 7 events of one instance split the run into segments (a launch each);
    # the grouped launches and the wavefront engine continue each other's
    # state
    wl = _instances()[3]
    wl.stims = [W.stim(10 + 9 * q, q, q, q + 10, q + 12, 1.0 - 0.1 * q)
                for q in range(7)]
    b = Batch([wl.p], [wl.fk], [wl.solid])
    b.set_wave(2)
    b.set_state(0, *wl.state0())
    b.run(60, [(0, s) for s in wl.stims])
    b.set_depth(1)
    assert b.wave()[0] == 0
    b.run(41, [(0, s) for s in wl.stims])
    b.set_wave(4, 6)
    b.run(33, [(0, s) for s in wl.stims])
    b.synchronize()
    got = b.get_state(0)
    ref = _single(wl, [60, 41, 33])
    for f in range(3):
        assert np.array_equal(got[f], ref[f]), f
    with pytest.raises(YolohtliError) as e:
        b.set_wave(3)
    assert e.value.status == A.YH_EINVAL
    b.close()
    narrow = A.fk_tissue_params(12, 16)  # 3 quads: no band for a 4th CTA
    b = Batch([narrow], [A.fk_defaults()])
    with pytest.raises(YolohtliError) as e:
        b.set_wave(4)
    assert e.value.status == A.YH_EUNSUPPORTED
    b.set_wave(2)
    b.close()


def test_wavefront_engine_on_the_benchmark_batch():
    """fk_batch_256 (all 256 instances, holes, per-instance D and time
    constants, the S2 moved inside the run) for 300 steps with the wavefront
    engine at 2 CTAs per instance: every 16th instance and the largest ones
    equal bit for bit to their single-grid solvers."""
    bw = W.fk_batch_256(nsteps=300)
    for w in bw.instances:
        for s in w.stims:
            s.step = 37 + s.step % 250
    b = Batch([w.p for w in bw.instances], [w.fk for w in bw.instances],
              [w.solid for w in bw.instances])
    b.set_wave(2)
    for k, w in enumerate(bw.instances):
        b.set_state(k, *w.state0())
    b.run(bw.nsteps, bw.stims())
    b.synchronize()
    assert b.launch_count() == 1
    big = sorted(range(len(bw.instances)), key=lambda k: -bw.instances[k].cells)[:3]
    for k in sorted(set(range(0, len(bw.instances), 16)) | set(big)):
        got = b.get_state(k)
        ref = _single(bw.instances[k], [bw.nsteps])
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (k, f)
    b.close()


def test_autotune_restores_the_state_and_keeps_the_bits():
    insts = _instances(seed=5)
    b = Batch([w.p for w in insts], [w.fk for w in insts],
              [w.solid for w in insts])
    for k, w in enumerate(insts):
        b.set_state(k, *w.state0())
    ev = [(k, st) for k, w in enumerate(insts) for st in w.stims]
    b.run(100, ev)
    b.synchronize()
    before = [b.get_state(k) for k in range(len(insts))]
    launches = b.launch_count()
    g, q, d = b.autotune(64)
    if d == 0:  # the wavefront engine, q CTAs per instance
        assert g == 0 and q in (1, 2, 4) and b.wave()[0] == q
    elif g == 0:  # one launch sequence per instance on q streams
        assert q in (6, 8, 12) and d in (1, 2) and b.wave()[0] == 0
    else:
        assert g in (1 << 18, 1 << 19, 1 << 20, 1 << 21) and q in (2, 3, 4)
        assert d in (1, 2) and b.wave()[0] == 0
    assert b.step_count() == 100 and b.launch_count() == launches
    for k in range(len(insts)):
        now = b.get_state(k)
        for f in range(3):
            assert np.array_equal(now[f], before[k][f]), (k, f)
    b.run(70, ev)
    b.synchronize()
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = _single(wl, [100, 70])
        for f in range(3):
            assert np.array_equal(got[f], ref[f]), (k, f)
    b.close()


def test_batch_against_the_fp64_oracle():
    insts = _instances(seed=11)[:3]
    nsteps = 200
    b = _batch(insts, [nsteps])
    for k, wl in enumerate(insts):
        got = b.get_state(k)
        ref = O.run(wl.p, wl.model, wl.fk, wl.state0(), nsteps, wl.stims,
                    wl.solid, dtype=np.float64)
        assert rel_l2(got[0], ref[0]) < 1e-5, k
    b.close()


def test_more_events_than_one_segment_holds():
    # 7 events on distinct steps for one instance: the run is split into
    # segments of at most 4 events per instance
    wl = _instances()[3]
    wl.stims = [W.stim(10 + 9 * q, q, q, q + 10, q + 12, 1.0 - 0.1 * q)
                for q in range(7)]
    b = _batch([wl], [100])
    got = b.get_state(0)
    ref = _single(wl, [100])
    for f in range(3):
        assert np.array_equal(got[f], ref[f])
    b.close()


def test_invalid_batches_are_rejected():
    p = A.fk_tissue_params(30, 32)  # nx % 4 != 0
    with pytest.raises(YolohtliError) as e:
        Batch([p], [A.fk_defaults()])
    assert e.value.status == A.YH_EUNSUPPORTED
    wl = _instances()[3]
    b = Batch([wl.p], [wl.fk])
    crowded = [(0, W.stim(5, 0, 0, 4, 4)) for _ in range(5)]  # 5 on one step
    with pytest.raises(YolohtliError) as e:
        b.run(10, crowded)
    assert e.value.status == A.YH_EOVERFLOW
    with pytest.raises(YolohtliError) as e:
        b.run(10, [(1, W.stim(5, 0, 0, 4, 4))])  # no instance 1
    assert e.value.status == A.YH_EINVAL
    b.close()


def test_config_sized_batch_matches_the_oracle():
    """The benchmark's batch (fk_batch_256, all 256 instances, per-instance
    D, time constants, holes and S2 time), 400 steps under the autotuned
    schedule: every instance equal bit for bit to its single-grid solver,
    and 8 instances (the smallest, the largest and six between) within
    1e-5 rel L2(u) of the FP64 oracle, or, where an S2 upstroke is under
    way at step 400, within twice what the oracle's own FP32 transcription
    of the step reaches against the FP64 oracle (the FK3V switches turn
    FP32 rounding into 1e-5 .. 4e-5 there: measured 1.4e-5 at 288^2, 3.4e-5
    at 704^2 with the S2 at steps 333 and 340)."""
    bw = W.fk_batch_256(nsteps=400)
    for w in bw.instances:
        for s in w.stims:
            s.step = s.step % 350  # the S2 inside the 400 steps
    b = Batch([w.p for w in bw.instances], [w.fk for w in bw.instances],
              [w.solid for w in bw.instances])
    for k, w in enumerate(bw.instances):
        b.set_state(k, *w.state0())
    b.autotune(64)
    for k, w in enumerate(bw.instances):
        b.set_state(k, *w.state0())
    b.run(bw.nsteps, bw.stims())
    order = sorted(range(len(bw.instances)), key=lambda k: bw.instances[k].cells)
    pick = [order[int(q)] for q in np.linspace(0, len(order) - 1, 8)]
    worst = 0.0
    for k in range(len(bw.instances)):
        got = b.get_state(k)
        if k in pick or k % 32 == 0:
            ref = _single(bw.instances[k], [400])
            for f in range(3):
                assert np.array_equal(got[f], ref[f]), (k, f)
        if k in pick:
            w = bw.instances[k]
            orc = O.run(w.p, w.model, w.fk, w.state0(), 400, w.stims,
                        solid=w.solid)
            o32 = O.run(w.p, w.model, w.fk, w.state0(), 400, w.stims,
                        solid=w.solid, dtype=np.float32)
            m = np.ones(w.cells, bool) if w.solid is None else w.solid != 0
            e = rel_l2(got[0][m], orc[0][m])
            e32 = rel_l2(o32[0][m], orc[0][m])
            print("instance %d (%d^2): rel L2(u) against the FP64 oracle %.2e "
                  "(FP32 transcription %.2e)" % (k, w.p.nx, e, e32))
            worst = max(worst, e)
            assert e < max(1e-5, 2.0 * e32), (k, w.p.nx, e, e32)
    print("batch of 256, 400 steps: largest rel L2(u) against the FP64 oracle "
          "over 8 instances %.2e" % worst)
    b.close()
