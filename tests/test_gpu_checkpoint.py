"""Checkpoint / resume and the finite check of the solver handle on the GPU.

A resumed run equals the uninterrupted one bit for bit. A checkpoint loads
only into a handle of the same problem. yh_check_finite counts planted NaN
and Inf values. run_checked rolls an unstable run back to its last finite
segment. Every non-finite value comes from the host (planted) or from an
explicit step that is unstable on purpose (rx = 0.8 > 1/4): the kernels
compute on it like on any other value and index nothing with it."""
import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import checkpoint as ck
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.ops import YolohtliError
from yolohtli_gb300.solver import Monodomain

pytestmark = pytest.mark.gpu


def case(nx=96, ny=80, seed=3, dt=0.05):
    rng = np.random.default_rng(seed)
    p = A.fk_tissue_params(nx, ny, dt=dt)
    solid = W.hole_mask(nx, ny, 6, 2.0, 5.0, rng)
    st = [np.zeros(nx * ny, np.float32), np.ones(nx * ny, np.float32),
          np.ones(nx * ny, np.float32)]
    for f in st:
        f[solid == 0] = 0
    stims = [W.stim(30, 0, 0, 8, ny), W.stim(130, 40, 30, 60, 50)]
    return p, A.fk_defaults(), st, solid, stims


def solver(p, fk, st, solid):
    m = Monodomain(p, A.YH_MODEL_FK3V, fk, solid=solid)
    m.set_state(*st)
    return m


def test_resume_equals_the_uninterrupted_run(tmp_path):
    p, fk, st, solid, stims = case()
    path = tmp_path / "s.yhck"
    a = solver(p, fk, st, solid)
    a.run(100, stims)
    a.save_checkpoint(path)
    a.run(100, stims)  # crosses the second stimulus
    want = a.get_state()
    assert a.step_count() == 200
    hd = ck.header(path)
    assert (hd.nx, hd.ny, hd.model, hd.has_mask, hd.step) == (
        p.nx, p.ny, A.YH_MODEL_FK3V, 1, 100)
    # a fresh handle of the same problem, and the same handle rolled back
    b = solver(p, fk, [np.full_like(f, 0.5) for f in st], solid)
    for m in (b, a):
        m.load_checkpoint(path)
        assert m.step_count() == 100
        m.run(100, stims)
        got = m.get_state()
        for x, y in zip(got, want):
            assert x.tobytes() == y.tobytes()
    # the file holds the state the handle had at step 100
    c = solver(p, fk, st, solid)
    c.run(100, stims)
    r = ck.read(path)
    for x, y in zip(r.fields, c.get_state()):
        assert x.tobytes() == y.tobytes()
    assert np.array_equal(r.mask != 0, solid != 0)
    for m in (a, b, c):
        m.close()


def test_load_refuses_another_problem(tmp_path):
    p, fk, st, solid, stims = case()
    path = tmp_path / "s.yhck"
    a = solver(p, fk, st, solid)
    a.run(10, stims)
    a.save_checkpoint(path)
    before = a.get_state()
    others = []
    q = A.fk_tissue_params(p.nx, p.ny, dt=0.04)                # other dt
    others.append(Monodomain(q, A.YH_MODEL_FK3V, fk, solid=solid))
    fk2 = A.fk_defaults()
    fk2.tau_d = 0.35                                           # other FK3V
    others.append(Monodomain(p, A.YH_MODEL_FK3V, fk2, solid=solid))
    s2 = solid.copy()
    s2[5] = 1 - s2[5]                                          # other mask
    others.append(Monodomain(p, A.YH_MODEL_FK3V, fk, solid=s2))
    others.append(Monodomain(p, A.YH_MODEL_FK3V, fk))          # no mask
    r = A.fk_tissue_params(p.nx + 4, p.ny)                     # other grid
    others.append(Monodomain(r, A.YH_MODEL_FK3V, fk))
    for m in others:
        with pytest.raises(YolohtliError) as e:
            m.load_checkpoint(path)
        assert e.value.status == A.YH_EINVAL
        assert m.step_count() == 0
        m.close()
    # a corrupt file leaves the handle as it was
    raw = bytearray(path.read_bytes())
    raw[-7] ^= 0x40
    bad = tmp_path / "bad.yhck"
    bad.write_bytes(bytes(raw))
    with pytest.raises(YolohtliError) as e:
        a.load_checkpoint(bad)
    assert e.value.status == A.YH_ECORRUPT
    assert a.step_count() == 10
    for x, y in zip(a.get_state(), before):
        assert x.tobytes() == y.tobytes()
    a.close()


def test_check_finite_counts_planted_values():
    p, fk, st, solid, stims = case()
    m = solver(p, fk, st, solid)
    assert m.check_finite() == 0
    u, v, w = [f.copy() for f in st]
    nx = p.nx
    # a tissue cell away from the edges whose row neighbours k-1..k+2 and
    # column neighbours are tissue too
    k = next(int(c) for c in np.flatnonzero(solid)
             if 2 <= c % nx < nx - 3 and nx <= c < solid.size - nx and
             all(solid[c + d] for d in (-1, 1, 2, -nx, nx)))
    u[k] = np.inf
    w[k + 1] = np.nan
    v[k + 2] = -np.inf
    m.set_state(u, v, w)
    assert m.check_finite() == 3
    m.run(1)  # the stencil carries them to the neighbours
    assert m.check_finite() > 3
    m.set_state(*st)
    assert m.check_finite() == 0
    m.close()


def test_run_checked_rolls_back_to_the_last_finite_segment():
    # rx = ry = 0.8: the explicit step is unstable. The rest state stays
    # exactly uniform (mirror boundaries, no holes) until the stimulus at
    # step 120 seeds the unstable mode; the oracle of the same run is
    # finite at step 100 and not at step 150.
    nx, ny = 96, 80
    p = A.fk_tissue_params(nx, ny, dt=0.5)
    fk = A.fk_defaults()
    st = [np.zeros(nx * ny, np.float32), np.ones(nx * ny, np.float32),
          np.ones(nx * ny, np.float32)]
    stims = [W.stim(120, 10, 10, 30, 30)]
    m = Monodomain(p, A.YH_MODEL_FK3V, fk)
    m.set_state(*st)
    with pytest.raises(YolohtliError) as e:
        m.run_checked(1000, stims, every=50)
    assert e.value.status == A.YH_ENONFINITE
    assert m.step_count() == 100
    assert m.check_finite() == 0
    ref = Monodomain(p, A.YH_MODEL_FK3V, fk)
    ref.set_state(*st)
    ref.run(100, stims)
    for x, y in zip(m.get_state(), ref.get_state()):
        assert x.tobytes() == y.tobytes()
    # a stable run goes through in whole segments
    q = A.fk_tissue_params(nx, ny)
    s = Monodomain(q, A.YH_MODEL_FK3V, fk)
    s.set_state(*st)
    assert s.run_checked(130, stims, every=50) == 3
    assert s.step_count() == 130 and s.check_finite() == 0
    for h in (m, ref, s):
        h.close()


def _batch_case(seed=5):
    """Three grids of different shapes, D, tau_d, masks and events."""
    rng = np.random.default_rng(seed)
    params, fks, masks, states, stims = [], [], [], [], []
    for k, (nx, ny) in enumerate([(64, 48), (96, 64), (32, 32)]):
        p = A.fk_tissue_params(nx, ny, D=float(rng.uniform(5e-4, 1.5e-3)))
        fk = A.fk_defaults()
        fk.tau_d *= float(rng.uniform(0.8, 1.2))
        solid = None if k == 1 else W.hole_mask(nx, ny, 3, 2.0, 4.0, rng)
        st = [np.zeros(nx * ny, np.float32), np.ones(nx * ny, np.float32),
              np.ones(nx * ny, np.float32)]
        if solid is not None:
            for f in st:
                f[solid == 0] = 0
        params.append(p)
        fks.append(fk)
        masks.append(solid)
        states.append(st)
        stims += [(k, W.stim(20 + 10 * k, 0, 0, nx // 2, ny // 2)),
                  (k, W.stim(90 + 5 * k, nx // 3, ny // 3, nx // 3 + 8,
                             ny // 3 + 6))]
    return params, fks, masks, states, stims


def _make_batch(params, fks, masks, states):
    from yolohtli_gb300.batch import Batch
    b = Batch(params, fks, masks)
    for k, st in enumerate(states):
        b.set_state(k, *st)
    return b


def test_batch_resume_equals_the_uninterrupted_run(tmp_path):
    params, fks, masks, states, stims = _batch_case()
    d = tmp_path / "batch"
    a = _make_batch(params, fks, masks, states)
    a.run(60, stims)
    a.save_checkpoint(d)
    a.run(60, stims)  # crosses every instance's second event
    want = [a.get_state(k) for k in range(3)]
    half = [[np.full_like(f, 0.5) for f in st] for st in states]
    b = _make_batch(params, fks, masks, half)
    b.load_checkpoint(d)
    assert b.step_count() == 60
    b.run(60, stims)
    for k in range(3):
        for x, y in zip(b.get_state(k), want[k]):
            assert x.tobytes() == y.tobytes()
    # another problem (instance 2's tau_d) is refused and changes nothing
    fks2 = [A.FKParams.from_buffer_copy(f) for f in fks]
    fks2[2].tau_d *= 1.1
    c = _make_batch(params, fks2, masks, states)
    with pytest.raises(YolohtliError) as e:
        c.load_checkpoint(d)
    assert e.value.status == A.YH_EINVAL
    assert c.step_count() == 0
    for k in range(3):
        for x, y in zip(c.get_state(k), states[k]):
            assert x.tobytes() == y.tobytes()
    # a corrupt file is reported and changes nothing
    f1 = d / "instance_0001.yhck"
    raw = bytearray(f1.read_bytes())
    raw[-1] ^= 1
    f1.write_bytes(bytes(raw))
    with pytest.raises(YolohtliError) as e:
        b.load_checkpoint(d)
    assert e.value.status == A.YH_ECORRUPT
    assert b.step_count() == 120
    for h in (a, b, c):
        h.close()
