"""GPU tests of the resident engine (a whole protocol in one cooperative
launch, state kept in shared memory) against the per-step engine."""
import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import ops
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.solver import Monodomain

from gpu_util import max_abs

pytestmark = pytest.mark.gpu


def case(nx, ny, holes, model=A.YH_MODEL_FK3V, seed=9):
    rng = np.random.default_rng(seed)
    if model == A.YH_MODEL_FK3V:
        p, fk = A.fk_tissue_params(nx, ny), A.fk_defaults()
    else:
        p, fk = A.param_defaults(nx, ny), None
        p.gateDiff = False
    st = [rng.uniform(0, 1, nx * ny).astype(np.float32) for _ in range(A.NFIELDS[model])]
    jj, ii = np.mgrid[0:ny, 0:nx]
    st[0][((ii - nx // 3) ** 2 + (jj - ny // 2) ** 2 < 200).ravel()] = 1.0
    solid = None
    if holes:
        solid = W.hole_mask(nx, ny, max(3, nx * ny // 4000), 2.0, 5.0, rng)
        p.solidSwitch = True
        for f in st:
            f[solid == 0] = 0
    return p, fk, st, solid


def run(p, fk, model, st, solid, nsteps, engine, stims=(), k=1, tips=False):
    m = Monodomain(p, model, fk, solid=solid)
    m.set_state(*st)
    m.set_engine(engine, k)
    m.run(nsteps, stims)
    out = m.get_state()
    t = None
    if tips:
        m.track_tips()
        t = m.get_tips()
    n = m.launch_count()
    m.close()
    return out, t, n


@pytest.mark.parametrize("nx,ny", [(256, 192), (97, 61), (1024, 1024)])
@pytest.mark.parametrize("holes", [False, True])
def test_resident_equals_step_engine(nx, ny, holes):
    p, fk, st, solid = case(nx, ny, holes)
    nsteps = 120
    a, _, _ = run(p, fk, A.YH_MODEL_FK3V, st, solid, nsteps, A.YH_ENGINE_STEP)
    b, _, nl = run(p, fk, A.YH_MODEL_FK3V, st, solid, nsteps, A.YH_ENGINE_RESIDENT)
    assert nl == 1
    for f in range(3):
        d = max_abs(a[f], b[f])
        assert d <= 1e-6, (f, d)


@pytest.mark.parametrize("nx,ny,nholes", [(1024, 1024, 300), (256, 304, 400), (128, 300, 60)])
def test_resident_split_passes_are_bitwise_the_step_engine(nx, ny, nholes):
    # FK3V with holes runs the plain quads and the hole quads in separate
    # passes (the hole quads listed per block, rows 0 and R-1 first): the
    # same bits as the step engine, with holes on the blocks' boundary rows,
    # dense hole masks and stimulus events inside the run
    rng = np.random.default_rng(nholes)
    p, fk = A.fk_tissue_params(nx, ny), A.fk_defaults()
    u, v, w = W._ic(nx, ny, rng)
    solid = W.hole_mask(nx, ny, nholes, 2.0, 7.0, rng)
    p.solidSwitch = True
    for f in (u, v, w):
        f[solid == 0] = 0.0
    stims = [W.stim(17, 0, 0, nx // 2, ny // 2), W.stim(60, nx // 3, 5, nx, ny // 3, 0.6)]
    st = [u, v, w]
    a, _, _ = run(p, fk, A.YH_MODEL_FK3V, st, solid, 150, A.YH_ENGINE_STEP, stims)
    b, _, nl = run(p, fk, A.YH_MODEL_FK3V, st, solid, 150, A.YH_ENGINE_RESIDENT, stims)
    assert nl == 1
    for f in range(3):
        assert np.array_equal(a[f], b[f]), f


def test_resident_ref2v_without_gate_diffusion():
    p, fk, st, solid = case(160, 130, True, model=A.YH_MODEL_REF2V)
    a, _, _ = run(p, fk, A.YH_MODEL_REF2V, st, solid, 200, A.YH_ENGINE_STEP)
    b, _, _ = run(p, fk, A.YH_MODEL_REF2V, st, solid, 200, A.YH_ENGINE_RESIDENT)
    for f in range(2):
        assert max_abs(a[f], b[f]) <= 1e-6


def test_resident_applies_many_stimuli_and_keeps_the_previous_level():
    p, fk, st, solid = case(320, 256, True)
    rng = np.random.default_rng(2)
    stims = [W.stim(int(rng.integers(0, 400)), int(rng.integers(0, 280)),
                    int(rng.integers(0, 220)), 0, 0) for _ in range(45)]
    for s in stims:  # 40 x 30 boxes, more events than one launch takes
        s.i1, s.j1 = s.i0 + 40, s.j0 + 30
    a, ta, _ = run(p, fk, A.YH_MODEL_FK3V, st, solid, 400, A.YH_ENGINE_STEP,
                   stims, tips=True)
    b, tb, nl = run(p, fk, A.YH_MODEL_FK3V, st, solid, 400, A.YH_ENGINE_RESIDENT,
                    stims, tips=True)
    assert nl >= 2  # split into launches of at most 32 events
    for f in range(3):
        assert max_abs(a[f], b[f]) <= 1e-6
    assert len(ta) == len(tb) and (len(ta) == 0 or np.abs(ta[:, :2] - tb[:, :2]).max() < 1e-4)


def test_resident_is_refused_where_it_does_not_apply():
    p = A.param_defaults(128, 128)  # REF2V with gate diffusion
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    with pytest.raises(ops.YolohtliError) as e:
        m.set_engine(A.YH_ENGINE_RESIDENT)
    assert e.value.status == A.YH_EUNSUPPORTED
    q = A.fk_tissue_params(4096, 4096)  # 16.8M cells: does not fit on chip
    m2 = Monodomain(q, A.YH_MODEL_FK3V, A.fk_defaults())
    with pytest.raises(ops.YolohtliError):
        m2.set_engine(A.YH_ENGINE_RESIDENT)


def test_fk_spiral_protocol_resident_vs_step_1500_steps():
    wl = W.fk_spiral_256(seed=0, n=256, nsteps=1500)
    wl.stims[0].step = 700
    a, _, _ = run(wl.p, wl.fk, wl.model, wl.state0(), None, wl.nsteps,
                  A.YH_ENGINE_STEP, wl.stims)
    b, _, _ = run(wl.p, wl.fk, wl.model, wl.state0(), None, wl.nsteps,
                  A.YH_ENGINE_RESIDENT, wl.stims)
    d = max_abs(a[0], b[0])
    print("FK3V 256^2 1500 steps: resident vs step max |du| = %.2e" % d)
    assert d <= 1e-5


def test_bounded_waits_report_a_timeout_and_leave_the_context_usable():
    # one block of a resident launch publishes none of its boundary rows: its
    # neighbours' waits run out after their 1 s bound and the launch ends
    # with YH_ETIMEOUT; the next launch on the same context runs normally
    import ctypes as C
    from yolohtli_gb300._loader import load
    muted, after = C.c_int(), C.c_int()
    rc = load().yh_selftest_resident_timeout(C.byref(muted), C.byref(after))
    if rc == A.YH_EUNSUPPORTED:
        pytest.skip("the resident engine does not run on this device")
    assert rc == A.YH_OK
    assert muted.value == A.YH_ETIMEOUT
    assert after.value == A.YH_OK
