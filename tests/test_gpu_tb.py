"""GPU tests of the temporally blocked step (K explicit steps per launch)
and of the time-block autotuner, through the solver handle."""
import numpy as np
import pytest

from oracle import oracle as O
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import workloads as W
from yolohtli_gb300.solver import Monodomain

from gpu_util import max_abs, rel_l2

pytestmark = pytest.mark.gpu


def fk_case(nx, ny, holes, seed=4):
    rng = np.random.default_rng(seed)
    p = A.fk_tissue_params(nx, ny)
    u = rng.uniform(0, 1, nx * ny).astype(np.float32)
    v = rng.uniform(0, 1, nx * ny).astype(np.float32)
    w = rng.uniform(0, 1, nx * ny).astype(np.float32)
    solid = None
    if holes:
        solid = W.hole_mask(nx, ny, 25, 2.0, 6.0, rng)
        p.solidSwitch = True
        for f in (u, v, w):
            f[solid == 0] = 0
    # a smooth excitation so that fronts move through tile boundaries
    jj, ii = np.mgrid[0:ny, 0:nx]
    u[((ii - nx // 3) ** 2 + (jj - ny // 2) ** 2 < 400).ravel()] = 1.0
    return p, [u, v, w], solid


def run(p, st, solid, nsteps, k, stims=()):
    m = Monodomain(p, A.YH_MODEL_FK3V, A.fk_defaults(), solid=solid)
    m.set_state(*st)
    m.set_time_block(k)
    assert m.time_block() == k
    m.run(nsteps, stims)
    out = m.get_state()
    m.close()
    return out


@pytest.mark.parametrize("nx,ny", [(300, 170), (256, 128), (97, 61)])
@pytest.mark.parametrize("holes", [False, True])
def test_blocked_steps_equal_single_steps(nx, ny, holes):
    p, st, solid = fk_case(nx, ny, holes)
    ref = run(p, st, solid, 96, 1)
    for k in range(2, 9):
        got = run(p, st, solid, 96, k)
        for f in range(3):
            d = max_abs(got[f], ref[f])
            assert d <= 2e-6, (k, f, d)


@pytest.mark.parametrize("nx,ny", [(300, 170), (68, 21), (256, 128), (8, 9),
                                   (160, 50)])
@pytest.mark.parametrize("holes", [False, True])
def test_two_step_kernel_is_bitwise_two_single_steps(nx, ny, holes):
    # depth 2 runs the two-step tile kernel (64 x 16 tiles, step 1 on a
    # 1-cell ring from a 2-cell halo), its inputs staged by TMA bulk tensor
    # copies where the rows allow (nx % 4; with holes nx % 16: 256, 160) and
    # by plain loads otherwise: the tiles at the domain's far edges are cut
    # (300 = 4 x 64 + 44, 170 = 10 x 16 + 10, 160 = 2 x 64 + 32), the
    # boxes can exceed the grid (8 x 9), the step count is odd (one single
    # step at the end), and every value must equal the single-step engine's
    # bits
    p, st, solid = fk_case(nx, ny, holes)
    ref = run(p, st, solid, 97, 1)
    got = run(p, st, solid, 97, 2)
    for f in range(3):
        assert np.array_equal(got[f], ref[f]), (f, max_abs(got[f], ref[f]))


def test_blocked_protocol_with_stimuli_matches_oracle():
    p, st, solid = fk_case(256, 192, True)
    stims = [W.stim(40, 10, 10, 60, 60), W.stim(133, 150, 100, 200, 150)]
    got = run(p, st, solid, 300, 6, stims)
    ref = O.run(p, A.YH_MODEL_FK3V, A.fk_defaults(), st, 300, stims, solid=solid)
    assert rel_l2(got[0], ref[0]) < 1e-5
    assert np.all(got[0][solid == 0] == 0)


def test_autotune_picks_an_engine_and_restores_the_state():
    p, st, solid = fk_case(512, 512, True)
    m = Monodomain(p, A.YH_MODEL_FK3V, A.fk_defaults(), solid=solid)
    m.set_state(*st)
    before = m.get_state()
    n0 = m.launch_count()
    e, k = m.autotune(128)
    after = m.get_state()
    assert e in A.ENGINE_NAMES and 1 <= k <= 8 and m.engine() == (e, k)
    print("autotune 512^2 FK3V with holes: engine %s, depth %d" % (A.ENGINE_NAMES[e], k))
    assert m.step_count() == 0 and m.launch_count() == n0
    for f in range(3):
        assert np.array_equal(before[f], after[f])
    m.close()


def test_ref2v_with_diffusing_v_stays_at_one_step_per_launch():
    p = A.param_defaults(64, 64)  # gateDiff = 1
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_time_block(6)
    assert m.time_block() == 1
    q = p.copy()
    q.gateDiff = False
    m2 = Monodomain(q, A.YH_MODEL_REF2V, None)
    m2.set_time_block(6)
    assert m2.time_block() == 6


@pytest.fixture(scope="module")
def reentry_state():
    """The 512^2 re-entry of the symmetry-reduced workload's start protocol
    (S1 at t = 0, S2 on the lower-left quadrant at 430 ms) at 1000 ms,
    where spiral tips are in the tissue."""
    wl = W.fk_sr_512()
    m = Monodomain(wl.p, wl.model, wl.fk)
    m.set_state(*wl.state0())
    m.run(wl.nsteps, wl.stims)
    st = m.get_state()
    m.close()
    return wl, st


@pytest.mark.parametrize("k", [2, 4])
@pytest.mark.parametrize("nsteps", [40, 41, 129])
def test_tips_after_a_blocked_run_use_the_previous_level(reentry_state, k,
                                                         nsteps):
    """yh_track_tips compares the state with the u level one step back,
    whatever the engine: a blocked run takes its last step on its own."""
    wl, st = reentry_state
    got = []
    for kk in (1, k):
        m = Monodomain(wl.p, wl.model, wl.fk)
        m.set_state(*st)
        m.set_time_block(kk)
        m.run(nsteps)
        m.track_tips()
        got.append(m.get_tips())
        m.close()
    assert len(got[0]) > 0
    assert len(got[0]) == len(got[1])
    assert np.array_equal(got[0][:, :2], got[1][:, :2])
