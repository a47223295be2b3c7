"""GPU parity of the symmetry-reduction operators (tips, fused phase
integrals + solve, comoving field, BFECC) and of the whole symmetry-reduced
step against the FP64 oracle, through the C ABI."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import ops
from yolohtli_gb300.solver import Monodomain

from gpu_util import dev, host, max_abs, rel_l2, smooth_state, tips_match

pytestmark = pytest.mark.gpu


def rotating_field(nx, ny, t, cx=0.3, cy=-0.2):
    jj, ii = np.mgrid[0:ny, 0:nx]
    x = ii - nx / 2 + cx
    y = jj - ny / 2 + cy
    th = np.arctan2(y, x)
    r = np.hypot(x, y)
    return (0.5 + 0.5 * np.cos(th - 0.35 * r - t)).ravel()


@pytest.mark.parametrize("holes", [False, True])
def test_tips_match_oracle(holes):
    import torch
    nx, ny = 96, 80
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 30
    past = rotating_field(nx, ny, 0.0).astype(np.float32)
    present = rotating_field(nx, ny, 0.3).astype(np.float32)
    solid = None
    if holes:
        p.solidSwitch = True
        solid = np.ones(nx * ny, np.uint8)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    ops.spiral_tip(p, dev(past), dev(present), cnt, vec, 4096, 2.5,
                   None if solid is None else dev(solid, torch.uint8))
    torch.cuda.synchronize()
    n = int(cnt.item())
    got = host(vec)[: 5 * n].reshape(n, 5)
    want = O.tips(p, past.astype(np.float64), present.astype(np.float64),
                  solid=solid, ptime=2.5)
    assert n >= 1
    assert tips_match(got, want, 1e-5)
    assert np.all(got[:, 4] == np.float32(2.5))


def sym_tensor(c_adv=(0, 0, 0), phi_adv=(0, 0, 0), phi=(0, 0, 0), centre=(0, 0), step=1):
    s = A.SymState()
    for k in range(3):
        s.c_adv[k], s.phi_adv[k], s.phi[k] = c_adv[k], phi_adv[k], phi[k]
    s.centre[0], s.centre[1] = centre
    s.step = step
    return ops.sym_to_tensor(s)


@pytest.mark.parametrize("model", [A.YH_MODEL_REF2V, A.YH_MODEL_FK3V])
@pytest.mark.parametrize("frozen", [False, True])
def test_phase_integrals_and_solve_match_oracle(model, frozen):
    import torch
    nx, ny = 96, 80
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 25
    nf = A.NFIELDS[model]
    st = [x.astype(np.float32) for x in smooth_state(nx, ny, 3, nf)]
    tan = [x.astype(np.float32) for x in smooth_state(nx, ny, 4, nf)]
    c_adv, phi_adv = (0.011, -0.02, 0.004), (0.0, 0.0, 0.6)
    phi = (0.1, 0.2, 0.9)
    centre = (41.3, 37.8)
    sym = sym_tensor(c_adv, phi_adv, phi, centre)
    ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
    ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
    ops.comoving_field(p, sym, ar, ac)  # from c_adv, phi_adv; no advance
    ws = torch.zeros(ops.phase_workspace_bytes(nx, ny), dtype=torch.uint8, device="cuda")
    templ = None
    st64 = [x.astype(np.float64) for x in st]
    if frozen:
        tmpl_state = [x.astype(np.float32) for x in smooth_state(nx, ny, 9, nf)]
        tx = [torch.zeros(nx * ny, device="cuda") for _ in range(nf)]
        ty = [torch.zeros_like(tx[0]) for _ in range(nf)]
        tt = [torch.zeros_like(tx[0]) for _ in range(nf)]
        ops.template_slices(p, model, [dev(x) for x in tmpl_state], tx, ty, tt)
        templ = (tx, ty, tt)
    ops.phase_integrals(p, model, [dev(x) for x in st], [dev(x) for x in tan],
                        ar, ac, sym, ws, templ=templ)
    torch.cuda.synchronize()
    s = ops.sym_from_bytes(sym)
    # oracle: slices of the same FP32 values in FP64, then integrals, solve
    sl = O.slices(p, st64, c_adv, phi_adv, centre)
    if frozen:
        q = p.copy()
        q.tipOffsetX = q.tipOffsetY = 4 * (nx + ny)
        tsl = O.slices(q, [x.astype(np.float64) for x in tmpl_state], (0, 0, 0),
                       (0, 0, 0), (nx / 2, ny / 2))
        sl["tx"], sl["ty"], sl["tt"] = tsl["tx"], tsl["ty"], tsl["tt"]
    I = O.integrals(p, sl, [x.astype(np.float64) for x in tan], centre)
    got = np.array(s.integrals[:])
    assert np.abs(got - I).max() <= 2e-6 * np.abs(I).max()
    c_ref = O.solve(I, phi)
    assert s.status == A.YH_OK
    assert np.allclose(np.array(s.c[:]), c_ref, rtol=1e-4, atol=1e-6 * np.abs(c_ref).max())
    assert tuple(s.c_adv[:]) == tuple(s.c[:])
    assert tuple(s.phi_adv[:]) == tuple(phi)


def test_singular_system_reports_status_and_keeps_c():
    import torch
    nx, ny = 48, 40
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 10
    zero = [torch.zeros(nx * ny, device="cuda") for _ in range(2)]  # flat state
    sym = sym_tensor(centre=(20.0, 20.0))
    ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
    ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
    ws = torch.zeros(ops.phase_workspace_bytes(nx, ny), dtype=torch.uint8, device="cuda")
    ops.phase_integrals(p, A.YH_MODEL_REF2V, zero, zero, ar, ac, sym, ws)
    torch.cuda.synchronize()
    s = ops.sym_from_bytes(sym)
    assert s.status == A.YH_ESINGULAR
    assert tuple(s.c[:]) == (0.0, 0.0, 0.0)


@pytest.mark.parametrize("model", [A.YH_MODEL_REF2V, A.YH_MODEL_FK3V])
def test_bfecc_matches_oracle(model):
    import torch
    nx, ny = 64, 52
    p = A.param_defaults(nx, ny)
    p.dt = 0.01
    A.param_derive(p)
    nf = A.NFIELDS[model]
    st = [x.astype(np.float32) for x in smooth_state(nx, ny, 5, nf)]
    c, phi = (1.3, -0.7, 0.02), (0.0, 0.0, 0.4)
    sym = sym_tensor(c, phi)
    ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
    ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
    arf = torch.zeros(ny, device="cuda")
    acf = torch.zeros(nx, device="cuda")
    ops.comoving_field(p, sym, ar, ac, arf, acf)
    inp = [dev(x) for x in st]
    out = [torch.zeros_like(inp[0]) for _ in range(nf)]
    uf = [torch.zeros_like(inp[0]) for _ in range(nf)]
    ue = [torch.zeros_like(inp[0]) for _ in range(nf)]
    ops.advect_bfecc(p, model, out, inp, arf, acf, uf, ue)
    torch.cuda.synchronize()
    want = O.bfecc(p, [x.astype(np.float64) for x in st], c, phi)
    for f in range(nf):
        assert max_abs(host(out[f]), want[f]) < 2e-6


@pytest.mark.parametrize("model", [A.YH_MODEL_REF2V, A.YH_MODEL_FK3V])
@pytest.mark.parametrize("holes", [False, True])
@pytest.mark.parametrize("shape", [(64, 52), (97, 61), (33, 17)])
def test_bfecc_one_launch_equals_three_launches(model, holes, shape):
    # the fused kernel (tiles with rings in shared memory) against the three
    # pass launches: the same bits, on grids that are no multiple of the tile
    import torch
    nx, ny = shape
    p = A.param_defaults(nx, ny)
    p.dt = 0.01
    A.param_derive(p)
    nf = A.NFIELDS[model]
    solid = None
    if holes:
        rng = np.random.default_rng(nx)
        jj, ii = np.mgrid[0:ny, 0:nx]
        m = np.ones((ny, nx), np.uint8)
        for _ in range(6):
            cx, cy, r = rng.uniform(0, nx), rng.uniform(0, ny), rng.uniform(1.5, 4)
            m[(ii - cx) ** 2 + (jj - cy) ** 2 <= r * r] = 0
        solid = dev(m.ravel(), torch.uint8)
        p.solidSwitch = True
    st = [x.astype(np.float32) for x in smooth_state(nx, ny, 7, nf)]
    for c, phi in (((1.3, -0.7, 0.02), (0.0, 0.0, 0.4)),
                   ((-2.1, 0.9, -0.05), (0.0, 0.0, 2.5))):
        sym = sym_tensor(c, phi)
        ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
        ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
        arf = torch.zeros(ny, device="cuda")
        acf = torch.zeros(nx, device="cuda")
        ops.comoving_field(p, sym, ar, ac, arf, acf)
        inp = [dev(x) for x in st]
        outs = []
        for three in (False, True):
            out = [torch.full_like(inp[0], 7.0) for _ in range(nf)]
            uf = [torch.zeros_like(inp[0]) for _ in range(nf)]
            ue = [torch.zeros_like(inp[0]) for _ in range(nf)]
            ops.advect_bfecc(p, model, out, inp, arf, acf, uf, ue, solid=solid,
                             three_launches=three)
            outs.append(out)
        torch.cuda.synchronize()
        for f in range(nf):
            assert torch.equal(outs[0][f], outs[1][f]), (f, c)


def ref2v_spiral(n, L=3.0, steps=6000):
    """A REF2V spiral grown from the reference's cross-field initial
    condition (main.cu:604-618) on an n x n grid of side L cm, with the FP32
    product kernels; returns the FP32 state and its parameters."""
    from yolohtli_gb300 import workloads as W
    p = A.param_defaults(n, n)
    p.Lx = p.Ly = L
    p.hx = p.hy = L / (n - 1)
    A.param_derive(p)
    u, v = W.ref2v_cross(n, n)
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(u, v)
    m.run(steps)
    st = m.get_state()
    m.close()
    return p, st


def test_sr_sequence_matches_oracle():
    n = 128
    p, st = ref2v_spiral(n)
    p.dt = 0.5 * p.dt  # the reference halves dt in SR mode (main.cu:148)
    A.param_derive(p)
    p.tipOffsetX = p.tipOffsetY = 30
    # start the disc at the spiral tip
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    m.run(1)
    m.track_tips()
    tips = m.get_tips()
    m.close()
    assert len(tips) >= 1
    p.tipx, p.tipy = float(tips[0, 0]), float(tips[0, 1])
    nsr = 40
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    m.sr_begin()
    m.sr_step(nsr)
    got = m.get_state()
    sg = m.get_sym()
    orc = O.SR(p, A.YH_MODEL_REF2V, None, [x.astype(np.float64) for x in st])
    orc.step(nsr)
    r = orc.get()
    print("SR %d steps: c gpu %s oracle %s; phi gpu %s oracle %s; rel L2(u) %.2e" % (
        nsr, list(sg.c), list(r["c"]), list(sg.phi), list(r["phi"]),
        rel_l2(got[0], r["state"][0])))
    assert sg.step == nsr and r["step"] == nsr
    assert sg.status == A.YH_OK
    assert np.allclose(list(sg.centre), r["centre"], atol=1e-3)
    # measured: c and phi within 8e-5 relative (the smallest component),
    # rel L2(u) 4.7e-7
    assert np.allclose(list(sg.c), r["c"], rtol=3e-4, atol=1e-6 * np.abs(r["c"]).max())
    assert np.allclose(list(sg.phi), r["phi"], rtol=3e-4, atol=1e-9)
    assert rel_l2(got[0], r["state"][0]) < 2e-6


def test_sr_frozen_template_runs_and_stays_finite():
    n = 96
    p, st = ref2v_spiral(n, L=2.25, steps=5000)
    p.dt *= 0.5
    A.param_derive(p)
    p.tipOffsetX = p.tipOffsetY = 20
    p.tipx, p.tipy = n / 2, n / 2
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    m.sr_begin(A.YH_TEMPLATE_FROZEN, template=st)
    m.sr_step(37)
    s = m.get_sym()
    got = m.get_state()
    assert s.step == 37
    assert np.all(np.isfinite(got[0])) and np.all(np.isfinite(list(s.c)))


def sr_spiral_case(n=128, L=3.0, radius=30):
    """A REF2V spiral (ref2v_spiral) with the symmetry-reduction parameters:
    dt halved as the reference does in SR mode (main.cu:148), a disc of
    `radius` cells started at the spiral's tip."""
    p, st = ref2v_spiral(n, L=L)
    p.dt = 0.5 * p.dt
    A.param_derive(p)
    p.tipOffsetX = p.tipOffsetY = radius
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    m.run(1)
    m.track_tips()
    tips = m.get_tips()
    m.close()
    assert len(tips) >= 1
    c = np.array([n / 2, n / 2])
    k = int(np.argmin(np.hypot(tips[:, 0] - c[0], tips[:, 1] - c[1])))
    p.tipx, p.tipy = float(tips[k, 0]), float(tips[k, 1])
    return p, st


def test_sr_enqueue_on_two_streams_equals_sr_step():
    # two handles on their own streams, their steps enqueued one after the
    # other without waiting (yh_sr_enqueue) and the status read at the end
    # (yh_sr_status): each the same bits as a handle stepped by yh_sr_step
    import torch
    p, st = sr_spiral_case(n=96, L=2.25, radius=20)
    ref = Monodomain(p, A.YH_MODEL_REF2V, None)
    ref.set_state(*st)
    ref.sr_begin()
    for _ in range(3):
        ref.sr_step(37)
    want, wsym = ref.get_state(), ref.get_sym()
    ref.close()
    streams = [torch.cuda.Stream() for _ in range(2)]
    hs = [Monodomain(p, A.YH_MODEL_REF2V, None, stream=s.cuda_stream) for s in streams]
    for m in hs:
        m.set_state(*st)
        m.sr_begin()
    for _ in range(3):
        for m in hs:
            m.sr_enqueue(37)
    for m in hs:
        m.sr_status()
        got, gsym = m.get_state(), m.get_sym()
        assert gsym.step == wsym.step == 111
        assert list(gsym.c) == list(wsym.c) and list(gsym.phi) == list(wsym.phi)
        for f in range(2):
            assert np.array_equal(got[f], want[f]), f
        m.close()


def test_sr_frozen_template_trajectory_matches_oracle():
    """BASELINE-style symmetry reduction (template frozen at the start
    state) over 2,000 SR steps on 128^2: the FP32 product's c, phi and u
    against the FP64 oracle's SR sequence (main.cu:894-954 with a fixed
    template) at several step counts."""
    p, st = sr_spiral_case()
    m = Monodomain(p, A.YH_MODEL_REF2V, None)
    m.set_state(*st)
    m.sr_begin(A.YH_TEMPLATE_FROZEN, template=st)
    st64 = [x.astype(np.float64) for x in st]
    orc = O.SR(p, A.YH_MODEL_REF2V, None, st64,
               template_mode=A.YH_TEMPLATE_FROZEN, template=st64)
    done, rows = 0, []
    for n in (250, 1000, 2000):
        m.sr_step(n - done)
        orc.step(n - done)
        done = n
        sg, r, got = m.get_sym(), orc.get(), m.get_state()
        cs = np.abs(r["c"]).max()
        rows.append((n, float(np.abs(np.array(sg.c) - r["c"]).max() / cs),
                     float(np.abs(np.array(sg.phi) - r["phi"]).max()),
                     rel_l2(got[0], r["state"][0]), sg.ntips, r["ntips"]))
        assert sg.status == A.YH_OK and sg.nsingular == 0
    print("frozen-template SR, FP32 vs FP64 oracle (N, max|dc|/max|c|, "
          "max|dphi|, rel L2(u), tips gpu/oracle):", rows)
    for n, dc, dphi, du, nt, nto in rows:
        assert nt >= 1 and nto >= 1
        assert dc <= 1e-3 and dphi <= 1e-3 and du <= 1e-4, (n, dc, dphi, du)


def test_sr_tips_reconstruct_the_lab_frame_trajectory():
    """The reconstruction of the reference's DATA/processSymmetry.m:80-115:
    the symmetry-reduced tip mapped back to the lab frame through phi,
    x = -phix + xt cos(-phit) - yt sin(-phit),
    y = -phiy + xt sin(-phit) + yt cos(-phit)   (physical units, corner
    origin), equals the plain-mode tip trajectory of the same start state
    and time step up to a constant offset."""
    p, st = sr_spiral_case()
    every, nsamp = 100, 30
    plain = Monodomain(p, A.YH_MODEL_REF2V, None)
    plain.set_state(*st)
    sr = Monodomain(p, A.YH_MODEL_REF2V, None)
    sr.set_state(*st)
    sr.sr_begin(A.YH_TEMPLATE_FROZEN, template=st)
    lab, rec = [], []
    prev = np.array([p.tipx, p.tipy])
    for _ in range(nsamp):
        plain.run(every)
        plain.track_tips()
        t = plain.get_tips()
        assert len(t) >= 1
        k = int(np.argmin(np.hypot(t[:, 0] - prev[0], t[:, 1] - prev[1])))
        prev = t[k, :2].astype(np.float64)
        lab.append(prev * p.hx)
        sr.sr_step(every)
        s = sr.get_sym()
        xt, yt = s.centre[0] * p.hx, s.centre[1] * p.hy
        ph = np.array(s.phi)
        rec.append([-ph[0] + xt * np.cos(-ph[2]) - yt * np.sin(-ph[2]),
                    -ph[1] + xt * np.sin(-ph[2]) + yt * np.cos(-ph[2])])
    plain.close()
    sr.close()
    lab, rec = np.array(lab), np.array(rec)
    off = (lab - rec).mean(axis=0)
    dev_cells = np.hypot(*(lab - rec - off).T) / p.hx
    span = np.hypot(*(lab - lab.mean(axis=0)).T).max() / p.hx
    print("reconstruction: lab-frame tip path spans %.2f cells; reconstructed "
          "path within %.3f cells (mean %.3f) after a constant offset" % (
              span, dev_cells.max(), dev_cells.mean()))
    assert span > 1.0
    assert dev_cells.max() < 0.5
