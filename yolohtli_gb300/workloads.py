"""Seeded synthetic workloads of the FK3V tissue benchmarks (no datasets:
every input is generated on the host from a seed with numpy's PCG64).

fk_spiral_256      256x256, 10,000 steps, S1 columns 0-9 at t=0, S2 lower-left
                   quadrant at t=320 ms: one spiral.
fk_holes_1024      1024x1024, 20,000 steps, 300 circular holes (r ~ U[2,6]
                   cells), 12 S2 patches of 40x40 at uniform positions and
                   times ~ U[200,400] ms: fibrillation-like.
fk_sr_512          512x512 start of the symmetry-reduced workload: S1 at
                   t = 0, S2 per tau_d (SR_PROTOCOLS), run to 1000 ms.
fk_adjoint_case    512x512 parameter estimation: D(x, y) of 8 seeded Gaussian
                   bumps in [5e-4, 1.5e-3] cm^2/ms, a plane wave from the
                   left edge (the adjoint's workload).
fk_batch_256       256 independent square grids, n ~ U{128, 160, ..., 768},
                   5,000 steps, D ~ U[5e-4, 1.5e-3] cm^2/ms, every FK time
                   constant scaled by exp(U[ln 0.8, ln 1.2]), 0-100 holes
                   each (r ~ U[2,6]), S2 on the lower-left quadrant at
                   t ~ U[280, 360] ms: the batched solver's workload.
All use dx = 0.025 cm, dt = 0.05 ms, u = U(-0.01, 0.01), v = w = 1, S1 on
columns 0-9; the single grids D = 0.001 cm^2/ms (D dt/dx^2 = 0.08) and the
Fenton-Karma BR-fit parameters.
"""
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A


@dataclass
class Workload:
    name: str
    p: A.ParamVar
    fk: A.FKParams
    model: int
    u0: np.ndarray
    v0: np.ndarray
    w0: np.ndarray
    solid: object  # np.uint8 mask (1 = tissue) or None
    stims: list = field(default_factory=list)
    nsteps: int = 0

    @property
    def cells(self):
        return self.p.nx * self.p.ny

    def state0(self):
        return [self.u0.copy(), self.v0.copy(), self.w0.copy()]


def _ic(nx, ny, rng):
    u = rng.uniform(-0.01, 0.01, size=nx * ny).astype(np.float32)
    v = np.ones(nx * ny, np.float32)
    w = np.ones(nx * ny, np.float32)
    # S1: u = 1 on columns 0-9 at t = 0
    u.reshape(ny, nx)[:, :10] = 1.0
    return u, v, w


def hole_mask(nx, ny, nholes, rmin, rmax, rng):
    """1 = tissue, 0 = hole: `nholes` discs, radius ~ U[rmin, rmax] cells,
    centres uniform over the grid (the reference's mask polarity, main.cu:679)."""
    solid = np.ones((ny, nx), np.uint8)
    jj, ii = np.mgrid[0:ny, 0:nx]
    cx = rng.uniform(0, nx, nholes)
    cy = rng.uniform(0, ny, nholes)
    r = rng.uniform(rmin, rmax, nholes)
    for k in range(nholes):
        x0, x1 = int(max(0, cx[k] - r[k] - 1)), int(min(nx, cx[k] + r[k] + 2))
        y0, y1 = int(max(0, cy[k] - r[k] - 1)), int(min(ny, cy[k] + r[k] + 2))
        sub = (ii[y0:y1, x0:x1] - cx[k]) ** 2 + (jj[y0:y1, x0:x1] - cy[k]) ** 2
        solid[y0:y1, x0:x1][sub <= r[k] ** 2] = 0
    return solid.ravel()


def stim(step, i0, j0, i1, j1, value=1.0):
    s = A.Stim()
    s.step, s.i0, s.j0, s.i1, s.j1, s.value = int(step), i0, j0, i1, j1, value
    return s


def fk_spiral_256(seed=0, n=256, nsteps=10000, s2_ms=320.0):
    """S1 on columns 0-9 at t = 0, S2 on the lower-left quadrant at s2_ms.
    With the BR-fit parameters on 256^2 (6.4 cm) the S2 at 320 ms makes
    tips for a few ms at the quadrant's corner and no S2 time leaves
    activity past 600 ms: the wavelength does not fit; 512^2 re-entry is
    in fk_sr_512."""
    rng = np.random.default_rng(seed)
    p = A.fk_tissue_params(n, n)
    u, v, w = _ic(n, n, rng)
    dt = p.dt
    s2 = stim(int(round(s2_ms / dt)), 0, 0, n // 2, n // 2)
    return Workload("fk_spiral_%d" % n, p, A.fk_defaults(), A.YH_MODEL_FK3V,
                    u, v, w, None, [s2], nsteps)


# Start protocols of the symmetry-reduced workload on 512^2, per tau_d:
# (S2 box, S2 time in ms). A sweep of S2 times 180-705 ms (every 15 ms) on
# the lower-left quadrant and on the lower half, run to 3000 ms on the
# GB300, found re-entry lasting past 3000 ms only for tau_d = 0.25 (lower
# half, S2 at 540-585 ms) and tau_d = 0.30 (S2 at 615 ms); with
# tau_d = 0.35, 0.40 and 0.45 every protocol's activity ends before
# 850 ms: the tissue stays refractory too long (v recovers with
# tau_v2- = 1000 ms below u_v) for a re-entrant path in 12.8 cm.
SR_PROTOCOLS = {0.25: ((0, 0, 512, 256), 585.0),
                0.30: ((0, 0, 256, 256), 615.0)}


def fk_sr_512(seed=0, tau_d=0.25):
    """The start of the symmetry-reduced workload: S1 on columns 0-9 at
    t = 0 and the S2 of SR_PROTOCOLS[tau_d] on 512^2, run to 1000 ms (the
    state there is the SR start and, frozen, its template). ValueError for
    a tau_d without a protocol that sustains re-entry."""
    if tau_d not in SR_PROTOCOLS:
        raise ValueError("no re-entry lasts on 512^2 with tau_d = %g" % tau_d)
    box, s2 = SR_PROTOCOLS[tau_d]
    wl = fk_spiral_256(seed=seed, n=512, nsteps=20000, s2_ms=s2)
    wl.fk.tau_d = tau_d
    s = wl.stims[0]
    s.i0, s.j0, s.i1, s.j1 = box
    wl.name = "fk_sr_512_td%g" % tau_d
    return wl


def fk_holes_1024(seed=0, n=1024, nsteps=20000, nholes=300, npatch=12):
    rng = np.random.default_rng(seed)
    p = A.fk_tissue_params(n, n)
    u, v, w = _ic(n, n, rng)
    solid = hole_mask(n, n, nholes, 2.0, 6.0, rng)
    p.solidSwitch = True
    u[solid == 0] = 0.0
    v[solid == 0] = 0.0
    w[solid == 0] = 0.0
    stims = []
    for _ in range(npatch):
        i0 = int(rng.integers(0, n - 40))
        j0 = int(rng.integers(0, n - 40))
        t = rng.uniform(200.0, 400.0)
        stims.append(stim(int(round(t / p.dt)), i0, j0, i0 + 40, j0 + 40))
    stims.sort(key=lambda s: s.step)
    return Workload("fk_holes_%d" % n, p, A.fk_defaults(), A.YH_MODEL_FK3V,
                    u, v, w, solid, stims, nsteps)


def ref2v_cross(nx, ny):
    """The reference's own initial condition: the cross-field stimulation of
    initGates (main.cu:604-618): u = 1 for i < nx/8, v = 1 for j >= ny/2."""
    u = np.zeros((ny, nx))
    v = np.zeros((ny, nx))
    u[:, : nx // 8] = 1.0
    v[ny // 2:, :] = 1.0
    return u.ravel(), v.ravel()


TAU_NAMES = ("tau_d", "tau_r", "tau_si", "tau_0", "tau_v_plus",
             "tau_v1_minus", "tau_v2_minus", "tau_w_plus", "tau_w_minus")


@dataclass
class BatchWorkload:
    name: str
    instances: list  # of Workload
    nsteps: int

    @property
    def cells(self):
        return sum(w.cells for w in self.instances)

    def stims(self):
        """(instance, Stim) pairs of every instance."""
        return [(k, s) for k, w in enumerate(self.instances) for s in w.stims]


def fk_batch_256(seed=0, count=256, nsteps=5000, sizes=range(128, 769, 32),
                 max_holes=100):
    rng = np.random.default_rng(seed)
    sizes = list(sizes)
    inst = []
    for k in range(count):
        n = int(sizes[int(rng.integers(0, len(sizes)))])
        D = float(rng.uniform(5e-4, 1.5e-3))
        p = A.fk_tissue_params(n, n, D=D)
        fk = A.fk_defaults()
        for name in TAU_NAMES:
            setattr(fk, name, getattr(fk, name) *
                    float(np.exp(rng.uniform(np.log(0.8), np.log(1.2)))))
        u, v, w = _ic(n, n, rng)
        nh = int(rng.integers(0, max_holes + 1))
        solid = None
        if nh:
            solid = hole_mask(n, n, nh, 2.0, 6.0, rng)
            p.solidSwitch = True
            for f in (u, v, w):
                f[solid.ravel() == 0] = 0.0
        t = float(rng.uniform(280.0, 360.0))
        s2 = stim(int(round(t / p.dt)), 0, 0, n // 2, n // 2)
        inst.append(Workload("fk_batch_%d" % k, p, fk, A.YH_MODEL_FK3V,
                             u, v, w, solid, [s2], nsteps))
    return BatchWorkload("fk_batch_%d" % count, inst, nsteps)


def fk_adjoint_case(n=512, seed=0, bumps=8):
    """(D, (u0, v0, w0)): the diffusion map and initial state of the
    adjoint workload."""
    rng = np.random.default_rng(seed)
    jj, ii = np.mgrid[0:n, 0:n] / n
    z = np.zeros((n, n))
    for _ in range(bumps):
        cx, cy = rng.uniform(0, 1, 2)
        s = rng.uniform(0.05, 0.2)
        z += rng.uniform(-1, 1) * np.exp(-((ii - cx) ** 2 + (jj - cy) ** 2) / (2 * s * s))
    z = (z - z.min()) / max(z.max() - z.min(), 1e-12)
    D = (5e-4 + 1e-3 * z).astype(np.float32).ravel()
    u = np.zeros((n, n), np.float32)
    u[:, :6] = 1.0
    v = np.ones((n, n), np.float32)
    w = np.ones((n, n), np.float32)
    return D, [u.ravel(), v.ravel(), w.ravel()]
