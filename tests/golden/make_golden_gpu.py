"""Generates tests/golden/ref_kernels.npz by running the reference's own CUDA
kernels (compiled unchanged for sm_103a by oracle/ref_build.sh, launched
headless by oracle/ref_harness.cpp) on seeded FP64 inputs.

Run on a GPU machine:  python tests/golden/make_golden_gpu.py [out.npz]
The npz is committed; the CPU tests check the oracle against it.

Cases (REF2V, Euler, 5-point, Neumann, gateDiff = 1, the reference's own
launch shapes):
  rd_sq / rd_holes    one step and 20 steps of reactionDiffusion_kernel,
                      square domain and with a hole mask
  tip                 spiralTip_kernel between two levels of a rotating field
  cxy                 Cxy_field_kernel for a given (c, phi)
  slice / trapz       slice_kernel (scheme 2, template re-taken) and the 12
                      trapz_kernel integrals around a given tip
  bfecc               advFDBFECC_kernel launched three times on the same
                      inputs: the scratch arrays uf/ue then hold the values
                      of the previous launch, so the third launch reproduces
                      the race-free three-pass result (one launch reads
                      neighbours written in the same launch)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import torch  # noqa: E402

from oracle import refgpu as R  # noqa: E402
from yolohtli_gb300 import _abi as A  # noqa: E402
from yolohtli_gb300 import workloads as W  # noqa: E402

NX, NY = 48, 40


def dev(x, dtype=torch.float64):
    return torch.tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def smooth_state(nx, ny, seed):
    rng = np.random.default_rng(seed)
    jj, ii = np.mgrid[0:ny, 0:nx]
    u = np.zeros((ny, nx))
    v = np.zeros((ny, nx))
    for _ in range(4):
        a, b, c, d = rng.uniform(0.05, 0.3, 4)
        u += 0.25 * np.sin(a * ii + b * jj + rng.uniform(0, 6))
        v += 0.1 * np.cos(c * ii - d * jj + rng.uniform(0, 6))
    return (0.5 + u).ravel(), (0.2 + v).ravel()


def holes(nx, ny, seed):
    rng = np.random.default_rng(seed)
    return W.hole_mask(nx, ny, 6, 1.5, 3.0, rng)


def run_rd(p, u, v, steps, solid=None):
    a = [dev(u), dev(v)]
    b = [torch.zeros_like(a[0]), torch.zeros_like(a[0])]
    J = [torch.zeros_like(a[0]), torch.zeros_like(a[0])]
    vt = [torch.zeros_like(a[0]), torch.zeros_like(a[0])]
    sol = None if solid is None else dev(solid, torch.uint8)
    R.set_params(p)
    for _ in range(steps):
        R.rd(p, b, a, J, vt, sol)
        a, b = b, a
    R.sync()
    return [t.cpu().numpy() for t in a], [t.cpu().numpy() for t in vt]


def rotating_field(nx, ny, t):
    jj, ii = np.mgrid[0:ny, 0:nx]
    x = ii - nx / 2 + 0.3
    y = jj - ny / 2 - 0.2
    th = np.arctan2(y, x)
    r = np.hypot(x, y)
    return (0.5 + 0.5 * np.cos(th - 0.35 * r - t)).ravel()


def main(out):
    g = {}
    # ------------------------------------------------------------ RD
    p = A.param_defaults(NX, NY)
    u, v = smooth_state(NX, NY, 1)
    g["rd_sq_p"] = np.frombuffer(bytes(p), np.uint8)
    g["rd_sq_u0"], g["rd_sq_v0"] = u, v
    for steps in (1, 20):
        st, vt = run_rd(p, u, v, steps)
        g["rd_sq_%d_u" % steps], g["rd_sq_%d_v" % steps] = st
        g["rd_sq_%d_tu" % steps], g["rd_sq_%d_tv" % steps] = vt
    ph = p.copy()
    ph.solidSwitch = True
    solid = holes(NX, NY, 2)
    g["rd_holes_p"] = np.frombuffer(bytes(ph), np.uint8)
    g["rd_holes_solid"] = solid
    for steps in (1, 20):
        st, vt = run_rd(ph, u, v, steps, solid)
        g["rd_holes_%d_u" % steps], g["rd_holes_%d_v" % steps] = st
        g["rd_holes_%d_tu" % steps], g["rd_holes_%d_tv" % steps] = vt
    # ------------------------------------------------------------ tips
    pt = A.param_defaults(NX, NY)
    past = rotating_field(NX, NY, 0.0)
    present = rotating_field(NX, NY, 0.25)
    R.set_params(pt)
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 4096, dtype=torch.float32, device="cuda")
    plot = torch.zeros(NX * NY, dtype=torch.uint8, device="cuda")
    R.tip(pt, dev(past), dev(present), plot, cnt, vec, 1.5)
    R.sync()
    n = int(cnt.item())
    tips = vec[: 5 * n].cpu().numpy().reshape(n, 5)
    g["tip_past"], g["tip_present"] = past, present
    g["tip_tips"] = tips[np.lexsort((tips[:, 0], tips[:, 1]))]
    # ------------------------------------------------------------ Cxy
    pc = A.param_defaults(NX, NY)
    c = np.array([0.013, -0.021, 0.0045])
    phi = np.array([0.2, -0.1, 0.7])
    ax = torch.zeros(NX * NY, dtype=torch.float64, device="cuda")
    ay = torch.zeros_like(ax)
    R.set_params(pc)
    R.cxy(pc, ax, ay, c, phi)
    R.sync()
    g["cxy_c"], g["cxy_phi"] = c, phi
    g["cxy_x"], g["cxy_y"] = ax.cpu().numpy(), ay.cpu().numpy()
    # ------------------------------------------------------------ slices + trapz
    ps = A.param_defaults(NX, NY)
    ps.tipOffsetX = ps.tipOffsetY = 14
    ps.tipx, ps.tipy = 20.3, 18.6
    R.set_params(ps)
    su, sv = smooth_state(NX, NY, 3)
    gt = [dev(su), dev(sv)]
    slc = [torch.zeros(NX * NY, dtype=torch.float64, device="cuda") for _ in range(6)]
    slc0 = [torch.zeros_like(slc[0]) for _ in range(6)]
    tip1 = torch.tensor([25.7, 21.2, 0, 0, 0], dtype=torch.float32, device="cuda")
    cnt1 = torch.ones(1, dtype=torch.int32, device="cuda")
    intgl = torch.zeros(NX * NY, dtype=torch.uint8, device="cuda")
    tu, tv = smooth_state(NX, NY, 4)
    vtan = [dev(tu), dev(tv)]
    for count in (0, 7):
        R.slice_(ps, gt, slc, slc0, ax, ay, intgl, cnt1, tip1, count)
        R.sync()
        I = R.integrals(ps, slc, slc0, vtan, cnt1, tip1, count)
        g["slice_%d_cur" % count] = np.stack([t.cpu().numpy() for t in slc])
        g["slice_%d_tmpl" % count] = np.stack([t.cpu().numpy() for t in slc0])
        g["trapz_%d" % count] = I
    g["slice_p"] = np.frombuffer(bytes(ps), np.uint8)
    g["slice_u"], g["slice_v"] = su, sv
    g["slice_tu"], g["slice_tv"] = tu, tv
    g["slice_tip"] = np.array([25.7, 21.2], np.float32)
    # ------------------------------------------------------------ BFECC
    pb = A.param_defaults(NX, NY)
    pb.dt = 0.01
    A.param_derive(pb)
    R.set_params(pb)
    bu, bv = smooth_state(NX, NY, 5)
    cb = np.array([1.3, -0.7, 0.02])
    phib = np.array([0.0, 0.0, 0.4])
    R.cxy(pb, ax, ay, cb, phib)
    gin = [dev(bu), dev(bv)]
    gout = [torch.zeros_like(gin[0]) for _ in range(2)]
    uf = [torch.zeros_like(gin[0]) for _ in range(2)]
    ub = [torch.zeros_like(gin[0]) for _ in range(2)]
    ue = [torch.zeros_like(gin[0]) for _ in range(2)]
    for _ in range(3):
        R.bfecc(pb, gout, gin, ax, ay, uf, ub, ue)
    R.sync()
    g["bfecc_p"] = np.frombuffer(bytes(pb), np.uint8)
    g["bfecc_u0"], g["bfecc_v0"] = bu, bv
    g["bfecc_c"], g["bfecc_phi"] = cb, phib
    g["bfecc_u"], g["bfecc_v"] = [t.cpu().numpy() for t in gout]
    g["bfecc_ue_u"] = ue[0].cpu().numpy()
    np.savez_compressed(out, **g)
    print("wrote", out, len(g), "arrays")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.path.join(ROOT, "tests", "golden", "ref_kernels.npz"))
