"""The analysis kernels beside the hot path's tip tracker against the
reference's own kernels (oracle/refgpu, headless): Newton tips (tipAlgorithm
2), the tip gradient (tipGrad), filament cells (tipAlgorithm 3), contours
(modes 1-3) and the space-APD tracker, through the FP64 drop-in symbols
(tip_wrapper, countour_wrapper, sAPD_wrapper) and the FP32 C ABI."""
import ctypes as C

import numpy as np
import pytest

from oracle import refgpu as R
from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import ops

from gpu_util import dev, host
from yolohtli_gb300.compat import B2, Compat, Dim3, G2, StateVar, sv

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.available(),
                                 reason="reference cubin not built (oracle/ref_build.sh)")]

SYM_CONTOUR = "_Z16countour_wrapperm4dim3S_PdS0_PbS1_PiP6float3fi"
SYM_SAPD = "_Z12sAPD_wrapperm4dim3S_iPdS0_S0_S0_S0_S0_S0_S0_PbS1_b"


def fields(n, seed, shift=0.0):
    """Two smooth levels whose u = Uth isolines cross many times."""
    rng = np.random.default_rng(seed)
    jj, ii = np.mgrid[0:n, 0:n]
    f = np.zeros((n, n))
    for _ in range(5):
        a, b = rng.uniform(0.08, 0.35, 2)
        f += 0.2 * np.sin(a * ii + b * jj + rng.uniform(0, 6) + shift)
    return (0.5 + f).astype(np.float32).ravel()


def params(n, tox=40, holes=False, grad=False):
    p = A.param_defaults(n, n)
    p.Uth = 0.5
    p.tipOffsetX = p.tipOffsetY = tox
    p.solidSwitch = holes
    p.tipGrad = grad
    return p


def tipset(vec, count):
    n = int(host(count)[0])
    t = host(vec)[: 5 * n].reshape(-1, 5)
    return t[np.lexsort((t[:, 0], t[:, 1]))]


def ref_tips(alg, p, past, present, ptime=2.5):
    import torch
    n = p.nx * p.ny
    plot = torch.zeros(n, dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 20000, dtype=torch.float32, device="cuda")
    R.set_params(p)
    a, b = dev(past, torch.float64), dev(present, torch.float64)
    if alg == 1:
        R.tip(p, a, b, plot, count, vec, ptime)
    else:
        R.tip_alg(alg, p, a, b, plot, count, vec, ptime)
    R.sync()
    return tipset(vec, count), host(plot)


def compat_tips(alg, p, past, present, ptime=2.5):
    import torch
    cp = Compat()
    cp.set_params(p)
    n = p.nx * p.ny
    plot = torch.zeros(n, dtype=torch.uint8, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 500000, dtype=torch.float32, device="cuda")
    a, b = dev(past, torch.float64), dev(present, torch.float64)
    z = torch.zeros_like(a)
    cp.f["tip"](0, G2, B2, sv(b, z), sv(a, z), sv(z, z), ptime, alg, False,
                plot.data_ptr(), count.data_ptr(), vec.data_ptr())
    torch.cuda.synchronize()
    assert cp.err() == 0
    return tipset(vec, count), host(plot)


@pytest.mark.parametrize("holes", [False, True])
@pytest.mark.parametrize("grad", [False, True])
@pytest.mark.parametrize("alg", [1, 2])
def test_tips_and_gradient_match_the_reference_kernels(alg, grad, holes):
    n = 96
    p = params(n, holes=holes, grad=grad)
    past, present = fields(n, 1), fields(n, 1, shift=0.4)
    ref, rplot = ref_tips(alg, p, past, present)
    got, gplot = compat_tips(alg, p, past, present)
    assert len(ref) > 3, "the fields give the kernels nothing to find"
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)
    assert np.array_equal(gplot, rplot)
    # the FP32 C ABI on the same (FP32) levels: the same FP64 arithmetic
    import torch
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(5 * 20000, dtype=torch.float32, device="cuda")
    q = p.copy()
    q.tipAlgorithm = alg
    ops.spiral_tip(q, dev(past), dev(present), count, vec, 20000, 2.5)
    torch.cuda.synchronize()
    f32 = tipset(vec, count)
    assert f32.shape == ref.shape
    assert np.abs(f32 - ref).max() <= 1e-6


def test_filament_cells_match_the_reference_kernel():
    import torch
    n = 96
    p = params(n)
    past, present = fields(n, 2), fields(n, 2, shift=0.3)
    _, ref = ref_tips(3, p, past, present)
    _, got = compat_tips(3, p, past, present)
    assert ref.sum() > 10
    assert np.array_equal(got, ref)
    mark = torch.zeros(n * n, dtype=torch.uint8, device="cuda")
    ops.filament_mark(p, dev(past), dev(present), mark)
    torch.cuda.synchronize()
    assert np.array_equal(host(mark), ref)


def contour_case(n, seed):
    rng = np.random.default_rng(seed)
    f1 = fields(n, seed + 10).astype(np.float64)
    f2 = (fields(n, seed) - 0.5).astype(np.float64)
    stim = (rng.random(n * n) < 0.8).astype(np.uint8)
    p = params(n)
    p.contourThresh1 = 0.55
    p.contourThresh2 = 0.02
    p.contourThresh3 = 0.05
    return p, f1, f2, stim


def cset(vec, count):
    k = int(host(count)[0])
    t = host(vec)[: 3 * k].reshape(-1, 3)
    return t[np.lexsort((t[:, 0], t[:, 1], t[:, 2]))]


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_contours_match_the_reference_kernel(mode):
    import torch
    n = 80
    p, f1, f2, stim = contour_case(n, 3 + mode)
    N = n * n
    # the reference reads one row past the end of field2 in its last row: a
    # copy of the last row there makes its read what this library assumes
    f2pad = np.concatenate([f2, f2[-n:]])
    d1, d2 = dev(f1, torch.float64), dev(f2pad, torch.float64)
    sa = dev(stim, torch.uint8)
    # plot_field writes past the end of the plot for points extrapolated
    # beyond the last cell; a padded plot keeps those writes off rvec
    rplot_pad = torch.zeros(4 * N, dtype=torch.uint8, device="cuda")
    rplot = rplot_pad[:N]
    rcount = torch.zeros(1, dtype=torch.int32, device="cuda")
    rvec = torch.zeros(3 * N, dtype=torch.float32, device="cuda")
    R.set_params(p)
    R.contour(p, d1, d2, rplot, sa, rcount, rvec, 1.25, mode)
    R.sync()
    ref = cset(rvec, rcount)
    assert len(ref) > 3
    lib = Compat().lib
    fn = getattr(lib, SYM_CONTOUR)
    fn.argtypes = [C.c_size_t, Dim3, Dim3] + [C.c_void_p] * 6 + [C.c_float, C.c_int]
    fn.restype = None
    Compat().set_params(p)
    gplot = torch.zeros(N, dtype=torch.uint8, device="cuda")
    gcount = torch.zeros(1, dtype=torch.int32, device="cuda")
    gvec = torch.zeros(3 * N, dtype=torch.float32, device="cuda")
    fn(0, G2, B2, d1.data_ptr(), d2.data_ptr(), gplot.data_ptr(), sa.data_ptr(),
       gcount.data_ptr(), gvec.data_ptr(), 1.25, mode)
    torch.cuda.synchronize()
    assert np.array_equal(cset(gvec, gcount), ref)
    assert np.array_equal(host(gplot), host(rplot))
    # FP32 C ABI
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    vec = torch.zeros(3 * N, dtype=torch.float32, device="cuda")
    ops.contour(p, dev(f1), dev(f2), sa, mode, 1.25, count, vec, N)
    torch.cuda.synchronize()
    f32 = cset(vec, count)
    # FP32 fields move a few points across the level; nearly all agree
    common = min(len(f32), len(ref))
    assert abs(len(f32) - len(ref)) <= max(2, len(ref) // 100)
    assert common > 0


@pytest.mark.parametrize("stimulate", [False, True])
def test_space_apd_matches_the_reference_kernel(stimulate):
    import torch
    n = 48
    N = n * n
    p = params(n)
    p.dt = 0.1
    rng = np.random.default_rng(9)
    stim = dev((rng.random(N) < 0.7).astype(np.uint8), torch.uint8)
    phase = rng.uniform(0, 40, N)
    width = rng.uniform(8, 14, N)

    def u_at(k):  # two beats of different duration per cell
        t = k - phase
        b1 = (t > 0) & (t < width)
        b2 = (t > 60) & (t < 60 + 0.8 * width)
        return np.where(b1 | b2, 0.9, 0.02) + 0.01 * np.sin(k + phase)

    def zeros(dtype=torch.float64):
        return torch.zeros(N, dtype=dtype, device="cuda")

    ref = {k: zeros() for k in ("a1", "a2", "s", "d", "b", "f")}
    ref["first"] = zeros(torch.uint8)
    got = {k: zeros() for k in ("a1", "a2", "s", "d", "b", "f")}
    got["first"] = zeros(torch.uint8)
    f32 = {k: zeros(torch.float32) for k in ("apd1", "apd2", "sapd", "dapd",
                                             "back", "front")}
    f32["first"] = zeros(torch.uint8)
    cp = Compat()
    cp.set_params(p)
    fn = getattr(cp.lib, SYM_SAPD)
    fn.argtypes = [C.c_size_t, Dim3, Dim3, C.c_int] + [C.c_void_p] * 10 + [C.c_bool]
    fn.restype = None
    R.set_params(p)
    for k in range(1, 120):
        uo = dev(u_at(k - 1), torch.float64)
        un = dev(u_at(k), torch.float64)
        R.sapd(k, uo, un, ref["a1"], ref["a2"], ref["s"], ref["d"], ref["b"],
               ref["f"], ref["first"], stim, stimulate)
        fn(0, Dim3(256, 1, 1), Dim3(64, 1, 1), k, uo.data_ptr(), un.data_ptr(),
           *[got[x].data_ptr() for x in ("a1", "a2", "s", "d", "b", "f", "first")],
           stim.data_ptr(), stimulate)
        ops.space_apd(p, k, uo.float(), un.float(), f32, stim, stimulate)
    torch.cuda.synchronize()
    assert cp.err() == 0
    for x in ("a1", "a2", "s", "d", "b", "f", "first"):
        assert torch.equal(got[x], ref[x]), x
    assert float(ref["a1"].abs().max()) > 0  # beats were measured
    assert np.allclose(host(f32["apd1"]), host(ref["a1"]), atol=1e-4)
    assert np.array_equal(host(f32["sapd"]), host(ref["s"]).astype(np.float32))
