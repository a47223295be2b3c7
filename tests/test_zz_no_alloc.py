"""yh_phase_integrals_noalloc: the phase-integral operator for callers that
may not allocate device memory (a host whose GPU memory belongs to its own
pool, or code in a section where cudaMalloc, which can synchronize the
device, is not allowed). It keeps its scratch in a fixed array compiled into
the library instead of a workspace argument. These checks call it through
the C ABI twice in a row, each time against yh_phase_integrals with a
workspace on the same inputs, and check that a disc too large for the fixed
scratch is refused. The file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import load, ops

from gpu_util import dev, smooth_state

pytestmark = pytest.mark.gpu


def _sym(c_adv, phi_adv, phi, centre):
    s = A.SymState()
    for k in range(3):
        s.c_adv[k], s.phi_adv[k], s.phi[k] = c_adv[k], phi_adv[k], phi[k]
    s.centre[0], s.centre[1] = centre
    s.step = 1
    return ops.sym_to_tensor(s)


def test_noalloc_matches_the_workspace_entry_point_on_two_calls():
    import torch
    lib = load()
    nx, ny = 160, 128
    p = A.param_defaults(nx, ny)
    p.tipOffsetX = p.tipOffsetY = 40
    model = A.YH_MODEL_FK3V
    cases = [
        (3, 4, (0.011, -0.02, 0.004), (0.0, 0.0, 0.6), (0.1, 0.2, 0.9), (70.3, 61.8)),
        (5, 6, (-0.03, 0.01, -0.002), (0.0, 0.0, -1.1), (0.0, 0.0, 0.2), (90.6, 50.2)),
    ]
    ws = torch.zeros(ops.phase_workspace_bytes(nx, ny), dtype=torch.uint8, device="cuda")
    for seed_s, seed_t, c_adv, phi_adv, phi, centre in cases:
        st = [dev(x.astype(np.float32)) for x in smooth_state(nx, ny, seed_s, 3)]
        tan = [dev(x.astype(np.float32)) for x in smooth_state(nx, ny, seed_t, 3)]
        sym_a = _sym(c_adv, phi_adv, phi, centre)
        sym_b = _sym(c_adv, phi_adv, phi, centre)
        ar = torch.zeros(ny, dtype=torch.float64, device="cuda")
        ac = torch.zeros(nx, dtype=torch.float64, device="cuda")
        ops.comoving_field(p, sym_a, ar, ac)
        ops.phase_integrals(p, model, st, tan, ar, ac, sym_a, ws)
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        rc = lib.yh_phase_integrals_noalloc(
            C.byref(p), model, ops.fields(st), ops.fields(tan), A.Fields(),
            A.Fields(), A.Fields(), ar.data_ptr(), ac.data_ptr(), None,
            sym_b.data_ptr(), stream)
        assert rc == A.YH_OK
        torch.cuda.synchronize()
        a, b = ops.sym_from_bytes(sym_a), ops.sym_from_bytes(sym_b)
        Ia, Ib = np.array(a.integrals[:]), np.array(b.integrals[:])
        # the tolerance of the other phase-integral tests (2e-6 of the
        # largest integral); the two paths run the same deterministic kernel
        assert np.abs(Ia - Ib).max() <= 2e-6 * np.abs(Ia).max()
        assert a.status == b.status == A.YH_OK
        assert np.allclose(list(a.c), list(b.c), rtol=1e-6, atol=0)


def test_noalloc_refuses_a_disc_larger_than_its_scratch():
    lib = load()
    p = A.param_defaults(4096, 4096)
    p.tipOffsetX = p.tipOffsetY = 2000  # needs about 60,000 blocks of partials
    f = A.Fields(1, 1, 1)  # never dereferenced: refused before any launch
    rc = lib.yh_phase_integrals_noalloc(
        C.byref(p), A.YH_MODEL_FK3V, f, f, A.Fields(), A.Fields(), A.Fields(),
        1, 1, None, 1, None)
    assert rc == A.YH_EINVAL
    assert lib.yh_phase_integrals_noalloc_limit() == 256 + 4096 * 12 * 8
