"""The JSON-lines run log: segment bookkeeping and rates on the CPU with a
stand-in solver, and one logged run of the real solver on the GPU."""
import json

import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import runlog


class FakeSolver:
    """The calls run_logged and sr_logged make, with a fixed clock."""

    def __init__(self, nx=64, ny=32, model=A.YH_MODEL_FK3V, mask=True):
        self.p = A.fk_tissue_params(nx, ny)
        self.model = model
        self.has_mask = mask
        self.step = 0
        self.runs = []

    def synchronize(self):
        pass

    def run(self, n, stims=()):
        self.runs.append((self.step, n, tuple(stims)))
        self.step += n

    def sr_step(self, n):
        self.step += n

    def step_count(self):
        return self.step

    def track_tips(self):
        pass

    def get_tips(self):
        return np.zeros((self.step % 3, 5), np.float32)

    def check_finite(self):
        return 0

    def get_sym(self):
        s = A.SymState()
        s.c[0], s.phi[2], s.ntips = 0.5, 0.25, 1
        return s


def test_bytes_per_cell_step():
    assert runlog.bytes_per_cell_step(A.YH_MODEL_FK3V, False) == 24
    assert runlog.bytes_per_cell_step(A.YH_MODEL_FK3V, True) == 25
    assert runlog.bytes_per_cell_step(A.YH_MODEL_REF2V, False) == 16


def test_plain_segments_and_rates(tmp_path, monkeypatch):
    clock = iter(np.arange(0.0, 100.0, 0.5))  # every segment takes 0.5 s
    monkeypatch.setattr(runlog.time, "perf_counter", lambda: next(clock))
    sim = FakeSolver()
    path = tmp_path / "run.jsonl"
    with runlog.RunLog(path) as log:
        lines = runlog.run_logged(sim, 250, log, stims=("s",), every=100,
                                  peak_gbs=1000.0)
    assert [r["step"] for r in lines] == [100, 200, 250]
    assert [r["steps"] for r in lines] == [100, 100, 50]
    assert sim.runs == [(0, 100, ("s",)), (100, 100, ("s",)),
                        (200, 50, ("s",))]
    rate = 64 * 32 * 100 / 0.5
    assert lines[0]["gcell_steps_per_s"] == round(rate / 1e9, 3)
    assert lines[0]["gbps"] == round(rate * 25 / 1e9, 1)
    assert lines[0]["hbm_frac"] == round(rate * 25 / 1e9 / 1000.0, 3)
    assert [r["ntips"] for r in lines] == [1, 2, 1]
    assert all(r["nonfinite"] == 0 for r in lines)
    on_disk = [json.loads(x) for x in path.read_text().splitlines()]
    assert on_disk == lines


def test_sr_lines_carry_the_frame(tmp_path):
    sim = FakeSolver()
    with runlog.RunLog(tmp_path / "sr.jsonl") as log:
        lines = runlog.sr_logged(sim, 30, log, every=16)
    assert [r["step"] for r in lines] == [16, 30]
    assert lines[0]["c"] == [0.5, 0.0, 0.0]
    assert lines[0]["phi"] == [0.0, 0.0, 0.25]
    assert lines[0]["status"] == "YH_OK" and lines[0]["ntips"] == 1


@pytest.mark.gpu
def test_logged_run_on_the_gpu(tmp_path):
    from yolohtli_gb300 import workloads as W
    from yolohtli_gb300.solver import Monodomain
    wl = W.fk_spiral_256(n=128, nsteps=400)
    sim = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid)
    sim.set_state(*wl.state0())
    with runlog.RunLog(tmp_path / "run.jsonl") as log:
        lines = runlog.run_logged(sim, 400, log, stims=wl.stims, every=100,
                                  peak_gbs=6778.7)
    assert [r["step"] for r in lines] == [100, 200, 300, 400]
    assert all(r["nonfinite"] == 0 and r["gcell_steps_per_s"] > 0
               for r in lines)
    ref = Monodomain(wl.p, wl.model, wl.fk, solid=wl.solid)
    ref.set_state(*wl.state0())
    ref.run(400, wl.stims)
    for x, y in zip(sim.get_state(), ref.get_state()):
        assert x.tobytes() == y.tobytes()
    sim.close()
    ref.close()
