"""The reference's interchange files (layer 4 of include/yolohtli.h) against
the reference's own writers and readers: tests/golden/io/ was written by
printParameters, loadParamValues, print2D2column, print2DSubWindow, printSym
and loadData themselves (tests/golden/make_golden_io.py). No GPU."""
import json
import os

import numpy as np
import pytest

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import refio
from yolohtli_gb300.ops import YolohtliError

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")

# the parameter sets of make_golden_io.params()
import importlib.util  # noqa: E402
_spec = importlib.util.spec_from_file_location(
    "make_golden_io", os.path.join(os.path.dirname(G), "make_golden_io.py"))
MG = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(MG)


def _read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("case", [0, 1])
def test_param_csv_is_byte_identical_to_the_references(tmp_path, case):
    p = MG.params()[case]
    name = ("default", "sr")[case]
    out = tmp_path / "dataparamcsv.csv"
    ic = "initCond/dataA/dataSpiral.dat" if p.load else None
    res = "out/" if p.save else None
    refio.write_param_csv(out, p, ic, res)
    assert _read(out) == _read(os.path.join(G, "dataparamcsv_%s.csv" % name))


def test_param_csv_reads_as_the_references_reader():
    q = refio.read_param_csv(os.path.join(G, "dataparamcsv_sr.csv"))
    want = json.load(open(os.path.join(G, "param_read_sr.json")))
    # the fields the reference's reader sets (others keep the start values)
    for f in ("saveEveryIt", "plotTip", "recordTip", "reduceSym", "reduceSymStart",
              "solidSwitch", "neumannBC", "gateDiff", "tipAlgorithm", "lap4",
              "timeIntOrder", "nx", "ny", "Lx", "Ly", "hx", "hy", "dt", "Dxx",
              "Dyy", "rx", "ry", "rscale", "invdx", "invdy", "startRecTime",
              "eSize", "point", "stimPeriod", "fibThreshold", "tipOffsetX",
              "tipOffsetY", "itPerFrame", "sample", "tipx", "tipy", "Uth", "tc",
              "alpha", "beta", "gamma", "delta", "eps", "mu", "theta", "count",
              "physicalTime", "animate"):
        x = getattr(q, f)
        if hasattr(x, "x"):
            x = [x.x, x.y]
        assert x == want[f], (f, x, want[f])
    # a round trip through this library's writer and reader
    p = MG.params()[1]
    assert q.nx == p.nx and q.tipOffsetY == p.tipOffsetY
    assert [q.point.x, q.point.y] == [p.point.y, p.point.x]  # the reference's swap


def test_raw_data_window_and_sym_list_are_byte_identical(tmp_path):
    inp = np.load(os.path.join(G, "inputs.npz"))
    p = MG.params()[1]
    refio.write_raw_data(tmp_path / "raw_data.dat", p, inp["u"], inp["v"])
    assert _read(tmp_path / "raw_data.dat") == _read(os.path.join(G, "raw_data.dat"))
    refio.write_raw_window(tmp_path / "w.dat", p, inp["u"], inp["v"])
    assert _read(tmp_path / "w.dat") == _read(os.path.join(G, "raw_window.dat"))
    refio.write_sym_list(tmp_path / "s.dat", inp["c"], inp["phi"])
    assert _read(tmp_path / "s.dat") == _read(os.path.join(G, "c_phi_list_sym.dat"))


def test_raw_data_reads_as_the_references_loader(tmp_path):
    p = MG.params()[1]
    u, v = refio.read_raw_data(os.path.join(G, "raw_data.dat"), p)
    ref = np.load(os.path.join(G, "load_data.npz"))
    assert np.array_equal(u, ref["u"].astype(np.float32))
    assert np.array_equal(v, ref["v"].astype(np.float32))


def test_tip_files_append_as_the_reference_does(tmp_path):
    # printTip (printFunctions.cu:149-197): "x y vx vy t" per tip with %f,
    # the count on the size file only when there are tips, truncated on the
    # first save and appended after
    a, b = tmp_path / "dataTip.dat", tmp_path / "dataTipSize.dat"
    t1 = [(1.5, 2.25, 0.0, -1.0, 10.0), (3.0, 4.0, 0.5, 0.25, 10.0)]
    refio.write_tips(a, b, t1, append=False)
    refio.write_tips(a, b, [], append=True)
    refio.write_tips(a, b, [(7.125, 8.0, 1.0, 2.0, 12.5)], append=True)
    assert a.read_text() == ("1.500000 2.250000 0.000000 -1.000000 10.000000\n"
                             "3.000000 4.000000 0.500000 0.250000 10.000000\n"
                             "7.125000 8.000000 1.000000 2.000000 12.500000\n")
    assert b.read_text() == "2\n1\n"
    refio.write_tips(a, b, t1[:1], append=False)
    assert b.read_text() == "1\n"


def test_bad_paths_and_windows_are_refused(tmp_path):
    p = MG.params()[1]
    u = np.zeros(p.nx * p.ny, np.float32)
    with pytest.raises(YolohtliError):
        refio.read_param_csv(tmp_path / "missing.csv")
    q = p.copy()
    q.tipx = 2.0  # the window would start left of the grid
    with pytest.raises(YolohtliError):
        refio.write_raw_window(tmp_path / "w.dat", q, u, u)
    short = tmp_path / "short.csv"
    short.write_text("a,1\nb,2\n")
    with pytest.raises(YolohtliError):
        refio.read_param_csv(short)
