"""Writes tests/golden/io/: the reference's own host code (oracle/_ref/
libref_host.so, built from the reference sources by oracle/ref_build.sh)
run on fixed inputs:

  dataparamcsv_default.csv / _sr.csv  printParameters (printFunctions.cu:266-403)
                                      on two parameter sets
  param_read_sr.json                  loadParamValues (saveFiles.cu:540-711)
                                      of dataparamcsv_sr.csv: every field it sets
  raw_data.dat                        print2D2column (printFunctions.cu:58-78)
  raw_window.dat                      print2DSubWindow (printFunctions.cu:80-103)
  c_phi_list_sym.dat                  printSym (printFunctions.cu:249-264)
  load_data.npz                       loadData (saveFiles.cu:507-537) of raw_data.dat
  inputs.npz                          the inputs of the above

Run in the container that has the reference (the GPU machine does not need it):
    python tests/golden/make_golden_io.py
"""
import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from yolohtli_gb300 import _abi as A  # noqa: E402

OUT = os.path.join(HERE, "io")
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_host.so")


class FileVar(C.Structure):  # fileVar (typeDefinition.cuh:30-33)
    _fields_ = [(n, C.c_char * 100) for n in (
        "read", "readcsv", "p1D", "p2D", "p2DG", "tip1", "tip2", "sym",
        "contour1", "contour2", "paramFile")]


class StateVar(C.Structure):  # stateVar (typeDefinition.cuh:7-9)
    _fields_ = [("u", C.c_void_p), ("v", C.c_void_p)]


class Real3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("t", C.c_double)]


class StdVector(C.Structure):
    """libstdc++'s std::vector<T>: begin, end, end of storage."""
    _fields_ = [("b", C.c_void_p), ("e", C.c_void_p), ("c", C.c_void_p)]


def params():
    d = A.param_defaults(40, 30)
    s = A.param_defaults(64, 48)
    s.reduceSym = True
    s.solidSwitch = True
    s.recordTip = True
    s.tipAlgorithm = 2
    s.dt = 0.0125
    s.diff_par = 1.0e-3
    s.Dxx = s.Dyy = 1.0e-3
    s.rx, s.ry = 0.0823, 0.0761
    s.point.x, s.point.y = 17, 29
    s.stimPeriod = 312.5
    s.sample = 0.123456789
    s.startRecTime = 7
    s.tipx, s.tipy = 31.75, 22.25
    s.tipOffsetX, s.tipOffsetY = 9, 7
    s.Uth = -0.35
    s.alpha, s.beta = 0.2, 1.1
    s.load, s.save = True, True
    return d, s


FIELDS = [f for f, _ in A.ParamVar._fields_ if not f.startswith("_")]


def main():
    lib = C.CDLL(LIB)
    os.makedirs(OUT, exist_ok=True)
    d, s = params()
    rng = np.random.default_rng(11)
    nx, ny = s.nx, s.ny
    u = rng.uniform(-0.2, 1.2, nx * ny).astype(np.float32).astype(np.float64)
    v = rng.uniform(0.0, 1.0, nx * ny).astype(np.float32).astype(np.float64)
    c = rng.normal(0, 0.05, (7, 3))
    phi = np.cumsum(rng.normal(0, 0.3, (7, 3)), axis=0)
    np.savez(os.path.join(OUT, "inputs.npz"), u=u.astype(np.float32),
             v=v.astype(np.float32), c=c, phi=phi)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            os.makedirs("out")
            pp = lib._Z15printParameters7fileVarP8paramVar
            for name, p in (("default", d), ("sr", s)):
                fv = FileVar()
                fv.paramFile = b"out/"
                fv.read = b"initCond/dataA/dataSpiral.dat"
                pp.argtypes = [FileVar, C.POINTER(A.ParamVar)]
                pp(fv, C.byref(p))
                os.replace("out/dataparamcsv.csv",
                           os.path.join(OUT, "dataparamcsv_%s.csv" % name))
            # the reference's reader on the second file
            q = A.param_defaults(4, 4)
            lp = lib._Z15loadParamValuesPKcP8paramVar
            lp.argtypes = [C.c_char_p, C.POINTER(A.ParamVar)]
            lp(os.path.join(OUT, "dataparamcsv_sr.csv").encode(), C.byref(q))
            got = {}
            for f in FIELDS:
                x = getattr(q, f)
                if hasattr(x, "x") and hasattr(x, "y"):
                    got[f] = [x.x, x.y]
                else:
                    got[f] = x if not isinstance(x, float) else float(x)
            with open(os.path.join(OUT, "param_read_sr.json"), "w") as fh:
                json.dump(got, fh, indent=0, sort_keys=True)
            g = StateVar(u.ctypes.data, v.ctypes.data)
            p2 = lib._Z14print2D2columnPKc8stateVarP8paramVar
            p2.argtypes = [C.c_char_p, StateVar, C.POINTER(A.ParamVar)]
            p2(os.path.join(OUT, "raw_data.dat").encode(), g, C.byref(s))
            pw = lib._Z16print2DSubWindowPKc8stateVarP8paramVar
            pw.argtypes = [C.c_char_p, StateVar, C.POINTER(A.ParamVar)]
            pw(os.path.join(OUT, "raw_window.dat").encode(), g, C.byref(s))
            cl = (Real3 * len(c))(*[Real3(*r) for r in c])
            pl = (Real3 * len(phi))(*[Real3(*r) for r in phi])
            vc = StdVector(C.addressof(cl), C.addressof(cl) + C.sizeof(cl),
                           C.addressof(cl) + C.sizeof(cl))
            vp = StdVector(C.addressof(pl), C.addressof(pl) + C.sizeof(pl),
                           C.addressof(pl) + C.sizeof(pl))
            ps = lib._Z8printSymPKcRSt6vectorI5REAL3SaIS2_EES5_
            ps.argtypes = [C.c_char_p, C.POINTER(StdVector), C.POINTER(StdVector)]
            ps(os.path.join(OUT, "c_phi_list_sym.dat").encode(), C.byref(vc),
               C.byref(vp))
            # loadData of the raw_data file
            ur, vr = np.zeros(nx * ny), np.zeros(nx * ny)
            fv = FileVar()
            fv.read = os.path.join(OUT, "raw_data.dat").encode()
            ld = lib._Z8loadData8stateVar7fileVarP8paramVar
            ld.argtypes = [StateVar, FileVar, C.POINTER(A.ParamVar)]
            ld(StateVar(ur.ctypes.data, vr.ctypes.data), fv, C.byref(s))
            np.savez(os.path.join(OUT, "load_data.npz"), u=ur, v=vr)
        finally:
            os.chdir(cwd)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
