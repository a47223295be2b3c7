"""Generates tests/golden/ref_host.npz from the reference's own host code
(oracle/_ref/libref_host.so, built from the reference sources by
oracle/ref_build.sh; x86 only, so it runs in the build container):
  param_*   every field of parameterSetup() (saveFiles.cu:105-231)
  solve_*   solve_matrix() (symmetryReduction.cu:329-420) on seeded 3x3
            systems of phase integrals, rotated by phi.t
Run:  python tests/golden/make_golden_host.py [out.npz]
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from yolohtli_gb300 import _abi as A  # noqa: E402


class Real3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("t", C.c_double)]


def main(out):
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_host.so"))
    ps = lib._Z14parameterSetup8paramVar  # paramVar parameterSetup(paramVar)
    ps.restype = A.ParamVar
    ps.argtypes = [A.ParamVar]
    sm = lib._Z12solve_matrix5REAL3S_Pd  # REAL3 solve_matrix(REAL3, REAL3, REAL*)
    sm.restype = Real3
    sm.argtypes = [Real3, Real3, C.POINTER(C.c_double)]
    g = {}
    q = ps(A.ParamVar())
    g["param_bytes"] = np.frombuffer(bytes(q), np.uint8)
    rng = np.random.default_rng(11)
    Is, phis, cs = [], [], []
    for k in range(40):
        I = rng.standard_normal(12)
        if k % 4 == 0:  # realistic scale: integrals ~ 1e-2..1e2
            I *= 10.0 ** rng.uniform(-2, 2, 12)
        phi = np.array([0.0, 0.0, rng.uniform(-7, 7)])
        c = sm(Real3(0, 0, 0), Real3(*phi), I.ctypes.data_as(C.POINTER(C.c_double)))
        Is.append(I)
        phis.append(phi)
        cs.append([c.x, c.y, c.t])
    g["solve_I"] = np.array(Is)
    g["solve_phi"] = np.array(phis)
    g["solve_c"] = np.array(cs)
    np.savez_compressed(out, **g)
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.path.join(ROOT, "tests", "golden", "ref_host.npz"))
