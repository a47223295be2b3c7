"""The C ABI: the library loads, exports every symbol the headers declare,
and its structs match the reference's layout (CPU only, no compute calls)."""
import ctypes as C
import json
import os
import re

import numpy as np

from yolohtli_gb300 import _abi as A
from yolohtli_gb300 import load

from conftest import GOLDEN, ROOT


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(yh_[a-z0-9_]+)\s*\(", src)))


def test_library_loads_and_exports_all_declared_symbols():
    lib = load()
    names = declared("yolohtli.h")
    assert len(names) > 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []


REFERENCE_HOST_SYMBOLS = [  # hostPrototypes.h:22-42, as the reference exports them
    "_Z25reactionDiffusion_wrapperm4dim3S_8stateVarS0_S0_S0_bPbbPdb4int2",
    "_Z11tip_wrapperm4dim3S_8stateVarS0_S0_dibPbPiP7vec5dyn",
    "_Z13slice_wrapperm4dim3S_8stateVar8sliceVarS1_bb6advVariPbPiP7vec5dyni",
    "_Z17Cxy_field_wrapperm4dim3S_6advVar5REAL3S1_Pb",
    "_Z18advFDBFECC_wrapperm4dim3S_8stateVarS0_6advVarS0_S0_S0_Pb",
    "_Z12solve_matrix5REAL3S_Pd",
    "_Z13trapz_wrapper4dim3S_8sliceVarS0_8stateVarPdS2_PiP7vec5dyni",
    # the contour / space-APD analysis (hostPrototypes.h:46-51)
    "_Z16countour_wrapperm4dim3S_PdS0_PbS1_PiP6float3fi",
    "_Z12sAPD_wrapperm4dim3S_iPdS0_S0_S0_S0_S0_S0_S0_PbS1_b",
]


def test_compat_exports_the_reference_host_symbols():
    lib = load()
    for name in REFERENCE_HOST_SYMBOLS + declared("yolohtli_compat.h"):
        assert hasattr(lib, name), name
    ref = os.path.join(ROOT, "oracle", "_ref", "libref_host.so")
    if os.path.exists(ref):  # the reference's own host library, built here
        r = C.CDLL(ref)
        for name in REFERENCE_HOST_SYMBOLS:
            assert hasattr(r, name), name


def test_struct_sizes_match_ctypes():
    lib = load()
    for name, ct in [("yh_param_var", A.ParamVar), ("yh_fk_params", A.FKParams),
                     ("yh_tip", A.Tip), ("yh_fields", A.Fields), ("yh_fields64", A.Fields64),
                     ("yh_sym_state", A.SymState), ("yh_stim", A.Stim),
                     ("yh_batch_stim", A.BatchStim),
                     ("yh_checkpoint_header", A.CheckpointHeader)]:
        assert lib.yh_sizeof(name.encode()) == C.sizeof(ct), name


def test_param_layout_is_the_references_paramVar():
    ref = json.load(open(os.path.join(GOLDEN, "paramvar_layout.json")))
    assert ref["sizeof"] == C.sizeof(A.ParamVar)
    for name, off in ref["offsets"].items():
        assert getattr(A.ParamVar, name).offset == off, name
    assert set(ref["offsets"]) == set(A.PARAM_FIELD_NAMES)


def test_param_defaults_match_reference_parameterSetup(golden_host):
    ref = A.ParamVar()
    raw = golden_host["param_bytes"].tobytes()
    C.memmove(C.byref(ref), raw, C.sizeof(ref))
    lib = load()
    p = A.ParamVar()
    assert lib.yh_param_defaults(C.byref(p), ref.nx, ref.ny) == 0
    # this path runs Euler / 5-point (the reference defaults to RK4 / lap4)
    assert (ref.timeIntOrder, ref.lap4) == (4, 4)
    assert (p.timeIntOrder, p.lap4) == (1, 0)
    for name in A.PARAM_FIELD_NAMES:
        # memSize is set later by main.cu:213, not by parameterSetup
        if name in ("timeIntOrder", "lap4", "point", "pointStim", "memSize"):
            continue
        a, b = getattr(p, name), getattr(ref, name)
        if isinstance(a, float):
            assert a == b or abs(a - b) <= 1e-15 * abs(b), name
        else:
            assert a == b, name
    assert (p.point.x, p.point.y) == (ref.point.x, ref.point.y)
    q = A.param_defaults(ref.nx, ref.ny)
    assert bytes(q) == bytes(p)


def test_status_strings_and_fk_defaults():
    lib = load()
    assert lib.yh_status_string(A.YH_ESINGULAR) == b"singular drift/rotation system"
    fk = A.FKParams()
    assert lib.yh_fk_defaults(C.byref(fk)) == 0
    assert bytes(fk) == bytes(A.fk_defaults())


def test_invalid_arguments_are_rejected_without_a_gpu():
    lib = load()
    p = A.param_defaults(64, 64)
    h = C.c_void_p()
    fk = A.fk_defaults()
    assert lib.yh_create(C.byref(p), 7, C.byref(fk), None, None, C.byref(h)) == A.YH_EINVAL
    q = p.copy()
    q.timeIntOrder = 4
    assert lib.yh_create(C.byref(q), 0, None, None, None, C.byref(h)) == A.YH_EUNSUPPORTED
    q = p.copy()
    q.nx = 2
    assert lib.yh_create(C.byref(q), 0, None, None, None, C.byref(h)) == A.YH_EINVAL
    q = p.copy()
    q.solidSwitch = True  # holes requested without a mask
    assert lib.yh_create(C.byref(q), 0, None, None, None, C.byref(h)) == A.YH_EINVAL
    assert lib.yh_create(C.byref(p), 1, None, None, None, C.byref(h)) == A.YH_EINVAL


C_PROGRAM = r"""
#include <stdio.h>
#include "yolohtli.h"
int main(void) {
  yh_param_var p;
  int rc = yh_param_defaults(&p, 64, 48);
  printf("%d %d %d %s\n", rc, p.nx, p.ny, yh_status_string(YH_EINVAL));
  return rc;
}
"""


def test_header_is_c_and_a_c_program_links_against_the_library(tmp_path):
    # the C ABI as a C caller sees it: the header compiles as pedantic C99
    # and as C++11, and a C program links against the library and calls its
    # host-side functions (no GPU needed)
    import shutil
    import subprocess
    import pytest
    if shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("no C compiler")
    inc = os.path.join(ROOT, "include")
    src = tmp_path / "prog.c"
    src.write_text(C_PROGRAM)
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror",
                           "-pedantic", "-fsyntax-only", "-I", inc, str(src)])
    subprocess.check_call(["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror",
                           "-fsyntax-only", "-I", inc, "-x", "c++", str(src)])
    libdir = os.path.dirname(load()._name)
    exe = tmp_path / "prog"
    subprocess.check_call(["gcc", "-std=c99", "-I", inc, str(src), "-o", str(exe),
                           "-L", libdir, "-lyolohtli_gb300",
                           "-Wl,-rpath," + libdir])
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True)
    assert out.stdout.split()[:3] == ["0", "64", "48"]
    assert "invalid" in out.stdout
