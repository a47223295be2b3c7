"""Builds libyolohtli_gb300.so in-tree with nvcc for sm_103a.

One nvcc process per translation unit, run in parallel, then one link.
Output: yolohtli_gb300/_build/libyolohtli_gb300.so (git-ignored)."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libyolohtli_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
SOURCES = ["yh_rd.cu", "yh_rd_2s.cu", "yh_rd_tb.cu", "yh_io.cu", "yh_analysis.cu", "yh_rd_resident.cu", "yh_sr.cu", "yh_api.cu", "yh_noalloc.cu", "yh_batch.cu", "yh_adjoint.cu",
           "yh_solver.cu", "yh_compat.cu"]


def _compile(src, out_dir=OUT_DIR, defines=()):
    obj = os.path.join(out_dir, src.replace(".cu", ".o"))
    cmd = ([NVCC] + ARCH + FLAGS + ["-D" + d for d in defines] +
           ["-c", os.path.join(CSRC, src), "-o", obj])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd),
                                                          r.stderr))
    return obj, r.stderr


def build(verbose=False, out_dir=OUT_DIR, defines=()):
    """Compiles every source into out_dir and links
    out_dir/libyolohtli_gb300.so; `defines` are extra -D macros."""
    os.makedirs(out_dir, exist_ok=True)
    lib = os.path.join(out_dir, os.path.basename(LIB))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, out_dir, defines), srcs))
    if verbose:
        for obj, err in results:
            if err.strip():
                sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    subprocess.check_call(cmd)
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
