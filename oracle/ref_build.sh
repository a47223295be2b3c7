#!/bin/sh
# Compiles the reference's kernel sources, unchanged, where they lie, into
#   oracle/_ref/yolohtli_ref.cubin  (sm_103a device code, loaded by
#                                    oracle/ref_harness.cpp on the GPU machine)
#   oracle/_ref/libref_host.so      (x86 host code of the same sources, for
#                                    CPU checks of solve_matrix and
#                                    parameterSetup in this container)
# Needs the reference sources (YH_REFERENCE, default: where this build
# mounts them); writes only into oracle/_ref/. Nothing of the reference is
# copied. With --if-present it exits 0 without building when the sources
# are not there (the GPU machine, which uses the prebuilt cubin).
set -e
REF=${YH_REFERENCE:-/root/reference}
here=$(cd "$(dirname "$0")" && pwd)
out="$here/_ref"
if [ ! -d "$REF" ]; then
  [ "$1" = "--if-present" ] && exit 0
  echo "reference sources not found at $REF (set YH_REFERENCE)" >&2
  exit 1
fi
mkdir -p "$out/obj"
ARCH="-gencode arch=compute_103a,code=sm_103a"
# the __constant__ definitions of main.cu:40-51 and the globals the kernel
# translation units reference (main.cu is not compiled: it needs GL/GLUT)
cat > "$out/obj/ref_stub.cu" <<STUB
#include "$REF/typeDefinition.cuh"
__constant__ int nx_d, ny_d;
__constant__ REAL dt_d, rx_d, ry_d, hx_d, hy_d, Lx_d, Ly_d, qx4_d, qy4_d, fx4_d, fy4_d;
__constant__ REAL rxy_d, rbx_d, rby_d, rscale_d;
__constant__ REAL invdx_d, invdy_d;
__constant__ REAL tc_d, alpha_d, beta_d, delta_d, eps_d, mu_d, gamma_d, theta_d;
__constant__ REAL boundaryVal_d;
__constant__ bool solidSwitch_d, neumannBC_d, gateDiff_d, anisotropy_d, tipGrad_d;
__constant__ int tipOffsetX_d, tipOffsetY_d;
__constant__ float minVarColor_d, maxVarColor_d;
__constant__ float tipx0_d, tipy0_d;
__constant__ REAL Uth_d, conTh1_d, conTh2_d, conTh3_d;
__constant__ int lap4_d, timeIntOrder_d;
paramVar param;
extern "C" int SOIL_save_screenshot(const char *, int, int, int, int, int) { return 0; }
STUB
KERNEL_TUS="reactionDiffusion advFDBFECC symmetryReduction integralTrapz tipTracker helper_functions spaceAPD"
cubins=""
for tu in $KERNEL_TUS; do
  nvcc $ARCH -rdc=true -std=c++11 -cubin -w "$REF/$tu.cu" -o "$out/obj/$tu.cubin"
  cubins="$cubins $out/obj/$tu.cubin"
done
nvcc $ARCH -rdc=true -std=c++11 -cubin -w "$out/obj/ref_stub.cu" -o "$out/obj/ref_stub.cubin"
nvlink -arch=sm_103a $cubins "$out/obj/ref_stub.cubin" -o "$out/yolohtli_ref.cubin"
# host library: the same sources plus the host-only ones the hot path uses
HOST_TUS="$KERNEL_TUS linearSolver saveFiles printFunctions"
objs=""
for tu in $HOST_TUS; do
  nvcc $ARCH -rdc=true -std=c++11 -Xcompiler -fPIC -w -c "$REF/$tu.cu" -o "$out/obj/$tu.o"
  objs="$objs $out/obj/$tu.o"
done
nvcc $ARCH -rdc=true -std=c++11 -Xcompiler -fPIC -w -c "$out/obj/ref_stub.cu" -o "$out/obj/ref_stub.o"
nvcc $ARCH -rdc=true -shared -Xcompiler -fPIC $objs "$out/obj/ref_stub.o" -o "$out/libref_host.so"
echo "built $out/yolohtli_ref.cubin $out/libref_host.so"
