// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// Headless runner of the reference's own CUDA kernels. oracle/ref_build.sh
// compiles the reference's kernel sources unchanged for sm_103a and links
// them into oracle/_ref/yolohtli_ref.cubin; this harness loads that cubin
// with the CUDA driver API, uploads the reference's __constant__ parameters
// from a paramVar exactly as main.cu:309-402 does, and launches the kernels
// with the reference's launch shapes. No GL, no GLUT, no stdin menu.
//
// Built on the GPU machine by oracle/build_harness.sh (links libcuda). Only the
// GPU parity tests and the fixture generator in tests/golden/ use it.
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../include/yolohtli.h"

namespace {

// The reference's by-value argument structs (typeDefinition.cuh:5-20).
struct StateVar { double *u, *v; };
struct AdvVar { double *x, *y; };
struct SliceVar { double *ux, *uy, *ut, *vx, *vy, *vt; };
struct Real3 { double x, y, t; };
struct alignas(8) Int2 { int x, y; };

CUmodule g_mod = nullptr;
CUfunction g_rd, g_tip, g_slice, g_trapz, g_cxy, g_bfecc;
// analysis kernels (tipTracker.cu:244-517, spaceAPD.cu:18-374); null when
// the cubin predates them
CUfunction g_newton, g_abouzar, g_contour, g_sapd;
char g_err[512];

int fail(const char *what, CUresult r) {
  const char *s = nullptr;
  cuGetErrorString(r, &s);
  snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
  return -1;
}

#define CK(x)                          \
  do {                                 \
    CUresult r_ = (x);                 \
    if (r_ != CUDA_SUCCESS) return fail(#x, r_); \
  } while (0)

template <typename T>
int set_const(const char *name, const T &v) {
  CUdeviceptr d;
  size_t sz;
  CUresult r = cuModuleGetGlobal(&d, &sz, g_mod, name);
  if (r != CUDA_SUCCESS) return fail(name, r);
  if (sz != sizeof(T)) {
    snprintf(g_err, sizeof(g_err), "%s: size %zu != %zu", name, sz, sizeof(T));
    return -1;
  }
  CK(cuMemcpyHtoD(d, &v, sizeof(T)));
  return 0;
}

int launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, unsigned by,
           void **args) {
  if (!f) {
    snprintf(g_err, sizeof(g_err), "kernel not in the cubin (rebuild oracle/_ref)");
    return -1;
  }
  CK(cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, nullptr, args, nullptr));
  return 0;
}

}  // namespace

extern "C" {

const char *refh_error(void) { return g_err; }

int refh_open(const char *cubin_path) {
  if (g_mod) return 0;
  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  CK(cuModuleLoad(&g_mod, cubin_path));
  // Itanium-mangled names of the reference kernels (devicePrototypes.cuh)
  CK(cuModuleGetFunction(&g_rd, g_mod,
                         "_Z24reactionDiffusion_kernelm8stateVarS_S_S_bPbbPdb4int2"));
  CK(cuModuleGetFunction(&g_tip, g_mod, "_Z16spiralTip_kernelmPdS_PbPiP7vec5dynd"));
  CK(cuModuleGetFunction(&g_slice, g_mod,
                         "_Z12slice_kernel8stateVar8sliceVarS0_bb6advVariPbPiP7vec5dyni"));
  CK(cuModuleGetFunction(&g_trapz, g_mod, "_Z12trapz_kernelPdS_S_S_S_S_PiP7vec5dyni"));
  CK(cuModuleGetFunction(&g_cxy, g_mod, "_Z16Cxy_field_kernel6advVar5REAL3S0_Pb"));
  CK(cuModuleGetFunction(&g_bfecc, g_mod,
                         "_Z17advFDBFECC_kernelm8stateVarS_6advVarS_S_S_Pb"));
  if (cuModuleGetFunction(&g_newton, g_mod,
                          "_Z22spiralTipNewton_kernelmPdS_PbPiP7vec5dynd") != CUDA_SUCCESS)
    g_newton = nullptr;
  if (cuModuleGetFunction(&g_abouzar, g_mod,
                          "_Z17abouzarTip_kernelmPdS_PbPiP7vec5dynd") != CUDA_SUCCESS)
    g_abouzar = nullptr;
  if (cuModuleGetFunction(&g_contour, g_mod,
                          "_Z15countour_kernelmPdS_PbS0_PiP6float3fi") != CUDA_SUCCESS)
    g_contour = nullptr;
  if (cuModuleGetFunction(&g_sapd, g_mod,
                          "_Z11sAPD_kernelmiPdS_S_S_S_S_S_S_PbS0_b") != CUDA_SUCCESS)
    g_sapd = nullptr;
  return 0;
}

// The __constant__ uploads of main.cu:309-402 (plus tipx0/tipy0, :373-376).
int refh_set_params(const yh_param_var *p) {
  if (!g_mod) return -1;
  int rc = 0;
  rc |= set_const("nx_d", p->nx);
  rc |= set_const("ny_d", p->ny);
  rc |= set_const("rx_d", p->rx);
  rc |= set_const("ry_d", p->ry);
  rc |= set_const("qx4_d", p->qx4);
  rc |= set_const("qy4_d", p->qy4);
  rc |= set_const("fx4_d", p->fx4);
  rc |= set_const("fy4_d", p->fy4);
  rc |= set_const("hx_d", p->hx);
  rc |= set_const("hy_d", p->hy);
  rc |= set_const("dt_d", p->dt);
  rc |= set_const("invdx_d", p->invdx);
  rc |= set_const("invdy_d", p->invdy);
  rc |= set_const("Lx_d", p->Lx);
  rc |= set_const("Ly_d", p->Ly);
  rc |= set_const("rxy_d", p->rxy);
  rc |= set_const("rbx_d", p->rbx);
  rc |= set_const("rby_d", p->rby);
  rc |= set_const("rscale_d", p->rscale);
  rc |= set_const("boundaryVal_d", p->boundaryVal);
  rc |= set_const("solidSwitch_d", p->solidSwitch);
  rc |= set_const("neumannBC_d", p->neumannBC);
  rc |= set_const("gateDiff_d", p->gateDiff);
  rc |= set_const("anisotropy_d", p->anisotropy);
  rc |= set_const("tipGrad_d", p->tipGrad);
  rc |= set_const("lap4_d", p->lap4);
  rc |= set_const("timeIntOrder_d", p->timeIntOrder);
  rc |= set_const("tipOffsetX_d", p->tipOffsetX);
  rc |= set_const("tipOffsetY_d", p->tipOffsetY);
  rc |= set_const("minVarColor_d", p->minVarColor);
  rc |= set_const("maxVarColor_d", p->maxVarColor);
  rc |= set_const("tipx0_d", p->tipx);
  rc |= set_const("tipy0_d", p->tipy);
  rc |= set_const("Uth_d", p->Uth);
  rc |= set_const("conTh1_d", p->contourThresh1);
  rc |= set_const("conTh2_d", p->contourThresh2);
  rc |= set_const("conTh3_d", p->contourThresh3);
  rc |= set_const("tc_d", p->tc);
  rc |= set_const("alpha_d", p->alpha);
  rc |= set_const("beta_d", p->beta);
  rc |= set_const("gamma_d", p->gamma);
  rc |= set_const("delta_d", p->delta);
  rc |= set_const("eps_d", p->eps);
  rc |= set_const("mu_d", p->mu);
  rc |= set_const("theta_d", p->theta);
  return rc ? -1 : 0;
}

int refh_sync(void) {
  CK(cuCtxSynchronize());
  return 0;
}

// reactionDiffusion_kernel<<<grid2D, block2D>>> (reactionDiffusion.cu:573)
int refh_rd(unsigned gx, unsigned gy, unsigned bx, unsigned by, double *out_u,
            double *out_v, double *in_u, double *in_v, double *J_u,
            double *J_v, double *vt_u, double *vt_v, int reduceSym,
            uint8_t *solid, int stimLock, double *stim, int stimLockMouse,
            int px, int py) {
  size_t pitch = 0;
  StateVar gout{out_u, out_v}, gin{in_u, in_v}, J{J_u, J_v}, vt{vt_u, vt_v};
  bool rs = reduceSym != 0, sl = stimLock != 0, slm = stimLockMouse != 0;
  bool *sol = reinterpret_cast<bool *>(solid);
  Int2 pt{px, py};
  void *args[] = {&pitch, &gout, &gin, &J, &vt, &rs, &sol, &sl, &stim, &slm, &pt};
  return launch(g_rd, gx, gy, bx, by, args);
}

// spiralTip_kernel(pitch, g_past, g_present, tip_plot, tip_count, tip_vector,
// physicalTime) (tipTracker.cu:20); the caller zeroes tip_count first as
// tip_wrapper does (tipTracker.cu:573).
int refh_tip(unsigned gx, unsigned gy, unsigned bx, unsigned by,
             double *g_past, double *g_present, uint8_t *tip_plot,
             int *tip_count, void *tip_vector, double ptime) {
  size_t pitch = 0;
  bool *plot = reinterpret_cast<bool *>(tip_plot);
  void *args[] = {&pitch, &g_past, &g_present, &plot, &tip_count, &tip_vector,
                  &ptime};
  return launch(g_tip, gx, gy, bx, by, args);
}

// slice_kernel (symmetryReduction.cu:72)
int refh_slice(unsigned gx, unsigned gy, unsigned bx, unsigned by, double *gu,
               double *gv, double **slice, double **slice0, int reduceSym,
               int reduceSymStart, double *advx, double *advy, int scheme,
               uint8_t *intglArea, int *tip_count, void *tip_vector,
               int count) {
  StateVar g{gu, gv};
  SliceVar s{slice[0], slice[1], slice[2], slice[3], slice[4], slice[5]};
  SliceVar s0{slice0[0], slice0[1], slice0[2], slice0[3], slice0[4], slice0[5]};
  bool rs = reduceSym != 0, rss = reduceSymStart != 0;
  AdvVar adv{advx, advy};
  bool *ia = reinterpret_cast<bool *>(intglArea);
  void *args[] = {&g,     &s,  &s0,        &rs,         &rss,  &adv,
                  &scheme, &ia, &tip_count, &tip_vector, &count};
  return launch(g_slice, gx, gy, bx, by, args);
}

// trapz_kernel(f, g, h, w, dot, coeffTrapz, tip_count, tip_vector, count)
// (integralTrapz.cu:17); *dot must be zeroed first.
int refh_trapz(unsigned gx, unsigned bx, double *f, double *g, double *h,
               double *w, double *dot, double *coeff, int *tip_count,
               void *tip_vector, int count) {
  void *args[] = {&f, &g, &h, &w, &dot, &coeff, &tip_count, &tip_vector,
                  &count};
  return launch(g_trapz, gx, 1, bx, 1, args);
}

// Cxy_field_kernel(adv, c, phi, solid) (symmetryReduction.cu:20)
int refh_cxy(unsigned gx, unsigned gy, unsigned bx, unsigned by, double *advx,
             double *advy, const double *c, const double *phi,
             uint8_t *solid) {
  AdvVar adv{advx, advy};
  Real3 cc{c[0], c[1], c[2]}, pp{phi[0], phi[1], phi[2]};
  bool *sol = reinterpret_cast<bool *>(solid);
  void *args[] = {&adv, &cc, &pp, &sol};
  return launch(g_cxy, gx, gy, bx, by, args);
}

// advFDBFECC_kernel(pitch, g_out, g_in, adv, uf, ub, ue, solid)
// (advFDBFECC.cu:18)
int refh_bfecc(unsigned gx, unsigned gy, unsigned bx, unsigned by,
               double *out_u, double *out_v, double *in_u, double *in_v,
               double *advx, double *advy, double *uf_u, double *uf_v,
               double *ub_u, double *ub_v, double *ue_u, double *ue_v,
               uint8_t *solid) {
  size_t pitch = 0;
  StateVar gout{out_u, out_v}, gin{in_u, in_v}, uf{uf_u, uf_v},
      ub{ub_u, ub_v}, ue{ue_u, ue_v};
  AdvVar adv{advx, advy};
  bool *sol = reinterpret_cast<bool *>(solid);
  void *args[] = {&pitch, &gout, &gin, &adv, &uf, &ub, &ue, &sol};
  return launch(g_bfecc, gx, gy, bx, by, args);
}

// spiralTipNewton_kernel (tipTracker.cu:244, tipAlgorithm 2) and
// abouzarTip_kernel (tipTracker.cu:434, tipAlgorithm 3), the arguments of
// spiralTip_kernel
int refh_tip_alg(int alg, unsigned gx, unsigned gy, unsigned bx, unsigned by,
                 double *g_past, double *g_present, uint8_t *tip_plot,
                 int *tip_count, void *tip_vector, double ptime) {
  size_t pitch = 0;
  bool *plot = reinterpret_cast<bool *>(tip_plot);
  void *args[] = {&pitch, &g_past, &g_present, &plot, &tip_count, &tip_vector,
                  &ptime};
  return launch(alg == 2 ? g_newton : g_abouzar, gx, gy, bx, by, args);
}

// countour_kernel(pitch, field1, field2, contour_plot, stimArea,
// contour_count, contour_vector, physicalTime, mode) (spaceAPD.cu:18)
int refh_contour(unsigned gx, unsigned gy, unsigned bx, unsigned by,
                 double *field1, double *field2, uint8_t *plot,
                 uint8_t *stim_area, int *count, void *vec, float ptime,
                 int mode) {
  size_t pitch = 0;
  bool *pl = reinterpret_cast<bool *>(plot);
  bool *sa = reinterpret_cast<bool *>(stim_area);
  void *args[] = {&pitch, &field1, &field2, &pl, &sa, &count, &vec, &ptime,
                  &mode};
  return launch(g_contour, gx, gy, bx, by, args);
}

// sAPD_kernel(pitch, count, uold, unew, APD1, APD2, sAPD, dAPD, back, front,
// first, stimArea, stimulate) (spaceAPD.cu:278)
int refh_sapd(unsigned gx, unsigned bx, int count, double *uold, double *unew,
              double *apd1, double *apd2, double *sapd, double *dapd,
              double *back, double *front, uint8_t *first,
              uint8_t *stim_area, int stimulate) {
  size_t pitch = 0;
  bool *fi = reinterpret_cast<bool *>(first);
  bool *sa = reinterpret_cast<bool *>(stim_area);
  bool st = stimulate != 0;
  void *args[] = {&pitch, &count, &uold, &unew, &apd1, &apd2, &sapd, &dapd,
                  &back, &front, &fi, &sa, &st};
  return launch(g_sapd, gx, 1, bx, 1, args);
}

}  // extern "C"
