// C ABI of include/yolohtli.h: parameter helpers, stateless operators and
// the solver handle.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "yh_kernels.cuh"

namespace yh {

template <typename Real>
StepCoeffs<Real> make_step_coeffs(const yh_param_var &p, int model,
                                  const yh_fk_params *fk) {
  StepCoeffs<Real> a;
  memset(&a, 0, sizeof(a));
  a.nx = p.nx;
  a.ny = p.ny;
  a.model = model;
  a.gate_diff = p.gateDiff ? 1 : 0;
  a.rx = (Real)p.rx;
  a.ry = (Real)p.ry;
  a.rscale = (Real)p.rscale;
  a.dt = (Real)p.dt;
  a.tc = (Real)p.tc;
  a.inv_dt = (Real)(1.0 / p.dt);
  a.mu = (Real)p.mu;
  a.alpha = (Real)p.alpha;
  a.eps = (Real)p.eps;
  a.delta = (Real)p.delta;
  a.gamma = (Real)p.gamma;
  a.beta = (Real)p.beta;
  a.theta = (Real)p.theta;
  {
    // -dt I_sum = dt u (mu (1 - u)(u - alpha) - v) with
    // mu (1 - u)(u - alpha) = -mu u^2 + mu (1 + alpha) u - mu alpha;
    // -dt I_v = dt eps (delta (u - gamma)(beta - u) - v - theta) with
    // delta (u - gamma)(beta - u) = -delta u^2 + delta (beta + gamma) u
    // - delta beta gamma
    const double K = p.dt, Ke = K * p.eps;
    a.pu2 = (Real)(-K * p.mu);
    a.pu1 = (Real)(K * p.mu * (1.0 + p.alpha));
    a.pu0 = (Real)(-K * p.mu * p.alpha);
    a.puv = (Real)(-K);
    a.pv2 = (Real)(-Ke * p.delta);
    a.pv1 = (Real)(Ke * p.delta * (p.beta + p.gamma));
    a.pv0 = (Real)(-Ke * (p.delta * p.beta * p.gamma + p.theta));
    a.pvv = (Real)(-Ke);
    a.rxs = (Real)(p.rx * p.rscale);
    a.rys = (Real)(p.ry * p.rscale);
  }
  if (fk) {
    a.u_c = (Real)fk->u_c;
    a.u_v = (Real)fk->u_v;
    a.u_csi = (Real)fk->u_csi;
    a.k_exp2 = (Real)(-2.0 * fk->k / log(2.0));
    a.inv_td = (Real)(1.0 / fk->tau_d);
    a.inv_tr = (Real)(1.0 / fk->tau_r);
    a.inv_to = (Real)(1.0 / fk->tau_0);
    a.inv_tsi = (Real)(1.0 / fk->tau_si);
    a.inv_tvp = (Real)(1.0 / fk->tau_v_plus);
    a.inv_tv1m = (Real)(1.0 / fk->tau_v1_minus);
    a.inv_tv2m = (Real)(1.0 / fk->tau_v2_minus);
    a.inv_twp = (Real)(1.0 / fk->tau_w_plus);
    a.inv_twm = (Real)(1.0 / fk->tau_w_minus);
    const double s = p.tc * p.dt;
    a.s_td = (Real)(s / fk->tau_d);
    a.s_tr = (Real)(s / fk->tau_r);
    a.s_to = (Real)(s / fk->tau_0);
    a.s_tsi = (Real)(s / fk->tau_si);
    a.s_tvp = (Real)(s / fk->tau_v_plus);
    a.s_tv1m = (Real)(s / fk->tau_v1_minus);
    a.s_tv2m = (Real)(s / fk->tau_v2_minus);
    a.s_twp = (Real)(s / fk->tau_w_plus);
    a.s_twm = (Real)(s / fk->tau_w_minus);
  }
  return a;
}
template StepCoeffs<float> make_step_coeffs<float>(const yh_param_var &, int,
                                                   const yh_fk_params *);
template StepCoeffs<double> make_step_coeffs<double>(const yh_param_var &,
                                                     int, const yh_fk_params *);

// Options this path implements (Euler, 5-point, Neumann, no anisotropy).
int check_params(const yh_param_var *p, int model, const yh_fk_params *fk) {
  if (!p) return YH_EINVAL;
  if (p->nx < 5 || p->ny < 5) return YH_EINVAL;
  if ((long long)p->nx * p->ny > (1LL << 31) - 1) return YH_EINVAL;
  if (model != YH_MODEL_REF2V && model != YH_MODEL_FK3V) return YH_EINVAL;
  if (model == YH_MODEL_FK3V && !fk) return YH_EINVAL;
  if (!(p->dt > 0.0) || !(p->hx > 0.0) || !(p->hy > 0.0)) return YH_EINVAL;
  if (p->timeIntOrder != 1 || p->lap4 != 0 || p->anisotropy || !p->neumannBC)
    return YH_EUNSUPPORTED;
  return YH_OK;
}

static inline int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return YH_OK;
  if (e == cudaErrorMemoryAllocation) return YH_ENOMEM;
  return YH_ECUDA;
}

static inline int nfields(int model) { return model == YH_MODEL_FK3V ? 3 : 2; }

static inline Fld<float> to_fld(const yh_fields &x) {
  return make_fld<float>(x.u, x.v, x.w);
}

}  // namespace yh

using namespace yh;

// ---------------------------------------------------------------------------
// Parameter helpers
// ---------------------------------------------------------------------------

extern "C" int yh_param_derive(yh_param_var *p) {
  if (!p || !(p->hx > 0) || !(p->hy > 0)) return YH_EINVAL;
  // main.cu:149-155 and saveFiles.cu:157-170
  p->rx = p->dt * p->Dxx / (p->hx * p->hx);
  p->ry = p->dt * p->Dyy / (p->hy * p->hy);
  p->rxy = 2.0 * p->Dxy * p->dt / (4.0 * p->hx * p->hy);
  p->rbx = p->Dxx != 0.0 ? p->hx * p->Dxy / (p->Dxx * p->hy) : 0.0;
  p->rby = p->Dyy != 0.0 ? p->hy * p->Dxy / (p->Dyy * p->hx) : 0.0;
  p->invdx = 0.5 / p->hx;
  p->invdy = 0.5 / p->hy;
  p->qx4 = p->dt * p->Dyy / (p->hy * p->hy * 12.0);
  p->qy4 = p->dt * p->Dxx / (p->hx * p->hx * 12.0);
  p->fx4 = p->dt / 12.0;
  p->fy4 = p->dt / 12.0;
  p->memSize = p->nx * p->ny * (int)sizeof(double);
  return YH_OK;
}

extern "C" int yh_param_defaults(yh_param_var *p, int nx, int ny) {
  if (!p || nx < 5 || ny < 5) return YH_EINVAL;
  memset(p, 0, sizeof(*p));
  // saveFiles.cu:105-231, with the Euler / 5-point options of this path.
  p->animate = true;
  p->plotTip = true;
  p->plotTimeSeries = true;
  p->neumannBC = true;
  p->gateDiff = true;
  p->tipAlgorithm = 1;
  p->contourMode = 3;
  p->lap4 = 0;
  p->timeIntOrder = 1;
  p->counterclock = true;
  p->firstFPS = true;
  p->firstIterTip = true;
  p->firstIterContour = true;
  p->nx = nx;
  p->ny = ny;
  p->Lx = 12.0;
  p->Ly = 12.0;
  p->hx = p->Lx / (nx - 1.0);
  p->hy = p->Ly / (ny - 1.0);
  p->dt = 0.02;
  p->diff_par = 0.001;
  p->diff_per = 0.001;
  const double th = p->degrad * 3.14159265359 / 180.0;
  p->Dxx = p->diff_par * cos(th) * cos(th) + p->diff_per * sin(th) * sin(th);
  p->Dyy = p->diff_par * sin(th) * sin(th) + p->diff_per * cos(th) * cos(th);
  p->Dxy = (p->diff_par - p->diff_per) * sin(th) * cos(th);
  p->rscale = 0.01;
  p->physicalTimeLim = 100000.0;
  p->eSize = 2;
  p->point.x = nx / 2;
  p->point.y = ny / 2;
  p->stimPeriod = 600.0;
  p->stimMag = 2.0;
  p->stimDuration = 10.0;
  p->fibThreshold = true;
  p->nc = 100;
  p->stcx = 0.25 * p->Lx;
  p->stcy = 0.25 * p->Ly;
  p->rdomStim = 0.03 * p->Lx;
  p->rdomAPD = 0.15 * p->Lx;
  p->tipOffsetX = 160;
  p->tipOffsetY = 160;
  p->rdomTrapz = 0.5 * ((p->tipOffsetX + p->tipOffsetY) * p->hx);
  p->itPerFrame = 50;
  p->sample = 2.0;
  p->minVarColor = -0.1f;
  p->maxVarColor = 1.1f;
  p->wnx = nx;
  p->wny = ny;
  p->uMin = -0.1f;
  p->uMax = 1.1f;
  p->vMin = -0.1f;
  p->vMax = 0.5f;
  p->contourThresh1 = 0.8;
  p->contourThresh2 = 0.85;
  p->contourThresh3 = 0.7;
  p->Uth = 0.7;
  p->tc = 1.0;
  p->alpha = 0.2;
  p->beta = 1.1;
  p->gamma = 0.0;
  p->delta = 1.0;
  p->eps = 0.005;
  p->mu = 1.0;
  p->theta = 0.0;
  return yh_param_derive(p);
}

extern "C" int yh_fk_defaults(yh_fk_params *fk) {
  if (!fk) return YH_EINVAL;
  fk->tau_d = 0.25;
  fk->tau_r = 50.0;
  fk->tau_si = 45.0;
  fk->tau_0 = 8.3;
  fk->tau_v_plus = 3.33;
  fk->tau_v1_minus = 19.6;
  fk->tau_v2_minus = 1000.0;
  fk->tau_w_plus = 667.0;
  fk->tau_w_minus = 11.0;
  fk->u_c = 0.13;
  fk->u_v = 0.055;
  fk->u_csi = 0.85;
  fk->k = 10.0;
  return YH_OK;
}

extern "C" const char *yh_status_string(int s) {
  switch (s) {
    case YH_OK: return "ok";
    case YH_EINVAL: return "invalid argument";
    case YH_ECUDA: return "CUDA error";
    case YH_ENOMEM: return "out of memory";
    case YH_ESINGULAR: return "singular drift/rotation system";
    case YH_ENONFINITE: return "non-finite state";
    case YH_EOVERFLOW: return "tip buffer overflow";
    case YH_EUNSUPPORTED: return "option not supported on this path";
    case YH_ENOTREADY: return "call order";
    case YH_ETIMEOUT: return "device-side wait timed out";
    case YH_ECORRUPT: return "corrupt checkpoint file";
  }
  return "unknown status";
}

extern "C" const char *yh_version(void) { return "yolohtli_gb300 0.1.0 sm_103a"; }

extern "C" size_t yh_sizeof(const char *type_name) {
  if (!type_name) return 0;
  if (!strcmp(type_name, "yh_param_var")) return sizeof(yh_param_var);
  if (!strcmp(type_name, "yh_fk_params")) return sizeof(yh_fk_params);
  if (!strcmp(type_name, "yh_tip")) return sizeof(yh_tip);
  if (!strcmp(type_name, "yh_fields")) return sizeof(yh_fields);
  if (!strcmp(type_name, "yh_fields64")) return sizeof(yh_fields64);
  if (!strcmp(type_name, "yh_sym_state")) return sizeof(yh_sym_state);
  if (!strcmp(type_name, "yh_stim")) return sizeof(yh_stim);
  if (!strcmp(type_name, "yh_batch_stim")) return sizeof(yh_batch_stim);
  if (!strcmp(type_name, "yh_checkpoint_header"))
    return sizeof(yh_checkpoint_header);
  return 0;
}

// ---------------------------------------------------------------------------
// Stateless operators
// ---------------------------------------------------------------------------

static bool fields_ok(const yh_fields &x, int model) {
  return x.u && x.v && (model != YH_MODEL_FK3V || x.w);
}

extern "C" int yh_reaction_diffusion(const yh_param_var *p, int model,
                                     const yh_fk_params *fk, yh_fields out,
                                     yh_fields in, yh_fields vel_tan,
                                     const uint8_t *solid, void *stream) {
  int st = check_params(p, model, fk);
  if (st) return st;
  if (!fields_ok(out, model) || !fields_ok(in, model)) return YH_EINVAL;
  if (vel_tan.u && !fields_ok(vel_tan, model)) return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  const StepCoeffs<float> a = make_step_coeffs<float>(*p, model, fk);
  return cuda_status(launch_rd_step<float>(
      a, to_fld(in), to_fld(out), to_fld(vel_tan),
      p->solidSwitch ? solid : nullptr, (cudaStream_t)stream));
}

extern "C" int yh_spiral_tip(const yh_param_var *p, const float *g_past,
                             const float *g_present, double physical_time,
                             int *tip_count, yh_tip *tip_vector, int capacity,
                             const uint8_t *solid, void *stream) {
  if (!p || !g_past || !g_present || !tip_count || !tip_vector || capacity < 0)
    return YH_EINVAL;
  if (p->nx < 5 || p->ny < 5) return YH_EINVAL;
  if (p->tipAlgorithm != 1 && p->tipAlgorithm != 2) return YH_EUNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(tip_count, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e);
  (void)solid;  // the hole branch uses a disc, not the mask
  return cuda_status(launch_tips<float>(*p, g_past, g_present,
                                        p->solidSwitch, physical_time,
                                        tip_count, tip_vector,
                                        capacity, nullptr, nullptr, s));
}

extern "C" int yh_pick_centre(const int *tip_count, const yh_tip *tip_vector,
                              int capacity, yh_sym_state *sym, void *stream) {
  if (!tip_count || !tip_vector || !sym || capacity < 0) return YH_EINVAL;
  return cuda_status(launch_pick_centre(tip_count, tip_vector, capacity, sym,
                                        (cudaStream_t)stream));
}

extern "C" size_t yh_phase_integrals_workspace(int nx, int ny) {
  yh_param_var p;
  memset(&p, 0, sizeof(p));
  p.nx = nx;
  p.ny = ny;
  p.tipOffsetX = 160;
  p.tipOffsetY = 160;
  // the largest box: the disc never needs more than twice the grid
  p.tipOffsetX = p.tipOffsetY = 2 * (nx > ny ? nx : ny) + 2;
  return phase_workspace_bytes(p);
}

extern "C" int yh_phase_integrals(const yh_param_var *p, int model,
                                  yh_fields state, yh_fields vel_tan,
                                  yh_fields templ_x, yh_fields templ_y,
                                  yh_fields templ_t, const double *adv_x_rows,
                                  const double *adv_y_cols,
                                  const uint8_t *solid, yh_sym_state *sym,
                                  void *workspace, void *stream) {
  if (!p || !sym || !workspace || !adv_x_rows || !adv_y_cols) return YH_EINVAL;
  if (p->nx < 5 || p->ny < 5) return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  if (!fields_ok(state, model) || !fields_ok(vel_tan, model)) return YH_EINVAL;
  if (templ_x.u && (!fields_ok(templ_x, model) || !fields_ok(templ_y, model) ||
                    !fields_ok(templ_t, model)))
    return YH_EINVAL;
  return cuda_status(launch_phase<float>(
      *p, nfields(model), to_fld(state), to_fld(vel_tan), to_fld(templ_x),
      to_fld(templ_y), to_fld(templ_t), adv_x_rows, adv_y_cols,
      p->solidSwitch ? solid : nullptr, sym, workspace,
      (cudaStream_t)stream));
}

extern "C" int yh_template_slices(const yh_param_var *p, int model,
                                  yh_fields state, yh_fields templ_x,
                                  yh_fields templ_y, yh_fields templ_t,
                                  void *stream) {
  if (!p || !fields_ok(state, model) || !fields_ok(templ_x, model) ||
      !fields_ok(templ_y, model) || !fields_ok(templ_t, model))
    return YH_EINVAL;
  return cuda_status(launch_template<float>(
      *p, nfields(model), to_fld(state), to_fld(templ_x), to_fld(templ_y),
      to_fld(templ_t), (cudaStream_t)stream));
}

extern "C" int yh_comoving_field(const yh_param_var *p, yh_sym_state *sym,
                                 double *adv_x_rows, double *adv_y_cols,
                                 float *adv_x_rows_f32, float *adv_y_cols_f32,
                                 int advance_phi, void *stream) {
  if (!p || !sym || !adv_x_rows || !adv_y_cols) return YH_EINVAL;
  return cuda_status(launch_comoving(*p, sym, adv_x_rows, adv_y_cols,
                                     adv_x_rows_f32, adv_y_cols_f32,
                                     advance_phi != 0, (cudaStream_t)stream));
}

extern "C" int yh_advect_bfecc(const yh_param_var *p, int model,
                               yh_fields out, yh_fields in,
                               const float *adv_x_rows_f32,
                               const float *adv_y_cols_f32,
                               const uint8_t *solid, yh_fields uf,
                               yh_fields ue, void *stream) {
  if (!p || !adv_x_rows_f32 || !adv_y_cols_f32) return YH_EINVAL;
  if (!fields_ok(out, model) || !fields_ok(in, model) ||
      !fields_ok(uf, model) || !fields_ok(ue, model))
    return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  const Fld<float> fi = to_fld(in), fo = to_fld(out);
  bool alias = false;
  for (int f = 0; f < nfields(model); ++f)
    for (int g = 0; g < nfields(model); ++g) alias |= fi.f[f] == fo.f[g];
  if (alias || p->nx < 2 || p->ny < 2)  // in place: the three launches
    return cuda_status(launch_bfecc<float>(
        *p, nfields(model), fi, fo, adv_x_rows_f32, adv_y_cols_f32,
        p->solidSwitch ? solid : nullptr, to_fld(uf), to_fld(ue),
        (cudaStream_t)stream));
  return cuda_status(launch_bfecc_fused(
      *p, nfields(model), fi, fo, adv_x_rows_f32, adv_y_cols_f32,
      p->solidSwitch ? solid : nullptr, (cudaStream_t)stream));
}

extern "C" int yh_advect_bfecc_3pass(const yh_param_var *p, int model,
                                     yh_fields out, yh_fields in,
                                     const float *adv_x_rows_f32,
                                     const float *adv_y_cols_f32,
                                     const uint8_t *solid, yh_fields uf,
                                     yh_fields ue, void *stream) {
  if (!p || !adv_x_rows_f32 || !adv_y_cols_f32) return YH_EINVAL;
  if (!fields_ok(out, model) || !fields_ok(in, model) ||
      !fields_ok(uf, model) || !fields_ok(ue, model))
    return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  return cuda_status(launch_bfecc<float>(
      *p, nfields(model), to_fld(in), to_fld(out), adv_x_rows_f32,
      adv_y_cols_f32, p->solidSwitch ? solid : nullptr, to_fld(uf),
      to_fld(ue), (cudaStream_t)stream));
}

extern "C" int yh_sym_advance(const yh_param_var *p, yh_sym_state *sym,
                              void *stream) {
  if (!p || !sym) return YH_EINVAL;
  return cuda_status(launch_sym_advance(*p, sym, (cudaStream_t)stream));
}

extern "C" int yh_stimulate_box(const yh_param_var *p, float *u,
                                const uint8_t *solid, int i0, int j0, int i1,
                                int j1, float value, void *stream) {
  if (!p || !u) return YH_EINVAL;
  return cuda_status(launch_stimulate<float>(
      u, p->solidSwitch ? solid : nullptr, p->nx, p->ny, i0, j0, i1, j1, value,
      (cudaStream_t)stream));
}

// FP64 instances of the operators above (the same kernel templates).
static bool fields64_ok(const yh_fields64 &x, int model) {
  return x.u && x.v && (model != YH_MODEL_FK3V || x.w);
}

extern "C" int yh_reaction_diffusion_f64(const yh_param_var *p, int model,
                                         const yh_fk_params *fk,
                                         yh_fields64 out, yh_fields64 in,
                                         yh_fields64 vel_tan,
                                         const uint8_t *solid, void *stream) {
  int st = check_params(p, model, fk);
  if (st) return st;
  if (!fields64_ok(out, model) || !fields64_ok(in, model)) return YH_EINVAL;
  if (vel_tan.u && !fields64_ok(vel_tan, model)) return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  const StepCoeffs<double> a = make_step_coeffs<double>(*p, model, fk);
  return cuda_status(launch_rd_step<double>(
      a, make_fld<double>(in.u, in.v, in.w),
      make_fld<double>(out.u, out.v, out.w),
      make_fld<double>(vel_tan.u, vel_tan.v, vel_tan.w),
      p->solidSwitch ? solid : nullptr, (cudaStream_t)stream, nullptr));
}

extern "C" int yh_spiral_tip_f64(const yh_param_var *p, const double *g_past,
                                 const double *g_present,
                                 double physical_time, int *tip_count,
                                 yh_tip *tip_vector, int capacity,
                                 const uint8_t *solid, void *stream) {
  if (!p || !g_past || !g_present || !tip_count || !tip_vector || capacity < 0)
    return YH_EINVAL;
  if (p->nx < 5 || p->ny < 5) return YH_EINVAL;
  if (p->tipAlgorithm != 1 && p->tipAlgorithm != 2) return YH_EUNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(tip_count, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_status(e);
  (void)solid;  // the hole branch uses a disc, not the mask
  return cuda_status(launch_tips<double>(*p, g_past, g_present,
                                         p->solidSwitch, physical_time,
                                         tip_count, tip_vector, capacity,
                                         nullptr, nullptr, s));
}

extern "C" int yh_stimulate_box_f64(const yh_param_var *p, double *u,
                                    const uint8_t *solid, int i0, int j0,
                                    int i1, int j1, double value,
                                    void *stream) {
  if (!p || !u) return YH_EINVAL;
  return cuda_status(launch_stimulate<double>(
      u, p->solidSwitch ? solid : nullptr, p->nx, p->ny, i0, j0, i1, j1, value,
      (cudaStream_t)stream));
}
