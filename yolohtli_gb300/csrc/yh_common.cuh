// Shared device definitions of the yolohtli_gb300 kernels (sm_103a).
//
// Fields are structure-of-arrays, row-major, idx = i + nx*j (the reference's
// I2D, typeDefinition.cuh:129). Every kernel is a template on the element
// type `Real`: float is the product path; double instantiates the same code
// for the FP64 drop-in of the reference's own symbols (yh_compat.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/yolohtli.h"

namespace yh {

// Maximum number of state variables of any model (FK3V: u, v, w).
constexpr int kMaxFields = 3;

template <typename Real>
struct Fld {
  Real *f[kMaxFields];
};

template <typename Real>
__host__ __device__ inline Fld<Real> make_fld(Real *u, Real *v, Real *w) {
  Fld<Real> r;
  r.f[0] = u;
  r.f[1] = v;
  r.f[2] = w;
  return r;
}

// Mirror index about the edge cell, coord_i/coord_j of the reference
// (helper_functions.cu:69-79), valid for -2 <= i <= n+1 and n >= 3.
__host__ __device__ __forceinline__ int mirror(int i, int n) {
  return i < 0 ? -i : (i >= n ? 2 * (n - 1) - i : i);
}

// Coefficients of one explicit step, computed on the host from the
// parameter struct and passed by value (the reference keeps them in
// process-global __constant__ memory, main.cu:40-51, which rules out
// several grids or parameter sets in one process).
template <typename Real>
struct StepCoeffs {
  int nx, ny;
  int model;       // YH_MODEL_*
  int gate_diff;   // REF2V: v diffuses with rscale
  Real rx, ry, rscale, dt, tc, inv_dt;
  // REF2V (reactionDiffusion.cu:131-141)
  Real mu, alpha, eps, delta, gamma, beta, theta;
  // FK3V (Fenton & Karma 1998) with reciprocals precomputed
  Real u_c, u_v, u_csi;
  Real k_exp2;      // -2*k*log2(e): 1 + tanh(k x) = 2/(1 + 2^(k_exp2 x))
  Real inv_td, inv_tr, inv_to, inv_tsi, inv_tvp, inv_tv1m, inv_tv2m;
  Real inv_twp, inv_twm;
  // the same rates pre-multiplied by tc*dt (FP32 update, fk3v_update)
  Real s_td, s_tr, s_to, s_tsi, s_tvp, s_tv1m, s_tv2m, s_twp, s_twm;
};

// Hole coefficients along one axis (reactionDiffusion.cu:162-169):
// weights (lo, centre, hi) for the neighbours on each side. Equivalent to a
// mirror ghost at a hole face and no flux through a cell with holes on both
// sides.
template <typename Real>
__device__ __forceinline__ void hole_coeffs(bool lo, bool c, bool hi,
                                            Real &wlo, Real &wc, Real &whi) {
  wlo = (lo && hi) && (lo && c) ? Real(1) : ((lo && c) ? Real(2) : Real(0));
  wc = c ? ((lo || hi) ? Real(2) : Real(0)) : Real(0);
  whi = (lo && hi) && (c && hi) ? Real(1) : ((c && hi) ? Real(2) : Real(0));
}

// Reaction right-hand sides (multiplied by dt where the reference does):
//   REF2V: ru = -dt*I_sum, rv = -dt*I_v (reactionDiffusion.cu:131-141,498-499)
//   FK3V:  ru = -dt*J_ion, rv = dt*dv/dt, rw = dt*dw/dt
template <typename Real>
__device__ __forceinline__ void ref2v_currents(const StepCoeffs<Real> &a,
                                               Real u, Real v, Real &I_sum,
                                               Real &I_v) {
  I_sum = -(a.mu * u * (Real(1) - u) * (u - a.alpha) - u * v);
  I_v = -(a.eps * (a.delta * (u - a.gamma) * (a.beta - u) - v - a.theta));
}

// Programmatic dependent launch (PTX griddepcontrol, sm_90+). A kernel
// launched with programmatic stream serialization may start while its
// predecessor drains; grid_dep_wait blocks until the predecessor grid has
// completed and its writes are visible, so it goes before the first global
// access. grid_dep_launch lets the successor's blocks be scheduled once
// every block of this grid has issued it. Both are no-ops in a kernel
// launched without the attribute.
__device__ __forceinline__ void grid_dep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void grid_dep_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// PTX approximate base-2 exponential and reciprocal (one MUFU operation
// each; relative error below 2^-22), enough for the 1e-5 FP32 budget.
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float fk_sigmoid(const StepCoeffs<float> &a,
                                            float u) {
  // (1 + tanh(k (u - u_csi))) / 2 = 1 / (1 + exp(-2k (u - u_csi)))
  return rcp_approx(1.0f + ex2_approx(a.k_exp2 * (u - a.u_csi)));
}
__device__ __forceinline__ double fk_sigmoid(const StepCoeffs<double> &a,
                                             double u) {
  return 1.0 / (1.0 + exp2(a.k_exp2 * (u - a.u_csi)));
}

// FK3V: ionic current J and gate rates (Fenton & Karma 1998, eqs. 2-6).
template <typename Real>
__device__ __forceinline__ void fk3v_rates(const StepCoeffs<Real> &a, Real u,
                                           Real v, Real w, Real &J, Real &gv,
                                           Real &gw) {
  const bool p = u >= a.u_c;
  const bool q = u >= a.u_v;
  const Real jfi = p ? -v * (Real(1) - u) * (u - a.u_c) * a.inv_td : Real(0);
  const Real jso = p ? a.inv_tr : u * a.inv_to;
  const Real jsi = -w * fk_sigmoid(a, u) * a.inv_tsi;
  J = jfi + jso + jsi;
  const Real itvm = q ? a.inv_tv1m : a.inv_tv2m;
  gv = p ? -v * a.inv_tvp : (Real(1) - v) * itvm;
  gw = p ? -w * a.inv_twp : (Real(1) - w) * a.inv_twm;
}

// One FK3V Euler update in FP32 with the rates pre-scaled by tc*dt:
//   u' = u + tc*du - tc*dt*J,  v' = v + tc*dt*dv/dt,  w' = w + tc*dt*dw/dt
// (the same step as fk3v_rates + the reference's update
// u0 += tc*rhs, reactionDiffusion.cu:498-513, with fewer operations).
// du is the scaled Laplacian rx*(..) + ry*(..). Returns the tangent rhs/dt
// pieces through ru, rv, rw when the caller needs them.
__device__ __forceinline__ void fk3v_update(const StepCoeffs<float> &a,
                                            float u, float v, float w,
                                            float du, float &un, float &vn,
                                            float &wn) {
  const bool p = u >= a.u_c;
  const bool q = u >= a.u_v;
  const float sig = fk_sigmoid(a, u);
  const float jfi = -v * ((1.f - u) * (u - a.u_c)) * a.s_td;
  const float Jd = (p ? jfi + a.s_tr : u * a.s_to) - w * sig * a.s_tsi;
  un = fmaf(a.tc, du, u) - Jd;
  const float sv = q ? a.s_tv1m : a.s_tv2m;
  vn = p ? v - v * a.s_tvp : fmaf(1.f - v, sv, v);
  wn = p ? w - w * a.s_twp : fmaf(1.f - w, a.s_twm, w);
}

// Hole pattern of one axis as 2 bits: 0 (1,2,1), 1 (2,2,0), 2 (0,2,2),
// 3 (0,0,0) — the coefficient triples of reactionDiffusion.cu:162-169.
__device__ __forceinline__ uint32_t hole_pattern(bool lo, bool c, bool hi) {
  if (!c) return 3u;
  return lo ? (hi ? 0u : 1u) : (hi ? 2u : 3u);
}
__device__ __forceinline__ void pattern_weights(uint32_t pat, float &wlo,
                                                float &wc, float &whi) {
  wlo = pat == 0u ? 1.f : (pat == 1u ? 2.f : 0.f);
  whi = pat == 0u ? 1.f : (pat == 2u ? 2.f : 0.f);
  wc = pat == 3u ? 0.f : 2.f;
}

// New u, v, w of one cell from its scaled Laplacian du: the FP32 FK3V
// update of the single-step kernels (fk3v_update), or the reference form
// for REF2V without gate diffusion (reactionDiffusion.cu:131-141,498-513).
template <int MODEL>
__device__ __forceinline__ void tb_update(const StepCoeffs<float> &a, float u,
                                          float v, float w, float du,
                                          float &un, float &vn, float &wn) {
  if (MODEL == YH_MODEL_FK3V) {
    fk3v_update(a, u, v, w, du, un, vn, wn);
  } else {
    float I_sum, I_v;
    ref2v_currents(a, u, v, I_sum, I_v);
    un = u + a.tc * (du - a.dt * I_sum);
    vn = v + a.tc * (0.f - a.dt * I_v);
    wn = 0.f;
  }
}

// Parameters of the symmetry-reduction kernels.
template <typename Real>
struct SymCoeffs {
  int nx, ny;
  int nf;
  int r2;          // tipOffsetX*tipOffsetY: disc radius squared (cells)
  int box;         // side of the disc's bounding box (cells)
  Real hx, hy, invdx, invdy, dt, tc;
  Real Rx_scale, Ry_scale;  // dt/hx, dt/hy
  double hxhy;
  double Uth;
};

}  // namespace yh
