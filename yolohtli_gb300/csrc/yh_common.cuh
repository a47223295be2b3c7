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
  // the REF2V reaction terms as polynomials in u with dt folded in
  // (ref2v_rhs_poly), and the gate's diffusion coefficients rx*rscale,
  // ry*rscale
  Real pu2, pu1, pu0, puv, pv2, pv1, pv0, pvv, rxs, rys;
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

// The REF2V right-hand sides r0 = du - dt I_sum, r1 = dv - dt I_v
// (reactionDiffusion.cu:131-141,498-499) with the currents expanded into
// polynomials of u and dt folded into their coefficients
// (make_step_coeffs):
//   r0 = du + u (pu2 u^2 + pu1 u + pu0 + puv v)
//   r1 = dv + pv2 u^2 + pv1 u + pv0 + pvv v
// in Horner form: 8 FP64 operations against the reference order's 15; the
// two orders round differently (about 1e-16 relative a step).
template <typename Real>
__device__ __forceinline__ void ref2v_rhs_poly(const StepCoeffs<Real> &a,
                                               Real u, Real v, Real du,
                                               Real dv, Real &r0, Real &r1) {
  r0 = fma(u, fma(a.puv, v, fma(fma(a.pu2, u, a.pu1), u, a.pu0)), du);
  r1 = fma(a.pvv, v, fma(fma(a.pv2, u, a.pv1), u, a.pv0)) + dv;
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
// du is the scaled Laplacian (lap5). Every operation is written with its
// rounding (__f*_rn), so the scalar form and the two-cell f32x2 form
// (fk3v_update2) give the same bits:
//   x = (u - u_csi) k2;  sig = 1 / (2^x + 1)
//   a4 = v ((1 - u)(u - u_c));  J1 = p ? s_tr - a4 s_td : u s_to
//   Jd = J1 - (w sig) s_tsi;  u' = (u + du tc) - Jd
//   v' = p ? v - v s_tvp : v + (1 - v) (q ? s_tv1m : s_tv2m)
//   w' = p ? w - w s_twp : w + (1 - w) s_twm
// with p = u >= u_c, q = u >= u_v.
__device__ __forceinline__ void fk3v_update(const StepCoeffs<float> &a,
                                            float u, float v, float w,
                                            float du, float &un, float &vn,
                                            float &wn) {
  const bool p = u >= a.u_c, q = u >= a.u_v;
  const float x = __fmul_rn(__fsub_rn(u, a.u_csi), a.k_exp2);
  const float sig = rcp_approx(__fadd_rn(ex2_approx(x), 1.f));
  const float a4 = __fmul_rn(v, __fmul_rn(__fsub_rn(1.f, u), __fsub_rn(u, a.u_c)));
  const float jp = __fmaf_rn(a4, -a.s_td, a.s_tr);
  const float jn = __fmul_rn(u, a.s_to);
  const float Jd = __fmaf_rn(__fmul_rn(w, sig), -a.s_tsi, p ? jp : jn);
  un = __fsub_rn(__fmaf_rn(du, a.tc, u), Jd);
  const float vp = __fmaf_rn(v, -a.s_tvp, v);
  const float vm = __fmaf_rn(__fsub_rn(1.f, v), q ? a.s_tv1m : a.s_tv2m, v);
  vn = p ? vp : vm;
  const float wp = __fmaf_rn(w, -a.s_twp, w);
  const float wm = __fmaf_rn(__fsub_rn(1.f, w), a.s_twm, w);
  wn = p ? wp : wm;
}

// Two FP32 lanes in one 64-bit register for the sm_100+ packed f32x2
// arithmetic (PTX add/sub/mul/fma .rn.f32x2: each lane rounds as the scalar
// instruction does, two lanes per issued instruction).
struct F2 {
  unsigned long long r;
};
__device__ __forceinline__ F2 f2(float lo, float hi) {
  F2 p;
  asm("mov.b64 %0, {%1, %2};" : "=l"(p.r) : "f"(lo), "f"(hi));
  return p;
}
__device__ __forceinline__ F2 f2(float x) { return f2(x, x); }
__device__ __forceinline__ void f2_split(F2 p, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(p.r));
}
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
  return d;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
  return d;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.r) : "l"(a.r), "l"(b.r));
  return d;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  F2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.r) : "l"(a.r), "l"(b.r), "l"(c.r));
  return d;
}

// Coefficients of the packed FK3V update as f32x2 lane pairs (each value
// in both lanes) and the scalars of its lane selects, read through one
// interface from two sources: FkPairsAt builds each pair where it is used
// (from the coefficients in a kernel parameter or shared memory), FkPairs
// holds them built once, for a kernel that updates many cells per thread
// and keeps them in registers. Both give the same values.
struct FkPairsAt {
  const StepCoeffs<float> &a;
  __device__ __forceinline__ F2 one() const { return f2(1.f); }
  __device__ __forceinline__ F2 m2() const { return f2(-2.f); }
  __device__ __forceinline__ F2 u_csi() const { return f2(a.u_csi); }
  __device__ __forceinline__ F2 k_exp2() const { return f2(a.k_exp2); }
  __device__ __forceinline__ F2 u_c() const { return f2(a.u_c); }
  __device__ __forceinline__ F2 m_s_td() const { return f2(-a.s_td); }
  __device__ __forceinline__ F2 s_tr() const { return f2(a.s_tr); }
  __device__ __forceinline__ F2 s_to() const { return f2(a.s_to); }
  __device__ __forceinline__ F2 m_s_tsi() const { return f2(-a.s_tsi); }
  __device__ __forceinline__ F2 tc() const { return f2(a.tc); }
  __device__ __forceinline__ F2 m_s_tvp() const { return f2(-a.s_tvp); }
  __device__ __forceinline__ F2 m_s_twp() const { return f2(-a.s_twp); }
  __device__ __forceinline__ F2 s_twm() const { return f2(a.s_twm); }
  __device__ __forceinline__ F2 rx() const { return f2(a.rx); }
  __device__ __forceinline__ F2 ry() const { return f2(a.ry); }
  __device__ __forceinline__ float u_c1() const { return a.u_c; }
  __device__ __forceinline__ float u_v1() const { return a.u_v; }
  __device__ __forceinline__ float s_tv1m() const { return a.s_tv1m; }
  __device__ __forceinline__ float s_tv2m() const { return a.s_tv2m; }
};
struct FkPairs {
  F2 p_one, p_m2, p_u_csi, p_k_exp2, p_u_c, p_m_s_td, p_s_tr, p_s_to,
      p_m_s_tsi, p_tc, p_m_s_tvp, p_m_s_twp, p_s_twm, p_rx, p_ry;
  float p_u_c1, p_u_v1, p_s_tv1m, p_s_tv2m;
  __device__ __forceinline__ explicit FkPairs(const StepCoeffs<float> &a) {
    const FkPairsAt c{a};
    p_one = c.one();
    p_m2 = c.m2();
    p_u_csi = c.u_csi();
    p_k_exp2 = c.k_exp2();
    p_u_c = c.u_c();
    p_m_s_td = c.m_s_td();
    p_s_tr = c.s_tr();
    p_s_to = c.s_to();
    p_m_s_tsi = c.m_s_tsi();
    p_tc = c.tc();
    p_m_s_tvp = c.m_s_tvp();
    p_m_s_twp = c.m_s_twp();
    p_s_twm = c.s_twm();
    p_rx = c.rx();
    p_ry = c.ry();
    p_u_c1 = c.u_c1();
    p_u_v1 = c.u_v1();
    p_s_tv1m = c.s_tv1m();
    p_s_tv2m = c.s_tv2m();
  }
  __device__ __forceinline__ F2 one() const { return p_one; }
  __device__ __forceinline__ F2 m2() const { return p_m2; }
  __device__ __forceinline__ F2 u_csi() const { return p_u_csi; }
  __device__ __forceinline__ F2 k_exp2() const { return p_k_exp2; }
  __device__ __forceinline__ F2 u_c() const { return p_u_c; }
  __device__ __forceinline__ F2 m_s_td() const { return p_m_s_td; }
  __device__ __forceinline__ F2 s_tr() const { return p_s_tr; }
  __device__ __forceinline__ F2 s_to() const { return p_s_to; }
  __device__ __forceinline__ F2 m_s_tsi() const { return p_m_s_tsi; }
  __device__ __forceinline__ F2 tc() const { return p_tc; }
  __device__ __forceinline__ F2 m_s_tvp() const { return p_m_s_tvp; }
  __device__ __forceinline__ F2 m_s_twp() const { return p_m_s_twp; }
  __device__ __forceinline__ F2 s_twm() const { return p_s_twm; }
  __device__ __forceinline__ F2 rx() const { return p_rx; }
  __device__ __forceinline__ F2 ry() const { return p_ry; }
  __device__ __forceinline__ float u_c1() const { return p_u_c1; }
  __device__ __forceinline__ float u_v1() const { return p_u_v1; }
  __device__ __forceinline__ float s_tv1m() const { return p_s_tv1m; }
  __device__ __forceinline__ float s_tv2m() const { return p_s_tv2m; }
};

// fk3v_update of two cells, the same operations lane by lane in f32x2.
template <class CP>
__device__ __forceinline__ void fk3v_update2(const CP &c, F2 U, F2 V, F2 W,
                                             F2 D, F2 &UN, F2 &VN, F2 &WN) {
  float u0, u1;
  f2_split(U, u0, u1);
  const bool p0 = u0 >= c.u_c1(), p1 = u1 >= c.u_c1();
  const bool q0 = u0 >= c.u_v1(), q1 = u1 >= c.u_v1();
  const F2 x = mul2(sub2(U, c.u_csi()), c.k_exp2());
  float x0, x1, e0, e1;
  f2_split(x, x0, x1);
  f2_split(add2(f2(ex2_approx(x0), ex2_approx(x1)), c.one()), e0, e1);
  const F2 sig = f2(rcp_approx(e0), rcp_approx(e1));
  const F2 a4 = mul2(V, mul2(sub2(c.one(), U), sub2(U, c.u_c())));
  float jp0, jp1, jn0, jn1;
  f2_split(fma2(a4, c.m_s_td(), c.s_tr()), jp0, jp1);
  f2_split(mul2(U, c.s_to()), jn0, jn1);
  const F2 Jd = fma2(mul2(W, sig), c.m_s_tsi(),
                     f2(p0 ? jp0 : jn0, p1 ? jp1 : jn1));
  UN = sub2(fma2(D, c.tc(), U), Jd);
  float vp0, vp1, vm0, vm1, wp0, wp1, wm0, wm1;
  f2_split(fma2(V, c.m_s_tvp(), V), vp0, vp1);
  f2_split(fma2(sub2(c.one(), V),
                f2(q0 ? c.s_tv1m() : c.s_tv2m(), q1 ? c.s_tv1m() : c.s_tv2m()),
                V),
           vm0, vm1);
  VN = f2(p0 ? vp0 : vm0, p1 ? vp1 : vm1);
  f2_split(fma2(W, c.m_s_twp(), W), wp0, wp1);
  f2_split(fma2(sub2(c.one(), W), c.s_twm(), W), wm0, wm1);
  WN = f2(p0 ? wp0 : wm0, p1 ? wp1 : wm1);
}
__device__ __forceinline__ void fk3v_update2(const StepCoeffs<float> &a, F2 U,
                                             F2 V, F2 W, F2 D, F2 &UN, F2 &VN,
                                             F2 &WN) {
  fk3v_update2(FkPairsAt{a}, U, V, W, D, UN, VN, WN);
}

// Scaled 5-point Laplacian rx (lo - 2c + hi)_x + ry (lo - 2c + hi)_y with
// explicit rounding: h = (-2 c + lo) + hi per axis, du = hx rx + hy ry. The
// hole form weights (wlo, wc, whi) per axis, (wlo lo - wc c) + whi hi, gives
// the same bits for the weights (1, 2, 1).
__device__ __forceinline__ float lap_axis(float lo, float c, float hi) {
  return __fadd_rn(__fmaf_rn(-2.f, c, lo), hi);
}
__device__ __forceinline__ float lap_axis(float lo, float c, float hi,
                                          float wlo, float wc, float whi) {
  return __fmaf_rn(whi, hi, __fmaf_rn(-wc, c, __fmul_rn(wlo, lo)));
}
__device__ __forceinline__ float lap5(const StepCoeffs<float> &a, float hx,
                                      float hy) {
  return __fmaf_rn(hx, a.rx, __fmul_rn(hy, a.ry));
}
template <class CP>
__device__ __forceinline__ F2 lap5_2(const CP &c, F2 W, F2 C, F2 E, F2 N,
                                     F2 S) {
  const F2 hx = add2(fma2(c.m2(), C, W), E);
  const F2 hy = add2(fma2(c.m2(), C, N), S);
  return fma2(hx, c.rx(), mul2(hy, c.ry()));
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

// FK3V update of 4 consecutive cells (u[k], with west/east neighbours uw,
// ue and the rows above/below un, us). plain: all four cells tissue with
// tissue neighbours; else `code` holds the four hole codes (byte k: bit 0
// tissue, bits 1-2 x pattern, bits 3-4 y pattern) and cells outside tissue
// are set to 0. c: a's coefficients as lane pairs (FkPairsAt or FkPairs).
template <class CP>
__device__ __forceinline__ void fk3v_cells4(const StepCoeffs<float> &a,
                                            const CP &c, bool plain,
                                            uint32_t code, const float (&u)[4],
                                            float uw, float ue,
                                            const float (&un)[4],
                                            const float (&us)[4],
                                            const float (&v)[4],
                                            const float (&w)[4],
                                            float (&ou)[4], float (&ov)[4],
                                            float (&ow)[4]) {
  F2 D01, D23;
  if (plain) {
    D01 = lap5_2(c, f2(uw, u[0]), f2(u[0], u[1]), f2(u[1], u[2]),
                 f2(un[0], un[1]), f2(us[0], us[1]));
    D23 = lap5_2(c, f2(u[1], u[2]), f2(u[2], u[3]), f2(u[3], ue),
                 f2(un[2], un[3]), f2(us[2], us[3]));
  } else {
    float du[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t cc = code >> (8 * k);
      float cxw, cxc, cxe, cyn, cyc, cys;
      pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
      pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
      const float uW = k == 0 ? uw : u[k - 1];
      const float uE = k == 3 ? ue : u[k + 1];
      du[k] = lap5(a, lap_axis(uW, u[k], uE, cxw, cxc, cxe),
                   lap_axis(un[k], u[k], us[k], cyn, cyc, cys));
    }
    D01 = f2(du[0], du[1]);
    D23 = f2(du[2], du[3]);
  }
  F2 un2, vn2, wn2;
  fk3v_update2(c, f2(u[0], u[1]), f2(v[0], v[1]), f2(w[0], w[1]), D01, un2,
               vn2, wn2);
  f2_split(un2, ou[0], ou[1]);
  f2_split(vn2, ov[0], ov[1]);
  f2_split(wn2, ow[0], ow[1]);
  fk3v_update2(c, f2(u[2], u[3]), f2(v[2], v[3]), f2(w[2], w[3]), D23, un2,
               vn2, wn2);
  f2_split(un2, ou[2], ou[3]);
  f2_split(vn2, ov[2], ov[3]);
  f2_split(wn2, ow[2], ow[3]);
  if (!plain) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (((code >> (8 * k)) & 1u) == 0u) ou[k] = ov[k] = ow[k] = 0.f;
  }
}
__device__ __forceinline__ void fk3v_cells4(const StepCoeffs<float> &a,
                                            bool plain, uint32_t code,
                                            const float (&u)[4], float uw,
                                            float ue, const float (&un)[4],
                                            const float (&us)[4],
                                            const float (&v)[4],
                                            const float (&w)[4],
                                            float (&ou)[4], float (&ov)[4],
                                            float (&ow)[4]) {
  fk3v_cells4(a, FkPairsAt{a}, plain, code, u, uw, ue, un, us, v, w, ou, ov,
              ow);
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
