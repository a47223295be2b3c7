// Adjoint of the FK3V explicit solver with a per-cell diffusion map
// (include/yolohtli.h, layer 5): the gradient of a probe loss with respect
// to D(x, y), for parameter estimation. No reference counterpart (the
// reference has constant D and no gradients).
//
// Forward step (finite-volume form of div(D grad u), no-flux edges by the
// reference's mirror ghosts, helper_functions.cu:69-79):
//   r_i = dt D_i / h^2,  k_f = (r_i + r_m(f)) / 2 for face f of cell i
//   towards its (mirrored) neighbour m(f),
//   du_i = sum_f k_f (u_m(f) - u_i),
// then the FK3V update with du (Fenton & Karma 1998, tc-scaled Euler):
//   u' = u + tc du - dt tc J(u, v, w),  v' = v + dt tc g_v,  w' = w + dt tc g_w
// in exact arithmetic (exp2 and division, no approximate MUFU forms), so the
// reverse step differentiates exactly what the forward step computes. The
// model's switches H(u - u_c), H(u - u_v) are steps (smooth = 0) or, for a
// loss that stays differentiable over long horizons, (1 + tanh(x/eps))/2:
// with steps the derivative exists almost everywhere but leaves out the
// threshold-crossing times that move the fronts, and it grows with the
// horizon (the upstroke's local instability).
//
// Loss: L = sum over frames f (the states after every `frame` steps) of
// sum over probes p (cells (px*sp + sp/2, py*sp + sp/2)) of
// (u_f,p - target_f,p)^2.
//
// Reverse step n (gather form, one kernel per step): from lambda^{n+1} and
// the state x^n it forms lambda^n = (dF/dx^n)^T lambda^{n+1} + dL/dx^n and
// adds (dF/dr)^T lambda^{n+1} to the gradient with respect to r. The
// forward states of a segment are recomputed from a checkpoint (every
// `ck` steps) before the segment's reverse sweep, on a second stream, one
// segment ahead of the sweep (the recompute of segment k - 1 runs beside
// the reverse sweep of segment k; at one 512^2 instance both are bound by
// launch latency, not by the SMs); the forward pass writes the last
// segment's states where the sweep reads them. Memory: the checkpoints
// plus two segments of states. The whole sequence (~3 nsteps launches and
// the checkpoint copies) is captured once per handle as a CUDA graph and
// replayed.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <utility>

#include "yh_kernels.cuh"

namespace yh {
template <typename Real>
StepCoeffs<Real> make_step_coeffs(const yh_param_var &p, int model,
                                  const yh_fk_params *fk);
int check_params(const yh_param_var *p, int model, const yh_fk_params *fk);
}  // namespace yh

using namespace yh;

namespace {

template <typename Real>
struct AdjCoeffs {
  int nx, ny;
  Real eps;  // width of the smoothed switches H(u - u_c), H(u - u_v); 0: steps
  Real sw_k, sw_d;  // eps > 0: -2 / (eps ln 2) and 2 / eps
  Real tc, dt;
  Real u_c, u_v, u_csi, k2;  // k2: -2k log2(e) of the sigmoid's 2^(k2 (u - u_csi))
  Real s_td, s_tr, s_to, s_tsi, s_tvp, s_tv1m, s_tv2m, s_twp, s_twm;
};

template <typename Real>
__device__ __forceinline__ Real ex2(Real x);
template <>
__device__ __forceinline__ float ex2<float>(float x) { return exp2f(x); }
template <>
__device__ __forceinline__ double ex2<double>(double x) { return exp2(x); }

// The switch H(x) of the model (a step at 0) and its derivative: with a
// smoothing width eps > 0, H = (1 + tanh(x / eps)) / 2, evaluated as the
// logistic function 1 / (1 + 2^(sw_k x)), sw_k = -2 / (eps ln 2) (the same
// function), dH = sw_d H (1 - H), sw_d = 2 / eps.
template <typename Real>
__device__ __forceinline__ void heaviside(const AdjCoeffs<Real> &a, Real x,
                                          Real &H, Real &dH) {
  if (a.eps > Real(0)) {
    const Real e = ex2<Real>(a.sw_k * x);
    H = Real(1) / (Real(1) + e);
    dH = a.sw_d * H * (Real(1) - H);
  } else {
    H = x >= Real(0) ? Real(1) : Real(0);
    dH = Real(0);
  }
}

// The switches and the sigmoid of one cell's u, shared by the update, its
// derivatives and the parameter terms.
template <typename Real>
struct FkSwitch {
  Real H1, dH1, H2, dH2, sig;
};
template <typename Real>
__device__ __forceinline__ FkSwitch<Real> fk_switch(const AdjCoeffs<Real> &a,
                                                    Real u) {
  FkSwitch<Real> s;
  heaviside(a, u - a.u_c, s.H1, s.dH1);
  heaviside(a, u - a.u_v, s.H2, s.dH2);
  const Real e = ex2<Real>(a.k2 * (u - a.u_csi));
  s.sig = Real(1) / (Real(1) + e);
  return s;
}

// The pointwise FK3V update and its partial derivatives.
template <typename Real>
struct FkLocal {
  Real un, vn, wn;
  Real dun_du, dun_dv, dun_dw;  // of un (du held fixed)
  Real dvn_du, dvn_dv, dwn_du, dwn_dw;
};

// J1 = H1 jp + (1 - H1) jn, v' = H1 vp + (1 - H1) vm, w' = H1 wp + (1 - H1) wm
// with H1 = H(u - u_c) and the v time constant H2 s_tv1m + (1 - H2) s_tv2m,
// H2 = H(u - u_v): the FK3V update (fk3v_update) when eps = 0.
template <typename Real>
__device__ __forceinline__ FkLocal<Real> fk_local(const AdjCoeffs<Real> &a,
                                                  const FkSwitch<Real> &S,
                                                  Real u, Real v, Real w,
                                                  Real du) {
  FkLocal<Real> r;
  const Real H1 = S.H1, dH1 = S.dH1, H2 = S.H2, dH2 = S.dH2, sig = S.sig;
  // d sig / du = -ln2 k2 e / (1 + e)^2 = -ln2 k2 sig (1 - sig)
  const Real dsig = -Real(0.69314718055994530942) * a.k2 * sig * (Real(1) - sig);
  const Real jp = a.s_tr - v * (Real(1) - u) * (u - a.u_c) * a.s_td;
  const Real jn = u * a.s_to;
  const Real djp_du = -a.s_td * v * (Real(1) - Real(2) * u + a.u_c);
  const Real djp_dv = -a.s_td * (Real(1) - u) * (u - a.u_c);
  const Real J1 = H1 * jp + (Real(1) - H1) * jn;
  const Real dJ1_du = H1 * djp_du + (Real(1) - H1) * a.s_to + dH1 * (jp - jn);
  const Real dJ1_dv = H1 * djp_dv;
  const Real Jd = J1 - w * sig * a.s_tsi;
  r.un = u + a.tc * du - Jd;
  r.dun_du = Real(1) - (dJ1_du - w * dsig * a.s_tsi);
  r.dun_dv = -dJ1_dv;
  r.dun_dw = sig * a.s_tsi;
  const Real sv = H2 * a.s_tv1m + (Real(1) - H2) * a.s_tv2m;
  const Real vp = v - v * a.s_tvp, vm = v + (Real(1) - v) * sv;
  r.vn = H1 * vp + (Real(1) - H1) * vm;
  r.dvn_dv = H1 * (Real(1) - a.s_tvp) + (Real(1) - H1) * (Real(1) - sv);
  r.dvn_du = dH1 * (vp - vm) +
             (Real(1) - H1) * (Real(1) - v) * dH2 * (a.s_tv1m - a.s_tv2m);
  const Real wp = w - w * a.s_twp, wm = w + (Real(1) - w) * a.s_twm;
  r.wn = H1 * wp + (Real(1) - H1) * wm;
  r.dwn_dw = H1 * (Real(1) - a.s_twp) + (Real(1) - H1) * (Real(1) - a.s_twm);
  r.dwn_du = dH1 * (wp - wm);
  return r;
}

// The raw FK3V parameters of the update, in the order of yh_fk_params:
// the nine rates s_X = tc dt / tau_X (tau_d, tau_r, tau_si, tau_0,
// tau_v_plus, tau_v1_minus, tau_v2_minus, tau_w_plus, tau_w_minus), then
// u_c, u_v, u_csi and k2 = -2k / ln 2. kNumFk of them.
constexpr int kNumFk = 13;

// g[q] = lu dun/dp_q + lv dvn/dp_q + lw dwn/dp_q for the raw parameters p_q
// at one cell: (lu, lv, lw) is the adjoint of (un, vn, wn).
template <typename Real>
__device__ __forceinline__ void fk_param_terms(const AdjCoeffs<Real> &a,
                                               const FkSwitch<Real> &S,
                                               Real u, Real v, Real w,
                                               Real lu, Real lv, Real lw,
                                               Real g[kNumFk]) {
  const Real H1 = S.H1, dH1 = S.dH1, H2 = S.H2, dH2 = S.dH2, sig = S.sig;
  const Real ln2 = Real(0.69314718055994530942);
  const Real ss = sig * (Real(1) - sig);
  const Real q = v * (Real(1) - u) * (u - a.u_c);  // jp = s_tr - q s_td
  const Real jp = a.s_tr - q * a.s_td;
  const Real jn = u * a.s_to;
  const Real sv = H2 * a.s_tv1m + (Real(1) - H2) * a.s_tv2m;
  const Real vp = v - v * a.s_tvp, vm = v + (Real(1) - v) * sv;
  const Real wp = w - w * a.s_twp, wm = w + (Real(1) - w) * a.s_twm;
  const Real L1 = Real(1) - H1;
  g[0] = lu * H1 * q;                          // s_td
  g[1] = -lu * H1;                             // s_tr
  g[2] = lu * w * sig;                         // s_tsi
  g[3] = -lu * L1 * u;                         // s_to
  g[4] = -lv * H1 * v;                         // s_tvp
  g[5] = lv * L1 * (Real(1) - v) * H2;         // s_tv1m
  g[6] = lv * L1 * (Real(1) - v) * (Real(1) - H2);  // s_tv2m
  g[7] = -lw * H1 * w;                         // s_twp
  g[8] = lw * L1 * (Real(1) - w);              // s_twm
  g[9] = lu * (dH1 * (jp - jn) - H1 * v * (Real(1) - u) * a.s_td) -
         lv * dH1 * (vp - vm) - lw * dH1 * (wp - wm);  // u_c
  g[10] = -lv * L1 * (Real(1) - v) * dH2 * (a.s_tv1m - a.s_tv2m);  // u_v
  g[11] = lu * w * a.s_tsi * ln2 * a.k2 * ss;       // u_csi
  g[12] = -lu * w * a.s_tsi * ln2 * (u - a.u_csi) * ss;  // k2
}

// du of cell (i, j): the four faces towards the mirrored neighbours.
template <typename Real>
__device__ __forceinline__ Real diffusion(const AdjCoeffs<Real> &a,
                                          const Real *__restrict__ u,
                                          const Real *__restrict__ r, int i,
                                          int j) {
  const int nx = a.nx, ny = a.ny, c = i + nx * j;
  const int m[4] = {mirror(i - 1, nx) + nx * j, mirror(i + 1, nx) + nx * j,
                    i + nx * mirror(j - 1, ny), i + nx * mirror(j + 1, ny)};
  const Real uc = u[c], rc = r[c];
  Real du = Real(0);
#pragma unroll
  for (int f = 0; f < 4; ++f) du += Real(0.5) * (rc + r[m[f]]) * (u[m[f]] - uc);
  return du;
}

template <typename Real>
__global__ void adj_forward_kernel(const AdjCoeffs<Real> a,
                                   const Real *__restrict__ r,
                                   const Real *__restrict__ u,
                                   const Real *__restrict__ v,
                                   const Real *__restrict__ w, Real *__restrict__ uo,
                                   Real *__restrict__ vo, Real *__restrict__ wo) {
  grid_dep_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.nx || j >= a.ny) return;
  const size_t off = (size_t)blockIdx.z * a.nx * a.ny;  // instance
  r += off;
  u += off;
  v += off;
  w += off;
  uo += off;
  vo += off;
  wo += off;
  const int c = i + a.nx * j;
  const Real uc = u[c];
  const FkLocal<Real> f = fk_local(a, fk_switch(a, uc), uc, v[c], w[c],
                                   diffusion(a, u, r, i, j));
  uo[c] = f.un;
  vo[c] = f.vn;
  wo[c] = f.wn;
}

// Reverse step: lambda_in = lambda^{n+1} (lu, lv, lw), x^n = (u, v, w);
// writes lambda^n (without the loss term) and adds to gr (the gradient
// with respect to r).
// With PARAMS the block also adds its cells' fk_param_terms to its own
// accumulators gp[block][0..12] (FP64; one slot per block, so the sum over
// steps keeps a fixed order).
// FP32: 32 registers, 8 blocks of 256 per SM, so a 512^2 step (1024
// blocks) is one wave of the GPU's 152 SMs (at the default 40 registers it
// was 1.1 waves, and 19 % slower a gradient).
template <typename Real, bool PARAMS>
__global__ void __launch_bounds__(256, sizeof(Real) == 4 ? 8 : 4)
    adj_reverse_kernel(const AdjCoeffs<Real> a, const Real *__restrict__ r,
                       const Real *__restrict__ u, const Real *__restrict__ v,
                       const Real *__restrict__ w, const Real *__restrict__ lu,
                       const Real *__restrict__ lv, const Real *__restrict__ lw,
                       Real *__restrict__ lu_o, Real *__restrict__ lv_o,
                       Real *__restrict__ lw_o, Real *__restrict__ gr,
                       double *__restrict__ gp) {
  grid_dep_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  {
    const size_t off = (size_t)blockIdx.z * nx * ny;  // instance
    r += off;
    u += off;
    v += off;
    w += off;
    lu += off;
    lv += off;
    lw += off;
    lu_o += off;
    lv_o += off;
    lw_o += off;
    gr += off;
  }
  // the cell's state and switches, shared by the parameter terms and the
  // update's derivatives
  const bool in = i < nx && j < ny;
  const int c = in ? i + nx * j : 0;
  Real uc = Real(0), vc = Real(0), wc = Real(0);
  FkSwitch<Real> S{};
  if (in) {
    uc = u[c];
    vc = v[c];
    wc = w[c];
    S = fk_switch(a, uc);
  }
  if (PARAMS) {
    // the block's 256 x 13 terms through shared memory, transposed: warp
    // q (0-7) sums rows q and q + 8 (8 values a lane, then a shuffle tree),
    // far fewer instructions than 13 shuffle trees in every warp
    __shared__ Real s_g[kNumFk][256];  // blockDim (32, 8)
    const int t = threadIdx.x + 32 * threadIdx.y;
    {
      Real g[kNumFk];
      if (in) {
        fk_param_terms(a, S, uc, vc, wc, lu[c], lv[c], lw[c], g);
      } else {
#pragma unroll
        for (int k = 0; k < kNumFk; ++k) g[k] = Real(0);
      }
#pragma unroll
      for (int k = 0; k < kNumFk; ++k) s_g[k][t] = g[k];
    }
    __syncthreads();
    const int lane = threadIdx.x, warp = threadIdx.y;
    const size_t blk =
        blockIdx.x + gridDim.x * (blockIdx.y + (size_t)gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = warp; q < kNumFk; q += 8) {
      Real sum = Real(0);
#pragma unroll
      for (int m = 0; m < 8; ++m) sum += s_g[q][lane + 32 * m];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
        sum += __shfl_down_sync(0xffffffffu, sum, off);
      if (lane == 0) gp[blk * 16 + q] += (double)sum;
    }
  }
  if (!in) return;
  // pointwise part at c (the derivatives do not depend on du)
  const FkLocal<Real> f = fk_local(a, S, uc, vc, wc, Real(0));
  const Real lun = lu[c];
  Real gu = lun * f.dun_du + lv[c] * f.dvn_du + lw[c] * f.dwn_du;
  const Real gv = lun * f.dun_dv + lv[c] * f.dvn_dv;
  const Real gw = lun * f.dun_dw + lw[c] * f.dwn_dw;
  // diffusion part: mu_j = tc * lambda_u^{n+1}_j is the adjoint of du_j.
  // du_j = sum_f (r_j + r_m(j,f)) / 2 (u_m(j,f) - u_j): cell c enters as
  // j itself (-k_f per face, and r_j in every k_f), and as m(j, f) of the
  // cells j whose face f points (through the mirror) at c.
  const Real muc = a.tc * lun;
  const Real rc = r[c];
  const int m[4] = {mirror(i - 1, nx) + nx * j, mirror(i + 1, nx) + nx * j,
                    i + nx * mirror(j - 1, ny), i + nx * mirror(j + 1, ny)};
  Real g = Real(0);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const Real k = Real(0.5) * (rc + r[m[q]]);
    gu -= muc * k;
    g += Real(0.5) * muc * (u[m[q]] - uc);
  }
  if (i >= 2 && i < nx - 2 && j >= 2 && j < ny - 2) {
    // interior: m(c, q) is the neighbour in direction q, and exactly one
    // of its faces (the opposite one) points back at c: the general loop
    // below in fewer instructions, with the same operations in the same
    // order (the same bits)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const Real muj = a.tc * lu[m[q]];
      const Real uj = u[m[q]], rj = r[m[q]];
      gu += muj * Real(0.5) * (rj + rc);  // d du_j / d u_c
      g += muj * Real(0.5) * (uc - uj);   // d du_j / d r_c
    }
    lu_o[c] = gu;
    lv_o[c] = gv;
    lw_o[c] = gw;
    gr[c] += g;
    return;
  }
  // neighbours j of c (the cells whose faces can point at c): the four
  // physical neighbours in range; for each, the faces f with m(j, f) == c
  const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int ii = i + di[q], jj = j + dj[q];
    if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;
    const int cj = ii + nx * jj;
    const int mj[4] = {mirror(ii - 1, nx) + nx * jj, mirror(ii + 1, nx) + nx * jj,
                       ii + nx * mirror(jj - 1, ny), ii + nx * mirror(jj + 1, ny)};
    const Real muj = a.tc * lu[cj];
    const Real uj = u[cj], rj = r[cj];
#pragma unroll
    for (int fq = 0; fq < 4; ++fq) {
      if (mj[fq] != c) continue;
      gu += muj * Real(0.5) * (rj + rc);  // d du_j / d u_c
      g += muj * Real(0.5) * (uc - uj);   // d du_j / d r_c
    }
  }
  lu_o[c] = gu;
  lv_o[c] = gv;
  lw_o[c] = gw;
  gr[c] += g;
}

// Probe loss of one frame (one block of 256 threads per instance,
// fixed-order sum) and, with lu != null, its adjoint 2 (u - target) added at
// the probes. u, lu: instance stride n; target: instance stride tstride;
// loss: one per instance.
template <typename Real>
__global__ void adj_probe_kernel(int nx, int sp, int npx, int npy, int n,
                                 size_t tstride, const Real *__restrict__ u,
                                 const float *__restrict__ target,
                                 double *loss, Real *lu) {
  grid_dep_wait();
  u += (size_t)blockIdx.x * n;
  target += (size_t)blockIdx.x * tstride;
  if (lu) lu += (size_t)blockIdx.x * n;
  if (loss) loss += blockIdx.x;
  __shared__ double s[256];
  double acc = 0.0;
  const int np = npx * npy;
  for (int p = threadIdx.x; p < np; p += 256) {
    const int px = p % npx, py = p / npx;
    const int c = (px * sp + sp / 2) + nx * (py * sp + sp / 2);
    const double d = (double)u[c] - (double)target[p];
    acc += d * d;
    if (lu) lu[c] += (Real)(2.0 * d);
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0 && loss) *loss += s[0];
}

template <typename Real>
__global__ void adj_scale_kernel(int n, Real scale, const Real *__restrict__ x,
                                 float *__restrict__ y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] = (float)(scale * x[k]);
}

template <typename Real>
__global__ void adj_to_r_kernel(int n, Real scale, const float *__restrict__ D,
                                Real *__restrict__ r) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) r[k] = scale * (Real)D[k];
}

template <typename Real>
__global__ void adj_widen_kernel(int n, const float *__restrict__ x,
                                 Real *__restrict__ y) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] = (Real)x[k];
}

// The probe values of one frame (instance blockIdx.y: u stride n, out
// stride ostride).
template <typename Real>
__global__ void adj_gather_kernel(int nx, int sp, int npx, int npy, int n,
                                  size_t ostride, const Real *__restrict__ u,
                                  float *__restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  u += (size_t)blockIdx.y * n;
  out += (size_t)blockIdx.y * ostride;
  if (p >= npx * npy) return;
  const int px = p % npx, py = p / npx;
  out[p] = (float)u[(px * sp + sp / 2) + nx * (py * sp + sp / 2)];
}

// Sum of the per-block parameter accumulators, in block order.
__global__ void adj_param_reduce_kernel(int nb, const double *__restrict__ gp,
                                        double *__restrict__ out) {
  const int k = threadIdx.x;
  gp += (size_t)blockIdx.x * nb * 16;  // instance
  out += (size_t)blockIdx.x * 16;
  if (k >= kNumFk) return;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += gp[(size_t)b * 16 + k];
  out[k] = s;
}

inline int st(cudaError_t e) {
  if (e == cudaSuccess) return YH_OK;
  if (e == cudaErrorMemoryAllocation) return YH_ENOMEM;
  return YH_ECUDA;
}

}  // namespace

struct yh_adjoint {
  int fp64 = 0;
  int nx = 0, ny = 0, n = 0;
  int batch = 1;  // instances: same grid, steps and FK parameters
  int nsteps = 0, frame = 0, sp = 0, npx = 0, npy = 0, ck = 0;
  double rscale = 0;  // r = rscale * D
  cudaStream_t s = nullptr;
  bool own_stream = false;
  // the recompute stream and its events (fork, segment ready per buffer,
  // segment consumed per buffer, join)
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev_ready[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  AdjCoeffs<float> af{};
  AdjCoeffs<double> ad{};
  // Every state is [field][instance][cell].
  void *ckpt = nullptr;   // checkpoints: (nsteps - 1) / ck + 1 states
  void *seg = nullptr;    // two segments of ck + 1 states (one if ck == 1)
  size_t seg_states = 0;  // states per segment buffer
  void *lam = nullptr;    // two adjoint states (ping-pong)
  void *r = nullptr;      // r = dt D / h^2, [instance][cell]
  void *gr = nullptr;     // gradient with respect to r
  float *target = nullptr;  // [instance][frame][probe]
  double *loss = nullptr;   // [instance]
  double *gp = nullptr;   // per-block FK-parameter accumulators (16 each)
  double *gfk = nullptr;  // their sums: dL/d(raw FK parameters), 16 each
  int nrev = 0;           // blocks of the reverse launch per instance
  int frames = 0;
  // the whole forward (+ reverse) sequence on the handle's own buffers,
  // captured once: [0] loss only, [1] loss and dL/dD, [2] also the FK
  // parameters
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  yh_fk_params fk{};
  yh_param_var pv{};
  double smooth = 0;
  double tcdt = 0;  // s_X = tcdt / tau_X
};

namespace {

// States of all instances: f(state, field) is the base of batch * n cells.
template <typename Real>
struct View {
  Real *p;
  size_t n;  // cells of one field over all instances
  Real *f(int state, int field) const { return p + ((size_t)state * 3 + field) * n; }
};

template <typename Real>
const AdjCoeffs<Real> &coeffs(const yh_adjoint *h);
template <>
const AdjCoeffs<float> &coeffs<float>(const yh_adjoint *h) { return h->af; }
template <>
const AdjCoeffs<double> &coeffs<double>(const yh_adjoint *h) { return h->ad; }

template <typename Real>
cudaError_t fwd(const yh_adjoint *h, const Real *r, const Real *const *x,
                Real *const *y, cudaStream_t s) {
  const dim3 b(32, 8), g((h->nx + 31) / 32, (h->ny + 7) / 8, h->batch);
  return launch_pdl(adj_forward_kernel<Real>, g, b, 0, s, coeffs<Real>(h),
                    r, x[0], x[1], x[2], y[0], y[1], y[2]);
}
template <typename Real>
cudaError_t fwd(const yh_adjoint *h, const Real *r, const Real *const *x,
                Real *const *y) {
  return fwd<Real>(h, r, x, y, h->s);
}

// Loss of frame f (1-based step / frame) from u, and with lu its adjoint.
template <typename Real>
cudaError_t probe(const yh_adjoint *h, int f, const Real *u, double *loss,
                  Real *lu) {
  const size_t np = (size_t)h->npx * h->npy;
  return launch_pdl(adj_probe_kernel<Real>, dim3(h->batch), dim3(256), 0,
                    h->s, h->nx, h->sp, h->npx, h->npy, h->n,
                    (size_t)h->frames * np, (const Real *)u,
                    (const float *)(h->target + (size_t)(f - 1) * np), loss,
                    lu);
}

template <typename Real, bool PARAMS>
cudaError_t rev(const yh_adjoint *h, const Real *r, const Real *const *x,
                const Real *const *lin, Real *const *lout, Real *gr) {
  const dim3 b(32, 8), g((h->nx + 31) / 32, (h->ny + 7) / 8, h->batch);
  return launch_pdl(adj_reverse_kernel<Real, PARAMS>, g, b, 0, h->s,
                    coeffs<Real>(h), r, (const Real *)x[0], (const Real *)x[1],
                    (const Real *)x[2], (const Real *)lin[0],
                    (const Real *)lin[1], (const Real *)lin[2], lout[0],
                    lout[1], lout[2], gr, PARAMS ? h->gp : (double *)nullptr);
}

// The forward pass (checkpoints, loss) and, with grad, the reverse sweep,
// on the handle's buffers only: r and checkpoint 0 hold the inputs. Its
// launches are captured into a CUDA graph by run_t. With ck == 1 every
// state is kept (no recompute): the checkpoints are states 0 .. T-1 and
// the forward pass writes them in place. Otherwise segment k (states
// k ck .. min((k + 1) ck, T)) lives in segment buffer k % 2: the forward
// pass fills the last segment's buffer itself, and the recompute stream
// refills buffer k % 2 with segment k - 2 once the sweep of segment k is
// done with it.
template <typename Real>
cudaError_t run_body(yh_adjoint *h, bool grad, bool params) {
  const size_t n = (size_t)h->n * h->batch;
  const int T = h->nsteps, ck = h->ck;
  const bool all = ck == 1;
  const View<Real> C{(Real *)h->ckpt, n}, S{(Real *)h->seg, n}, L{(Real *)h->lam, n};
  auto buf = [&](int k) {
    return View<Real>{(Real *)h->seg + (size_t)(k & 1) * h->seg_states * 3 * n, n};
  };
  Real *r = (Real *)h->r, *gr = (Real *)h->gr;
  auto st3 = [](const View<Real> &V, int k, Real **out) {
    for (int q = 0; q < 3; ++q) out[q] = V.f(k, q);
  };
  const int K = (T - 1) / ck + 1, sl = (K - 1) * ck;  // segments; last start
  cudaError_t e = cudaMemsetAsync(h->loss, 0, h->batch * sizeof(double), h->s);
  // forward: checkpoints every ck steps, the loss at every frame
  if (all) {
    for (int t = 0; t < T && e == cudaSuccess; ++t) {
      Real *x[3], *y[3];
      st3(C, t, x);
      if (t + 1 < T) st3(C, t + 1, y); else st3(S, 0, y);
      e = fwd<Real>(h, r, x, y);
      if (e == cudaSuccess && (t + 1) % h->frame == 0)
        e = probe<Real>(h, (t + 1) / h->frame, y[0], h->loss, nullptr);
    }
  } else {
    // states before sl ping-pong in the other buffer's first two slots;
    // states sl .. T go to the last segment's buffer
    const View<Real> BL = buf(K - 1), BO = buf(K);
    Real *cur[3], *nxt[3];
    st3(sl == 0 ? BL : BO, 0, cur);
    st3(BO, 1, nxt);
    for (int q = 0; q < 3 && e == cudaSuccess; ++q)
      e = cudaMemcpyAsync(cur[q], C.f(0, q), n * sizeof(Real),
                          cudaMemcpyDeviceToDevice, h->s);
    for (int t = 0; t < T && e == cudaSuccess; ++t) {
      const int step = t + 1;
      if (step >= sl) {
        Real *y[3];
        st3(BL, step - sl, y);
        e = fwd<Real>(h, r, cur, y);
        for (int q = 0; q < 3; ++q) cur[q] = y[q];
      } else {
        e = fwd<Real>(h, r, cur, nxt);
        for (int q = 0; q < 3; ++q) std::swap(cur[q], nxt[q]);
      }
      if (e == cudaSuccess && step % h->frame == 0)
        e = probe<Real>(h, step / h->frame, cur[0], h->loss, nullptr);
      if (e == cudaSuccess && step % ck == 0 && step < sl)
        for (int q = 0; q < 3 && e == cudaSuccess; ++q)
          e = cudaMemcpyAsync(C.f(step / ck, q), cur[q], n * sizeof(Real),
                              cudaMemcpyDeviceToDevice, h->s);
      // the forward pass is done with the other buffer: the recompute of
      // segment K - 2 may start beside the last segment's steps
      if (e == cudaSuccess && step == sl && grad)
        e = cudaEventRecord(h->ev_fork, h->s);
    }
  }
  if (e != cudaSuccess || !grad) return e;
  // reverse, one segment at a time from the last: lambda^T = dL/dx^T
  e = cudaMemsetAsync(L.f(0, 0), 0, 3 * n * sizeof(Real), h->s);
  if (e == cudaSuccess) e = cudaMemsetAsync(gr, 0, n * sizeof(Real), h->s);
  if (e == cudaSuccess && params)
    e = cudaMemsetAsync(h->gp, 0, (size_t)h->batch * h->nrev * 16 * sizeof(double),
                        h->s);
  int li = 0;  // lambda^{t+1} lives in L state li
  // one reverse step: lambda^t += dL/dx^t (u^t = ut), then lambda^{t-1}
  // from lambda^t and x^{t-1}
  auto back = [&](int t, const Real *ut, Real *const *xp) {
    cudaError_t er = cudaSuccess;
    if (t % h->frame == 0) er = probe<Real>(h, t / h->frame, ut, nullptr, L.f(li, 0));
    Real *lin[3], *lout[3];
    st3(L, li, lin);
    st3(L, li ^ 1, lout);
    if (er == cudaSuccess)
      er = params ? rev<Real, true>(h, r, xp, lin, lout, gr)
                  : rev<Real, false>(h, r, xp, lin, lout, gr);
    li ^= 1;
    return er;
  };
  if (all) {
    for (int t = T; t > 0 && e == cudaSuccess; --t) {
      Real *xp[3];
      st3(C, t - 1, xp);
      e = back(t, t == T ? S.f(0, 0) : C.f(t, 0), xp);
    }
  } else {
    cudaStream_t s2 = h->s2;
    // segment k (k <= K - 2) from its checkpoint into buffer k % 2, on s2
    auto recompute = [&](int k) {
      const View<Real> B = buf(k);
      const int s0 = k * ck, s1 = s0 + ck;
      cudaError_t er = cudaSuccess;
      for (int q = 0; q < 3 && er == cudaSuccess; ++q)
        er = cudaMemcpyAsync(B.f(0, q), C.f(k, q), n * sizeof(Real),
                             cudaMemcpyDeviceToDevice, s2);
      for (int t = s0; t < s1 && er == cudaSuccess; ++t) {
        Real *x[3], *y[3];
        st3(B, t - s0, x);
        st3(B, t - s0 + 1, y);
        er = fwd<Real>(h, r, x, y, s2);
      }
      if (er == cudaSuccess) er = cudaEventRecord(h->ev_ready[k & 1], s2);
      return er;
    };
    const bool forked = K >= 2;
    if (forked) {
      e = cudaStreamWaitEvent(s2, h->ev_fork, 0);
      if (e == cudaSuccess) e = recompute(K - 2);
    }
    for (int k = K - 1; k >= 0 && e == cudaSuccess; --k) {
      const View<Real> B = buf(k);
      const int s0 = k * ck, s1 = std::min(s0 + ck, T);  // states s0 .. s1
      if (k <= K - 2) e = cudaStreamWaitEvent(h->s, h->ev_ready[k & 1], 0);
      for (int t = s1; t > s0 && e == cudaSuccess; --t) {
        Real *xp[3];
        st3(B, t - 1 - s0, xp);
        e = back(t, B.f(t - s0, 0), xp);
      }
      if (e == cudaSuccess && k >= 2) {
        e = cudaEventRecord(h->ev_free[k & 1], h->s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, h->ev_free[k & 1], 0);
        if (e == cudaSuccess) e = recompute(k - 2);
      }
    }
    if (forked) {  // join s2 back (also after an error, so the capture ends)
      const cudaError_t ej = cudaEventRecord(h->ev_join, s2);
      const cudaError_t ew = cudaStreamWaitEvent(h->s, h->ev_join, 0);
      if (e == cudaSuccess) e = ej != cudaSuccess ? ej : ew;
    }
  }
  if (e == cudaSuccess && params) {
    adj_param_reduce_kernel<<<h->batch, 32, 0, h->s>>>(h->nrev, h->gp, h->gfk);
    e = cudaGetLastError();
  }
  return e;
}

// The inputs (D, u0, v0, w0: batch * n floats each) into r and state 0 of
// the checkpoints.
template <typename Real>
cudaError_t load_inputs(yh_adjoint *h, const float *D, const float *u0,
                        const float *v0, const float *w0, Real *state0) {
  const size_t n = (size_t)h->n * h->batch;
  const int nb = (int)((n + 255) / 256);
  adj_to_r_kernel<Real><<<nb, 256, 0, h->s>>>((int)n, (Real)h->rscale, D, (Real *)h->r);
  const float *x0[3] = {u0, v0, w0};
  for (int q = 0; q < 3; ++q)
    adj_widen_kernel<Real><<<nb, 256, 0, h->s>>>((int)n, x0[q], state0 + q * n);
  return cudaGetLastError();
}

template <typename Real>
int run_t(yh_adjoint *h, const float *D, const float *u0, const float *v0,
          const float *w0, double *loss_out, float *grad, double *graw) {
  const size_t n = (size_t)h->n * h->batch;
  const int nb = (int)((n + 255) / 256);
  // the inputs into the handle's buffers (outside the graph: the caller's
  // pointers may change from run to run)
  cudaError_t e = load_inputs<Real>(h, D, u0, v0, w0, (Real *)h->ckpt);
  if (e != cudaSuccess) return st(e);
  const bool want_grad = grad != nullptr || graw != nullptr;
  cudaGraphExec_t &ex = h->graph[graw ? 2 : (want_grad ? 1 : 0)];
  if (!ex) {
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return st(e);
    const cudaError_t eb = run_body<Real>(h, want_grad, graw != nullptr);
    e = cudaStreamEndCapture(h->s, &g);
    if (eb != cudaSuccess || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return st(eb != cudaSuccess ? eb : e);
    }
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ex = nullptr;
      return st(e);
    }
  }
  e = cudaGraphLaunch(ex, h->s);
  if (e == cudaSuccess && grad) {
    // dL/dD = dL/dr * dt / h^2
    adj_scale_kernel<Real><<<nb, 256, 0, h->s>>>((int)n, (Real)h->rscale,
                                                 (const Real *)h->gr, grad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && loss_out)
    e = cudaMemcpyAsync(loss_out, h->loss, h->batch * sizeof(double),
                        cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess && graw)
    e = cudaMemcpyAsync(graw, h->gfk, (size_t)h->batch * 16 * sizeof(double),
                        cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  return st(e);
}

// A forward run that gathers the probe values of every frame (a target).
template <typename Real>
int record_t(yh_adjoint *h, const float *D, const float *u0, const float *v0,
             const float *w0, float *probes) {
  const size_t n = (size_t)h->n * h->batch;
  const int T = h->nsteps, np = h->npx * h->npy;
  const View<Real> S{(Real *)h->seg, n};
  Real *r = (Real *)h->r;
  cudaError_t e = load_inputs<Real>(h, D, u0, v0, w0, S.f(0, 0));
  Real *cur[3] = {S.f(0, 0), S.f(0, 1), S.f(0, 2)};
  Real *nxt[3] = {S.f(1, 0), S.f(1, 1), S.f(1, 2)};
  for (int t = 0; t < T && e == cudaSuccess; ++t) {
    e = fwd<Real>(h, r, cur, nxt);
    for (int q = 0; q < 3; ++q) std::swap(cur[q], nxt[q]);
    if (e == cudaSuccess && (t + 1) % h->frame == 0) {
      const int f = (t + 1) / h->frame - 1;
      adj_gather_kernel<Real><<<dim3((np + 255) / 256, h->batch), 256, 0, h->s>>>(
          h->nx, h->sp, h->npx, h->npy, h->n, (size_t)h->frames * np, cur[0],
          probes + (size_t)f * np);
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  return st(e);
}

// The step coefficients of the handle from its parameters and fk.
void set_coeffs(yh_adjoint *h, const yh_fk_params *fk) {
  h->fk = *fk;
  const StepCoeffs<double> sd =
      make_step_coeffs<double>(h->pv, YH_MODEL_FK3V, fk);
  auto fill = [&](auto &a) {
    using R = decltype(a.tc);
    a.nx = h->nx;
    a.ny = h->ny;
    a.eps = (R)h->smooth;
    a.sw_k = (R)(h->smooth > 0.0 ? -2.0 / (h->smooth * log(2.0)) : 0.0);
    a.sw_d = (R)(h->smooth > 0.0 ? 2.0 / h->smooth : 0.0);
    a.tc = (R)sd.tc;
    a.dt = (R)sd.dt;
    a.u_c = (R)sd.u_c;
    a.u_v = (R)sd.u_v;
    a.u_csi = (R)sd.u_csi;
    a.k2 = (R)sd.k_exp2;
    a.s_td = (R)sd.s_td;
    a.s_tr = (R)sd.s_tr;
    a.s_to = (R)sd.s_to;
    a.s_tsi = (R)sd.s_tsi;
    a.s_tvp = (R)sd.s_tvp;
    a.s_tv1m = (R)sd.s_tv1m;
    a.s_tv2m = (R)sd.s_tv2m;
    a.s_twp = (R)sd.s_twp;
    a.s_twm = (R)sd.s_twm;
  };
  fill(h->af);
  fill(h->ad);
}

}  // namespace

extern "C" int yh_adjoint_destroy(yh_adjoint *h) {
  if (!h) return YH_EINVAL;
  if (h->s) cudaStreamSynchronize(h->s);
  for (auto &g : h->graph)
    if (g) cudaGraphExecDestroy(g);
  cudaFree(h->ckpt);
  cudaFree(h->seg);
  cudaFree(h->lam);
  cudaFree(h->r);
  cudaFree(h->gr);
  cudaFree(h->target);
  cudaFree(h->loss);
  cudaFree(h->gp);
  cudaFree(h->gfk);
  if (h->s2) cudaStreamDestroy(h->s2);
  for (cudaEvent_t ev : {h->ev_fork, h->ev_join, h->ev_ready[0], h->ev_ready[1],
                         h->ev_free[0], h->ev_free[1]})
    if (ev) cudaEventDestroy(ev);
  if (h->own_stream && h->s) cudaStreamDestroy(h->s);
  delete h;
  return YH_OK;
}

extern "C" int yh_adjoint_create_batch(const yh_param_var *p,
                                       const yh_fk_params *fk, int batch,
                                       int nsteps, int frame_steps,
                                       int probe_spacing, int checkpoint_steps,
                                       int fp64, double smooth, void *stream,
                                       yh_adjoint **out) {
  if (!out) return YH_EINVAL;
  *out = nullptr;
  int rc = check_params(p, YH_MODEL_FK3V, fk);
  if (rc) return rc;
  if (p->hx != p->hy || batch < 1 || batch > 4096 || nsteps < 1 ||
      frame_steps < 1 || probe_spacing < 1 || probe_spacing > p->nx ||
      probe_spacing > p->ny || checkpoint_steps < 1 || !(smooth >= 0.0))
    return YH_EINVAL;
  yh_adjoint *h = new (std::nothrow) yh_adjoint();
  if (!h) return YH_ENOMEM;
  h->fp64 = fp64 ? 1 : 0;
  h->smooth = smooth;
  h->nx = p->nx;
  h->ny = p->ny;
  h->n = p->nx * p->ny;
  h->batch = batch;
  h->nsteps = nsteps;
  h->frame = frame_steps;
  h->sp = probe_spacing;
  h->npx = p->nx / probe_spacing;
  h->npy = p->ny / probe_spacing;
  h->ck = checkpoint_steps;
  h->frames = nsteps / frame_steps;
  h->rscale = p->dt / (p->hx * p->hx);
  h->tcdt = p->tc * p->dt;
  h->nrev = ((p->nx + 31) / 32) * ((p->ny + 7) / 8);
  h->pv = *p;
  set_coeffs(h, fk);
  const size_t es = h->fp64 ? sizeof(double) : sizeof(float);
  const size_t cells = (size_t)h->n * batch;
  const size_t state = 3 * cells * es;
  const size_t nck = (size_t)(nsteps - 1) / checkpoint_steps + 1;
  h->seg_states = checkpoint_steps == 1 ? 2 : (size_t)checkpoint_steps + 1;
  const size_t tgt = (size_t)std::max(1, h->frames) * h->npx * h->npy * batch;
  cudaError_t e = cudaSuccess;
  h->s = (cudaStream_t)stream;
  if (!h->s) {
    e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking);
    h->own_stream = e == cudaSuccess;
  }
  if (e == cudaSuccess) e = cudaMalloc(&h->ckpt, nck * state);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->seg, (checkpoint_steps == 1 ? 1 : 2) * h->seg_states * state);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->s2, cudaStreamNonBlocking);
  for (cudaEvent_t *ev : {&h->ev_fork, &h->ev_join, &h->ev_ready[0], &h->ev_ready[1],
                          &h->ev_free[0], &h->ev_free[1]})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&h->lam, 2 * state);
  if (e == cudaSuccess) e = cudaMalloc(&h->r, cells * es);
  if (e == cudaSuccess) e = cudaMalloc(&h->gr, cells * es);
  if (e == cudaSuccess) e = cudaMalloc(&h->target, tgt * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h->loss, batch * sizeof(double));
  if (e == cudaSuccess)
    e = cudaMalloc(&h->gp, (size_t)batch * h->nrev * 16 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->gfk, (size_t)batch * 16 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(h->target, 0, tgt * sizeof(float), h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) {
    yh_adjoint_destroy(h);
    return st(e);
  }
  *out = h;
  return YH_OK;
}

extern "C" int yh_adjoint_create(const yh_param_var *p, const yh_fk_params *fk,
                                 int nsteps, int frame_steps, int probe_spacing,
                                 int checkpoint_steps, int fp64, double smooth,
                                 void *stream, yh_adjoint **out) {
  return yh_adjoint_create_batch(p, fk, 1, nsteps, frame_steps, probe_spacing,
                                 checkpoint_steps, fp64, smooth, stream, out);
}

extern "C" int yh_adjoint_set_target(yh_adjoint *h, const float *target) {
  if (!h || !target) return YH_EINVAL;
  cudaError_t e = cudaMemcpyAsync(
      h->target, target,
      (size_t)h->batch * h->frames * h->npx * h->npy * sizeof(float),
      cudaMemcpyDefault, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  return st(e);
}

extern "C" int yh_adjoint_probes(yh_adjoint *h, int *frames, int *probes_x,
                                 int *probes_y) {
  if (!h) return YH_EINVAL;
  if (frames) *frames = h->frames;
  if (probes_x) *probes_x = h->npx;
  if (probes_y) *probes_y = h->npy;
  return YH_OK;
}

extern "C" int yh_adjoint_batch(yh_adjoint *h, int *batch) {
  if (!h || !batch) return YH_EINVAL;
  *batch = h->batch;
  return YH_OK;
}

extern "C" int yh_adjoint_run(yh_adjoint *h, const float *D, const float *u0,
                              const float *v0, const float *w0, double *loss,
                              float *grad_D) {
  if (!h || !D || !u0 || !v0 || !w0) return YH_EINVAL;
  return h->fp64 ? run_t<double>(h, D, u0, v0, w0, loss, grad_D, nullptr)
                 : run_t<float>(h, D, u0, v0, w0, loss, grad_D, nullptr);
}

extern "C" int yh_adjoint_run_fk(yh_adjoint *h, const float *D,
                                 const float *u0, const float *v0,
                                 const float *w0, double *loss, float *grad_D,
                                 yh_fk_params *grad_fk) {
  if (!h || !D || !u0 || !v0 || !w0 || !grad_fk) return YH_EINVAL;
  double *g = new (std::nothrow) double[(size_t)h->batch * 16];
  if (!g) return YH_ENOMEM;
  const int rc = h->fp64 ? run_t<double>(h, D, u0, v0, w0, loss, grad_D, g)
                         : run_t<float>(h, D, u0, v0, w0, loss, grad_D, g);
  if (rc) {
    delete[] g;
    return rc;
  }
  // chain rule from the raw parameters: s_X = tc dt / tau_X, so
  // ds_X/dtau_X = -s_X / tau_X; k2 = -2k / ln 2
  const yh_fk_params &f = h->fk;
  const double tau[9] = {f.tau_d, f.tau_r, f.tau_si, f.tau_0, f.tau_v_plus,
                         f.tau_v1_minus, f.tau_v2_minus, f.tau_w_plus,
                         f.tau_w_minus};
  for (int b = 0; b < h->batch; ++b) {
    const double *gb = g + (size_t)b * 16;
    double o[9];
    for (int q = 0; q < 9; ++q) o[q] = -gb[q] * h->tcdt / (tau[q] * tau[q]);
    yh_fk_params &d = grad_fk[b];
    d.tau_d = o[0];
    d.tau_r = o[1];
    d.tau_si = o[2];
    d.tau_0 = o[3];
    d.tau_v_plus = o[4];
    d.tau_v1_minus = o[5];
    d.tau_v2_minus = o[6];
    d.tau_w_plus = o[7];
    d.tau_w_minus = o[8];
    d.u_c = gb[9];
    d.u_v = gb[10];
    d.u_csi = gb[11];
    d.k = gb[12] * (-2.0 / log(2.0));
  }
  delete[] g;
  return YH_OK;
}

extern "C" int yh_adjoint_set_fk(yh_adjoint *h, const yh_fk_params *fk) {
  if (!h || !fk) return YH_EINVAL;
  const int rc = check_params(&h->pv, YH_MODEL_FK3V, fk);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  set_coeffs(h, fk);
  // the captured graphs hold the old coefficients as kernel arguments
  for (auto &g : h->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return YH_OK;
}

extern "C" int yh_adjoint_record(yh_adjoint *h, const float *D, const float *u0,
                                 const float *v0, const float *w0,
                                 float *probes) {
  if (!h || !D || !u0 || !v0 || !w0 || !probes) return YH_EINVAL;
  return h->fp64 ? record_t<double>(h, D, u0, v0, w0, probes)
                 : record_t<float>(h, D, u0, v0, w0, probes);
}
