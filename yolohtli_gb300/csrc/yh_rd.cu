// Explicit Euler reaction-diffusion step (the reference's
// reactionDiffusion_kernel, reactionDiffusion.cu:26-566, on its Euler /
// Neumann / 5-point path) and the stimulus box.
//
// rd_step_scalar: one cell per thread, any nx; also the FP64 instance (the
//                 REF2V FP64 step with its currents in the polynomial form
//                 of ref2v_rhs_poly and velTan as rhs * (1/dt)).
// rd_step_vec4:   FP32, four cells per thread with float4 loads/stores of
//                 the centre row and of the rows above and below (nx % 4 == 0).
// Both read the inputs through the read-only path and write every output
// exactly once (the reference rewrites g_in in place, reactionDiffusion.cu:117-118,508-509).
#include "yh_kernels.cuh"

namespace yh {

template <int MODEL, typename Real>
__device__ __forceinline__ void reaction(const StepCoeffs<Real> &a, Real u,
                                         Real v, Real w, Real du, Real dv,
                                         Real r[kMaxFields]) {
  if (MODEL == YH_MODEL_REF2V) {
    Real I_sum, I_v;
    ref2v_currents(a, u, v, I_sum, I_v);
    du -= a.dt * I_sum;
    dv -= a.dt * I_v;
    r[0] = du;
    r[1] = dv;
    r[2] = Real(0);
  } else {
    Real J, gv, gw;
    fk3v_rates(a, u, v, w, J, gv, gw);
    r[0] = du - a.dt * J;
    r[1] = a.dt * gv;
    r[2] = a.dt * gw;
  }
}

// velTan = rhs/dt (reactionDiffusion.cu:529-530) as rhs * (1/dt): one
// multiplication in place of a division (within an ulp of it).
__device__ __forceinline__ double tangent(const StepCoeffs<double> &a,
                                          double r) {
  return r * a.inv_dt;
}
__device__ __forceinline__ float tangent(const StepCoeffs<float> &a, float r) {
  return r * a.inv_dt;
}

// New values nv of one cell from its scaled Laplacians du, dv, and the
// tangent rhs/dt when TAN. The FP32 FK3V update without tangent takes the
// pre-scaled form (fk3v_update); every other case follows the reference's
// rhs / u0 += tc*rhs form (reactionDiffusion.cu:498-513).
template <int MODEL, bool TAN, typename Real>
__device__ __forceinline__ void cell_update(const StepCoeffs<Real> &a, Real u,
                                            Real v, Real w, Real du, Real dv,
                                            Real nv[kMaxFields],
                                            Real tv[kMaxFields]) {
  if constexpr (MODEL == YH_MODEL_FK3V && std::is_same<Real, float>::value &&
                !TAN) {
    fk3v_update(a, u, v, w, du, nv[0], nv[1], nv[2]);
  } else {
    Real r[kMaxFields];
    reaction<MODEL>(a, u, v, w, du, dv, r);
    const Real x0[3] = {u, v, w};
#pragma unroll
    for (int f = 0; f < kMaxFields; ++f) {
      nv[f] = x0[f] + a.tc * r[f];
      if (TAN) tv[f] = tangent(a, r[f]);
    }
  }
}

template <int MODEL, typename Real, bool HOLES, bool TAN>
__global__ void __launch_bounds__(256)
    rd_step_scalar(const StepCoeffs<Real> a, const Fld<Real> in,
                   const Fld<Real> out, const Fld<Real> tan,
                   const uint8_t *__restrict__ solid, int *reset) {
  constexpr int NF = MODEL == YH_MODEL_FK3V ? 3 : 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (reset && i == 0 && j == 0) *reset = 0;
  const int nx = a.nx, ny = a.ny;
  if (i >= nx || j >= ny) return;
  const int C = i + nx * j;
  const int W = mirror(i - 1, nx) + nx * j;
  const int E = mirror(i + 1, nx) + nx * j;
  const int S = i + nx * mirror(j - 1, ny);
  const int N = i + nx * mirror(j + 1, ny);
  const Real *__restrict__ U = in.f[0];
  const Real *__restrict__ V = in.f[1];
  const Real u = __ldg(U + C), v = __ldg(V + C);
  const Real w = NF > 2 ? __ldg(in.f[2] + C) : Real(0);
  bool sc = true;
  Real du, dv = Real(0);
  constexpr bool F32 = std::is_same<Real, float>::value;
  if constexpr (MODEL == YH_MODEL_REF2V && !F32) {
    if (HOLES) {
      sc = solid[C] != 0;
      Real cxw, cxc, cxe, cyn, cyc, cys;
      hole_coeffs(solid[W] != 0, sc, solid[E] != 0, cxw, cxc, cxe);
      hole_coeffs(solid[N] != 0, sc, solid[S] != 0, cyn, cyc, cys);
      du = (cxw * __ldg(U + W) - cxc * u + cxe * __ldg(U + E)) * a.rx +
           (cyn * __ldg(U + N) - cyc * u + cys * __ldg(U + S)) * a.ry;
      if (a.gate_diff)
        dv = (cxw * __ldg(V + W) - cxc * v + cxe * __ldg(V + E)) * a.rxs +
             (cyn * __ldg(V + N) - cyc * v + cys * __ldg(V + S)) * a.rys;
    } else {
      const Real hx = fma(Real(-2), u, __ldg(U + W) + __ldg(U + E));
      const Real hy = fma(Real(-2), u, __ldg(U + N) + __ldg(U + S));
      du = fma(hx, a.rx, hy * a.ry);
      if (a.gate_diff) {
        const Real gx = fma(Real(-2), v, __ldg(V + W) + __ldg(V + E));
        const Real gy = fma(Real(-2), v, __ldg(V + N) + __ldg(V + S));
        dv = fma(gx, a.rxs, gy * a.rys);
      }
    }
    Real r0, r1;
    ref2v_rhs_poly(a, u, v, du, dv, r0, r1);
    out.f[0][C] = sc ? fma(a.tc, r0, u) : Real(0);
    out.f[1][C] = sc ? fma(a.tc, r1, v) : Real(0);
    if (TAN) {
      tan.f[0][C] = sc ? r0 * a.inv_dt : Real(0);
      tan.f[1][C] = sc ? r1 * a.inv_dt : Real(0);
    }
    return;
  }
  if (HOLES) {
    sc = solid[C] != 0;
    Real cxw, cxc, cxe, cyn, cyc, cys;
    hole_coeffs(solid[W] != 0, sc, solid[E] != 0, cxw, cxc, cxe);
    hole_coeffs(solid[N] != 0, sc, solid[S] != 0, cyn, cyc, cys);
    if constexpr (F32)
      du = lap5(a, lap_axis(__ldg(U + W), u, __ldg(U + E), cxw, cxc, cxe),
                lap_axis(__ldg(U + N), u, __ldg(U + S), cyn, cyc, cys));
    else
      du = (cxw * __ldg(U + W) - cxc * u + cxe * __ldg(U + E)) * a.rx +
           (cyn * __ldg(U + N) - cyc * u + cys * __ldg(U + S)) * a.ry;
    if (MODEL == YH_MODEL_REF2V && a.gate_diff)
      dv = (cxw * __ldg(V + W) - cxc * v + cxe * __ldg(V + E)) * a.rx *
               a.rscale +
           (cyn * __ldg(V + N) - cyc * v + cys * __ldg(V + S)) * a.ry *
               a.rscale;
  } else {
    if constexpr (F32)
      du = lap5(a, lap_axis(__ldg(U + W), u, __ldg(U + E)),
                lap_axis(__ldg(U + N), u, __ldg(U + S)));
    else
      du = (__ldg(U + W) - Real(2) * u + __ldg(U + E)) * a.rx +
           (__ldg(U + N) - Real(2) * u + __ldg(U + S)) * a.ry;
    if (MODEL == YH_MODEL_REF2V && a.gate_diff)
      dv = (__ldg(V + W) - Real(2) * v + __ldg(V + E)) * a.rx * a.rscale +
           (__ldg(V + N) - Real(2) * v + __ldg(V + S)) * a.ry * a.rscale;
  }
  Real nv[kMaxFields], tv[kMaxFields];
  cell_update<MODEL, TAN>(a, u, v, w, du, dv, nv, tv);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    out.f[f][C] = sc ? nv[f] : Real(0);
    if (TAN) tan.f[f][C] = sc ? tv[f] : Real(0);
  }
}

#ifndef YH_PDL
#define YH_PDL 1
#endif

// Per-cell hole codes of a mask, computed once per grid: bit 0 tissue,
// bits 1-2 the x pattern and bits 3-4 the y pattern of hole_pattern (the
// coefficient triples of reactionDiffusion.cu:162-169 with mirrored
// neighbours at the domain edge). 0x01 is a tissue cell with four tissue
// neighbours.
__global__ void hole_codes_kernel(const uint8_t *__restrict__ solid, int nx,
                                  int ny, uint8_t *__restrict__ codes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t row = (size_t)nx * j;
  const bool sc = solid[row + i] != 0;
  const bool sw = solid[row + mirror(i - 1, nx)] != 0;
  const bool se = solid[row + mirror(i + 1, nx)] != 0;
  const bool sn = solid[(size_t)nx * mirror(j + 1, ny) + i] != 0;
  const bool ss = solid[(size_t)nx * mirror(j - 1, ny) + i] != 0;
  codes[row + i] = (uint8_t)((sc ? 1u : 0u) | (hole_pattern(sw, sc, se) << 1) |
                             (hole_pattern(sn, sc, ss) << 3));
}

cudaError_t launch_hole_codes(const uint8_t *solid, int nx, int ny,
                              uint8_t *codes, cudaStream_t s) {
  const dim3 block(32, 8);
  const dim3 grid((nx + 31) / 32, (ny + 7) / 8);
  hole_codes_kernel<<<grid, block, 0, s>>>(solid, nx, ny, codes);
  return cudaGetLastError();
}

// FP32 fast path: thread (tx, j) owns cells 4*tx .. 4*tx+3 of row j.
// CODES: `solid` holds the per-cell hole codes of hole_codes_kernel instead
// of the mask; a thread whose 4 cells are all 0x01 takes the select-free
// expression (the same bits as the coefficient form with (1, 2, 1)).
template <int MODEL, bool HOLES, bool TAN, bool CODES>
__global__ void __launch_bounds__(256)
    rd_step_vec4(const StepCoeffs<float> a, const Fld<float> in,
                 const Fld<float> out, const Fld<float> tan,
                 const uint8_t *__restrict__ solid, int *reset) {
  constexpr int NF = MODEL == YH_MODEL_FK3V ? 3 : 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;  // float4 column
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny, nq = nx >> 2;
  if (q >= nq || j >= ny) return;
  const int i0 = q << 2;
  const int row = nx * j;
  const int rowS = nx * mirror(j - 1, ny);
  const int rowN = nx * mirror(j + 1, ny);
  const int iw = mirror(i0 - 1, nx), ie = mirror(i0 + 4, nx);
  grid_dep_wait();
  grid_dep_launch();
  if (reset && q == 0 && j == 0) *reset = 0;
  const float *__restrict__ U = in.f[0];
  const float4 uc = __ldg(reinterpret_cast<const float4 *>(U + row + i0));
  const float4 un = __ldg(reinterpret_cast<const float4 *>(U + rowN + i0));
  const float4 us = __ldg(reinterpret_cast<const float4 *>(U + rowS + i0));
  const float uw = __ldg(U + row + iw), ue = __ldg(U + row + ie);
  float4 fv[NF];
#pragma unroll
  for (int f = 1; f < NF; ++f)
    fv[f] = __ldg(reinterpret_cast<const float4 *>(in.f[f] + row + i0));
  fv[0] = uc;
  float4 vn, vs;
  float vw = 0.f, ve = 0.f;
  const bool vdiff = MODEL == YH_MODEL_REF2V && a.gate_diff;
  if (vdiff) {
    const float *__restrict__ V = in.f[1];
    vn = __ldg(reinterpret_cast<const float4 *>(V + rowN + i0));
    vs = __ldg(reinterpret_cast<const float4 *>(V + rowS + i0));
    vw = __ldg(V + row + iw);
    ve = __ldg(V + row + ie);
  }
  uchar4 mc, mn, ms;
  uint8_t mw = 1, me = 1;
  uint32_t code4 = 0x01010101u;
  if (HOLES && CODES) {
    code4 = __ldg(reinterpret_cast<const unsigned int *>(solid + row + i0));
  } else if (HOLES) {
    mc = *reinterpret_cast<const uchar4 *>(solid + row + i0);
    mn = *reinterpret_cast<const uchar4 *>(solid + rowN + i0);
    ms = *reinterpret_cast<const uchar4 *>(solid + rowS + i0);
    mw = solid[row + iw];
    me = solid[row + ie];
  }
  const bool plain = HOLES && CODES && code4 == 0x01010101u;
  const float ucv[4] = {uc.x, uc.y, uc.z, uc.w};
  const float unv[4] = {un.x, un.y, un.z, un.w};
  const float usv[4] = {us.x, us.y, us.z, us.w};
  if constexpr (MODEL == YH_MODEL_FK3V && !TAN) {
    // two f32x2 pairs; the mask form builds the hole codes on the fly
    if (HOLES && !CODES) {
      const uint8_t c8[4] = {mc.x, mc.y, mc.z, mc.w};
      const uint8_t n8[4] = {mn.x, mn.y, mn.z, mn.w};
      const uint8_t s8[4] = {ms.x, ms.y, ms.z, ms.w};
      code4 = 0u;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool sc = c8[k] != 0;
        const bool sw = (k == 0 ? mw : c8[k - 1]) != 0;
        const bool se = (k == 3 ? me : c8[k + 1]) != 0;
        code4 |= ((sc ? 1u : 0u) | (hole_pattern(sw, sc, se) << 1) |
                  (hole_pattern(n8[k] != 0, sc, s8[k] != 0) << 3))
                 << (8 * k);
      }
    }
    const float vv[4] = {fv[1].x, fv[1].y, fv[1].z, fv[1].w};
    const float ww[4] = {fv[2].x, fv[2].y, fv[2].z, fv[2].w};
    float ou[4], ov[4], ow[4];
    fk3v_cells4(a, !HOLES || code4 == 0x01010101u, code4, ucv, uw, ue, unv,
                usv, vv, ww, ou, ov, ow);
    *reinterpret_cast<float4 *>(out.f[0] + row + i0) =
        make_float4(ou[0], ou[1], ou[2], ou[3]);
    *reinterpret_cast<float4 *>(out.f[1] + row + i0) =
        make_float4(ov[0], ov[1], ov[2], ov[3]);
    *reinterpret_cast<float4 *>(out.f[2] + row + i0) =
        make_float4(ow[0], ow[1], ow[2], ow[3]);
    return;
  }
  float res[NF][4], tres[NF][4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float u = ucv[k];
    const float uW = k == 0 ? uw : ucv[k - 1];
    const float uE = k == 3 ? ue : ucv[k + 1];
    float x[3];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const float4 t = fv[f];
      x[f] = k == 0 ? t.x : (k == 1 ? t.y : (k == 2 ? t.z : t.w));
    }
    if (NF < 3) x[2] = 0.f;
    bool sc = true;
    float du, dv = 0.f;
    if (HOLES && !plain) {
      float cxw, cxc, cxe, cyn, cyc, cys;
      if (CODES) {
        const uint32_t cc = code4 >> (8 * k);
        sc = (cc & 1u) != 0u;
        pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
        pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
      } else {
        const uint8_t c8[4] = {mc.x, mc.y, mc.z, mc.w};
        const uint8_t n8[4] = {mn.x, mn.y, mn.z, mn.w};
        const uint8_t s8[4] = {ms.x, ms.y, ms.z, ms.w};
        sc = c8[k] != 0;
        const bool sw = (k == 0 ? mw : c8[k - 1]) != 0;
        const bool se = (k == 3 ? me : c8[k + 1]) != 0;
        hole_coeffs(sw, sc, se, cxw, cxc, cxe);
        hole_coeffs(n8[k] != 0, sc, s8[k] != 0, cyn, cyc, cys);
      }
      du = lap5(a, lap_axis(uW, u, uE, cxw, cxc, cxe),
                lap_axis(unv[k], u, usv[k], cyn, cyc, cys));
      if (vdiff) {
        const float4 vc = fv[1];
        const float vcv[4] = {vc.x, vc.y, vc.z, vc.w};
        const float vnv[4] = {vn.x, vn.y, vn.z, vn.w};
        const float vsv[4] = {vs.x, vs.y, vs.z, vs.w};
        const float vW = k == 0 ? vw : vcv[k - 1];
        const float vE = k == 3 ? ve : vcv[k + 1];
        dv = (cxw * vW - cxc * vcv[k] + cxe * vE) * a.rx * a.rscale +
             (cyn * vnv[k] - cyc * vcv[k] + cys * vsv[k]) * a.ry * a.rscale;
      }
    } else {
      du = lap5(a, lap_axis(uW, u, uE), lap_axis(unv[k], u, usv[k]));
      if (vdiff) {
        const float4 vc = fv[1];
        const float vcv[4] = {vc.x, vc.y, vc.z, vc.w};
        const float vnv[4] = {vn.x, vn.y, vn.z, vn.w};
        const float vsv[4] = {vs.x, vs.y, vs.z, vs.w};
        const float vW = k == 0 ? vw : vcv[k - 1];
        const float vE = k == 3 ? ve : vcv[k + 1];
        dv = (vW - 2.f * vcv[k] + vE) * a.rx * a.rscale +
             (vnv[k] - 2.f * vcv[k] + vsv[k]) * a.ry * a.rscale;
      }
    }
    float nv[kMaxFields], tv[kMaxFields];
    cell_update<MODEL, TAN>(a, x[0], x[1], x[2], du, dv, nv, tv);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      res[f][k] = sc ? nv[f] : 0.f;
      if (TAN) tres[f][k] = sc ? tv[f] : 0.f;
    }
  }
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    *reinterpret_cast<float4 *>(out.f[f] + row + i0) =
        make_float4(res[f][0], res[f][1], res[f][2], res[f][3]);
    if (TAN)
      *reinterpret_cast<float4 *>(tan.f[f] + row + i0) =
          make_float4(tres[f][0], tres[f][1], tres[f][2], tres[f][3]);
  }
}

template <typename Real>
__global__ void stimulate_box_kernel(Real *u, const uint8_t *solid, int nx,
                                     int i0, int j0, int i1, int j1,
                                     Real value) {
  const int i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = j0 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= i1 || j >= j1) return;
  const int C = i + nx * j;
  if (!solid || solid[C]) u[C] = value;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

template <int MODEL, typename Real, bool HOLES, bool TAN>
static cudaError_t launch_rd_t(const StepCoeffs<Real> &a, const Fld<Real> &in,
                               const Fld<Real> &out, const Fld<Real> &tan,
                               const uint8_t *solid, const uint8_t *codes,
                               cudaStream_t s, int *reset) {
  if constexpr (std::is_same<Real, float>::value) {
    const uint8_t *m = HOLES && codes ? codes : solid;
    if ((a.nx % 4) == 0 && aligned16(in, MODEL) && aligned16(out, MODEL) &&
        (!TAN || aligned16(tan, MODEL)) &&
        (!HOLES || (reinterpret_cast<uintptr_t>(m) & 3) == 0)) {
      const dim3 block(64, 4);
      const dim3 grid((a.nx / 4 + block.x - 1) / block.x,
                      (a.ny + block.y - 1) / block.y);
      // Programmatic stream serialization: the next step's blocks are
      // scheduled while this one drains and wait in grid_dep_wait.
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = grid;
      cfg.blockDim = block;
      cfg.stream = s;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = YH_PDL;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      if (HOLES && codes)
        return cudaLaunchKernelEx(&cfg, rd_step_vec4<MODEL, HOLES, TAN, true>,
                                  a, in, out, tan, codes, reset);
      return cudaLaunchKernelEx(&cfg, rd_step_vec4<MODEL, HOLES, TAN, false>,
                                a, in, out, tan, solid, reset);
    }
  }
  {
    const dim3 block(32, 8);
    const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8);
    rd_step_scalar<MODEL, Real, HOLES, TAN>
        <<<grid, block, 0, s>>>(a, in, out, tan, solid, reset);
  }
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_rd_step(const StepCoeffs<Real> &a, const Fld<Real> &in,
                           const Fld<Real> &out, const Fld<Real> &tan,
                           const uint8_t *solid, cudaStream_t s,
                           const uint8_t *codes, int *reset) {
  const bool holes = solid != nullptr;
  const bool t = tan.f[0] != nullptr;
#define YH_RD_CASE(M, H, T)                                             \
  if (a.model == M && holes == H && t == T)                             \
    return launch_rd_t<M, Real, H, T>(a, in, out, tan, solid, codes, s, reset);
  YH_RD_CASE(YH_MODEL_REF2V, false, false)
  YH_RD_CASE(YH_MODEL_REF2V, false, true)
  YH_RD_CASE(YH_MODEL_REF2V, true, false)
  YH_RD_CASE(YH_MODEL_REF2V, true, true)
  YH_RD_CASE(YH_MODEL_FK3V, false, false)
  YH_RD_CASE(YH_MODEL_FK3V, false, true)
  YH_RD_CASE(YH_MODEL_FK3V, true, false)
  YH_RD_CASE(YH_MODEL_FK3V, true, true)
#undef YH_RD_CASE
  return cudaErrorInvalidValue;
}

template <typename Real>
cudaError_t launch_stimulate(Real *u, const uint8_t *solid, int nx, int ny,
                             int i0, int j0, int i1, int j1, Real value,
                             cudaStream_t s) {
  i0 = i0 < 0 ? 0 : i0;
  j0 = j0 < 0 ? 0 : j0;
  i1 = i1 > nx ? nx : i1;
  j1 = j1 > ny ? ny : j1;
  if (i1 <= i0 || j1 <= j0) return cudaSuccess;
  const dim3 block(32, 8);
  const dim3 grid((i1 - i0 + 31) / 32, (j1 - j0 + 7) / 8);
  stimulate_box_kernel<Real>
      <<<grid, block, 0, s>>>(u, solid, nx, i0, j0, i1, j1, value);
  return cudaGetLastError();
}

template cudaError_t launch_rd_step<float>(const StepCoeffs<float> &,
                                           const Fld<float> &,
                                           const Fld<float> &,
                                           const Fld<float> &,
                                           const uint8_t *, cudaStream_t,
                                           const uint8_t *, int *);
template cudaError_t launch_rd_step<double>(const StepCoeffs<double> &,
                                            const Fld<double> &,
                                            const Fld<double> &,
                                            const Fld<double> &,
                                            const uint8_t *, cudaStream_t,
                                            const uint8_t *, int *);
template cudaError_t launch_stimulate<float>(float *, const uint8_t *, int,
                                             int, int, int, int, int, float,
                                             cudaStream_t);
template cudaError_t launch_stimulate<double>(double *, const uint8_t *, int,
                                              int, int, int, int, int, double,
                                              cudaStream_t);

}  // namespace yh
