// Temporally blocked reaction-diffusion step: K explicit Euler steps per
// launch (FP32, models where only u diffuses: FK3V, or REF2V with
// gateDiff = 0).
//
// A block of 512 threads (16 warps) owns a 128 x 64 region of cells: an
// interior of (128 - 2K) x (64 - 2K) cells and a halo of K cells on each
// side. Thread (lane, warp) owns the 4 x 4 cells of columns 4*lane .. +3
// and rows 4*warp .. +3 for all K sub-steps: their u in registers, their v
// and w in the thread's own float4 slots of shared memory (no other thread
// reads them: only u diffuses). Neighbours come from the thread's registers, from the
// adjacent lanes by one warp shuffle per row (W of column 0, E of column 3),
// and from the adjacent warps by one float4 row exchange in shared memory
// per sub-step (S of the first row, N of the last): one __syncthreads per
// sub-step.
// After sub-step s the cells at distance >= s from the region edge are
// exact, so after K sub-steps the interior is, and only the interior is
// stored. At the domain edge the mirror ghost (helper_functions.cu:69-79)
// reads inward, so the region does not shrink on that side. Global traffic
// per interior cell-step is about (13 B x 128*64/interior + 12 B) / K
// instead of 25 B.
#include "yh_kernels.cuh"

namespace yh {

constexpr int kTbW = 128, kTbH = 64, kTbThreads = 512, kTbMaxK = 8;
constexpr int kTbWarps = kTbThreads / 32;
constexpr int kR = kTbH / kTbWarps;  // rows per thread
// edge rows [2 buffers][bottom/top][warps][128 floats], then the region's
// v and w [2][64][128]
constexpr int kTbEdge = 2 * 2 * kTbWarps * kTbW;
constexpr int kTbSmem = (kTbEdge + 2 * kTbW * kTbH) * 4;

int rd_tb_max_steps() { return kTbMaxK; }

__device__ __forceinline__ float4 f4(const float x[4]) {
  return make_float4(x[0], x[1], x[2], x[3]);
}

template <int MODEL, bool HOLES>
__global__ void __launch_bounds__(kTbThreads, 1)
    rd_tb_kernel(const StepCoeffs<float> a, const Fld<float> in,
                 const Fld<float> out, const uint8_t *__restrict__ solid,
                 const int K, const bool vec_ok) {
  extern __shared__ float4 smem4[];
  float *edge = reinterpret_cast<float *>(smem4);  // [2][2][16][128]
  float *vs = edge + kTbEdge;                      // [64][128]
  float *ws = vs + kTbW * kTbH;                    // [64][128]
  const int nx = a.nx, ny = a.ny;
  const int TX = kTbW - 2 * K, TY = kTbH - 2 * K;
  const int x0 = (int)blockIdx.x * TX - K, y0 = (int)blockIdx.y * TY - K;
  const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
  const int lx0 = 4 * lane, ly0 = kR * wy;
  const int gx0 = x0 + lx0, gy0 = y0 + ly0;
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;

  // domain-edge flags: bit k of xw/xe: column k is the first/last column;
  // bit r of ys/yn: row r is the first/last row; inx/iny: inside the domain
  uint32_t xw = 0, xe = 0, ys = 0, yn = 0, inx = 0, iny = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int gx = gx0 + k;
    xw |= (gx == 0 ? 1u : 0u) << k;
    xe |= (gx == nx - 1 ? 1u : 0u) << k;
    inx |= ((unsigned)gx < (unsigned)nx ? 1u : 0u) << k;
  }
#pragma unroll
  for (int r = 0; r < kR; ++r) {
    const int gy = gy0 + r;
    ys |= (gy == 0 ? 1u : 0u) << r;
    yn |= (gy == ny - 1 ? 1u : 0u) << r;
    iny |= ((unsigned)gy < (unsigned)ny ? 1u : 0u) << r;
  }

  float u[kR][4], v[4], w[4];
  uint32_t m[kR];  // tissue bits of the 4 cells of a row
  // float4 loads need a 16-byte aligned address: every row start is one
  // only when nx % 4 == 0 and the fields are 16-byte aligned (vec_ok, from
  // the host), and this thread's first column must be a multiple of 4
  const bool vec = vec_ok && ((x0 & 3) == 0) && inx == 0xFu;
#pragma unroll
  for (int r = 0; r < kR; ++r) {
    m[r] = 0u;
    const bool rowin = (iny >> r) & 1u;
    const size_t base = (size_t)(gy0 + r) * nx + gx0;
    if (rowin && vec) {
      const float4 q0 = __ldg(reinterpret_cast<const float4 *>(in.f[0] + base));
      const float4 q1 = __ldg(reinterpret_cast<const float4 *>(in.f[1] + base));
      u[r][0] = q0.x; u[r][1] = q0.y; u[r][2] = q0.z; u[r][3] = q0.w;
      v[0] = q1.x; v[1] = q1.y; v[2] = q1.z; v[3] = q1.w;
      if (W3) {
        const float4 q2 = __ldg(reinterpret_cast<const float4 *>(in.f[2] + base));
        w[0] = q2.x; w[1] = q2.y; w[2] = q2.z; w[3] = q2.w;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool ok = rowin && ((inx >> k) & 1u);
        u[r][k] = ok ? __ldg(in.f[0] + base + k) : 0.f;
        v[k] = ok ? __ldg(in.f[1] + base + k) : 0.f;
        w[k] = (W3 && ok) ? __ldg(in.f[2] + base + k) : 0.f;
      }
    }
    *reinterpret_cast<float4 *>(vs + (ly0 + r) * kTbW + lx0) = f4(v);
    if (W3) *reinterpret_cast<float4 *>(ws + (ly0 + r) * kTbW + lx0) = f4(w);
    if (HOLES) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const bool ok = rowin && ((inx >> k) & 1u);
        m[r] |= (ok && solid[base + k] ? 1u : 0u) << k;
      }
    }
  }

  // per-cell hole codes (bit 0 tissue, bits 1-2 x pattern, bits 3-4 y
  // pattern), from the tissue bits of the cell and its mirrored neighbours
  uint32_t code[kR];
#pragma unroll
  for (int r = 0; r < kR; ++r) code[r] = 0u;
  if (HOLES) {
    uint32_t *eb = reinterpret_cast<uint32_t *>(edge);
    eb[wy * 32 + lane] = m[0];                       // bottom rows
    eb[kTbWarps * 32 + wy * 32 + lane] = m[kR - 1];  // top rows
    __syncthreads();
    const uint32_t mS = wy > 0 ? eb[kTbWarps * 32 + (wy - 1) * 32 + lane] : m[0];
    const uint32_t mN = wy < kTbWarps - 1 ? eb[(wy + 1) * 32 + lane] : m[kR - 1];
#pragma unroll
    for (int r = 0; r < kR; ++r) {
      const uint32_t left = __shfl_up_sync(0xffffffffu, m[r], 1);
      const uint32_t right = __shfl_down_sync(0xffffffffu, m[r], 1);
      const uint32_t below = r > 0 ? m[r - 1] : mS;
      const uint32_t above = r < kR - 1 ? m[r + 1] : mN;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        bool sw = k > 0 ? (m[r] >> (k - 1)) & 1u : (left >> 3) & 1u;
        bool se = k < 3 ? (m[r] >> (k + 1)) & 1u : right & 1u;
        bool ss = (below >> k) & 1u, sn = (above >> k) & 1u;
        const bool tw = sw, ts = ss;
        if ((xw >> k) & 1u) sw = se;  // mirror: W of the first column is E
        if ((xe >> k) & 1u) se = tw;
        if ((ys >> r) & 1u) ss = sn;
        if ((yn >> r) & 1u) sn = ts;
        const bool sc = (m[r] >> k) & 1u;
        const uint32_t px = hole_pattern(sw, sc, se);
        const uint32_t py = hole_pattern(sn, sc, ss);
        code[r] |= ((sc ? 1u : 0u) | (px << 1) | (py << 3)) << (8 * k);
      }
    }
    __syncthreads();
  }

  // rows whose 4 cells are inside the domain, off its edges, tissue with
  // tissue neighbours: the common case, updated without selects
  uint32_t plain = 0u;
#pragma unroll
  for (int r = 0; r < kR; ++r) {
    const bool p = xw == 0u && xe == 0u && inx == 0xFu && ((iny >> r) & 1u) &&
                   !((ys >> r) & 1u) && !((yn >> r) & 1u) &&
                   (!HOLES || code[r] == 0x01010101u);
    plain |= (p ? 1u : 0u) << r;
  }

  for (int s = 0; s < K; ++s) {
    float *bot = edge + (s & 1) * 2 * kTbWarps * kTbW;
    float *top = bot + kTbWarps * kTbW;
    *reinterpret_cast<float4 *>(bot + wy * kTbW + lx0) = f4(u[0]);
    *reinterpret_cast<float4 *>(top + wy * kTbW + lx0) = f4(u[kR - 1]);
    __syncthreads();
    const float4 qs = wy > 0 ? *reinterpret_cast<const float4 *>(top + (wy - 1) * kTbW + lx0)
                             : f4(u[0]);
    const float4 qn = wy < kTbWarps - 1
                          ? *reinterpret_cast<const float4 *>(bot + (wy + 1) * kTbW + lx0)
                          : f4(u[kR - 1]);
    const float rowN[4] = {qn.x, qn.y, qn.z, qn.w};
    // rows are updated in place, bottom to top: `prev` keeps the old values
    // of the row below, which its own update has overwritten
    float prev[4] = {qs.x, qs.y, qs.z, qs.w};
#pragma unroll
    for (int r = 0; r < kR; ++r) {
      const float left = __shfl_up_sync(0xffffffffu, u[r][3], 1);
      const float right = __shfl_down_sync(0xffffffffu, u[r][0], 1);
      float4 *vp = reinterpret_cast<float4 *>(vs + (ly0 + r) * kTbW + lx0);
      float4 *wp = reinterpret_cast<float4 *>(ws + (ly0 + r) * kTbW + lx0);
      const float4 v4 = *vp;
      const float4 w4 = W3 ? *wp : make_float4(0.f, 0.f, 0.f, 0.f);
      float v[4] = {v4.x, v4.y, v4.z, v4.w};
      float w[4] = {w4.x, w4.y, w4.z, w4.w};
      float un[4];
      if ((plain >> r) & 1u) {
        // interior tissue row away from the domain edge: no selects
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float uc = u[r][k];
          const float uW = k > 0 ? u[r][k - 1] : left;
          const float uE = k < 3 ? u[r][k + 1] : right;
          const float uN = r < kR - 1 ? u[r + 1][k] : rowN[k];
          const float du =
              lap5(a, lap_axis(uW, uc, uE), lap_axis(uN, uc, prev[k]));
          tb_update<MODEL>(a, uc, v[k], w[k], du, un[k], v[k], w[k]);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float uc = u[r][k];
          float uW = k > 0 ? u[r][k - 1] : left;
          float uE = k < 3 ? u[r][k + 1] : right;
          float uS = prev[k];
          float uN = r < kR - 1 ? u[r + 1][k] : rowN[k];
          const float tW = uW, tS = uS;
          if ((xw >> k) & 1u) uW = uE;
          if ((xe >> k) & 1u) uE = tW;
          if ((ys >> r) & 1u) uS = uN;
          if ((yn >> r) & 1u) uN = tS;
          float du;
          bool sc = true;
          if (HOLES) {
            const uint32_t c = code[r] >> (8 * k);
            sc = (c & 1u) != 0u;
            float cxw, cxc, cxe, cyn, cyc, cys;
            pattern_weights((c >> 1) & 3u, cxw, cxc, cxe);
            pattern_weights((c >> 3) & 3u, cyn, cyc, cys);
            du = lap5(a, lap_axis(uW, uc, uE, cxw, cxc, cxe),
                      lap_axis(uN, uc, uS, cyn, cyc, cys));
          } else {
            du = lap5(a, lap_axis(uW, uc, uE), lap_axis(uN, uc, uS));
          }
          float nu, nv, nw;
          tb_update<MODEL>(a, uc, v[k], w[k], du, nu, nv, nw);
          const bool live = sc && ((inx >> k) & 1u) && ((iny >> r) & 1u);
          un[k] = live ? nu : 0.f;
          v[k] = live ? nv : 0.f;
          w[k] = live ? nw : 0.f;
        }
      }
      *vp = f4(v);
      if (W3) *wp = f4(w);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        prev[k] = u[r][k];
        u[r][k] = un[k];
      }
    }
  }

  // store the interior
#pragma unroll
  for (int r = 0; r < kR; ++r) {
    const int ly = ly0 + r;
    if (ly < K || ly >= kTbH - K || !((iny >> r) & 1u)) continue;
    const size_t base = (size_t)(gy0 + r) * nx + gx0;
    const float *vr = vs + ly * kTbW + lx0;
    const float *wr = ws + ly * kTbW + lx0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int lx = lx0 + k;
      if (lx >= K && lx < kTbW - K && ((inx >> k) & 1u)) {
        out.f[0][base + k] = u[r][k];
        out.f[1][base + k] = vr[k];
        if (W3) out.f[2][base + k] = wr[k];
      }
    }
  }
}

template <int MODEL, bool HOLES>
static cudaError_t launch_tb_t(const StepCoeffs<float> &a,
                               const Fld<float> &in, const Fld<float> &out,
                               const uint8_t *solid, int K, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(
        rd_tb_kernel<MODEL, HOLES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        kTbSmem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int TX = kTbW - 2 * K, TY = kTbH - 2 * K;
  const dim3 grid((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY);
  const bool vec_ok = (a.nx % 4) == 0 && aligned16(in, MODEL);
  rd_tb_kernel<MODEL, HOLES>
      <<<grid, kTbThreads, kTbSmem, s>>>(a, in, out, solid, K, vec_ok);
  return cudaGetLastError();
}

// K steps out <- in in one launch; cudaErrorNotSupported when the model
// diffuses more than u (REF2V with gateDiff) or K is out of [1, kTbMaxK].
cudaError_t launch_rd_tb(const StepCoeffs<float> &a, const Fld<float> &in,
                         const Fld<float> &out, const uint8_t *solid, int K,
                         cudaStream_t s) {
  if (K < 1 || K > kTbMaxK) return cudaErrorNotSupported;
  if (a.model == YH_MODEL_REF2V && a.gate_diff) return cudaErrorNotSupported;
  const bool holes = solid != nullptr;
  if (a.model == YH_MODEL_FK3V)
    return holes ? launch_tb_t<YH_MODEL_FK3V, true>(a, in, out, solid, K, s)
                 : launch_tb_t<YH_MODEL_FK3V, false>(a, in, out, solid, K, s);
  return holes ? launch_tb_t<YH_MODEL_REF2V, true>(a, in, out, solid, K, s)
               : launch_tb_t<YH_MODEL_REF2V, false>(a, in, out, solid, K, s);
}

}  // namespace yh
