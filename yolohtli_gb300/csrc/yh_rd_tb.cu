// Temporally blocked reaction-diffusion step: K explicit Euler steps per
// launch (FP32, models where only u diffuses: FK3V, or REF2V with
// gateDiff = 0).
//
// A block of 512 threads owns a 128 x 64 region of cells: an interior of
// (128 - 2K) x (64 - 2K) cells and a halo of K cells on each side. Each
// thread owns 16 cells (4 columns lane + 32k x 4 rows) and keeps their v, w
// in registers for all K sub-steps; u lives in a double-buffered
// shared-memory copy of the region (64 KB), the only field exchanged. After sub-step
// s the cells at distance >= s from the region edge are exact, so after K
// sub-steps the interior is, and only the interior is stored. At the domain
// edge the mirror ghost (helper_functions.cu:69-79) reads inward, so the
// region does not shrink on that side. Global traffic per interior
// cell-step is about (13 B x 128*64/interior + 12 B) / K instead of 25 B.
#include "yh_kernels.cuh"

namespace yh {

constexpr int kTbW = 128, kTbH = 64, kTbThreads = 512, kTbMaxK = 8;
constexpr int kTbSmem = 2 * kTbW * kTbH * 4 + kTbW * kTbH;  // u x2 + mask

int rd_tb_max_steps() { return kTbMaxK; }

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

template <int MODEL, bool HOLES>
__global__ void __launch_bounds__(kTbThreads, 1)
    rd_tb_kernel(const StepCoeffs<float> a, const Fld<float> in,
                 const Fld<float> out, const uint8_t *__restrict__ solid,
                 const int K) {
  extern __shared__ float4 smem4[];
  float *us0 = reinterpret_cast<float *>(smem4);
  float *us1 = us0 + kTbW * kTbH;
  uint8_t *ms = reinterpret_cast<uint8_t *>(us1 + kTbW * kTbH);
  const int nx = a.nx, ny = a.ny;
  const int TX = kTbW - 2 * K, TY = kTbH - 2 * K;
  const int x0 = (int)blockIdx.x * TX - K, y0 = (int)blockIdx.y * TY - K;
  const int lane = threadIdx.x & 31, wy = threadIdx.x >> 5;  // wy in 0..15
  const float *__restrict__ U = in.f[0];
  const float *__restrict__ V = in.f[1];
  const float *__restrict__ Wf = in.f[2];
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;

  float v[4][4], w[4][4];
  // load the region: u to shared memory, v, w to registers
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int ly = wy * 4 + r, gy = y0 + ly;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int lx = lane + 32 * k, gx = x0 + lx;
      const bool inside = (unsigned)gx < (unsigned)nx && (unsigned)gy < (unsigned)ny;
      const size_t idx = (size_t)gy * nx + gx;
      v[r][k] = inside ? __ldg(V + idx) : 0.f;
      w[r][k] = (W3 && inside) ? __ldg(Wf + idx) : 0.f;
      us0[ly * kTbW + lx] = inside ? __ldg(U + idx) : 0.f;
      if (HOLES) ms[ly * kTbW + lx] = inside ? solid[idx] : 0;
    }
  }
  __syncthreads();

  // per-cell hole codes (bit 0 tissue, bits 1-2 x pattern, bits 3-4 y
  // pattern), computed once from the mask and kept in shared memory in
  // place of the mask: 1 byte per cell instead of 4 registers per thread
  if (HOLES) {
    uint32_t code[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int ly = wy * 4 + r, gy = y0 + ly;
      const int lyS = min(max(gy == 0 ? ly + 1 : ly - 1, 0), kTbH - 1);
      const int lyN = min(max(gy == ny - 1 ? ly - 1 : ly + 1, 0), kTbH - 1);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int lx = lane + 32 * k, gx = x0 + lx;
        const int lxW = min(max(gx == 0 ? lx + 1 : lx - 1, 0), kTbW - 1);
        const int lxE = min(max(gx == nx - 1 ? lx - 1 : lx + 1, 0), kTbW - 1);
        const bool sc = ms[ly * kTbW + lx] != 0;
        const uint32_t px = hole_pattern(ms[ly * kTbW + lxW] != 0, sc,
                                         ms[ly * kTbW + lxE] != 0);
        const uint32_t py = hole_pattern(ms[lyN * kTbW + lx] != 0, sc,
                                         ms[lyS * kTbW + lx] != 0);
        code[r] |= ((sc ? 1u : 0u) | (px << 1) | (py << 3)) << (8 * k);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int k = 0; k < 4; ++k)
        ms[(wy * 4 + r) * kTbW + lane + 32 * k] = (uint8_t)(code[r] >> (8 * k));
    __syncthreads();
  }

  for (int s = 0; s < K; ++s) {
    const float *src = (s & 1) ? us1 : us0;
    float *dst = (s & 1) ? us0 : us1;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int ly = wy * 4 + r, gy = y0 + ly;
      const int lyS = min(max(gy == 0 ? ly + 1 : ly - 1, 0), kTbH - 1);
      const int lyN = min(max(gy == ny - 1 ? ly - 1 : ly + 1, 0), kTbH - 1);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int lx = lane + 32 * k, gx = x0 + lx;
        const bool inside = (unsigned)gx < (unsigned)nx && (unsigned)gy < (unsigned)ny;
        const int lxW = min(max(gx == 0 ? lx + 1 : lx - 1, 0), kTbW - 1);
        const int lxE = min(max(gx == nx - 1 ? lx - 1 : lx + 1, 0), kTbW - 1);
        const float uc = src[ly * kTbW + lx];
        const float uW = src[ly * kTbW + lxW], uE = src[ly * kTbW + lxE];
        const float uN = src[lyN * kTbW + lx], uS = src[lyS * kTbW + lx];
        float du;
        bool sc = true;
        if (HOLES) {
          const uint32_t c = ms[ly * kTbW + lx];
          sc = (c & 1u) != 0u;
          float cxw, cxc, cxe, cyn, cyc, cys;
          pattern_weights((c >> 1) & 3u, cxw, cxc, cxe);
          pattern_weights((c >> 3) & 3u, cyn, cyc, cys);
          du = (cxw * uW - cxc * uc + cxe * uE) * a.rx +
               (cyn * uN - cyc * uc + cys * uS) * a.ry;
        } else {
          du = (uW - 2.f * uc + uE) * a.rx + (uN - 2.f * uc + uS) * a.ry;
        }
        float ru, rv, rw;
        if (W3) {
          float J, gv, gw;
          fk3v_rates(a, uc, v[r][k], w[r][k], J, gv, gw);
          ru = du - a.dt * J;
          rv = a.dt * gv;
          rw = a.dt * gw;
        } else {
          float I_sum, I_v;
          ref2v_currents(a, uc, v[r][k], I_sum, I_v);
          ru = du - a.dt * I_sum;
          rv = 0.f - a.dt * I_v;
          rw = 0.f;
        }
        const bool live = inside && sc;
        const float un = live ? uc + a.tc * ru : 0.f;
        v[r][k] = live ? v[r][k] + a.tc * rv : 0.f;
        if (W3) w[r][k] = live ? w[r][k] + a.tc * rw : 0.f;
        dst[ly * kTbW + lx] = un;
      }
    }
    __syncthreads();
  }

  // store the interior; the last sub-step wrote us1 when K is odd
  const float *ufin = (K & 1) ? us1 : us0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int ly = wy * 4 + r, gy = y0 + ly;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int lx = lane + 32 * k, gx = x0 + lx;
      const bool keep = lx >= K && lx < kTbW - K && ly >= K && ly < kTbH - K &&
                        (unsigned)gx < (unsigned)nx && (unsigned)gy < (unsigned)ny;
      if (keep) {
        const size_t idx = (size_t)gy * nx + gx;
        out.f[0][idx] = ufin[ly * kTbW + lx];
        out.f[1][idx] = v[r][k];
        if (W3) out.f[2][idx] = w[r][k];
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
  rd_tb_kernel<MODEL, HOLES>
      <<<grid, kTbThreads, kTbSmem, s>>>(a, in, out, solid, K);
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
