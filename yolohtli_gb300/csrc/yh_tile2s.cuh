// The two-step tile scheme shared by the single-grid and batched kernels:
// 64 x 16 output tiles of 256 threads, u with a 2-cell halo and v, w, hole
// codes over the tile and its 1-cell ring in shared memory, step 1 on the
// tile and the ring, step 2 on the tile; the arithmetic of the single-step
// kernels (the same bits as two single steps). The inputs arrive by plain
// loads or by TMA bulk tensor copies (helpers below).
#pragma once

#include <cuda.h>          // CUtensorMap and its enums (types only)
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled

#include "yh_kernels.cuh"

namespace yh {
namespace tile2s {

constexpr int kTW = 64, kTH = 16;          // output tile (cells)
constexpr int kThreads = 256;              // one quad of the tile each
constexpr int kW0 = kTW + 4, kH0 = kTH + 4;  // u with a 2-cell halo
constexpr int kW1 = kTW + 2, kH1 = kTH + 2;  // step-1 u with a 1-cell ring
constexpr int kRing = 2 * kW1 + 2 * kTH;     // 164 ring cells
// Shared rows are 72 floats; U0 column c lives at c + 2 and U1 column c at
// c + 3, so that every quad's first cell is 16-byte aligned.
constexpr int kS = 72;

// Steps 1 and 2 of a tile once U0 (u with its 2-cell halo, mirror ghosts
// in place), the quad's v, w, hole codes and the ring cell's v, w, code are
// loaded: the arithmetic of the single-step kernels.
struct NoHook {
  __device__ void operator()(float *) const {}
};

// hook(U1) runs after step 1, before the mirror ghosts of U1 are copied
// (the batched kernel applies the next step's stimulus events there).
template <bool HOLES, class Hook = NoHook>
__device__ __forceinline__ void two_steps(
    const StepCoeffs<float> &a, const Fld<float> &out, const float *U0,
    float *U1, int x0, int y0, int t, int qx, int ty, int gi0, int gj,
    bool quad_ok, const float (&vv)[4], const float (&ww)[4], uint32_t code4,
    int rr, int rc, bool ring_ok, float rv, float rw, uint32_t rcode,
    Hook hook = Hook()) {
  const int nx = a.nx, ny = a.ny;
  // step 1: the quad (v, w kept in registers) and the ring cell
  float u1[4], v1[4], w1[4];
  const bool plain = !HOLES || code4 == 0x01010101u;
  if (quad_ok) {
    const float *c0 = U0 + (ty + 2) * kS + 4 * qx + 4;  // first cell
    const float4 c = *reinterpret_cast<const float4 *>(c0);
    const float4 n = *reinterpret_cast<const float4 *>(c0 + kS);
    const float4 s = *reinterpret_cast<const float4 *>(c0 - kS);
    const float uc[4] = {c.x, c.y, c.z, c.w};
    const float un[4] = {n.x, n.y, n.z, n.w};
    const float us[4] = {s.x, s.y, s.z, s.w};
    fk3v_cells4(a, plain, code4, uc, c0[-1], c0[4], un, us, vv, ww, u1, v1,
                w1);
    *reinterpret_cast<float4 *>(U1 + (ty + 1) * kS + 4 * qx + 4) =
        make_float4(u1[0], u1[1], u1[2], u1[3]);
  }
  if (ring_ok) {
    const float *c0 = U0 + (rr + 1) * kS + rc + 3;
    float cxw, cxc, cxe, cyn, cyc, cys;
    pattern_weights((rcode >> 1) & 3u, cxw, cxc, cxe);
    pattern_weights((rcode >> 3) & 3u, cyn, cyc, cys);
    const float du = lap5(a, lap_axis(c0[-1], c0[0], c0[1], cxw, cxc, cxe),
                          lap_axis(c0[kS], c0[0], c0[-kS], cyn, cyc, cys));
    float ou, ov, ow;
    fk3v_update(a, c0[0], rv, rw, du, ou, ov, ow);
    U1[rr * kS + rc + 3] = (rcode & 1u) ? ou : 0.f;
  }
  __syncthreads();
  hook(U1);
  // mirror ghosts of the step-1 u outside the domain (x = -1 <- 1,
  // x = nx <- nx - 2, the same in y); corners are not read
  if (t < kH1) {
    if (x0 == 0) U1[t * kS + 0 + 3] = U1[t * kS + 2 + 3];
    if (x0 + kTW >= nx) {
      const int c = nx - x0 + 1;  // step-1 column of x = nx
      U1[t * kS + c + 3] = U1[t * kS + c - 2 + 3];
    }
  }
  __syncthreads();  // the y ghosts copy columns the x ghosts wrote
  if (t < kW1) {
    if (y0 == 0) U1[0 * kS + t + 3] = U1[2 * kS + t + 3];
    if (y0 + kTH >= ny) {
      const int r = ny - y0 + 1;  // step-1 row of y = ny
      U1[r * kS + t + 3] = U1[(r - 2) * kS + t + 3];
    }
  }
  __syncthreads();

  // step 2 on the quad
  if (quad_ok) {
    const float *c0 = U1 + (ty + 1) * kS + 4 * qx + 4;
    const float4 c = *reinterpret_cast<const float4 *>(c0);
    const float4 n = *reinterpret_cast<const float4 *>(c0 + kS);
    const float4 s = *reinterpret_cast<const float4 *>(c0 - kS);
    const float uc[4] = {c.x, c.y, c.z, c.w};
    const float un[4] = {n.x, n.y, n.z, n.w};
    const float us[4] = {s.x, s.y, s.z, s.w};
    float u2[4], v2[4], w2[4];
    fk3v_cells4(a, plain, code4, uc, c0[-1], c0[4], un, us, v1, w1, u2, v2,
                w2);
    const size_t g = (size_t)gj * nx + gi0;
    *reinterpret_cast<float4 *>(out.f[0] + g) = make_float4(u2[0], u2[1], u2[2], u2[3]);
    *reinterpret_cast<float4 *>(out.f[1] + g) = make_float4(v2[0], v2[1], v2[2], v2[3]);
    *reinterpret_cast<float4 *>(out.f[2] + g) = make_float4(w2[0], w2[1], w2[2], w2[3]);
  }
}

struct TileMaps {
  CUtensorMap u, v, w, c;
};

constexpr int kVW = 72, kVH = kTH + 2;  // v, w box: the tile and its ring
constexpr int kCW = 96;                 // hole-code box width (bytes)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map,
                                       int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::"
      "bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y),
      "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// true once phase 0 of the barrier completed; false after 1 s
__device__ __forceinline__ bool bar_wait0(uint64_t *bar) {
  const uint32_t b = smem_u32(bar);
  unsigned long long t0 = 0;
  for (int spin = 0;; ++spin) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; "
        "selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(b)
        : "memory");
    if (done) return true;
    if (spin == 0) t0 = gtimer();
    else if (gtimer() - t0 > 1000000000ull) return false;
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null when unavailable.
inline PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

inline bool encode_2d(CUtensorMap *m, const void *base, bool bytes, int nx, int ny,
               int bx, int by) {
  const PFN_cuTensorMapEncodeTiled_v12000 fn = encode_tiled();
  if (!fn) return false;
  const size_t es = bytes ? 1 : sizeof(float);
  const cuuint64_t dims[2] = {(cuuint64_t)nx, (cuuint64_t)ny};
  const cuuint64_t strides[1] = {(cuuint64_t)nx * es};
  const cuuint32_t box[2] = {(cuuint32_t)bx, (cuuint32_t)by};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, bytes ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
            2, const_cast<void *>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tile2s
}  // namespace yh
