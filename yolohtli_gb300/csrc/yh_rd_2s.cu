// Two explicit FK3V steps per launch (the blocked engine at depth 2).
//
// A block owns a 64 x 16 tile of cells. It loads u of the tile and a 2-cell
// halo into shared memory (mirrored at the domain edge, as the single-step
// kernels read it), takes step 1 on the tile and on the 1-cell ring around
// it (ring: 164 scalar cells, tile: one float4 quad per thread whose new v,
// w stay in registers), writes the mirror ghosts of the step-1 u that fall
// outside the domain, and takes step 2 on the tile. Per two steps a tile
// reads u over 68 x 20 cells and v, w, hole codes over 66 x 18, and writes
// u, v, w once: ~14 B per cell-step of L2/DRAM traffic against 25 for two
// single steps. Both steps use the operations of the single-step kernels
// (fk3v_cells4 / fk3v_update with lap5), so the result has the same bits as
// two launches of rd_step_vec4.
#include "yh_tile2s.cuh"

namespace yh {

using namespace tile2s;

namespace {

__device__ __forceinline__ int load_index(int i, int n) {
  i = mirror(i, n);  // -1 -> 1, n -> n - 2 (the reference's coord_i)
  return i < 0 ? 0 : (i >= n ? n - 1 : i);  // 2 cells out: never used
}

// The inputs by plain loads: u through mirrored, clamped indices, v, w and
// the hole codes of the quad (float4) and of the ring cell (scalars).
template <bool HOLES>
__global__ void __launch_bounds__(kThreads)
    rd_2s_kernel(const StepCoeffs<float> a, const Fld<float> in,
                 const Fld<float> out, const uint8_t *__restrict__ codes) {
  __shared__ __align__(16) float U0[kH0 * kS];
  __shared__ __align__(16) float U1[kH1 * kS];
  const int nx = a.nx, ny = a.ny;
  const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
  const int t = threadIdx.x;
  grid_dep_wait();
  grid_dep_launch();
  // u over the tile and a 2-cell halo
  for (int idx = t; idx < kH0 * kW0; idx += kThreads) {
    const int r = idx / kW0, c = idx - r * kW0;
    const int gi = load_index(x0 - 2 + c, nx), gj = load_index(y0 - 2 + r, ny);
    U0[r * kS + c + 2] = __ldg(in.f[0] + (size_t)gj * nx + gi);
  }
  // this thread's quad of the tile: row y0 + ty, cells x0 + 4 qx .. + 3
  const int qx = t & 15, ty = t >> 4;
  const int gi0 = x0 + 4 * qx, gj = y0 + ty;
  const bool quad_ok = gi0 < nx && gj < ny;  // nx % 4 == 0: all four or none
  float vv[4] = {0.f, 0.f, 0.f, 0.f}, ww[4] = {0.f, 0.f, 0.f, 0.f};
  uint32_t code4 = 0x01010101u;
  if (quad_ok) {
    const size_t g = (size_t)gj * nx + gi0;
    const float4 v4 = __ldg(reinterpret_cast<const float4 *>(in.f[1] + g));
    const float4 w4 = __ldg(reinterpret_cast<const float4 *>(in.f[2] + g));
    vv[0] = v4.x; vv[1] = v4.y; vv[2] = v4.z; vv[3] = v4.w;
    ww[0] = w4.x; ww[1] = w4.y; ww[2] = w4.z; ww[3] = w4.w;
    if (HOLES) code4 = __ldg(reinterpret_cast<const unsigned int *>(codes + g));
  }
  // this thread's ring cell (t < kRing), in step-1 tile coordinates
  int rr = 0, rc = 0;
  if (t < kW1) {
    rr = 0; rc = t;                              // row above the tile
  } else if (t < 2 * kW1) {
    rr = kH1 - 1; rc = t - kW1;                  // row below
  } else if (t < 2 * kW1 + kTH) {
    rr = 1 + t - 2 * kW1; rc = 0;                // column left
  } else {
    rr = 1 + t - 2 * kW1 - kTH; rc = kW1 - 1;    // column right
  }
  const int rgi = x0 - 1 + rc, rgj = y0 - 1 + rr;
  const bool ring_ok = t < kRing && rgi >= 0 && rgi < nx && rgj >= 0 && rgj < ny;
  float rv = 0.f, rw = 0.f;
  uint32_t rcode = 1u;
  if (ring_ok) {
    const size_t g = (size_t)rgj * nx + rgi;
    rv = __ldg(in.f[1] + g);
    rw = __ldg(in.f[2] + g);
    if (HOLES) rcode = __ldg(codes + g);
  }
  __syncthreads();
  two_steps<HOLES>(a, out, U0, U1, x0, y0, t, qx, ty, gi0, gj, quad_ok, vv,
                   ww, code4, rr, rc, ring_ok, rv, rw, rcode);
}

// The same two steps with the tile's inputs staged by the tensor memory
// accelerator: one thread issues four 2D bulk tensor copies (u over the
// tile and a 2-cell halo, 72 x 20 from (x0 - 4, y0 - 2); v and w over the
// tile and its ring, 72 x 18 from (x0 - 4, y0 - 1); the hole codes, 96 x 18
// bytes from (x0 - 16, y0 - 1)) on one mbarrier, in place of the threads'
// ~11 loads each. Every box starts at an x that is a multiple of 16 bytes
// (x0 is a multiple of 64). Cells outside the grid arrive as zeros; the
// mirror ghosts at x = -1, nx and y = -1, ny are then copied in shared
// memory (the cells two out are never read). The wait is bounded by 1 s
// of %globaltimer, after which the block sets *err and returns. Compiled
// for 8 blocks per SM (32 registers, a few bytes spilled): 455 against
// 423 Gcell-steps/s at 5 blocks per SM on the 4096^2 holes workload.
template <bool HOLES>
__global__ void __launch_bounds__(kThreads, 8)
    rd_2s_tma_kernel(const StepCoeffs<float> a, const __grid_constant__ TileMaps m,
                     const Fld<float> out, int *err) {
  __shared__ __align__(128) float U0[kH0 * kS];
  __shared__ __align__(128) float Vs[kVH * kVW];
  __shared__ __align__(128) float Ws[kVH * kVW];
  __shared__ __align__(128) uint8_t Cs[kVH * kCW];
  __shared__ __align__(16) float U1[kH1 * kS];
  __shared__ __align__(8) uint64_t bar;
  const int nx = a.nx, ny = a.ny;
  const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
  const int t = threadIdx.x;
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar))
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  grid_dep_wait();
  grid_dep_launch();
  if (t == 0) {
    const uint32_t bytes = (uint32_t)(sizeof(float) * (kH0 * kS + 2 * kVH * kVW) +
                                      (HOLES ? kVH * kCW : 0));
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_u32(&bar)),
        "r"(bytes)
        : "memory");
    tma_2d(U0, &m.u, x0 - 4, y0 - 2, &bar);
    tma_2d(Vs, &m.v, x0 - 4, y0 - 1, &bar);
    tma_2d(Ws, &m.w, x0 - 4, y0 - 1, &bar);
    if (HOLES) tma_2d(Cs, &m.c, x0 - 16, y0 - 1, &bar);
  }
  if (!bar_wait0(&bar)) {
    if (t == 0) atomicExch(err, 1);
    return;
  }
  // mirror ghosts of u: x = -1 <- 1, x = nx <- nx - 2 (columns), then the
  // rows y = -1 <- 1, y = ny <- ny - 2 (U0 row r is y0 - 2 + r, column s is
  // x0 - 4 + s)
  if (t < kH0) {
    if (x0 == 0) U0[t * kS + 3] = U0[t * kS + 5];
    const int sR = nx - x0 + 4;
    if (sR < kS) U0[t * kS + sR] = U0[t * kS + sR - 2];
  }
  __syncthreads();
  if (t < kS) {
    if (y0 == 0) U0[1 * kS + t] = U0[3 * kS + t];
    const int rT = ny - y0 + 2;
    if (rT < kH0) U0[rT * kS + t] = U0[(rT - 2) * kS + t];
  }
  // this thread's quad of the tile: row y0 + ty, cells x0 + 4 qx .. + 3
  const int qx = t & 15, ty = t >> 4;
  const int gi0 = x0 + 4 * qx, gj = y0 + ty;
  const bool quad_ok = gi0 < nx && gj < ny;
  const float4 v4 = *reinterpret_cast<const float4 *>(Vs + (ty + 1) * kVW + 4 * qx + 4);
  const float4 w4 = *reinterpret_cast<const float4 *>(Ws + (ty + 1) * kVW + 4 * qx + 4);
  const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
  const float ww[4] = {w4.x, w4.y, w4.z, w4.w};
  const uint32_t code4 =
      HOLES ? *reinterpret_cast<const uint32_t *>(Cs + (ty + 1) * kCW + 4 * qx + 16)
            : 0x01010101u;
  int rr = 0, rc = 0;
  if (t < kW1) {
    rr = 0; rc = t;
  } else if (t < 2 * kW1) {
    rr = kH1 - 1; rc = t - kW1;
  } else if (t < 2 * kW1 + kTH) {
    rr = 1 + t - 2 * kW1; rc = 0;
  } else {
    rr = 1 + t - 2 * kW1 - kTH; rc = kW1 - 1;
  }
  const int rgi = x0 - 1 + rc, rgj = y0 - 1 + rr;
  const bool ring_ok = t < kRing && rgi >= 0 && rgi < nx && rgj >= 0 && rgj < ny;
  const float rv = ring_ok ? Vs[rr * kVW + rc + 3] : 0.f;
  const float rw = ring_ok ? Ws[rr * kVW + rc + 3] : 0.f;
  const uint32_t rcode = (HOLES && ring_ok) ? Cs[rr * kCW + rc + 15] : 1u;
  __syncthreads();
  two_steps<HOLES>(a, out, U0, U1, x0, y0, t, qx, ty, gi0, gj, quad_ok, vv,
                   ww, code4, rr, rc, ring_ok, rv, rw, rcode);
}

}  // namespace

bool rd_2s_supported(const StepCoeffs<float> &a, const Fld<float> &in,
                     const Fld<float> &out, bool holes, const uint8_t *codes) {
  return a.model == YH_MODEL_FK3V && (a.nx % 4) == 0 && aligned16(in, a.model) &&
         aligned16(out, a.model) && (!holes || codes != nullptr) &&
         (!codes || (reinterpret_cast<uintptr_t>(codes) & 3) == 0);
}

// The tensor-memory-accelerator form needs 16-byte rows for every box:
// nx % 4 for the FP32 fields, nx % 16 for the hole codes.
static bool tma_ok(const StepCoeffs<float> &a, const uint8_t *codes) {
#ifdef YH_RD2S_NO_TMA
  (void)a; (void)codes;
  return false;
#else
  return (a.nx % 4) == 0 &&
         (!codes || ((a.nx % 16) == 0 &&
                     (reinterpret_cast<uintptr_t>(codes) & 15) == 0)) &&
         encode_tiled() != nullptr;
#endif
}

cudaError_t launch_rd_2s(const StepCoeffs<float> &a, const Fld<float> &in,
                         const Fld<float> &out, const uint8_t *codes,
                         int *err, cudaStream_t s) {
  if (err && tma_ok(a, codes)) {
    TileMaps m;
    bool ok = encode_2d(&m.u, in.f[0], false, a.nx, a.ny, kS, kH0) &&
              encode_2d(&m.v, in.f[1], false, a.nx, a.ny, kVW, kVH) &&
              encode_2d(&m.w, in.f[2], false, a.nx, a.ny, kVW, kVH);
    if (codes) ok = ok && encode_2d(&m.c, codes, true, a.nx, a.ny, kCW, kVH);
    else m.c = m.u;
    if (ok) {
      const dim3 grid((a.nx + kTW - 1) / kTW, (a.ny + kTH - 1) / kTH);
      if (codes)
        return launch_pdl(rd_2s_tma_kernel<true>, grid, dim3(kThreads), 0, s, a,
                          m, out, err);
      return launch_pdl(rd_2s_tma_kernel<false>, grid, dim3(kThreads), 0, s, a,
                        m, out, err);
    }
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((a.nx + kTW - 1) / kTW, (a.ny + kTH - 1) / kTH);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (codes) return cudaLaunchKernelEx(&cfg, rd_2s_kernel<true>, a, in, out, codes);
  return cudaLaunchKernelEx(&cfg, rd_2s_kernel<false>, a, in, out, codes);
}

}  // namespace yh
