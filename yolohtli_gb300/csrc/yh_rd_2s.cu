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
#include "yh_kernels.cuh"

namespace yh {

namespace {

constexpr int kTW = 64, kTH = 16;          // output tile (cells)
constexpr int kThreads = 256;              // one quad of the tile each
constexpr int kW0 = kTW + 4, kH0 = kTH + 4;  // u with a 2-cell halo
constexpr int kW1 = kTW + 2, kH1 = kTH + 2;  // step-1 u with a 1-cell ring
constexpr int kRing = 2 * kW1 + 2 * kTH;     // 164 ring cells
// Shared rows are 72 floats; U0 column c lives at c + 2 and U1 column c at
// c + 3, so that every quad's first cell is 16-byte aligned.
constexpr int kS = 72;

__device__ __forceinline__ int load_index(int i, int n) {
  i = mirror(i, n);  // -1 -> 1, n -> n - 2 (the reference's coord_i)
  return i < 0 ? 0 : (i >= n ? n - 1 : i);  // 2 cells out: never used
}

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

}  // namespace

bool rd_2s_supported(const StepCoeffs<float> &a, const Fld<float> &in,
                     const Fld<float> &out, bool holes, const uint8_t *codes) {
  return a.model == YH_MODEL_FK3V && (a.nx % 4) == 0 && aligned16(in, a.model) &&
         aligned16(out, a.model) && (!holes || codes != nullptr) &&
         (!codes || (reinterpret_cast<uintptr_t>(codes) & 3) == 0);
}

cudaError_t launch_rd_2s(const StepCoeffs<float> &a, const Fld<float> &in,
                         const Fld<float> &out, const uint8_t *codes,
                         cudaStream_t s) {
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
