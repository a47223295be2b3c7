// Resident solver: a whole protocol of explicit steps (with its stimulus
// events) in one cooperative launch, for grids whose state fits in the SMs'
// shared memory (FP32, models where only u diffuses: FK3V, or REF2V with
// gateDiff = 0).
//
// Block b of nb (one per SM, all co-resident: cooperative launch) owns the
// rows [r0, r0 + R) of the grid and keeps their u (double-buffered), v, w
// and hole codes in shared memory for all steps; nothing but two rows of u
// per block and step leaves the SM. Per step, a block
//   1. applies the stimulus events of this step to its rows,
//   2. updates its interior rows 1 .. R-2, which need no other block,
//   3. waits until both neighbours have published the step's boundary rows
//      (a per-block step counter, st.release / ld.acquire; the wait is
//      bounded by 1 s of %globaltimer, then it sets the error flag and the
//      kernel returns),
//   4. copies those two rows into its halo rows and updates rows 0, R-1,
//   5. publishes its new rows 0 and R-1 (double-buffered by step parity)
//      and its counter.
// The neighbour wait in 3 overlaps with the interior work of 2. A block can
// run at most one step ahead of its neighbours, so two halo buffers suffice.
// The cell update is the one of the single-step kernels (same expression,
// same bits). The mirror ghost rows at the domain's top and bottom are copies
// of the block's own rows 1 and R-2 (helper_functions.cu:69-79).
#include "yh_kernels.cuh"

namespace yh {

constexpr int kResThreads = 512;
constexpr unsigned long long kResWaitNs = 1000000000ull;  // 1 s

struct ResArgs {
  StepCoeffs<float> a;
  Fld<float> io;          // state: read at the start, written at the end
  float *prev_u;          // u before the last step (nullptr: not written)
  const uint8_t *solid;   // nullptr: no holes
  float *halo;            // [2][nb][2][nx]: published boundary rows of u
  unsigned int *flags;    // [nb]: 1 + steps whose boundary rows are published
  int *error;             // set to 1 when a wait gave up
  int nsteps, step0;
  int nb, rq, rrem, rmax;
  int nstims;
  yh_stim stims[kResMaxStims];
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Updates the cells of rows [lr0, lr1) (local rows) from `cur` into `nxt`.
// U buffers hold local rows -1 .. R, row lr at offset (lr + 1) * nx.
template <int MODEL, bool HOLES, bool VEC>
__device__ __forceinline__ void res_rows(const StepCoeffs<float> &a,
                                         const float *cur, float *nxt,
                                         float *Vs, float *Ws,
                                         const uint8_t *Cs, int lr0, int lr1) {
  const int nx = a.nx;
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;
  if (VEC) {
    const int nq = nx >> 2;
    const int items = (lr1 - lr0) * nq;
    for (int it = threadIdx.x; it < items; it += kResThreads) {
      const int lr = lr0 + it / nq;
      const int i0 = (it - (lr - lr0) * nq) << 2;
      const float *rc = cur + (lr + 1) * nx;
      const float4 c = *reinterpret_cast<const float4 *>(rc + i0);
      const float4 n = *reinterpret_cast<const float4 *>(rc + nx + i0);
      const float4 s = *reinterpret_cast<const float4 *>(rc - nx + i0);
      const float uw = rc[mirror(i0 - 1, nx)], ue = rc[mirror(i0 + 4, nx)];
      float4 *vp = reinterpret_cast<float4 *>(Vs + lr * nx + i0);
      float4 *wp = reinterpret_cast<float4 *>(Ws + lr * nx + i0);
      const float4 v4 = *vp;
      const float4 w4 = W3 ? *wp : make_float4(0.f, 0.f, 0.f, 0.f);
      uint32_t code = 0x01010101u;
      if (HOLES) code = *reinterpret_cast<const uint32_t *>(Cs + lr * nx + i0);
      const float uc[4] = {c.x, c.y, c.z, c.w};
      const float un_[4] = {n.x, n.y, n.z, n.w};
      const float us_[4] = {s.x, s.y, s.z, s.w};
      const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
      const float ww[4] = {w4.x, w4.y, w4.z, w4.w};
      float ou[4], ov[4], ow[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float uW = k == 0 ? uw : uc[k - 1];
        const float uE = k == 3 ? ue : uc[k + 1];
        float du;
        bool sc = true;
        if (HOLES && code != 0x01010101u) {
          const uint32_t cc = code >> (8 * k);
          sc = (cc & 1u) != 0u;
          float cxw, cxc, cxe, cyn, cyc, cys;
          pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
          pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
          du = (cxw * uW - cxc * uc[k] + cxe * uE) * a.rx +
               (cyn * un_[k] - cyc * uc[k] + cys * us_[k]) * a.ry;
        } else {
          du = (uW - 2.f * uc[k] + uE) * a.rx +
               (un_[k] - 2.f * uc[k] + us_[k]) * a.ry;
        }
        tb_update<MODEL>(a, uc[k], vv[k], ww[k], du, ou[k], ov[k], ow[k]);
        if (HOLES && !sc) ou[k] = ov[k] = ow[k] = 0.f;
      }
      *reinterpret_cast<float4 *>(nxt + (lr + 1) * nx + i0) =
          make_float4(ou[0], ou[1], ou[2], ou[3]);
      *vp = make_float4(ov[0], ov[1], ov[2], ov[3]);
      if (W3) *wp = make_float4(ow[0], ow[1], ow[2], ow[3]);
    }
  } else {
    const int items = (lr1 - lr0) * nx;
    for (int it = threadIdx.x; it < items; it += kResThreads) {
      const int lr = lr0 + it / nx;
      const int i = it - (lr - lr0) * nx;
      const float *rc = cur + (lr + 1) * nx;
      const float uc = rc[i];
      const float uW = rc[mirror(i - 1, nx)], uE = rc[mirror(i + 1, nx)];
      const float uN = rc[nx + i], uS = rc[-nx + i];
      const int C = lr * nx + i;
      float du;
      bool sc = true;
      if (HOLES && Cs[C] != 0x01u) {
        const uint32_t cc = Cs[C];
        sc = (cc & 1u) != 0u;
        float cxw, cxc, cxe, cyn, cyc, cys;
        pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
        pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
        du = (cxw * uW - cxc * uc + cxe * uE) * a.rx +
             (cyn * uN - cyc * uc + cys * uS) * a.ry;
      } else {
        du = (uW - 2.f * uc + uE) * a.rx + (uN - 2.f * uc + uS) * a.ry;
      }
      float ou, ov, ow;
      tb_update<MODEL>(a, uc, Vs[C], W3 ? Ws[C] : 0.f, du, ou, ov, ow);
      if (HOLES && !sc) ou = ov = ow = 0.f;
      nxt[(lr + 1) * nx + i] = ou;
      Vs[C] = ov;
      if (W3) Ws[C] = ow;
    }
  }
}

// u = value on the tissue cells of global row gy held in local buffer row
// `row` (a U buffer row of nx cells) that lie in the box of event e.
__device__ __forceinline__ void res_stim_row(float *row, int gy, int nx,
                                             const yh_stim &e,
                                             const uint8_t *solid) {
  if (gy < e.j0 || gy >= e.j1) return;
  const int i0 = e.i0 < 0 ? 0 : e.i0, i1 = e.i1 > nx ? nx : e.i1;
  for (int i = i0 + (int)threadIdx.x; i < i1; i += kResThreads)
    if (!solid || solid[(size_t)gy * nx + i]) row[i] = e.value;
}

template <int MODEL, bool HOLES, bool VEC>
__global__ void __launch_bounds__(kResThreads, 1)
    rd_resident_kernel(const ResArgs A) {
  extern __shared__ float4 sm4[];
  const StepCoeffs<float> &a = A.a;
  const int nx = a.nx, ny = a.ny;
  const int b = blockIdx.x, nb = A.nb, RM = A.rmax;
  const int r0 = b * A.rq + min(b, A.rrem);
  const int R = A.rq + (b < A.rrem ? 1 : 0);
  float *U0 = reinterpret_cast<float *>(sm4);
  float *U1 = U0 + (RM + 2) * nx;
  float *Vs = U1 + (RM + 2) * nx;
  float *Ws = Vs + RM * nx;
  uint8_t *Cs = reinterpret_cast<uint8_t *>(Ws + RM * nx);
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;
  __shared__ int s_abort;

  // load the block's rows; hole codes from the mask with mirrored neighbours
  for (int idx = threadIdx.x; idx < R * nx; idx += kResThreads) {
    const int lr = idx / nx, i = idx - lr * nx, gy = r0 + lr;
    const size_t g = (size_t)gy * nx + i;
    U0[(lr + 1) * nx + i] = A.io.f[0][g];
    Vs[idx] = A.io.f[1][g];
    if (W3) Ws[idx] = A.io.f[2][g];
    if (HOLES) {
      const uint8_t *S = A.solid;
      const bool sc = S[g] != 0;
      const bool sw = S[(size_t)gy * nx + mirror(i - 1, nx)] != 0;
      const bool se = S[(size_t)gy * nx + mirror(i + 1, nx)] != 0;
      const bool sn = S[(size_t)mirror(gy + 1, ny) * nx + i] != 0;
      const bool ss = S[(size_t)mirror(gy - 1, ny) * nx + i] != 0;
      Cs[idx] = (uint8_t)((sc ? 1u : 0u) | (hole_pattern(sw, sc, se) << 1) |
                          (hole_pattern(sn, sc, ss) << 3));
    }
  }
  // publish the initial boundary rows (state after 0 steps) in halo[0]
  {
    float *hb = A.halo + ((size_t)0 * nb + b) * 2 * nx;
    for (int i = threadIdx.x; i < nx; i += kResThreads) {
      hb[i] = A.io.f[0][(size_t)r0 * nx + i];
      hb[nx + i] = A.io.f[0][(size_t)(r0 + R - 1) * nx + i];
    }
  }
  __threadfence();
  if (threadIdx.x == 0) s_abort = 0;
  __syncthreads();
  if (threadIdx.x == 0) st_release(A.flags + b, 1u);

  for (int s = 0; s < A.nsteps; ++s) {
    const int gs = A.step0 + s;
    float *cur = (s & 1) ? U1 : U0;
    float *nxt = (s & 1) ? U0 : U1;
    // 1. stimulus events of this step on the block's own rows
    for (int e = 0; e < A.nstims; ++e)
      if (A.stims[e].step == gs)
        for (int lr = 0; lr < R; ++lr)
          res_stim_row(cur + (lr + 1) * nx, r0 + lr, nx, A.stims[e], A.solid);
    __syncthreads();
    // 2. interior rows
    if (R > 2) res_rows<MODEL, HOLES, VEC>(a, cur, nxt, Vs, Ws, Cs, 1, R - 1);
    // 3. neighbours' boundary rows of the state after s steps
    if (threadIdx.x == 0) {
      const unsigned need = (unsigned)s + 1u;
      const unsigned long long t0 = globaltimer();
      for (;;) {
        const bool lo = b == 0 || ld_acquire(A.flags + b - 1) >= need;
        const bool hi = b == nb - 1 || ld_acquire(A.flags + b + 1) >= need;
        if (lo && hi) break;
        if (*(volatile int *)A.error || globaltimer() - t0 > kResWaitNs) {
          atomicExch(A.error, 1);
          s_abort = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __syncthreads();
    if (s_abort) return;
    // 4. halo rows, then the block's first and last rows
    {
      const float *hp = A.halo + (size_t)(s & 1) * nb * 2 * nx;
      float *below = cur;                 // local row -1
      float *above = cur + (R + 1) * nx;  // local row R
      for (int i = threadIdx.x; i < nx; i += kResThreads) {
        below[i] = b > 0 ? __ldcg(hp + ((size_t)(b - 1) * 2 + 1) * nx + i)
                         : cur[2 * nx + i];          // mirror: row 1
        above[i] = b < nb - 1 ? __ldcg(hp + ((size_t)(b + 1) * 2) * nx + i)
                              : cur[(R - 1) * nx + i];  // mirror: row R-2
      }
      __syncthreads();
      for (int e = 0; e < A.nstims; ++e)
        if (A.stims[e].step == gs) {
          if (b > 0) res_stim_row(below, r0 - 1, nx, A.stims[e], A.solid);
          if (b < nb - 1) res_stim_row(above, r0 + R, nx, A.stims[e], A.solid);
        }
      __syncthreads();
      res_rows<MODEL, HOLES, VEC>(a, cur, nxt, Vs, Ws, Cs, 0, 1);
      if (R > 1)
        res_rows<MODEL, HOLES, VEC>(a, cur, nxt, Vs, Ws, Cs, R - 1, R);
    }
    __syncthreads();
    // 5. publish the new boundary rows (state after s + 1 steps)
    {
      float *hb = A.halo + ((size_t)((s + 1) & 1) * nb + b) * 2 * nx;
      for (int i = threadIdx.x; i < nx; i += kResThreads) {
        __stcg(hb + i, nxt[nx + i]);
        __stcg(hb + nx + i, nxt[R * nx + i]);
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) st_release(A.flags + b, (unsigned)s + 2u);
  }

  // write the state back (and u of the level before the last step)
  const float *fin = (A.nsteps & 1) ? U1 : U0;
  const float *pre = (A.nsteps & 1) ? U0 : U1;
  for (int idx = threadIdx.x; idx < R * nx; idx += kResThreads) {
    const int lr = idx / nx, i = idx - lr * nx;
    const size_t g = (size_t)(r0 + lr) * nx + i;
    A.io.f[0][g] = fin[(lr + 1) * nx + i];
    A.io.f[1][g] = Vs[idx];
    if (W3) A.io.f[2][g] = Ws[idx];
    if (A.prev_u) A.prev_u[g] = pre[(lr + 1) * nx + i];
  }
}

// Rows per block and shared memory of the resident solver on this device;
// ok = false when the grid does not fit (or the model diffuses v).
ResidentPlan resident_plan(const StepCoeffs<float> &a, int device) {
  ResidentPlan pl{};
  pl.ok = false;
  if (a.model == YH_MODEL_REF2V && a.gate_diff) return pl;
  int sms = 0, smem_optin = 0, coop = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess)
    return pl;
  if (!coop) return pl;
  int nb = sms < a.ny / 2 ? sms : a.ny / 2;  // at least 2 rows per block
  if (nb < 1) return pl;
  pl.nb = nb;
  pl.rq = a.ny / nb;
  pl.rrem = a.ny % nb;
  pl.rmax = pl.rq + (pl.rrem ? 1 : 0);
  pl.smem = (size_t)(2 * (pl.rmax + 2) + 2 * pl.rmax) * a.nx * sizeof(float) +
            (size_t)pl.rmax * a.nx + 64;
  pl.ok = pl.smem <= (size_t)smem_optin && pl.rq >= 2;
  return pl;
}

template <int MODEL, bool HOLES, bool VEC>
static cudaError_t launch_res_t(const ResArgs &A, size_t smem,
                                cudaStream_t s) {
  auto fn = rd_resident_kernel<MODEL, HOLES, VEC>;
  cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void *args[] = {const_cast<ResArgs *>(&A)};
  return cudaLaunchCooperativeKernel((const void *)fn, dim3(A.nb),
                                     dim3(kResThreads), args, smem, s);
}

cudaError_t launch_rd_resident(const StepCoeffs<float> &a, const Fld<float> &io,
                               float *prev_u, const uint8_t *solid,
                               int nsteps, int step0,
                               const yh_stim *stims, int nstims,
                               const ResidentPlan &pl, float *halo,
                               unsigned int *flags, int *error,
                               cudaStream_t s) {
  if (!pl.ok || nstims > kResMaxStims || nsteps < 0) return cudaErrorInvalidValue;
  if (nsteps == 0) return cudaSuccess;
  ResArgs A;
  A.a = a;
  A.io = io;
  A.prev_u = prev_u;
  A.solid = solid;
  A.halo = halo;
  A.flags = flags;
  A.error = error;
  A.nsteps = nsteps;
  A.step0 = step0;
  A.nb = pl.nb;
  A.rq = pl.rq;
  A.rrem = pl.rrem;
  A.rmax = pl.rmax;
  A.nstims = nstims;
  for (int k = 0; k < nstims; ++k) A.stims[k] = stims[k];
  cudaError_t e = cudaMemsetAsync(flags, 0, (size_t)pl.nb * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const bool vec = (a.nx % 4) == 0;
  const bool holes = solid != nullptr;
#define YH_RES(M, H, V)                                         \
  if (a.model == M && holes == H && vec == V)                   \
    return launch_res_t<M, H, V>(A, pl.smem, s);
  YH_RES(YH_MODEL_FK3V, false, true)
  YH_RES(YH_MODEL_FK3V, true, true)
  YH_RES(YH_MODEL_FK3V, false, false)
  YH_RES(YH_MODEL_FK3V, true, false)
  YH_RES(YH_MODEL_REF2V, false, true)
  YH_RES(YH_MODEL_REF2V, true, true)
  YH_RES(YH_MODEL_REF2V, false, false)
  YH_RES(YH_MODEL_REF2V, true, false)
#undef YH_RES
  return cudaErrorInvalidValue;
}

}  // namespace yh
