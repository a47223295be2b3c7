// Resident solver: a whole protocol of explicit steps (with its stimulus
// events) in one cooperative launch, for grids whose state fits in the SMs'
// shared memory (FP32, models where only u diffuses: FK3V, or REF2V with
// gateDiff = 0).
//
// Block b of nb (one per SM, all co-resident: cooperative launch) owns the
// rows [r0, r0 + R) of the grid and keeps their u (double-buffered), v, w
// and hole codes in shared memory for all steps; nothing but two rows of u
// per block and step leaves the SM. The block's warps have two roles:
//   - up to 16 compute warps update the block's rows for step s, rows 0 and R-1
//     first, and publish those two rows as soon as they are computed;
//   - 2 or 4 communication warps meanwhile receive the neighbours' boundary rows
//     of the state after s + 1 steps into the halo rows -1 and R of the
//     next buffer (the rows step s + 1 reads and step s does not touch).
// One barrier per step joins the two. A published row is a sequence of
// 64-bit words (step tag << 32 | bits of u): one relaxed gpu-scope store
// makes value and tag visible together, so a receiver polls the words
// themselves and needs no flag and no fence. Every wait is bounded by 1 s
// of %globaltimer; then the thread sets the error flag and the block
// returns. A block can run at most one step ahead of its neighbours (it
// needs their rows of its current step), so two buffers by step parity
// suffice; the buffers are reset to tag 0xffffffff before each launch, a
// tag no step uses. The cell update is the one of the single-step kernels
// (same expression, same bits). The mirror ghost rows at the domain's top
// and bottom (helper_functions.cu:69-79) are read from the block's own rows
// 1 and R-2.
#include <algorithm>

#include "yh_kernels.cuh"

namespace yh {

#ifndef YH_RES_THREADS
#define YH_RES_THREADS 512
#endif
#ifndef YH_RES_CELLS
#define YH_RES_CELLS 4
#endif
// Receivers back off 64 ns << min(spin, YH_RES_BACKOFF) between polls.
#ifndef YH_RES_BACKOFF
#define YH_RES_BACKOFF 4
#endif
constexpr int kResThreads = YH_RES_THREADS;  // most compute threads
constexpr int kResCommMax = 128;  // communication threads (64 or 128)
constexpr int kResBatch = 16;                // halo words per comm thread and pass
constexpr int kResCells = YH_RES_CELLS;  // cells per work item, rows nx % 4 == 0
constexpr unsigned long long kResWaitNs = 1000000000ull;  // 1 s

struct ResArgs {
  StepCoeffs<float> a;
  Fld<float> io;                // state: read at the start, written at the end
  float *prev_u;                // u before the last step (nullptr: not written)
  const uint8_t *solid;         // nullptr: no holes
  unsigned long long *halo;     // [2][nb][2][nx] tagged boundary rows of u
  int *error;                   // set to 1 when a wait gave up
  int mute;                     // a block that publishes nothing (-1: none)
  int threads;            // compute threads; the rest of the block receives
  int nsteps, step0;
  int nb, rq, rrem, rmax;
  int nstims;
  yh_stim stims[kResMaxStims];
};

__device__ __forceinline__ void st_tagged(unsigned long long *p, float v,
                                          unsigned tag) {
  const unsigned long long x =
      ((unsigned long long)tag << 32) | __float_as_uint(v);
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(x)
               : "memory");
}
// CW consecutive tagged words in one relaxed vector store (each 8-byte
// element is its own single-copy-atomic access); p is 8 * CW byte aligned.
template <int CW>
__device__ __forceinline__ void st_tagged_vec(unsigned long long *p,
                                              const float (&v)[CW],
                                              unsigned tag) {
  unsigned long long x[CW];
#pragma unroll
  for (int k = 0; k < CW; ++k)
    x[k] = ((unsigned long long)tag << 32) | __float_as_uint(v[k]);
  if constexpr (CW == 4)
    asm volatile("st.relaxed.gpu.global.v4.b64 [%0], {%1, %2, %3, %4};" ::"l"(p),
                 "l"(x[0]), "l"(x[1]), "l"(x[2]), "l"(x[3])
                 : "memory");
  else if constexpr (CW == 2)
    asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(p),
                 "l"(x[0]), "l"(x[1])
                 : "memory");
  else
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(x[0])
                 : "memory");
}
__device__ __forceinline__ unsigned long long ld_tagged(
    const unsigned long long *p) {
  unsigned long long x;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(x) : "l"(p)
               : "memory");
  return x;
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// One cell update of the single-step kernels from its five u values.
template <int MODEL, bool HOLES>
__device__ __forceinline__ void res_cell(const StepCoeffs<float> &a,
                                         uint32_t cc, float u, float uW,
                                         float uE, float uN, float uS,
                                         float v, float w, float &ou,
                                         float &ov, float &ow) {
  float du;
  bool sc = true;
  if (HOLES && cc != 0x01u) {
    sc = (cc & 1u) != 0u;
    float cxw, cxc, cxe, cyn, cyc, cys;
    pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
    pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
    du = lap5(a, lap_axis(uW, u, uE, cxw, cxc, cxe),
              lap_axis(uN, u, uS, cyn, cyc, cys));
  } else {
    du = lap5(a, lap_axis(uW, u, uE), lap_axis(uN, u, uS));
  }
  tb_update<MODEL>(a, u, v, w, du, ou, ov, ow);
  if (HOLES && !sc) ou = ov = ow = 0.f;
}

// res_cell for any hole code, without branches (weights by selects).
__device__ __forceinline__ void res_cell_coded(const StepCoeffs<float> &a,
                                               uint32_t cc, float u, float uW,
                                               float uE, float uN, float uS,
                                               float v, float w, float &ou,
                                               float &ov, float &ow, bool fk) {
  const bool sc = (cc & 1u) != 0u;
  float cxw, cxc, cxe, cyn, cyc, cys;
  pattern_weights((cc >> 1) & 3u, cxw, cxc, cxe);
  pattern_weights((cc >> 3) & 3u, cyn, cyc, cys);
  const float du = lap5(a, lap_axis(uW, u, uE, cxw, cxc, cxe),
                        lap_axis(uN, u, uS, cyn, cyc, cys));
  if (fk)
    tb_update<YH_MODEL_FK3V>(a, u, v, w, du, ou, ov, ow);
  else
    tb_update<YH_MODEL_REF2V>(a, u, v, w, du, ou, ov, ow);
  ou = sc ? ou : 0.f;
  ov = sc ? ov : 0.f;
  ow = sc ? ow : 0.f;
}

// CW consecutive floats (CW = 1, 2, 4; 4 CW-byte aligned) as one load/store.
template <int CW> struct CellVec;
template <> struct CellVec<1> { using T = float; using C = uint8_t; };
template <> struct CellVec<2> { using T = float2; using C = uint16_t; };
template <> struct CellVec<4> { using T = float4; using C = uint32_t; };
template <int CW>
__device__ __forceinline__ void ld_cells(const float *p, float (&x)[CW]) {
  const typename CellVec<CW>::T t = *reinterpret_cast<const typename CellVec<CW>::T *>(p);
  const float *f = reinterpret_cast<const float *>(&t);
#pragma unroll
  for (int k = 0; k < CW; ++k) x[k] = f[k];
}
template <int CW>
__device__ __forceinline__ void st_cells(float *p, const float (&x)[CW]) {
  typename CellVec<CW>::T t;
  float *f = reinterpret_cast<float *>(&t);
#pragma unroll
  for (int k = 0; k < CW; ++k) f[k] = x[k];
  *reinterpret_cast<typename CellVec<CW>::T *>(p) = t;
}

// One work item of a step: CW consecutive cells (from column q * CW) of
// local row lr. U buffers hold local rows -1 .. R, row lr at offset
// (lr + 1) * nx. Rows 0 and R-1 are also published, tagged `tag`, into
// `pub` (row 0 at pub[0 .. nx), row R-1 at pub[nx .. 2 nx)) when a
// neighbour reads them.
template <int MODEL, bool HOLES, int CW>
__device__ __forceinline__ void res_item(const StepCoeffs<float> &a, int lr,
                                         int q, int R, bool bottom, bool top,
                                         const float *cur, float *nxt,
                                         float *Vs, float *Ws,
                                         const uint8_t *Cs,
                                         unsigned long long *pub,
                                         unsigned tag) {
  const int nx = a.nx;
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;
  const float *rc = cur + (lr + 1) * nx;
  const float *rn = (top && lr == R - 1) ? rc - nx : rc + nx;   // mirror
  const float *rs = (bottom && lr == 0) ? rc + nx : rc - nx;    // mirror
  const bool publish = (lr == 0 && !bottom) || (lr == R - 1 && !top);
  unsigned long long *pp = pub + (lr == 0 ? 0 : nx);
  const int i0 = q * CW;
  float uc[CW], un_[CW], us_[CW], vv[CW], ww[CW];
  ld_cells<CW>(rc + i0, uc);
  ld_cells<CW>(rn + i0, un_);
  ld_cells<CW>(rs + i0, us_);
  const float uw = rc[mirror(i0 - 1, nx)], ue = rc[mirror(i0 + CW, nx)];
  float *vp = Vs + lr * nx + i0;
  float *wp = Ws + lr * nx + i0;
  ld_cells<CW>(vp, vv);
  if (W3) ld_cells<CW>(wp, ww);
  else
#pragma unroll
    for (int k = 0; k < CW; ++k) ww[k] = 0.f;
  uint32_t code = 0;
  if (HOLES)
    code = *reinterpret_cast<const typename CellVec<CW>::C *>(Cs + lr * nx + i0);
  float ou[CW], ov[CW], ow[CW];
  // all CW cells tissue with tissue neighbours: one branch for the item,
  // straight-line code over its cells
  constexpr uint32_t kPlain = CW == 4 ? 0x01010101u : (CW == 2 ? 0x0101u : 0x01u);
  if constexpr (CW == 4 && MODEL == YH_MODEL_FK3V) {
    fk3v_cells4(a, !HOLES || code == kPlain, code, uc, uw, ue, un_, us_, vv,
                ww, ou, ov, ow);
  } else if (!HOLES || code == kPlain) {
#pragma unroll
    for (int k = 0; k < CW; ++k) {
      const float uW = k == 0 ? uw : uc[k - 1];
      const float uE = k == CW - 1 ? ue : uc[k + 1];
      res_cell<MODEL, false>(a, 0x01u, uc[k], uW, uE, un_[k], us_[k], vv[k],
                             ww[k], ou[k], ov[k], ow[k]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < CW; ++k) {
      const float uW = k == 0 ? uw : uc[k - 1];
      const float uE = k == CW - 1 ? ue : uc[k + 1];
      res_cell_coded(a, (code >> (8 * k)) & 0xffu, uc[k], uW, uE, un_[k],
                     us_[k], vv[k], ww[k], ou[k], ov[k], ow[k],
                     MODEL == YH_MODEL_FK3V);
    }
  }
  st_cells<CW>(nxt + (lr + 1) * nx + i0, ou);
  st_cells<CW>(vp, ov);
  if (W3) st_cells<CW>(wp, ow);
  if (publish && pub) st_tagged_vec<CW>(pp + i0, ou, tag);
}

// u = value on the tissue cells of global row gy held in local buffer row
// `row` (a U buffer row of nx cells) that lie in the box of event e.
__device__ __forceinline__ void res_stim_row(float *row, int gy, int nx,
                                             const yh_stim &e,
                                             const uint8_t *solid) {
  if (gy < e.j0 || gy >= e.j1) return;
  const int i0 = e.i0 < 0 ? 0 : e.i0, i1 = e.i1 > nx ? nx : e.i1;
  for (int i = i0 + (int)threadIdx.x; i < i1; i += (int)blockDim.x)
    if (!solid || solid[(size_t)gy * nx + i]) row[i] = e.value;
}

// Events of the launch are sorted by step (stable, so events of one step
// keep their order). [e0, e1) is the run of events on step gs, found from
// cursor `ev` (the first event not before gs) in the block's copy of the
// event steps; empty when no event falls on gs.
__device__ __forceinline__ void stim_run(const int *ev_step, int nstims,
                                         int ev, int gs, int &e0, int &e1) {
  e0 = e1 = ev;
  while (e1 < nstims && ev_step[e1] == gs) ++e1;
}

// u of halo cell (gy, i) after the stimulus events [e0, e1) of one step.
__device__ __forceinline__ float res_stim_cell(const ResArgs &A, int e0,
                                               int e1, int gy, int i,
                                               float u) {
  for (int e = e0; e < e1; ++e) {
    const yh_stim &ev = A.stims[e];
    if (gy >= ev.j0 && gy < ev.j1 && i >= ev.i0 && i < ev.i1 &&
        (!A.solid || A.solid[(size_t)gy * A.a.nx + i]))
      u = ev.value;
  }
  return u;
}

// Communication threads: receive the halo rows of the state after s steps
// (words [0, nx): row R-1 of block b-1 into local row -1; [nx, 2 nx): row 0
// of block b+1 into local row R) into the U buffer `dst`, applying the
// stimulus events [e0, e1). Thread c of nc reads words
// p * kResBatch * nc + k * nc + c of pass p, consecutive threads
// consecutive words; each pass keeps kResBatch loads in flight and polls
// stale words until they carry tag s. Returns false when a wait gave up.
template <int CW>
__device__ __forceinline__ bool res_receive(const ResArgs &A, int s, int e0,
                                            int e1, int b, int r0, int R,
                                            bool bottom, bool top, float *dst,
                                            int c, int nc) {
  const int nx = A.a.nx;
  const unsigned long long *hp =
      A.halo + (size_t)(s & 1) * ((size_t)A.nb * 2 * nx);
  const unsigned long long *below = hp + ((size_t)(b - 1) * 2 + 1) * nx;
  const unsigned long long *above = hp + ((size_t)(b + 1) * 2) * nx;
  const unsigned want = (unsigned)s;
  for (int base = 0; base < 2 * nx; base += kResBatch * nc) {
    unsigned long long x[kResBatch];
#pragma unroll
    for (int k = 0; k < kResBatch; ++k) {
      const int e = base + k * nc + c;
      const bool up = e >= nx;
      const bool need = e < 2 * nx && (up ? !top : !bottom);
      x[k] = need ? ld_tagged(up ? above + (e - nx) : below + e)
                  : ((unsigned long long)want << 32);
    }
    unsigned long long t0 = 0;  // read on the first miss only
    for (int spin = 0;; ++spin) {
      bool ok = true;
#pragma unroll
      for (int k = 0; k < kResBatch; ++k) ok &= (unsigned)(x[k] >> 32) == want;
      if (ok) break;
      if (spin == 0) t0 = globaltimer();
      if (((spin & 15) == 15 && *(volatile int *)A.error) ||
          globaltimer() - t0 > kResWaitNs) {
        atomicExch(A.error, 1);
        return false;
      }
      // back off (64 ns doubling to 64 << YH_RES_BACKOFF ns) so that
      // polling takes few issue slots from the compute warps
      __nanosleep(64u << (spin < YH_RES_BACKOFF ? spin : YH_RES_BACKOFF));
#pragma unroll
      for (int k = 0; k < kResBatch; ++k)
        if ((unsigned)(x[k] >> 32) != want) {
          const int e = base + k * nc + c;
          const bool up = e >= nx;
          x[k] = ld_tagged(up ? above + (e - nx) : below + e);
        }
    }
#pragma unroll
    for (int k = 0; k < kResBatch; ++k) {
      const int e = base + k * nc + c;
      const bool up = e >= nx;
      if (!(e < 2 * nx && (up ? !top : !bottom))) continue;
      const int i = up ? e - nx : e;
      float u = __uint_as_float((unsigned)x[k]);
      if (e1 > e0) u = res_stim_cell(A, e0, e1, up ? r0 + R : r0 - 1, i, u);
      dst[(up ? R + 1 : 0) * nx + i] = u;
    }
  }
  return true;
}

template <int MODEL, bool HOLES, int CW, int NC>
__global__ void __launch_bounds__(kResThreads + NC, 1)
    rd_resident_kernel(const ResArgs A) {
  extern __shared__ float4 sm4[];
  const StepCoeffs<float> &a = A.a;
  const int nx = a.nx, ny = a.ny;
  const int b = blockIdx.x, nb = A.nb, RM = A.rmax;
  const int r0 = b * A.rq + min(b, A.rrem);
  const int R = A.rq + (b < A.rrem ? 1 : 0);
  const bool bottom = b == 0, top = b == nb - 1;
  float *U0 = reinterpret_cast<float *>(sm4);
  float *U1 = U0 + (RM + 2) * nx;
  float *Vs = U1 + (RM + 2) * nx;
  float *Ws = Vs + RM * nx;
  uint8_t *Cs = reinterpret_cast<uint8_t *>(Ws + RM * nx);
  constexpr bool W3 = MODEL == YH_MODEL_FK3V;
  const int t = threadIdx.x;
  const int T = A.threads;  // compute threads
  constexpr int nc = NC;    // receiving threads: the last warps
  const bool comm = t >= T;
  const int c = t - T;
  const int nq = nx / CW;
  const int vr0 = t / nq, q0 = t - vr0 * nq;
  const size_t par_stride = (size_t)nb * 2 * nx;  // words per step parity
  __shared__ int s_abort;
  __shared__ int s_ev_step[kResMaxStims];
  if (t == 0) s_abort = 0;
  if (t < A.nstims) s_ev_step[t] = A.stims[t].step;
  __syncthreads();

  // load the block's rows; hole codes from the mask with mirrored neighbours
  for (int idx = t; idx < R * nx; idx += (int)blockDim.x) {
    const int lr = idx / nx, i = idx - lr * nx, gy = r0 + lr;
    const size_t g = (size_t)gy * nx + i;
    const float u = A.io.f[0][g];
    U0[(lr + 1) * nx + i] = u;
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
    // the boundary rows of the state after 0 steps, tag 0, buffer 0
    if (lr == 0 && !bottom && b != A.mute)
      st_tagged(A.halo + (size_t)b * 2 * nx + i, u, 0u);
    if (lr == R - 1 && !top && b != A.mute)
      st_tagged(A.halo + (size_t)b * 2 * nx + nx + i, u, 0u);
  }
  // halo rows of the state after 0 steps
  int ev = 0;  // first event not before the current step
  {
    int e0, e1;
    stim_run(s_ev_step, A.nstims, ev, A.step0, e0, e1);
    if (comm && !res_receive<CW>(A, 0, e0, e1, b, r0, R, bottom, top, U0, c, nc))
      s_abort = 1;
  }
  __syncthreads();
  if (s_abort) return;

  for (int s = 0; s < A.nsteps; ++s) {
    const int gs = A.step0 + s;
    float *cur = (s & 1) ? U1 : U0;
    float *nxt = (s & 1) ? U0 : U1;
    // stimulus events of this step on the block's own rows (the halo rows
    // got theirs when they were received)
    int e0, e1;
    stim_run(s_ev_step, A.nstims, ev, gs, e0, e1);
    if (e1 > e0) {
      for (int e = e0; e < e1; ++e)
        for (int lr = 0; lr < R; ++lr)
          res_stim_row(cur + (lr + 1) * nx, r0 + lr, nx, A.stims[e], A.solid);
      __syncthreads();
    }
    ev = e1;
    if (!comm) {
      // rows 0 and R-1 (published, tag s + 1), then the interior rows, in
      // the order rows 0, R-1, 1 .. R-2 (virtual row vr), nq items per row,
      // thread t taking items t, t + T, ...
      unsigned long long *pub =
          b == A.mute ? nullptr
                      : A.halo + (size_t)((s + 1) & 1) * par_stride + (size_t)b * 2 * nx;
      for (int vr = vr0, q = q0; vr < R;) {
        const int lr = vr == 0 ? 0 : (vr == 1 ? R - 1 : vr - 1);
        res_item<MODEL, HOLES, CW>(a, lr, q, R, bottom, top, cur, nxt, Vs, Ws,
                                   Cs, pub, (unsigned)s + 1u);
        q += T;
        while (q >= nq) {
          q -= nq;
          ++vr;
        }
      }
    } else if (s + 1 < A.nsteps) {
      int n0, n1;
      stim_run(s_ev_step, A.nstims, ev, gs + 1, n0, n1);
      if (!res_receive<CW>(A, s + 1, n0, n1, b, r0, R, bottom, top, nxt, c, nc))
        s_abort = 1;
    }
    __syncthreads();
    if (s_abort) return;
  }

  // write the state back (and u of the level before the last step)
  const float *fin = (A.nsteps & 1) ? U1 : U0;
  const float *pre = (A.nsteps & 1) ? U0 : U1;
  for (int idx = t; idx < R * nx; idx += (int)blockDim.x) {
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
  // compute threads: the fewest rounds of work items at up to kResThreads
  // threads, then the fewest warps that keep that number of rounds (every
  // thread the same number of items where the rows allow it)
  const int cw = (a.nx % kResCells) == 0 ? kResCells : 1;
  const int items = pl.rmax * (a.nx / cw);
  const int rounds = (items + kResThreads - 1) / kResThreads;
  const int per = (items + rounds - 1) / rounds;
  pl.threads = ((per + 31) / 32) * 32;
  if (pl.threads > kResThreads) pl.threads = kResThreads;
  return pl;
}

size_t resident_halo_bytes(const ResidentPlan &pl, int nx) {
  return (size_t)2 * pl.nb * 2 * nx * sizeof(unsigned long long);
}

template <int MODEL, bool HOLES, int CW, int NC>
static cudaError_t launch_res_t(const ResArgs &A, size_t smem,
                                cudaStream_t s) {
  auto fn = rd_resident_kernel<MODEL, HOLES, CW, NC>;
  cudaError_t e =
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void *args[] = {const_cast<ResArgs *>(&A)};
  return cudaLaunchCooperativeKernel((const void *)fn, dim3(A.nb),
                                     dim3(A.threads + NC), args, smem, s);
}

cudaError_t launch_rd_resident(const StepCoeffs<float> &a, const Fld<float> &io,
                               float *prev_u, const uint8_t *solid,
                               int nsteps, int step0,
                               const yh_stim *stims, int nstims,
                               const ResidentPlan &pl,
                               unsigned long long *halo, int *error,
                               cudaStream_t s, int mute) {
  if (!pl.ok || nstims > kResMaxStims || nsteps < 0) return cudaErrorInvalidValue;
  if (nsteps == 0) return cudaSuccess;
  ResArgs A;
  A.mute = mute;
  A.a = a;
  A.io = io;
  A.prev_u = prev_u;
  A.solid = solid;
  A.halo = halo;
  A.error = error;
  A.nsteps = nsteps;
  A.step0 = step0;
  A.nb = pl.nb;
  A.rq = pl.rq;
  A.rrem = pl.rrem;
  A.rmax = pl.rmax;
  A.nstims = nstims;
  for (int k = 0; k < nstims; ++k) A.stims[k] = stims[k];
  // by step, stable: events of one step keep their order (a later event
  // overrides an earlier one on the cells both cover)
  std::stable_sort(A.stims, A.stims + nstims,
                   [](const yh_stim &x, const yh_stim &y) { return x.step < y.step; });
  cudaError_t e = cudaMemsetAsync(halo, 0xff, resident_halo_bytes(pl, a.nx), s);
  if (e != cudaSuccess) return e;
  const bool vec = (a.nx % kResCells) == 0;
  const bool holes = solid != nullptr;
  A.threads = pl.threads;
  // Receiving threads: 128 take the halo in one pass of loads; with a hole
  // mask the compute warps are the critical path and 64 (two passes, fewer
  // warps beside them) measured faster (FK3V 1024^2 on GB300: 3.41 vs 3.79
  // us per step with 300 holes; 3.03 vs 2.61 without).

#define YH_RES(M, H, V)                                         \
  if (a.model == M && holes == H && vec == V)                   \
    return launch_res_t<M, H, V ? kResCells : 1, H ? 64 : kResCommMax>(A, pl.smem, s);
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
