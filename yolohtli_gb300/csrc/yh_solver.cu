// Solver handle of include/yolohtli.h: owns the device buffers of one grid
// and runs plain and symmetry-reduced step sequences as captured CUDA graphs
// (the reference drives every kernel from the GLUT idle callback with a
// blocking copy per step, main.cu:862-1040).
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "yh_kernels.cuh"

namespace yh {
int check_params(const yh_param_var *p, int model, const yh_fk_params *fk);
}  // namespace yh

using namespace yh;

namespace {

constexpr int kPlainGraphSteps = 64;  // even: the state ends where it began
constexpr int kSrGraphSteps = 16;
constexpr int kTipCapacity = 1 << 16;

struct GraphCache {
  const float *key = nullptr;
  int len = 0;
  int tb = 0;
  long long kernels = 0;  // kernel launches one replay performs
  cudaGraphExec_t exec = nullptr;
};

inline int st(cudaError_t e) {
  if (e == cudaSuccess) return YH_OK;
  if (e == cudaErrorMemoryAllocation) return YH_ENOMEM;
  return YH_ECUDA;
}

}  // namespace

struct yh_solver {
  yh_param_var p;
  yh_fk_params fk;
  int model = 0, nf = 2;
  cudaStream_t s = nullptr;
  size_t n = 0, stride = 0;
  float *pool = nullptr;     // state ping-pong
  float *sr_pool = nullptr;  // tangent, BFECC scratch, template
  Fld<float> cur{}, nxt{}, tan{}, uf{}, ue{}, tx{}, ty{}, tt{};
  uint8_t *solid = nullptr;
  uint8_t *codes = nullptr;  // per-cell hole codes of solid (same allocation)
  int *tip_count = nullptr;
  yh_tip *tips = nullptr;
  unsigned int *tip_done = nullptr;
  yh_sym_state *sym = nullptr;
  void *ws = nullptr;
  double *adv_d = nullptr;  // ny rows then nx columns
  float *adv_f = nullptr;
  int step = 0;
  int sr_step = 0;
  int sr_nsingular = 0;  // the device state's nsingular at the last read
  int time_block = 1;
  bool sr_ready = false;
  bool frozen = false;
  long long launches = 0;  // kernels enqueued by this handle
  bool own_stream = false;
  int engine = YH_ENGINE_STEP;
  ResidentPlan plan{};       // resident solver layout (plan.ok: usable)
  unsigned long long *res_halo = nullptr;  // tagged boundary rows
  int *res_error = nullptr;  // device flag set when a bounded wait gave up
  unsigned long long *nonfinite = nullptr;  // yh_check_finite's count
  GraphCache plain[2];
  GraphCache sr[2];
};

static void free_graph(GraphCache &g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  g = GraphCache();
}

static Fld<float> carve(float *base, size_t stride, int nf, int slot) {
  Fld<float> f{};
  for (int k = 0; k < nf; ++k) f.f[k] = base + (size_t)(slot * nf + k) * stride;
  return f;
}

extern "C" int yh_create(const yh_param_var *p, int model,
                         const yh_fk_params *fk, const uint8_t *solid_host,
                         void *stream, yh_solver **out) {
  if (!out) return YH_EINVAL;
  *out = nullptr;
  int rc = check_params(p, model, fk);
  if (rc) return rc;
  if (p->solidSwitch && !solid_host) return YH_EINVAL;
  yh_solver *h = new (std::nothrow) yh_solver();
  if (!h) return YH_ENOMEM;
  h->p = *p;
  if (fk) h->fk = *fk; else memset(&h->fk, 0, sizeof(h->fk));
  h->model = model;
  h->nf = model == YH_MODEL_FK3V ? 3 : 2;
  h->s = (cudaStream_t)stream;
  h->n = (size_t)p->nx * p->ny;
  h->stride = (h->n + 63) & ~(size_t)63;  // 256-byte aligned fields
  cudaError_t e = cudaSuccess;
  if (!h->s) {
    // The legacy default stream cannot be captured into a graph: use a
    // blocking stream of our own, which still orders with it.
    e = cudaStreamCreate(&h->s);
    h->own_stream = e == cudaSuccess;
  }
  if (e == cudaSuccess)
    e = cudaMalloc(&h->pool, 2 * h->nf * h->stride * sizeof(float));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->pool, 0, 2 * h->nf * h->stride * sizeof(float),
                        h->s);
  if (e == cudaSuccess) {
    h->cur = carve(h->pool, h->stride, h->nf, 0);
    h->nxt = carve(h->pool, h->stride, h->nf, 1);
  }
  if (e == cudaSuccess && p->solidSwitch) {
    const size_t padded = (h->n + 255) & ~(size_t)255;
    e = cudaMalloc(&h->solid, 2 * padded);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h->solid, solid_host, h->n, cudaMemcpyHostToDevice,
                          h->s);
    if (e == cudaSuccess) {
      h->codes = h->solid + padded;
      e = launch_hole_codes(h->solid, p->nx, p->ny, h->codes, h->s);
    }
  }
  if (e == cudaSuccess) e = cudaMalloc(&h->tip_count, 256);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->tip_count, 0, 256, h->s);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->tips, (size_t)kTipCapacity * sizeof(yh_tip));
  if (e == cudaSuccess) h->tip_done = (unsigned int *)(h->tip_count + 32);
  if (e == cudaSuccess) e = cudaMalloc(&h->sym, sizeof(yh_sym_state));
  if (e == cudaSuccess) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
      h->plan = resident_plan(make_step_coeffs<float>(h->p, h->model, &h->fk), dev);
  }
  // the flag a bounded wait sets when it gives up (resident engine, TMA)
  if (e == cudaSuccess) e = cudaMalloc(&h->res_error, 256);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->res_error, 0, 256, h->s);
  if (e == cudaSuccess && h->plan.ok)
    e = cudaMalloc(&h->res_halo, resident_halo_bytes(h->plan, p->nx));
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) {
    yh_destroy(h);
    return st(e);
  }
  *out = h;
  return YH_OK;
}

extern "C" int yh_destroy(yh_solver *h) {
  if (!h) return YH_EINVAL;
  if (h->s) cudaStreamSynchronize(h->s); else cudaDeviceSynchronize();
  for (auto &g : h->plain) free_graph(g);
  for (auto &g : h->sr) free_graph(g);
  cudaFree(h->pool);
  cudaFree(h->sr_pool);
  cudaFree(h->solid);
  cudaFree(h->tip_count);
  cudaFree(h->tips);
  cudaFree(h->sym);
  cudaFree(h->ws);
  cudaFree(h->adv_d);
  cudaFree(h->adv_f);
  cudaFree(h->res_halo);
  cudaFree(h->res_error);
  cudaFree(h->nonfinite);
  if (h->own_stream) cudaStreamDestroy(h->s);
  delete h;
  return YH_OK;
}

// YH_ETIMEOUT if a resident launch gave up waiting (after a sync).
static int resident_status(yh_solver *h) {
  if (!h->res_error) return YH_OK;
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, h->res_error, sizeof(int),
                                  cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  return err ? YH_ETIMEOUT : YH_OK;
}

extern "C" int yh_synchronize(yh_solver *h) {
  if (!h) return YH_EINVAL;
  const int rc = st(cudaStreamSynchronize(h->s));
  return rc ? rc : resident_status(h);
}

extern "C" int yh_set_state(yh_solver *h, const float *u, const float *v,
                            const float *w) {
  if (!h) return YH_EINVAL;
  const float *src[3] = {u, v, w};
  for (int f = 0; f < h->nf; ++f) {
    if (!src[f]) continue;
    cudaError_t e = cudaMemcpyAsync(h->cur.f[f], src[f], h->n * sizeof(float),
                                    cudaMemcpyDefault, h->s);
    if (e != cudaSuccess) return st(e);
  }
  return YH_OK;
}

extern "C" int yh_get_state(yh_solver *h, float *u, float *v, float *w) {
  if (!h) return YH_EINVAL;
  float *dst[3] = {u, v, w};
  for (int f = 0; f < h->nf; ++f) {
    if (!dst[f]) continue;
    cudaError_t e = cudaMemcpyAsync(dst[f], h->cur.f[f], h->n * sizeof(float),
                                    cudaMemcpyDefault, h->s);
    if (e != cudaSuccess) return st(e);
  }
  const int rc = st(cudaStreamSynchronize(h->s));
  return rc ? rc : resident_status(h);
}

extern "C" int yh_state_device(yh_solver *h, yh_fields *cur) {
  if (!h || !cur) return YH_EINVAL;
  cur->u = h->cur.f[0];
  cur->v = h->cur.f[1];
  cur->w = h->nf > 2 ? h->cur.f[2] : nullptr;
  return YH_OK;
}

extern "C" int yh_get_step(yh_solver *h, int *step) {
  if (!h || !step) return YH_EINVAL;
  *step = h->step;
  return YH_OK;
}

extern "C" int yh_set_step(yh_solver *h, int step) {
  if (!h || step < 0) return YH_EINVAL;
  h->step = step;
  return YH_OK;
}

// The blocked kernel exchanges only u between sub-steps: models where v
// diffuses too (REF2V with gateDiff) take one launch per step.
static int max_time_block(const yh_solver *h) {
  if (h->model == YH_MODEL_REF2V && h->p.gateDiff) return 1;
  return rd_tb_max_steps();
}

extern "C" int yh_set_time_block(yh_solver *h, int k) {
  if (!h) return YH_EINVAL;
  if (k < 1) k = 1;
  const int kmax = max_time_block(h);
  h->time_block = k > kmax ? kmax : k;
  h->engine = h->time_block > 1 ? YH_ENGINE_BLOCKED : YH_ENGINE_STEP;
  return YH_OK;
}

extern "C" int yh_get_time_block(yh_solver *h, int *k) {
  if (!h || !k) return YH_EINVAL;
  *k = h->time_block;
  return YH_OK;
}

extern "C" int yh_set_engine(yh_solver *h, int engine, int steps_per_launch) {
  if (!h) return YH_EINVAL;
  switch (engine) {
    case YH_ENGINE_STEP:
      h->engine = engine;
      h->time_block = 1;
      return YH_OK;
    case YH_ENGINE_BLOCKED: {
      if (max_time_block(h) < 2) return YH_EUNSUPPORTED;
      yh_set_time_block(h, steps_per_launch < 2 ? 2 : steps_per_launch);
      return YH_OK;
    }
    case YH_ENGINE_RESIDENT:
      if (!h->plan.ok) return YH_EUNSUPPORTED;
      h->engine = engine;
      h->time_block = 1;
      return YH_OK;
  }
  return YH_EINVAL;
}

extern "C" int yh_get_engine(yh_solver *h, int *engine, int *steps_per_launch) {
  if (!h) return YH_EINVAL;
  if (engine) *engine = h->engine;
  if (steps_per_launch) *steps_per_launch = h->time_block;
  return YH_OK;
}

// nsteps resident steps from h->cur in place, events in [step, step+nsteps)
// applied inside the kernel (at most kResMaxStims per launch).
static int run_resident(yh_solver *h, int nsteps, const yh_stim *ev,
                        int nev) {
  const StepCoeffs<float> a = make_step_coeffs<float>(h->p, h->model, &h->fk);
  int done = 0, k = 0;
  while (done < nsteps) {
    int len = nsteps - done, m = nev - k;
    if (m > kResMaxStims) {  // stop before the first event that does not fit
      m = kResMaxStims;
      len = ev[k + m].step - (h->step);
    }
    // the state stays in h->cur; the previous u level goes to h->nxt (tips)
    cudaError_t e = launch_rd_resident(a, h->cur, h->nxt.f[0], h->solid, len,
                                       h->step, ev + k, m, h->plan,
                                       h->res_halo, h->res_error, h->s);
    if (e != cudaSuccess) return st(e);
    h->launches += 1;
    h->step += len;
    done += len;
    k += m;
  }
  return YH_OK;
}

// Failure self-test of the bounded device-side waits: a small FK3V grid on
// the resident engine, once with one block publishing nothing (its
// neighbours' waits run out after their 1 s bound, set the error flag and
// every block returns), once normally on the same context. No fault, trap
// or unbounded wait is involved.
extern "C" int yh_selftest_resident_timeout(int *muted_status,
                                            int *after_status) {
  if (!muted_status || !after_status) return YH_EINVAL;
  const int n = 128;
  yh_param_var p;
  yh_fk_params fk;
  int rc = yh_param_defaults(&p, n, n);
  if (!rc) rc = yh_fk_defaults(&fk);
  if (rc) return rc;
  p.hx = p.hy = 0.025;
  p.Lx = p.Ly = 0.025 * (n - 1);
  p.dt = 0.05;
  p.diff_par = p.diff_per = p.Dxx = p.Dyy = 0.001;
  p.Dxy = 0.0;
  p.gateDiff = false;
  rc = yh_param_derive(&p);
  if (rc) return rc;
  yh_solver *h = nullptr;
  rc = yh_create(&p, YH_MODEL_FK3V, &fk, nullptr, nullptr, &h);
  if (rc) return rc;
  if (!h->plan.ok || h->plan.nb < 3) {
    yh_destroy(h);
    return YH_EUNSUPPORTED;
  }
  const StepCoeffs<float> a = make_step_coeffs<float>(h->p, h->model, &h->fk);
  cudaError_t e = launch_rd_resident(a, h->cur, nullptr, h->solid, 4, 0,
                                     nullptr, 0, h->plan, h->res_halo,
                                     h->res_error, h->s, 1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  *muted_status = e == cudaSuccess ? resident_status(h) : st(e);
  e = cudaMemsetAsync(h->res_error, 0, sizeof(int), h->s);
  if (e == cudaSuccess)
    e = launch_rd_resident(a, h->cur, nullptr, h->solid, 4, 0, nullptr, 0,
                           h->plan, h->res_halo, h->res_error, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  *after_status = e == cudaSuccess ? resident_status(h) : st(e);
  yh_destroy(h);
  return YH_OK;
}

// `len` plain steps starting from h->cur, leaving the result in h->cur.
// With time_block > 1 the temporally blocked kernel takes that many steps
// per launch (its depth is fixed per launch, so the ping-pong flips once per
// launch).
static cudaError_t enqueue_plain(yh_solver *h, int len) {
  const StepCoeffs<float> a = make_step_coeffs<float>(h->p, h->model, &h->fk);
  const Fld<float> none{};
  int left = len;
  while (left > 0) {
    cudaError_t e;
    if (h->time_block > 1 && left >= 2) {
      const int k = std::min(left, h->time_block);
      if (k == 2 && rd_2s_supported(a, h->cur, h->nxt, h->solid != nullptr,
                                    h->codes))
        e = launch_rd_2s(a, h->cur, h->nxt, h->codes, h->res_error, h->s);
      else
        e = launch_rd_tb(a, h->cur, h->nxt, h->solid, k, h->s);
      left -= k;
    } else {
      e = launch_rd_step<float>(a, h->cur, h->nxt, none, h->solid, h->s,
                                h->codes);
      left -= 1;
    }
    if (e != cudaSuccess) return e;
    h->launches += 1;
    std::swap(h->cur, h->nxt);
  }
  return cudaSuccess;
}

static int graph_for(yh_solver *h, GraphCache *cache, int len,
                     cudaError_t (*body)(yh_solver *, int),
                     cudaGraphExec_t *exec) {
  for (int k = 0; k < 2; ++k)
    if (cache[k].exec && cache[k].key == h->cur.f[0] && cache[k].len == len &&
        cache[k].tb == h->time_block) {
      *exec = cache[k].exec;
      return YH_OK;
    }
  GraphCache &slot = cache[0].exec && !cache[1].exec ? cache[1] : cache[0];
  free_graph(slot);
  const float *key = h->cur.f[0];
  const Fld<float> save_cur = h->cur, save_nxt = h->nxt;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return st(e);
  const long long before = h->launches;
  cudaError_t eb = body(h, len);
  e = cudaStreamEndCapture(h->s, &g);
  const long long kernels = h->launches - before;
  h->launches = before;  // capturing launches nothing
  h->cur = save_cur;
  h->nxt = save_nxt;
  if (eb != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return st(eb);
  }
  if (e != cudaSuccess) return st(e);
  e = cudaGraphInstantiate(&slot.exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    slot = GraphCache();
    return st(e);
  }
  slot.key = key;
  slot.len = len;
  slot.tb = h->time_block;
  slot.kernels = kernels;
  *exec = slot.exec;
  return YH_OK;
}

// Replays a cached graph and counts its kernels.
static int replay(yh_solver *h, GraphCache *cache, cudaGraphExec_t ex) {
  cudaError_t e = cudaGraphLaunch(ex, h->s);
  if (e != cudaSuccess) return st(e);
  for (int k = 0; k < 2; ++k)
    if (cache[k].exec == ex) h->launches += cache[k].kernels;
  return YH_OK;
}

static cudaError_t plain_body(yh_solver *h, int len) {
  return enqueue_plain(h, len);
}

// Runs `len` plain steps: whole graphs of kPlainGraphSteps, then the rest
// launched directly. Returns with the state in h->cur.
static int run_plain(yh_solver *h, int len) {
  while (len >= kPlainGraphSteps) {
    cudaGraphExec_t ex = nullptr;
    int rc = graph_for(h, h->plain, kPlainGraphSteps, plain_body, &ex);
    if (rc) return rc;
    rc = replay(h, h->plain, ex);
    if (rc) return rc;
    // the graph is built so that an even number of flips returns the
    // state to h->cur; with temporal blocking the flips are per launch
    int flips = 0;
    {
      int left = kPlainGraphSteps;
      while (left > 0) {
        if (h->time_block > 1 && left >= 2) left -= std::min(left, h->time_block);
        else left -= 1;
        ++flips;
      }
    }
    if (flips & 1) std::swap(h->cur, h->nxt);
    len -= kPlainGraphSteps;
    h->step += kPlainGraphSteps;
  }
  if (len > 0) {
    cudaError_t e = enqueue_plain(h, len);
    if (e != cudaSuccess) return st(e);
    h->step += len;
  }
  return YH_OK;
}

// Times `probe_steps` plain steps from the current state for every engine
// and time block depth the model allows (a warm-up run each, CUDA events on
// the handle's stream), restores the state, step and launch counters, and
// keeps the fastest. Returns it in *engine, *steps_per_launch.
extern "C" int yh_autotune(yh_solver *h, int probe_steps, int *engine,
                           int *steps_per_launch) {
  if (!h || probe_steps < 1) return YH_EINVAL;
  const size_t bytes = h->n * sizeof(float);
  float *save = nullptr;
  cudaError_t e = cudaMalloc(&save, h->nf * bytes);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int f = 0; f < h->nf && e == cudaSuccess; ++f)
    e = cudaMemcpyAsync(save + f * h->n, h->cur.f[f], bytes,
                        cudaMemcpyDeviceToDevice, h->s);
  const int step0 = h->step;
  const long long launches0 = h->launches;
  const int kmax = max_time_block(h);
  // candidates: (engine, depth)
  std::vector<std::pair<int, int>> cand;
  cand.push_back({YH_ENGINE_STEP, 1});
  for (int k = 2; k <= kmax; ++k) cand.push_back({YH_ENGINE_BLOCKED, k});
  if (h->plan.ok) cand.push_back({YH_ENGINE_RESIDENT, 1});
  std::pair<int, int> best_c = cand[0];
  float best_ms = 1e30f;
  int rc = st(e);
  for (size_t c = 0; c < cand.size() && rc == YH_OK; ++c) {
    h->engine = cand[c].first;
    h->time_block = cand[c].second;
    float ms = 0.f;
    for (int rep = 0; rep < 2 && rc == YH_OK; ++rep) {
      for (int f = 0; f < h->nf && rc == YH_OK; ++f)
        rc = st(cudaMemcpyAsync(h->cur.f[f], save + f * h->n, bytes,
                                cudaMemcpyDeviceToDevice, h->s));
      if (rc == YH_OK) rc = st(cudaEventRecord(e0, h->s));
      if (rc == YH_OK)
        rc = h->engine == YH_ENGINE_RESIDENT
                 ? run_resident(h, probe_steps, nullptr, 0)
                 : run_plain(h, probe_steps);
      if (rc == YH_OK) rc = st(cudaEventRecord(e1, h->s));
      if (rc == YH_OK) rc = st(cudaEventSynchronize(e1));
      if (rc == YH_OK) rc = st(cudaEventElapsedTime(&ms, e0, e1));
      if (rc == YH_OK) rc = resident_status(h);
    }
    if (rc == YH_OK && ms < best_ms) {
      best_ms = ms;
      best_c = cand[c];
    }
  }
  for (int f = 0; f < h->nf && rc == YH_OK; ++f)
    rc = st(cudaMemcpyAsync(h->cur.f[f], save + f * h->n, bytes,
                            cudaMemcpyDeviceToDevice, h->s));
  if (rc == YH_OK) rc = st(cudaStreamSynchronize(h->s));
  h->step = step0;
  h->launches = launches0;
  h->engine = best_c.first;
  h->time_block = best_c.second;
  if (engine) *engine = best_c.first;
  if (steps_per_launch) *steps_per_launch = best_c.second;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  return rc;
}

extern "C" int yh_run(yh_solver *h, int nsteps, const yh_stim *stims,
                      int nstims) {
  if (!h || nsteps < 0 || (nstims > 0 && !stims)) return YH_EINVAL;
  const int end = h->step + nsteps;
  std::vector<yh_stim> ev;
  for (int k = 0; k < nstims; ++k)
    if (stims[k].step >= h->step && stims[k].step < end) ev.push_back(stims[k]);
  std::stable_sort(ev.begin(), ev.end(),
                   [](const yh_stim &a, const yh_stim &b) { return a.step < b.step; });
  if (h->engine == YH_ENGINE_RESIDENT && nsteps > 0) {
    const int rc = run_resident(h, nsteps, ev.data(), (int)ev.size());
    return rc ? rc : st(cudaGetLastError());
  }
  size_t k = 0;
  while (h->step < end) {
    while (k < ev.size() && ev[k].step == h->step) {
      cudaError_t e = launch_stimulate<float>(
          h->cur.f[0], h->solid, h->p.nx, h->p.ny, ev[k].i0, ev[k].j0,
          ev[k].i1, ev[k].j1, ev[k].value, h->s);
      if (e != cudaSuccess) return st(e);
      h->launches += 1;
      ++k;
    }
    const int next = k < ev.size() ? ev[k].step : end;
    int rc;
    if (next == end && h->time_block > 1 && end - h->step >= 2) {
      // the run's last step on its own: a launch of k steps leaves the u
      // level k steps back in h->nxt, yh_track_tips needs the previous one
      rc = run_plain(h, end - 1 - h->step);
      if (!rc) rc = run_plain(h, 1);
    } else {
      rc = run_plain(h, next - h->step);
    }
    if (rc) return rc;
  }
  return st(cudaGetLastError());
}

extern "C" int yh_track_tips(yh_solver *h) {
  if (!h) return YH_EINVAL;
  cudaError_t e = cudaMemsetAsync(h->tip_count, 0, sizeof(int), h->s);
  if (e != cudaSuccess) return st(e);
  // plain mode: x = new u (present), y = old u (past) (main.cu:963)
  e = launch_tips<float>(h->p, h->nxt.f[0], h->cur.f[0], h->p.solidSwitch,
                         h->p.dt * (double)h->step, h->tip_count, h->tips,
                         kTipCapacity, nullptr, nullptr, h->s);
  if (e == cudaSuccess) h->launches += 1;
  return st(e);
}

extern "C" int yh_get_launch_count(yh_solver *h, long long *n) {
  if (!h || !n) return YH_EINVAL;
  *n = h->launches;
  return YH_OK;
}

extern "C" int yh_get_tips(yh_solver *h, yh_tip *out, int capacity, int *n) {
  if (!h || !n || (capacity > 0 && !out)) return YH_EINVAL;
  int cnt = 0;
  cudaError_t e = cudaMemcpyAsync(&cnt, h->tip_count, sizeof(int),
                                  cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  const int have = std::min(cnt, kTipCapacity);
  std::vector<yh_tip> buf((size_t)have);
  if (have > 0) {
    e = cudaMemcpyAsync(buf.data(), h->tips, (size_t)have * sizeof(yh_tip),
                        cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return st(e);
  }
  // the atomic push order is not deterministic: return them sorted by (y, x)
  std::sort(buf.begin(), buf.end(), [](const yh_tip &a, const yh_tip &b) {
    return a.y < b.y || (a.y == b.y && a.x < b.x);
  });
  const int m = std::min(have, capacity);
  if (m > 0) memcpy(out, buf.data(), (size_t)m * sizeof(yh_tip));
  *n = cnt;
  return cnt > kTipCapacity || cnt > capacity ? YH_EOVERFLOW : YH_OK;
}

// ---------------------------------------------------------------------------
// Symmetry reduction
// ---------------------------------------------------------------------------

extern "C" int yh_sr_begin(yh_solver *h, int template_mode, const float *tu,
                           const float *tv, const float *tw) {
  if (!h) return YH_EINVAL;
  if (template_mode != YH_TEMPLATE_CURRENT && template_mode != YH_TEMPLATE_FROZEN)
    return YH_EINVAL;
  const bool frozen = template_mode == YH_TEMPLATE_FROZEN;
  if (frozen && (!tu || !tv || (h->nf > 2 && !tw))) return YH_EINVAL;
  cudaError_t e = cudaSuccess;
  if (!h->sr_pool) {
    // tan, uf, ue, tx, ty, tt
    e = cudaMalloc(&h->sr_pool, 6 * h->nf * h->stride * sizeof(float));
    if (e == cudaSuccess)
      e = cudaMemsetAsync(h->sr_pool, 0, 6 * h->nf * h->stride * sizeof(float),
                          h->s);
    if (e != cudaSuccess) return st(e);
    h->tan = carve(h->sr_pool, h->stride, h->nf, 0);
    h->uf = carve(h->sr_pool, h->stride, h->nf, 1);
    h->ue = carve(h->sr_pool, h->stride, h->nf, 2);
    h->tx = carve(h->sr_pool, h->stride, h->nf, 3);
    h->ty = carve(h->sr_pool, h->stride, h->nf, 4);
    h->tt = carve(h->sr_pool, h->stride, h->nf, 5);
    const size_t wsb = yh_phase_integrals_workspace(h->p.nx, h->p.ny);
    e = cudaMalloc(&h->ws, wsb);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->ws, 0, wsb, h->s);
    if (e == cudaSuccess)
      e = cudaMalloc(&h->adv_d, (size_t)(h->p.nx + h->p.ny) * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMalloc(&h->adv_f, (size_t)(h->p.nx + h->p.ny) * sizeof(float));
    if (e != cudaSuccess) return st(e);
  }
  e = cudaMemsetAsync(h->adv_d, 0, (size_t)(h->p.nx + h->p.ny) * sizeof(double), h->s);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->adv_f, 0, (size_t)(h->p.nx + h->p.ny) * sizeof(float), h->s);
  if (e != cudaSuccess) return st(e);
  if (frozen) {
    // the template state goes through the BFECC scratch uf
    const float *src[3] = {tu, tv, tw};
    for (int f = 0; f < h->nf; ++f) {
      e = cudaMemcpyAsync(h->uf.f[f], src[f], h->n * sizeof(float),
                          cudaMemcpyHostToDevice, h->s);
      if (e != cudaSuccess) return st(e);
    }
    e = launch_template<float>(h->p, h->nf, h->uf, h->tx, h->ty, h->tt, h->s);
    if (e != cudaSuccess) return st(e);
  }
  yh_sym_state s0;
  memset(&s0, 0, sizeof(s0));
  s0.centre[0] = h->p.tipx;  // tipx0_d (main.cu:373-376)
  s0.centre[1] = h->p.tipy;
  e = cudaMemcpyAsync(h->sym, &s0, sizeof(s0), cudaMemcpyHostToDevice, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  h->frozen = frozen;
  h->sr_step = 0;
  h->sr_nsingular = 0;
  h->sr_ready = true;
  for (auto &g : h->sr) free_graph(g);
  return YH_OK;
}

// One symmetry-reduced step (main.cu:894-954) on the stream.
static cudaError_t enqueue_sr_step(yh_solver *h, bool first) {
  const StepCoeffs<float> a = make_step_coeffs<float>(h->p, h->model, &h->fk);
  const Fld<float> none{};
  const Fld<float> tx = h->frozen ? h->tx : none;
  const Fld<float> ty = h->frozen ? h->ty : none;
  const Fld<float> tt = h->frozen ? h->tt : none;
  float *advf_rows = h->adv_f, *advf_cols = h->adv_f + h->p.ny;
  // 1. RD with tangent: cur -> nxt; it also zeroes the tip count
  cudaError_t e = launch_rd_step<float>(a, h->cur, h->nxt, h->tan, h->solid,
                                        h->s, h->codes, h->tip_count);
  if (e == cudaSuccess)  // 2. tips x = pre-RD u, y = post-RD u; centre
    e = launch_tips<float>(h->p, h->nxt.f[0], h->cur.f[0], h->p.solidSwitch, 0.0,
                           h->tip_count, h->tips, kTipCapacity, h->sym,
                           h->tip_done, h->s);
  // phase integrals + solve + comoving field, twice on the first step
  // (main.cu:910-926)
  const int reps = first ? 2 : 1;
  for (int r = 0; r < reps && e == cudaSuccess; ++r)
    e = launch_phase_comoving(h->p, h->nf, h->cur, h->tan, tx, ty, tt,
                              advf_rows, advf_cols, h->solid, h->sym, h->ws,
                              r == reps - 1, h->s);
  if (e == cudaSuccess)  // BFECC, three passes in one launch: nxt -> cur
    e = launch_bfecc_fused(h->p, h->nf, h->nxt, h->cur, advf_rows, advf_cols,
                           h->solid, h->s);
  // RD, tips, phase x reps, BFECC
  if (e == cudaSuccess) h->launches += 2 + reps + 1;
  return e;
}

static cudaError_t sr_body(yh_solver *h, int len) {
  for (int k = 0; k < len; ++k) {
    cudaError_t e = enqueue_sr_step(h, false);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The steps of yh_sr_step without the status read: enqueued on the
// handle's stream, nothing waited for.
static int sr_enqueue(yh_solver *h, int nsteps) {
  int left = nsteps;
  if (left > 0 && h->sr_step == 0) {
    cudaError_t e = enqueue_sr_step(h, true);
    if (e != cudaSuccess) return st(e);
    h->sr_step += 1;
    h->step += 1;
    left -= 1;
  }
  while (left >= kSrGraphSteps) {
    cudaGraphExec_t ex = nullptr;
    int rc = graph_for(h, h->sr, kSrGraphSteps, sr_body, &ex);
    if (rc) return rc;
    rc = replay(h, h->sr, ex);
    if (rc) return rc;
    left -= kSrGraphSteps;
    h->sr_step += kSrGraphSteps;
    h->step += kSrGraphSteps;
  }
  for (; left > 0; --left) {
    cudaError_t e = enqueue_sr_step(h, false);
    if (e != cudaSuccess) return st(e);
    h->sr_step += 1;
    h->step += 1;
  }
  return st(cudaGetLastError());
}

extern "C" int yh_sr_enqueue(yh_solver *h, int nsteps) {
  if (!h || nsteps < 0) return YH_EINVAL;
  if (!h->sr_ready) return YH_ENOTREADY;
  return sr_enqueue(h, nsteps);
}

// Waits for the handle's stream and reads the singular-solve count of the
// device state: YH_ESINGULAR when it grew since the last read.
extern "C" int yh_sr_status(yh_solver *h) {
  if (!h) return YH_EINVAL;
  if (!h->sr_ready) return YH_ENOTREADY;
  int ns = 0;
  cudaError_t e = cudaMemcpyAsync(&ns, &h->sym->nsingular, sizeof(int),
                                  cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  if (ns != h->sr_nsingular) {
    h->sr_nsingular = ns;
    return YH_ESINGULAR;
  }
  return YH_OK;
}

extern "C" int yh_sr_step(yh_solver *h, int nsteps) {
  if (!h || nsteps < 0) return YH_EINVAL;
  if (!h->sr_ready) return YH_ENOTREADY;
  const int rc = sr_enqueue(h, nsteps);
  if (rc || nsteps == 0) return rc;
  // the singular-solve count of the device state, read once per call
  return yh_sr_status(h);
}

extern "C" int yh_get_sym(yh_solver *h, yh_sym_state *out) {
  if (!h || !out) return YH_EINVAL;
  if (!h->sr_ready) return YH_ENOTREADY;
  cudaError_t e = cudaMemcpyAsync(out, h->sym, sizeof(*out),
                                  cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  return st(e);
}

// ---------------------------------------------------------------------------
// Finite check and checkpoint / resume
// ---------------------------------------------------------------------------

// Counts the non-finite values of field blockIdx.y (exponent bits all ones:
// Inf or NaN, IEEE 754 binary32), one atomic per warp that found any.
__global__ void __launch_bounds__(256)
    count_nonfinite_kernel(Fld<float> f, size_t n, unsigned long long *count) {
  const unsigned *a = (const unsigned *)f.f[blockIdx.y];
  unsigned c = 0;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    c += (a[k] & 0x7f800000u) == 0x7f800000u;
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, (unsigned long long)c);
}

extern "C" int yh_check_finite(yh_solver *h, long long *bad_values) {
  if (!h) return YH_EINVAL;
  cudaError_t e = cudaSuccess;
  if (!h->nonfinite) e = cudaMalloc(&h->nonfinite, sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->nonfinite, 0, sizeof(unsigned long long), h->s);
  if (e != cudaSuccess) return st(e);
  // 4 cells per thread, at most 8 blocks of 256 per SM of a 152-SM GB300
  const size_t per_block = 256 * 4;
  const size_t blocks = std::min<size_t>((h->n + per_block - 1) / per_block,
                                         152 * 8);
  count_nonfinite_kernel<<<dim3((unsigned)blocks, h->nf), 256, 0, h->s>>>(
      h->cur, h->n, h->nonfinite);
  h->launches += 1;
  unsigned long long c = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&c, h->nonfinite, sizeof(c), cudaMemcpyDeviceToHost,
                        h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) return st(e);
  const int rc = resident_status(h);
  if (rc) return rc;
  if (bad_values) *bad_values = (long long)c;
  return c ? YH_ENONFINITE : YH_OK;
}

// The handle's mask on the host (empty when it has none).
static int host_mask(yh_solver *h, std::vector<uint8_t> *mask) {
  mask->clear();
  if (!h->solid) return YH_OK;
  mask->resize(h->n);
  cudaError_t e = cudaMemcpyAsync(mask->data(), h->solid, h->n,
                                  cudaMemcpyDeviceToHost, h->s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  return st(e);
}

extern "C" int yh_save_checkpoint(yh_solver *h, const char *path) {
  if (!h || !path) return YH_EINVAL;
  std::vector<float> u(h->n), v(h->n), w(h->nf > 2 ? h->n : 0);
  std::vector<uint8_t> mask;
  int rc = yh_get_state(h, u.data(), v.data(), h->nf > 2 ? w.data() : nullptr);
  if (!rc) rc = host_mask(h, &mask);
  if (rc) return rc;
  return yh_write_checkpoint(path, &h->p, h->model,
                             h->model == YH_MODEL_FK3V ? &h->fk : nullptr,
                             mask.empty() ? nullptr : mask.data(), h->step,
                             u.data(), v.data(),
                             h->nf > 2 ? w.data() : nullptr);
}

// The parameters the step's coefficients are made of (make_step_coeffs).
static bool same_step(const yh_param_var &a, const yh_param_var &b) {
  return a.nx == b.nx && a.ny == b.ny && a.gateDiff == b.gateDiff &&
         a.rx == b.rx && a.ry == b.ry && a.rscale == b.rscale &&
         a.dt == b.dt && a.tc == b.tc && a.mu == b.mu && a.alpha == b.alpha &&
         a.eps == b.eps && a.delta == b.delta && a.gamma == b.gamma &&
         a.beta == b.beta && a.theta == b.theta;
}

static bool same_fk(const yh_fk_params &a, const yh_fk_params &b) {
  return a.tau_d == b.tau_d && a.tau_r == b.tau_r && a.tau_si == b.tau_si &&
         a.tau_0 == b.tau_0 && a.tau_v_plus == b.tau_v_plus &&
         a.tau_v1_minus == b.tau_v1_minus && a.tau_v2_minus == b.tau_v2_minus &&
         a.tau_w_plus == b.tau_w_plus && a.tau_w_minus == b.tau_w_minus &&
         a.u_c == b.u_c && a.u_v == b.u_v && a.u_csi == b.u_csi && a.k == b.k;
}

extern "C" int yh_checkpoint_same_problem(const yh_param_var *a, int model_a,
                                          const yh_fk_params *fk_a,
                                          const yh_param_var *b, int model_b,
                                          const yh_fk_params *fk_b) {
  if (!a || !b) return 0;
  if (model_a != model_b || !same_step(*a, *b)) return 0;
  if (model_a == YH_MODEL_FK3V && (!fk_a || !fk_b || !same_fk(*fk_a, *fk_b)))
    return 0;
  return 1;
}

extern "C" int yh_load_checkpoint(yh_solver *h, const char *path) {
  if (!h || !path) return YH_EINVAL;
  yh_checkpoint_header hd;
  int rc = yh_read_checkpoint_header(path, &hd);
  if (rc) return rc;
  if (hd.nx != h->p.nx || hd.ny != h->p.ny || hd.model != h->model ||
      hd.has_mask != (h->solid ? 1 : 0) || hd.step > 0x7fffffffLL)
    return YH_EINVAL;
  std::vector<float> u(h->n), v(h->n), w(h->nf > 2 ? h->n : 0);
  std::vector<uint8_t> mask(hd.has_mask ? h->n : 0), mine;
  yh_param_var p;
  yh_fk_params fk;
  int model = -1;
  long long step = 0;
  rc = yh_read_checkpoint(path, &p, &model, &fk,
                          hd.has_mask ? mask.data() : nullptr, &step, u.data(),
                          v.data(), h->nf > 2 ? w.data() : nullptr);
  if (rc) return rc;
  if (!same_step(p, h->p) || (h->model == YH_MODEL_FK3V && !same_fk(fk, h->fk)))
    return YH_EINVAL;
  rc = host_mask(h, &mine);
  if (rc) return rc;
  for (size_t k = 0; k < mine.size(); ++k)
    if ((mine[k] != 0) != (mask[k] != 0)) return YH_EINVAL;
  rc = yh_set_state(h, u.data(), v.data(), h->nf > 2 ? w.data() : nullptr);
  if (!rc) rc = st(cudaStreamSynchronize(h->s));
  if (rc) return rc;
  h->step = (int)step;
  return YH_OK;
}
