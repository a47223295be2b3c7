// yh_phase_integrals_noalloc: the fused phase-integral operator without a
// caller-provided workspace, for callers that cannot allocate device memory.
//
// Its scratch (the per-block FP64 partial sums and the completion counter
// of the deterministic two-level reduction) is the file-scope array below:
// a fixed 384 KiB + 256 B that every GPU loading this library holds until
// the process exits. The host cannot hand the array's name to a kernel (in
// host code it is a host-side stand-in, not a device address), so the first
// call on each device looks up the array's device address with
// cudaGetSymbolAddress while that device is current, and keeps it.
#include <mutex>

#include "yh_kernels.cuh"

namespace {

constexpr int kNoAllocMaxBlocks = 4096;  // 12 8-byte partial sums per block
constexpr size_t kNoAllocBytes = 256 + (size_t)kNoAllocMaxBlocks * 12 * sizeof(double);
constexpr int kMaxDevices = 64;

// counter in the first 256 bytes, then the block partials
static __device__ __align__(256) unsigned char g_phase_scratch[kNoAllocBytes];

std::mutex g_mu;
void *g_addr[kMaxDevices] = {};

// Device address of g_phase_scratch on the current device (looked up once
// per device).
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return YH_ECUDA;
  if (dev < 0 || dev >= kMaxDevices) return YH_EINVAL;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_phase_scratch);
    if (e != cudaSuccess || !p) return YH_ECUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return YH_OK;
}

}  // namespace

extern "C" size_t yh_phase_integrals_noalloc_limit(void) { return kNoAllocBytes; }

extern "C" int yh_phase_integrals_noalloc(
    const yh_param_var *p, int model, yh_fields state, yh_fields vel_tan,
    yh_fields templ_x, yh_fields templ_y, yh_fields templ_t,
    const double *adv_x_rows, const double *adv_y_cols, const uint8_t *solid,
    yh_sym_state *sym, void *stream) {
  if (!p || !sym || !adv_x_rows || !adv_y_cols) return YH_EINVAL;
  if (p->nx < 5 || p->ny < 5) return YH_EINVAL;
  const int nf = model == YH_MODEL_FK3V ? 3 : 2;
  if (model != YH_MODEL_REF2V && model != YH_MODEL_FK3V) return YH_EINVAL;
  if (!state.u || !state.v || (nf > 2 && !state.w) || !vel_tan.u ||
      !vel_tan.v || (nf > 2 && !vel_tan.w))
    return YH_EINVAL;
  if (templ_x.u && (!templ_x.v || !templ_y.u || !templ_y.v || !templ_t.u ||
                    !templ_t.v || (nf > 2 && (!templ_x.w || !templ_y.w ||
                                              !templ_t.w))))
    return YH_EINVAL;
  if (p->solidSwitch && !solid) return YH_EINVAL;
  // this disc needs more block partials than the fixed scratch holds
  if (yh::phase_workspace_bytes(*p) > kNoAllocBytes) return YH_EINVAL;
  void *ws = nullptr;
  int rc = scratch_address(&ws);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the completion counter must start at zero; the partials are rewritten
  cudaError_t e = cudaMemsetAsync(ws, 0, 256, s);
  if (e != cudaSuccess) return YH_ECUDA;
  e = yh::launch_phase<float>(
      *p, nf, yh::make_fld<float>(state.u, state.v, state.w),
      yh::make_fld<float>(vel_tan.u, vel_tan.v, vel_tan.w),
      yh::make_fld<float>(templ_x.u, templ_x.v, templ_x.w),
      yh::make_fld<float>(templ_y.u, templ_y.v, templ_y.w),
      yh::make_fld<float>(templ_t.u, templ_t.v, templ_t.w), adv_x_rows,
      adv_y_cols, p->solidSwitch ? solid : nullptr, sym, ws, s);
  return e == cudaSuccess ? YH_OK : YH_ECUDA;
}
