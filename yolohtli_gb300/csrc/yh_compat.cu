// The reference's seven hot-path host entry points (hostPrototypes.h:22-42)
// with identical C++ signatures, on this library's kernels in FP64
// (include/yolohtli_compat.h states the contract and the differences).
#include <string.h>

#include "../../include/yolohtli_compat.h"
#include "yh_kernels.cuh"

// The reference's ABI types (typeDefinition.cuh:4-20), declared with the same
// names and layouts so that the C++ symbols of the wrappers match its own.
typedef double REAL;
typedef struct REAL3 { REAL x, y, t; } REAL3;
typedef struct stateVar { REAL *u, *v; } stateVar;
typedef struct advVar { REAL *x, *y; } advVar;
typedef struct sliceVar { REAL *ux, *uy, *ut, *vx, *vy, *vt; } sliceVar;
typedef struct vec5dyn { float x, y, vx, vy, t; } vec5dyn;

static_assert(sizeof(vec5dyn) == sizeof(yh_tip), "vec5dyn layout");

namespace {

yh_param_var g_p;
bool g_have_params = false;
int g_err = YH_OK;
constexpr int kTipVecSize = 500000;  // TIPVECSIZE (typeDefinition.cuh:137)

int fail(int e) {
  g_err = e;
  return e;
}

int ready(bool needs_tip_algo = false) {
  g_err = YH_OK;
  if (!g_have_params) return fail(YH_ENOTREADY);
  const yh_param_var &p = g_p;
  if (p.timeIntOrder != 1 || p.lap4 != 0 || p.anisotropy || !p.neumannBC)
    return fail(YH_EUNSUPPORTED);
  if (needs_tip_algo && p.tipAlgorithm != 1) return fail(YH_EUNSUPPORTED);
  return YH_OK;
}

void cuda_check(cudaError_t e) {
  if (e != cudaSuccess) g_err = e == cudaErrorMemoryAllocation ? YH_ENOMEM : YH_ECUDA;
}

// Disc centre as slice_kernel / trapz_kernel take it
// (symmetryReduction.cu:98-104): tipx0/tipy0 at count == 0, else the last
// tip pushed; the initial centre when no tip exists.
__device__ __forceinline__ void compat_centre(int nx, int ny, float tipx0,
                                              float tipy0, int count,
                                              const int *tip_count,
                                              const yh_tip *tips, int &cx,
                                              int &cy) {
  float x = tipx0, y = tipy0;
  if (count != 0) {
    const int n = *tip_count;
    if (n > 0) {
      x = tips[n - 1].x;
      y = tips[n - 1].y;
    }
  }
  cx = __float2int_rn(x - (float)(nx / 2));
  cy = __float2int_rn(y - (float)(ny / 2));
}

struct CompatGeom {
  int nx, ny, r2;
  double hx, hy, invdx, invdy;
  float tipx0, tipy0;
};

CompatGeom geom() {
  CompatGeom g;
  g.nx = g_p.nx;
  g.ny = g_p.ny;
  g.r2 = g_p.tipOffsetX * g_p.tipOffsetY;
  g.hx = g_p.hx;
  g.hy = g_p.hy;
  g.invdx = g_p.invdx;
  g.invdy = g_p.invdy;
  g.tipx0 = g_p.tipx;
  g.tipy0 = g_p.tipy;
  return g;
}

// slice_kernel scheme 2 (symmetryReduction.cu:167-206): the 12 slice arrays.
__global__ void compat_slice_kernel(const CompatGeom g, const double *gu,
                                    const double *gv, sliceVar s,
                                    sliceVar s0, bool take_template,
                                    const double *advx, const double *advy,
                                    const int *tip_count, const yh_tip *tips,
                                    int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = g.nx, ny = g.ny;
  if (i >= nx || j >= ny) return;
  int cx, cy;
  compat_centre(nx, ny, g.tipx0, g.tipy0, count, tip_count, tips, cx, cy);
  const int C = i + nx * j;
  const int ic = i - nx / 2 - cx, jc = j - ny / 2 - cy;
  const bool sc = ic * ic + jc * jc < g.r2;
  const double x = (double)i, y = (double)j;
  const int row = nx * j;
  const int iE = row + yh::mirror(i + 1, nx), iW = row + yh::mirror(i - 1, nx);
  const int iEE = row + yh::mirror(i + 2, nx), iWW = row + yh::mirror(i - 2, nx);
  const int jN = i + nx * yh::mirror(j + 1, ny), jS = i + nx * yh::mirror(j - 1, ny);
  const int jNN = i + nx * yh::mirror(j + 2, ny), jSS = i + nx * yh::mirror(j - 2, ny);
  const double *f[2] = {gu, gv};
  double *cur[2][3] = {{s.ux, s.uy, s.ut}, {s.vx, s.vy, s.vt}};
  double *tm[2][3] = {{s0.ux, s0.uy, s0.ut}, {s0.vx, s0.vy, s0.vt}};
  for (int q = 0; q < 2; ++q) {
    const double *h = f[q];
    const double c = h[C];
    double dx = 0.0, dy = 0.0, dth = 0.0;
    if (sc) {
      dx = advx[C] > 0.0 ? (-3.0 * c + 4.0 * h[iE] - h[iEE]) * g.invdx
                         : (3.0 * c - 4.0 * h[iW] + h[iWW]) * g.invdx;
      dy = advy[C] > 0.0 ? (-3.0 * c + 4.0 * h[jN] - h[jNN]) * g.invdy
                         : (3.0 * c - 4.0 * h[jS] + h[jSS]) * g.invdy;
      dth = g.hx * x * dy - g.hy * y * dx;
    }
    cur[q][0][C] = dx;
    cur[q][1][C] = dy;
    cur[q][2][C] = dth;
    if (take_template) {
      double tx = 0.0, ty = 0.0, tt = 0.0;
      if (sc) {
        tx = (h[iEE] - 8.0 * h[iE] + 8.0 * h[iW] - h[iWW]) * g.invdx * (1.0 / 6.0);
        ty = (h[jNN] - 8.0 * h[jN] + 8.0 * h[jS] - h[jSS]) * g.invdy * (1.0 / 6.0);
        tt = g.hx * x * ty - g.hy * y * tx;
      }
      tm[q][0][C] = tx;
      tm[q][1][C] = ty;
      tm[q][2][C] = tt;
    }
  }
}

// Cxy_field_kernel (symmetryReduction.cu:20-62) as full arrays.
__global__ void compat_cxy_kernel(const CompatGeom g, double *advx,
                                  double *advy, REAL3 c, double cs,
                                  double sn, const uint8_t *solid) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.nx || j >= g.ny) return;
  const int C = i + g.nx * j;
  const double x = (double)i, y = (double)j;
  const bool sc = !solid || solid[C];
  advx[C] = sc ? g.hy * y * c.t - c.x * cs + c.y * sn : 0.0;
  advy[C] = sc ? -g.hx * x * c.t - c.x * sn - c.y * cs : 0.0;
}

// The 12 trapz_wrapper integrals (integralTrapz.cu:97-179) in one launch of
// one block: hx*hy * sum over the disc of f*g + h*w, in a fixed order.
__global__ void __launch_bounds__(256)
    compat_trapz_kernel(const CompatGeom g, sliceVar s, sliceVar s0,
                        stateVar vt, const int *tip_count, const yh_tip *tips,
                        int count, double *out) {
  int cx, cy;
  compat_centre(g.nx, g.ny, g.tipx0, g.tipy0, count, tip_count, tips, cx, cy);
  const double *T[3][2] = {{s0.ux, s0.vx}, {s0.uy, s0.vy}, {s0.ut, s0.vt}};
  const double *Cv[4][2] = {{s.ux, s.vx}, {s.uy, s.vy}, {s.ut, s.vt}, {vt.u, vt.v}};
  double acc[12];
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  const int n = g.nx * g.ny;
  for (int C = threadIdx.x; C < n; C += blockDim.x) {
    const int i = C % g.nx, j = C / g.nx;
    const int ic = i - g.nx / 2 - cx, jc = j - g.ny / 2 - cy;
    if (ic * ic + jc * jc >= g.r2) continue;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 4; ++b)
        acc[b < 3 ? 3 * a + b : 9 + a] +=
            T[a][0][C] * Cv[b][0][C] + T[a][1][C] * Cv[b][1][C];
  }
  __shared__ double red[12][256];
  for (int k = 0; k < 12; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if ((int)threadIdx.x < off)
      for (int k = 0; k < 12; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x < 12) out[threadIdx.x] = g.hx * g.hy * red[threadIdx.x][0];
}

double *g_trapz_out = nullptr;

}  // namespace

extern "C" int yh_compat_set_params(const yh_param_var *p) {
  if (!p) return YH_EINVAL;
  g_p = *p;
  g_have_params = true;
  return YH_OK;
}

extern "C" int yh_compat_last_error(void) { return g_err; }

void reactionDiffusion_wrapper(size_t pitch, dim3 grid2D, dim3 block2D,
                               stateVar gOut_d, stateVar gIn_d, stateVar J,
                               stateVar velTan, bool reduceSym, bool *solid,
                               bool stimLock, REAL *stim, bool stimLockMouse,
                               int2 point) {
  (void)pitch, (void)grid2D, (void)block2D, (void)J, (void)reduceSym;
  (void)stimLock, (void)stim, (void)point;
  if (ready()) return;
  if (stimLockMouse) {  // the mouse stimulus is a UI feature
    fail(YH_EUNSUPPORTED);
    return;
  }
  const yh::StepCoeffs<double> a =
      yh::make_step_coeffs<double>(g_p, YH_MODEL_REF2V, nullptr);
  const yh::Fld<double> in = yh::make_fld<double>(gIn_d.u, gIn_d.v, nullptr);
  const yh::Fld<double> out = yh::make_fld<double>(gOut_d.u, gOut_d.v, nullptr);
  // velTan is written only when gate diffusion is on (reactionDiffusion.cu:519-559)
  const yh::Fld<double> tan = g_p.gateDiff
      ? yh::make_fld<double>(velTan.u, velTan.v, nullptr)
      : yh::make_fld<double>(nullptr, nullptr, nullptr);
  cuda_check(yh::launch_rd_step<double>(
      a, in, out, tan,
      g_p.solidSwitch ? reinterpret_cast<const uint8_t *>(solid) : nullptr, 0));
}

void tip_wrapper(size_t pitch, dim3 grid2D, dim3 block2D, stateVar gOut_d,
                 stateVar gIn_d, stateVar velTan, REAL physicalTime,
                 int tipAlgorithm, bool recordTip, bool *tip_plot,
                 int *tip_count, vec5dyn *tip_vector) {
  (void)pitch, (void)grid2D, (void)block2D, (void)velTan, (void)recordTip;
  if (ready()) return;
  if (tipAlgorithm < 1 || tipAlgorithm > 3) {
    fail(YH_EUNSUPPORTED);
    return;
  }
  cuda_check(cudaMemsetAsync(tip_count, 0, sizeof(int), 0));
  uint8_t *plot = reinterpret_cast<uint8_t *>(tip_plot);
  if (tipAlgorithm == 3) {  // abouzarTip_kernel (tipTracker.cu:601-604)
    cuda_check(yh::launch_filament<double>(g_p, gIn_d.u, gOut_d.u, plot, 0));
    return;
  }
  // spiralTip_kernel / spiralTipNewton_kernel (g_past = gIn_d.u, g_present =
  // gOut_d.u) (tipTracker.cu:586-599)
  yh_param_var q = g_p;
  q.tipAlgorithm = tipAlgorithm;
  cuda_check(yh::launch_tips<double>(
      q, gIn_d.u, gOut_d.u, g_p.solidSwitch, physicalTime, tip_count,
      reinterpret_cast<yh_tip *>(tip_vector), kTipVecSize, nullptr, nullptr, 0,
      plot));
}

// countour_wrapper (spaceAPD.cu:257-276): count and plot reset, then
// countour_kernel; the reference's contour_vector holds nx*ny points.
void countour_wrapper(size_t pitch, dim3 grid2D, dim3 block2D, REAL *field1,
                      REAL *field2, bool *contour_plot, bool *stimArea,
                      int *contour_count, float3 *contour_vector,
                      float physicalTime, int mode) {
  (void)pitch, (void)grid2D, (void)block2D;
  if (ready()) return;
  if (mode < 1 || mode > 3) {
    fail(YH_EINVAL);
    return;
  }
  static_assert(sizeof(float3) == sizeof(yh_contour_pt), "float3 layout");
  cuda_check(cudaMemsetAsync(contour_count, 0, sizeof(int), 0));
  cuda_check(cudaMemsetAsync(contour_plot, 0, (size_t)g_p.nx * g_p.ny, 0));
  cuda_check(yh::launch_contour<double>(
      g_p, field1, field2, reinterpret_cast<const uint8_t *>(stimArea), mode,
      physicalTime, contour_count,
      reinterpret_cast<yh_contour_pt *>(contour_vector), g_p.nx * g_p.ny,
      reinterpret_cast<uint8_t *>(contour_plot), 0));
}

// sAPD_wrapper (spaceAPD.cu:376-383)
void sAPD_wrapper(size_t pitch, dim3 grid1D, dim3 block1D, int count,
                  REAL *uold, REAL *unew, REAL *APD1, REAL *APD2, REAL *sAPD,
                  REAL *dAPD, REAL *back, REAL *front, bool *first,
                  bool *stimArea, bool stimulate) {
  (void)pitch, (void)grid1D, (void)block1D;
  if (ready()) return;
  yh::ApdFields<double> f{APD1, APD2, sAPD, dAPD, back, front,
                          reinterpret_cast<uint8_t *>(first)};
  cuda_check(yh::launch_space_apd<double>(
      g_p, count, uold, unew, f, reinterpret_cast<const uint8_t *>(stimArea),
      stimulate, 0));
}

void slice_wrapper(size_t pitch, dim3 grid2D, dim3 block2D, stateVar g,
                   sliceVar slice, sliceVar slice0, bool reduceSym,
                   bool reduceSymStart, advVar adv, int scheme,
                   bool *intglArea, int *tip_count, vec5dyn *tip_vector,
                   int count) {
  (void)pitch, (void)grid2D, (void)block2D, (void)intglArea;
  if (ready()) return;
  if (scheme != 2) {
    fail(YH_EUNSUPPORTED);
    return;
  }
  if (!reduceSym) return;
  const dim3 block(32, 8);
  const dim3 grid((g_p.nx + 31) / 32, (g_p.ny + 7) / 8);
  compat_slice_kernel<<<grid, block>>>(
      geom(), g.u, g.v, slice, slice0, reduceSymStart, adv.x, adv.y, tip_count,
      reinterpret_cast<const yh_tip *>(tip_vector), count);
  cuda_check(cudaGetLastError());
}

void Cxy_field_wrapper(size_t pitch, dim3 grid2D, dim3 block2D, advVar adv,
                       REAL3 c, REAL3 phi, bool *solid) {
  (void)pitch, (void)grid2D, (void)block2D;
  if (ready()) return;
  const dim3 block(32, 8);
  const dim3 grid((g_p.nx + 31) / 32, (g_p.ny + 7) / 8);
  compat_cxy_kernel<<<grid, block>>>(
      geom(), adv.x, adv.y, c, cos(phi.t), sin(phi.t),
      g_p.solidSwitch ? reinterpret_cast<const uint8_t *>(solid) : nullptr);
  cuda_check(cudaGetLastError());
}

void advFDBFECC_wrapper(size_t pitch, dim3 grid2D, dim3 block2D,
                        stateVar gOut, stateVar gIn, advVar adv, stateVar uf,
                        stateVar ub, stateVar ue, bool *solid) {
  (void)pitch, (void)grid2D, (void)block2D, (void)ub;
  if (ready()) return;
  cuda_check(yh::launch_bfecc_2d<double>(
      g_p, 2, yh::make_fld<double>(gIn.u, gIn.v, nullptr),
      yh::make_fld<double>(gOut.u, gOut.v, nullptr), adv.x, adv.y,
      g_p.solidSwitch ? reinterpret_cast<const uint8_t *>(solid) : nullptr,
      yh::make_fld<double>(uf.u, uf.v, nullptr),
      yh::make_fld<double>(ue.u, ue.v, nullptr), 0));
}

REAL3 solve_matrix(REAL3 c, REAL3 phi, REAL *Int) {
  g_err = YH_OK;
  double out[3];
  const int st = yh::solve3(Int, phi.t, out);
  if (st != YH_OK) {
    fail(st);
    return c;  // unchanged on a singular system
  }
  REAL3 r;
  r.x = out[0];
  r.y = out[1];
  r.t = out[2];
  return r;
}

void trapz_wrapper(dim3 grid1D, dim3 block1D, sliceVar slice, sliceVar slice0,
                   stateVar velTan, REAL *integrals, REAL *coeffTrapz,
                   int *tip_count, vec5dyn *tip_vector, int count) {
  (void)grid1D, (void)block1D, (void)coeffTrapz;  // coeffTrapz is unused there too
  if (ready()) return;
  if (!g_trapz_out) {
    cudaError_t e = cudaMalloc(&g_trapz_out, 12 * sizeof(double));
    if (e != cudaSuccess) {
      g_trapz_out = nullptr;
      cuda_check(e);
      return;
    }
  }
  compat_trapz_kernel<<<1, 256>>>(geom(), slice, slice0, velTan, tip_count,
                                   reinterpret_cast<const yh_tip *>(tip_vector),
                                   count, g_trapz_out);
  cuda_check(cudaGetLastError());
  // one blocking copy of the 12 results (the reference makes 12)
  cuda_check(cudaMemcpy(integrals, g_trapz_out, 12 * sizeof(double),
                        cudaMemcpyDeviceToHost));
}
