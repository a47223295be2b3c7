// Analysis kernels beside the hot path's tip tracker:
//   filament_kernel   tipAlgorithm 3: cells whose 2x2 corners straddle both
//                     u = Uth and u_present = u_past (abouzarTip_kernel and
//                     abubuFilament, tipTracker.cu:434-517)
//   contour_kernel    isolines of a field (countour_kernel,
//                     spaceAPD.cu:18-153, modes 1-3)
//   space_apd_kernel  per-cell action potential duration of two successive
//                     beats and the sign of their difference (sAPD_kernel,
//                     spaceAPD.cu:278-374)
// Element-wise and HBM-bound; FP64 arithmetic where the reference has it
// (its REAL), on FP32 or FP64 fields.
#include "yh_kernels.cuh"

namespace yh {

namespace {

// ---------------------------------------------------------------------------
// tipAlgorithm 3
// ---------------------------------------------------------------------------

template <typename Real>
__global__ void filament_kernel(int nx, int ny, double Uth,
                                const Real *__restrict__ past,
                                const Real *__restrict__ present,
                                uint8_t *mark) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const int s0 = i + nx * j;
  const int sx = (i < nx - 1) ? s0 + 1 : s0;
  const int sy = (j < ny - 1) ? s0 + nx : s0;
  const int sxy = ((j < ny - 1) && (i < nx - 1)) ? s0 + nx + 1 : s0;
  const double v[4] = {(double)present[s0], (double)present[sx],
                       (double)present[sy], (double)present[sxy]};
  const double w[4] = {(double)past[s0], (double)past[sx], (double)past[sy],
                       (double)past[sxy]};
  // how many corners lie at or below u = Uth, and at or below the previous
  // level: the cell is marked when both counts are mixed (1 to 3 of 4)
  int below = 0, falling = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    below += (0.0 >= v[k] - Uth) ? 1 : 0;
    falling += (0.0 >= v[k] - w[k]) ? 1 : 0;
  }
  if (below >= 1 && below <= 3 && falling >= 1 && falling <= 3) mark[s0] = 1;
}

// ---------------------------------------------------------------------------
// Contours
// ---------------------------------------------------------------------------

struct ContourArgs {
  int nx, ny;
  double th1, th2, th3;  // contourThresh1..3
};

__device__ __forceinline__ void push_contour(int nx, int ny, float x, float y,
                                             float t, int *count,
                                             yh_contour_pt *vec, int cap,
                                             uint8_t *plot) {
  const int slot = atomicAdd(count, 1);
  if (slot < cap) {
    yh_contour_pt q;
    q.x = x;
    q.y = y;
    q.t = t;
    vec[slot] = q;
  }
  if (plot) {
    // plot_field's linear index (helper_functions.cu:45-51): a point past
    // the last column marks the next row as the reference does; a mark
    // outside the array, which the reference writes anyway, is dropped
    const long long k = (long long)floorf(x) + (long long)nx * (long long)floorf(y);
    if (k >= 0 && k < (long long)nx * ny) plot[k] = 1;
  }
}

// Sign changes of f2 (minus a threshold) towards the east and north
// neighbours. The reference reads the east value at i + 1 even in the last
// column (the first cell of the next row) and the north value past the end
// of the array in the last row; here a value past the end is taken as the
// cell's own (a product v0*v0 >= 0 the reference takes there anyway).
template <typename Real>
__global__ void contour_kernel(const ContourArgs a, const Real *__restrict__ f1,
                               const Real *__restrict__ f2,
                               const uint8_t *__restrict__ stim_area, int mode,
                               float time, int *count, yh_contour_pt *vec,
                               int cap, uint8_t *plot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  if (i >= nx || j >= ny) return;
  const long long n = (long long)nx * ny;
  const long long c = i + (long long)nx * j;
  const bool sc = stim_area[c] != 0;
  const double f0 = f2[c];
  const double fx = c + 1 < n ? (double)f2[c + 1] : f0;
  const double fy = c + nx < n ? (double)f2[c + nx] : f0;
  const bool xin = i < nx - 1, yin = j < ny - 1;
  if (mode == 1) {  // space APD contour: the zero level of f2
    const double zx = xin ? f0 * fx : f0 * f0;
    const double zy = yin ? f0 * fy : f0 * f0;
    if ((zx < 0.0) || ((zy < 0.0) && sc)) {  // the reference's precedence
      const double eps = 2.220446049250313e-16;  // MACHINE_EPS
      const double px = fabs(f0 - fx) > eps ? i + f0 / (f0 - fx) : (double)i;
      const double py = fabs(f0 - fy) > eps ? j + f0 / (f0 - fy) : (double)j;
      push_contour(nx, ny, (float)px, (float)py, time, count, vec, cap, plot);
    }
  } else if (mode == 2) {  // f2 = th2 where f1 < th1
    if (((double)f1[c] < a.th1) && sc) {
      const double v0 = f0 - a.th2, vx = fx - a.th2, vy = fy - a.th2;
      const double zx = xin ? v0 * vx : v0 * v0;
      const double zy = yin ? v0 * vy : v0 * v0;
      if ((zx < 0.0) || (zy < 0.0))
        push_contour(nx, ny, (float)i, (float)j, time, count, vec, cap, plot);
    }
  } else if (mode == 3) {  // f2 = 2 th2 and f2 = th2 - th3 near th2
    const double V0 = f0 - a.th2, Vx = fx - a.th2, Vy = fy - a.th2;
    const double band = a.th3 + 0.1;
    if (((double)f1[c] < a.th1) && (fabs(V0) < band) && (fabs(Vx) < band) &&
        (fabs(Vy) < band) && sc) {
      const double shift[2] = {-a.th2, a.th3};
      for (int k = 0; k < 2; ++k) {
        const double v0 = V0 + shift[k], vx = Vx + shift[k], vy = Vy + shift[k];
        const double zx = xin ? v0 * vx : v0 * v0;
        const double zy = yin ? v0 * vy : v0 * v0;
        if ((zx < 0.0) || (zy < 0.0))
          push_contour(nx, ny, (float)i, (float)j, time, count, vec, cap, plot);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Space APD
// ---------------------------------------------------------------------------

// Per cell: the times (dt * count, interpolated within the step) of the
// upstroke and downstroke through 0.15, two successive APDs and
// sign(APD1 - APD2); `stimulate` restricts it to the stimulus area and
// writes dAPD = APD2 (sAPD_kernel, spaceAPD.cu:278-374).
template <typename Real>
__global__ void space_apd_kernel(long long n, double dt, int count,
                                 const Real *__restrict__ uold,
                                 const Real *__restrict__ unew,
                                 ApdFields<Real> f,
                                 const uint8_t *__restrict__ stim_area,
                                 bool stimulate) {
  const double th = 0.15;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const double uo = uold[k], un = unew[k];
    const bool sc = !stimulate || stim_area[k] != 0;
    double front = f.front[k], back = f.back[k];
    bool first = f.first[k] != 0;
    if ((un > th) && (uo < th) && sc)
      front = dt * (count - (un - th) / (un - uo));
    if ((un < th) && (uo > th) && sc)
      back = dt * (count - (un - th) / (un - uo));
    double apd1 = f.apd1[k], apd2 = f.apd2[k];
    if ((back > 0.0) && (front > 0.0) && !first && sc) {
      apd1 = back - front;
      front = back = 0.0;
      first = true;
    }
    if ((back > 0.0) && (front > 0.0) && first && sc) {
      apd2 = back - front;
      front = back = 0.0;
      first = false;
    }
    f.front[k] = (Real)front;
    f.back[k] = (Real)back;
    f.first[k] = first ? 1 : 0;
    f.apd1[k] = (Real)apd1;
    f.apd2[k] = (Real)apd2;
    if (stimulate) {
      const double scv = stim_area[k] != 0 ? 1.0 : 0.0;
      f.sapd[k] = (Real)(((apd1 - apd2 > 0.0) && sc ? 1.0 : -1.0) * scv);
      f.dapd[k] = (Real)(apd2 * scv);
    } else {
      f.sapd[k] = (Real)((apd1 - apd2 > 0.0) ? 1.0 : -1.0);
    }
  }
}

}  // namespace

template <typename Real>
cudaError_t launch_filament(const yh_param_var &p, const Real *past,
                            const Real *present, uint8_t *mark,
                            cudaStream_t s) {
  const dim3 block(32, 8), grid((p.nx + 31) / 32, (p.ny + 7) / 8);
  filament_kernel<Real><<<grid, block, 0, s>>>(p.nx, p.ny, p.Uth, past, present,
                                               mark);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_contour(const yh_param_var &p, const Real *field1,
                           const Real *field2, const uint8_t *stim_area,
                           int mode, float time, int *count,
                           yh_contour_pt *vec, int cap, uint8_t *plot,
                           cudaStream_t s) {
  if (mode < 1 || mode > 3) return cudaErrorInvalidValue;
  ContourArgs a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.th1 = p.contourThresh1;
  a.th2 = p.contourThresh2;
  a.th3 = p.contourThresh3;
  const dim3 block(32, 8), grid((p.nx + 31) / 32, (p.ny + 7) / 8);
  contour_kernel<Real><<<grid, block, 0, s>>>(a, field1, field2, stim_area,
                                              mode, time, count, vec, cap,
                                              plot);
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch_space_apd(const yh_param_var &p, int count,
                             const Real *uold, const Real *unew,
                             const ApdFields<Real> &f,
                             const uint8_t *stim_area, bool stimulate,
                             cudaStream_t s) {
  const long long n = (long long)p.nx * p.ny;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  space_apd_kernel<Real><<<blocks, 256, 0, s>>>(n, p.dt, count, uold, unew, f,
                                                stim_area, stimulate);
  return cudaGetLastError();
}

#define YH_ANALYSIS_INST(Real)                                                 \
  template cudaError_t launch_filament<Real>(const yh_param_var &,             \
                                             const Real *, const Real *,       \
                                             uint8_t *, cudaStream_t);         \
  template cudaError_t launch_contour<Real>(                                   \
      const yh_param_var &, const Real *, const Real *, const uint8_t *, int,  \
      float, int *, yh_contour_pt *, int, uint8_t *, cudaStream_t);            \
  template cudaError_t launch_space_apd<Real>(                                 \
      const yh_param_var &, int, const Real *, const Real *,                   \
      const ApdFields<Real> &, const uint8_t *, bool, cudaStream_t);
YH_ANALYSIS_INST(float)
YH_ANALYSIS_INST(double)
#undef YH_ANALYSIS_INST

}  // namespace yh

using namespace yh;

namespace {
int status(cudaError_t e) {
  if (e == cudaSuccess) return YH_OK;
  if (e == cudaErrorMemoryAllocation) return YH_ENOMEM;
  if (e == cudaErrorInvalidValue) return YH_EINVAL;
  return YH_ECUDA;
}
}  // namespace

extern "C" int yh_filament_mark(const yh_param_var *p, const float *past,
                                const float *present, uint8_t *mark,
                                void *stream) {
  if (!p || !past || !present || !mark || p->nx < 2 || p->ny < 2)
    return YH_EINVAL;
  return status(launch_filament<float>(*p, past, present, mark,
                                       (cudaStream_t)stream));
}

extern "C" int yh_contour(const yh_param_var *p, const float *field1,
                          const float *field2, const uint8_t *stim_area,
                          int mode, float time, int *count,
                          yh_contour_pt *vec, int capacity, uint8_t *plot,
                          void *stream) {
  if (!p || !field2 || !stim_area || !count || !vec || capacity < 0 ||
      p->nx < 2 || p->ny < 2 || mode < 1 || mode > 3 ||
      (mode > 1 && !field1))
    return YH_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), s);
  if (e == cudaSuccess && plot)
    e = cudaMemsetAsync(plot, 0, (size_t)p->nx * p->ny, s);
  if (e == cudaSuccess)
    e = launch_contour<float>(*p, field1 ? field1 : field2, field2, stim_area,
                              mode, time, count, vec, capacity, plot, s);
  return status(e);
}

extern "C" int yh_space_apd(const yh_param_var *p, int count,
                            const float *uold, const float *unew,
                            yh_apd_fields f, const uint8_t *stim_area,
                            int stimulate, void *stream) {
  if (!p || !uold || !unew || !f.apd1 || !f.apd2 || !f.sapd || !f.back ||
      !f.front || !f.first || (stimulate && (!stim_area || !f.dapd)))
    return YH_EINVAL;
  ApdFields<float> a{f.apd1, f.apd2, f.sapd, f.dapd, f.back, f.front, f.first};
  return status(launch_space_apd<float>(*p, count, uold, unew, a, stim_area,
                                        stimulate != 0, (cudaStream_t)stream));
}
