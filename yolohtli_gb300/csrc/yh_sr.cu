// Symmetry-reduction kernels of the monodomain hot path:
//   tip_kernel     spiral tips, closed-form bilinear isoline intersection
//                  (spiralTip_kernel, tipTracker.cu:20-241) + the disc-centre
//                  choice in the last block;
//   phase_kernel   slices (symmetryReduction.cu:72-262) fused with the 12
//                  phase integrals (integralTrapz.cu:17-184) and the FP64
//                  3x3 solve (symmetryReduction.cu:329-420) in the last
//                  block: one launch instead of 2 + 12 launches, 12 blocking
//                  copies and a host solve; in the symmetry-reduced step
//                  the last block also writes the comoving field;
//   comoving_kernel the comoving field (Cxy_field_kernel,
//                  symmetryReduction.cu:20-62), which is separable: adv.x
//                  depends on the row, adv.y on the column, so it is two
//                  vectors of ny and nx values, not two full grids;
//   bfecc_pass1/2/3 BFECC advection (advFDBFECC.cu:18-353) as three passes,
//                  so no thread reads a neighbour written in the same launch.
//
// Reductions are deterministic: per-thread accumulators (float-float pairs
// for FP32 fields, doubles for FP64 fields), warp shuffles, per-block
// partials, a fixed-order sum by the last block to finish, FP64 from the
// 12 block-summed integrals on. The tip, phase and BFECC kernels are
// launched with programmatic stream serialization.
#include "yh_kernels.cuh"

namespace yh {

// ---------------------------------------------------------------------------
// Tips
// ---------------------------------------------------------------------------

struct TipArgs {
  int nx, ny, r2;
  int tox, toy;  // tipOffsetX/Y: the Newton search window
  double Uth;
  double invdx, invdy;  // 1/(2 hx), 1/(2 hy): the tip gradient
  double dt;     // with sym: time = dt * sym->step (graph-stable)
  double ptime;  // without sym: the time stamp of the tips
};

// Index (i, j) clamped into the grid: the gradient stencil below reaches
// i-1 at i = 0 and j+2 near the top, where the reference reads outside its
// arrays; inside the grid the indices are the reference's.
__device__ __forceinline__ int gidx(int nx, int ny, int i, int j) {
  i = i < 0 ? 0 : (i >= nx ? nx - 1 : i);
  j = j < 0 ? 0 : (j >= ny ? ny - 1 : j);
  return i + nx * j;
}

// Gradient of g at the tip (i + s, j + t): central differences at the four
// corners of the cell, blended bilinearly, with the reference's choice of
// stencil at the grid edges (gradient, tipTracker.cu:519-566).
template <typename Real>
__device__ float2 tip_gradient(const TipArgs &a, int i, int j, double s,
                               double t, const Real *__restrict__ g) {
  const int nx = a.nx, ny = a.ny;
  auto at = [&](int x, int y) { return (double)g[gidx(nx, ny, x, y)]; };
  const bool xl = i < nx - 1, xl2 = i < nx - 2, yl = j < ny - 1, yl2 = j < ny - 2;
  const double S = j > 0 ? at(i, j - 1) : at(i, j + 1);
  const double Sx = (j > 0 && xl) ? at(i + 1, j - 1) : at(i - 1, j + 1);
  const double Sy = at(i, j);
  const double Sxy = xl ? at(i + 1, j) : at(i - 1, j);
  const double N = yl ? at(i, j + 1) : at(i, j - 1);
  const double Nx = (xl && yl) ? at(i + 1, j + 1) : at(i - 1, j - 1);
  const double Ny = yl2 ? at(i, j + 2) : (j == ny - 2 ? at(i, j) : at(i, j - 1));
  const double Nxy = (xl && yl2) ? at(i + 1, j + 2)
                                 : (j == ny - 2 ? at(i - 1, j) : at(i - 1, j - 1));
  const double W = at(i - 1, j);
  const double Wx = at(i, j);
  const double Wy = (i > 0 && yl) ? at(i - 1, j + 1) : at(i + 1, j - 1);
  const double Wxy = yl ? at(i, j + 1) : at(i - 1, j);
  const double E = xl ? at(i + 1, j) : at(i - 1, j);
  const double Ex = xl2 ? at(i + 2, j) : (i == nx - 2 ? at(i, j) : at(i - 1, j));
  const double Ey = (xl && yl) ? at(i + 1, j + 1) : at(i - 1, j - 1);
  const double Exy = (xl2 && yl) ? at(i + 2, j + 1)
                                 : (i == nx - 2 ? at(i, j - 1) : at(i - 1, j - 1));
  const double gx1 = (E - W) * a.invdx, gy1 = (N - S) * a.invdy;
  const double gx2 = (Ex - Wx) * a.invdx, gy2 = (Nx - Sx) * a.invdy;
  const double gx3 = (Ey - Wy) * a.invdx, gy3 = (Ny - Sy) * a.invdy;
  const double gx4 = (Exy - Wxy) * a.invdx, gy4 = (Nxy - Sxy) * a.invdy;
  float2 r;
  r.x = (float)((1.0 - s) * (1.0 - t) * gx1 + s * (1.0 - t) * gx2 +
                t * (1.0 - s) * gx3 + s * t * gx4);
  r.y = (float)((1.0 - s) * (1.0 - t) * gy1 + s * (1.0 - t) * gy2 +
                t * (1.0 - s) * gy3 + s * t * gy4);
  return r;
}

// tipRecordPlane (tipTracker.cu:210-241): a tip strictly inside the cell is
// pushed (with the gradient of the present field when GRAD) and, with a
// plot array, its cell marked.
template <bool GRAD, typename Real>
__device__ __forceinline__ void tip_record(const TipArgs &a, int i, int j,
                                           float s, float t, float ptime,
                                           const Real *present, int *count,
                                           yh_tip *vec, int cap,
                                           uint8_t *plot) {
  if ((s > 0.0f && s < 1.0f) && (t > 0.0f && t < 1.0f)) {
    float2 g = make_float2(0.0f, 0.0f);
    if (GRAD) g = tip_gradient(a, i, j, (double)s, (double)t, present);
    yh_tip d;
    d.x = (float)i + s;
    d.y = (float)j + t;
    d.vx = g.x;
    d.vy = g.y;
    d.t = ptime;
    const int slot = atomicAdd(count, 1);
    if (slot < cap) vec[slot] = d;
    if (plot) {  // plot_field's linear index, marks outside the array dropped
      const long long k = (long long)floorf(d.x) + (long long)a.nx * (long long)floorf(d.y);
      if (k >= 0 && k < (long long)a.nx * a.ny) plot[k] = 1;
    }
  }
}

// Candidate tips of one cell; x = present corners, y = past corners in the
// order (i,j), (i+1,j), (i+1,j+1), (i,j+1) (tipTracker.cu:140-174), in FP64.
template <bool GRAD, typename Real>
__device__ __forceinline__ void tip_cell(const TipArgs &a, int i, int j,
                                         double x1, double x2, double x3,
                                         double x4, double y1, double y2,
                                         double y3, double y4, bool need_disc,
                                         float ptime, const Real *present,
                                         int *count, yh_tip *vec, int cap,
                                         uint8_t *plot) {
  const double Uth = a.Uth;
  const double x3y1 = x3 * y1, x4y1 = x4 * y1, x3y2 = x3 * y2, x4y2 = x4 * y2;
  const double x1y3 = x1 * y3, x2y3 = x2 * y3, x1y4 = x1 * y4, x2y4 = x2 * y4;
  const double x2y1 = x2 * y1, x1y2 = x1 * y2, x4y3 = x4 * y3, x3y4 = x3 * y4;
  const double den1 =
      2.0 * (x3y1 - x4y1 - x3y2 + x4y2 - x1y3 + x2y3 + x1y4 - x2y4);
  const double den2 =
      2.0 * (x2y1 - x3y1 - x1y2 + x4y2 + x1y3 - x4y3 - x2y4 + x3y4);
  const double ctn1 = x1 - x2 + x3 - x4 - y1 + y2 - y3 + y4;
  const double ctn2 = x3y1 - 2.0 * x4y1 + x4y2 - x1y3 + 2.0 * x1y4 - x2y4;
  const double disc =
      sqrt(4.0 * (x3y1 - x3y2 - x4y1 + x4y2 - x1y3 + x1y4 + x2y3 - x2y4) *
               (x4y1 - x1y4 + Uth * (x1 - x4 - y1 + y4)) +
           (-ctn2 + Uth * ctn1) * (-ctn2 + Uth * ctn1));
  const double px = ctn2 - Uth * ctn1;
  const double py =
      Uth * ctn1 - x3y1 + x4y2 + x1y3 - x2y4 + 2.0 * (x2y1 - x1y2);
  if (need_disc && !(disc >= 0.0)) return;
  tip_record<GRAD>(a, i, j, (float)((px + disc) / den1),
                   (float)((py + disc) / den2), ptime, present, count, vec,
                   cap, plot);
  tip_record<GRAD>(a, i, j, (float)((px - disc) / den1),
                   (float)((py - disc) / den2), ptime, present, count, vec,
                   cap, plot);
}

// tip_cell for FP32 levels, in fewer FP64 operations: the expanded sums
// factor into products of corner differences, which are exact in FP64
// for FP32 corners,
//   den1/2 = (x3-x4)(y1-y2) - (x1-x2)(y3-y4)   (also the factor under the root)
//   den2/2 = (x2-x3)(y1-y4) + (x4-x1)(y2-y3),
// so the quantities are at least as accurate as the expanded form's; the
// four root divisions run in FP32 on the rounded numerators and
// denominators (the roots kept lie in (0, 1): ~1e-7 of a cell). GB300's
// narrow FP64 pipe makes this chain the tip launch's critical path.
template <bool GRAD, typename Real>
__device__ __forceinline__ void tip_cell_f32div(
    const TipArgs &a, int i, int j, double x1, double x2, double x3, double x4,
    double y1, double y2, double y3, double y4, bool need_disc, float ptime,
    const Real *present, int *count, yh_tip *vec, int cap, uint8_t *plot) {
  const double Uth = a.Uth;
  const double d12 = x1 - x2, d34 = x3 - x4, e12 = y1 - y2, e34 = y3 - y4;
  const double A = d34 * e12 - d12 * e34;  // den1 / 2
  const double den2h = (x2 - x3) * (y1 - y4) + (x4 - x1) * (y2 - y3);
  const double ctn1 = (d12 + d34) - (e12 + e34);
  const double ctn2 =
      y1 * (x3 - 2.0 * x4) + x4 * y2 - x1 * y3 + y4 * (2.0 * x1 - x2);
  const double B = x4 * y1 - x1 * y4 + Uth * (x1 - x4 - y1 + y4);
  const double px = ctn2 - Uth * ctn1;
  const double disc = sqrt(4.0 * A * B + px * px);
  const double py = Uth * ctn1 + y1 * (2.0 * x2 - x3) + y2 * (x4 - 2.0 * x1) +
                    x1 * y3 - x2 * y4;
  if (need_disc && !(disc >= 0.0)) return;
  const float d1 = (float)(2.0 * A), d2 = (float)(2.0 * den2h);
  tip_record<GRAD>(a, i, j, __fdiv_rn((float)(px + disc), d1),
                   __fdiv_rn((float)(py + disc), d2), ptime, present, count,
                   vec, cap, plot);
  tip_record<GRAD>(a, i, j, __fdiv_rn((float)(px - disc), d1),
                   __fdiv_rn((float)(py - disc), d2), ptime, present, count,
                   vec, cap, plot);
}

__device__ __forceinline__ bool near(double x, double y, double tol) {
  return x == y || (x <= y + tol && x >= y - tol);  // equals (helper_functions.cu:58-62)
}

// Newton's method for the crossing of the two bilinear isolines x = Uth and
// y = Uth in one cell (spiralTipNewton_kernel, tipTracker.cu:287-333): four
// iterations from the cell centre, clamped to the cell, accepted when both
// interpolants hit Uth to 1e-15; the reference's expressions in FP64.
template <bool GRAD, typename Real>
__device__ __forceinline__ void tip_cell_newton(
    const TipArgs &a, int i, int j, double px1, double px2, double px3,
    double px4, double py1, double py2, double py3, double py4, float ptime,
    const Real *present, int *count, yh_tip *vec, int cap, uint8_t *plot) {
  const double Uth = a.Uth;
  double s = 0.5, t = 0.5;
  for (int k = 0; k < 4; ++k) {
    const double r1 = px1 * (1.0 - s) * (1.0 - t) + px2 * s * (1.0 - t) +
                      px3 * s * t + px4 * (1.0 - s) * t - Uth;
    const double r2 = py1 * (1.0 - s) * (1.0 - t) + py2 * s * (1.0 - t) +
                      py3 * s * t + py4 * (1.0 - s) * t - Uth;
    const double J11 = -px1 * (1.0 - t) + px2 * (1.0 - t) + px3 * t - px4 * t;
    const double J21 = -py1 * (1.0 - t) + py2 * (1.0 - t) + py3 * t - py4 * t;
    const double J12 = -px1 * (1.0 - s) - px2 * s + px3 * s + px4 * (1.0 - s);
    const double J22 = -py1 * (1.0 - s) - py2 * s + py3 * s + py4 * (1.0 - s);
    const double detJ = J11 * J22 - J12 * J21;
    if (!near(detJ, 0.0, 1e-14)) {
      s -= (J22 * r1 - J12 * r2) / detJ;
      t -= (-J21 * r1 + J11 * r2) / detJ;
      s = fmin(fmax(s, 0.0), 1.0);
      t = fmin(fmax(t, 0.0), 1.0);
    } else {
      s = -1.0;
      t = -1.0;
    }
  }
  const bool in = (s >= 0.0) && (s <= 1.0) && (t >= 0.0) && (t <= 1.0);
  const double u1 = in ? px1 * (1 - s) * (1.0 - t) + px2 * s * (1.0 - t) +
                             px3 * s * t + px4 * (1.0 - s) * t
                       : 0.0;
  const double u2 = in ? py1 * (1 - s) * (1.0 - t) + py2 * s * (1.0 - t) +
                             py3 * s * t + py4 * (1.0 - s) * t
                       : 0.0;
  if (near(u1, Uth, 1e-15) && near(u2, Uth, 1e-15))
    tip_record<GRAD>(a, i, j, (float)s, (float)t, ptime, present, count, vec,
                     cap, plot);
}

// Block-wide argmin (256 threads, linear id t) of the tip nearest to the
// current centre, ties broken by (y, x); writes the new centre unless no tip
// was found or this is step 0 (slice_kernel uses tipx0/tipy0 at count == 0,
// symmetryReduction.cu:98-101).
// (d, y, x) lexicographically smaller: a total order, so the nearest tip
// does not depend on the order the tips were found or compared in.
__device__ __forceinline__ bool tip_before(double d, float y, float x,
                                           double db, float yb, float xb) {
  return d < db || (d == db && (y < yb || (y == yb && x < xb)));
}

// Warp 0 of the calling block: the nearest tip to the current centre,
// lanes over the tips then a shuffle arg-min (no block-wide barrier); the
// other threads return at once.
__device__ void pick_centre_block(int t, const int *count, const yh_tip *vec,
                                  int cap, yh_sym_state *sym) {
  if (t >= 32) return;
  const int n0 = *(volatile const int *)count;
  const int n = n0 < cap ? n0 : cap;
  const float cx = sym->centre[0], cy = sym->centre[1];
  double bd = 1e300;
  float bx = 0.f, by = 0.f;
  for (int k = t; k < n; k += 32) {
    const float tx = ((volatile const float *)&vec[k].x)[0];
    const float ty = ((volatile const float *)&vec[k].y)[0];
    const double dx = (double)tx - cx, dy = (double)ty - cy;
    const double d = dx * dx + dy * dy;
    if (tip_before(d, ty, tx, bd, by, bx)) {
      bd = d;
      bx = tx;
      by = ty;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const double d = __shfl_down_sync(0xffffffffu, bd, off);
    const float x = __shfl_down_sync(0xffffffffu, bx, off);
    const float y = __shfl_down_sync(0xffffffffu, by, off);
    if (tip_before(d, y, x, bd, by, bx)) {
      bd = d;
      bx = x;
      by = y;
    }
  }
  if (t == 0) {
    sym->ntips = n0;
    if (n > 0 && sym->step > 0) {
      sym->centre[0] = bx;
      sym->centre[1] = by;
    }
  }
}

// HOLES: the disc around the grid centre, all cells (tipTracker.cu:47-122,
// :262-266); otherwise, closed form (ALG 1): i in [1,nx-3], j in [1,ny-3]
// (tipTracker.cu:124-204), Newton (ALG 2): the 2 tipOffset window around
// the grid centre (tipTracker.cu:339-341).
template <bool HOLES, int ALG>
__device__ __forceinline__ bool tip_active(const TipArgs &a, int i, int j) {
  const int nx = a.nx, ny = a.ny;
  if (HOLES) {
    const int ic = i - nx / 2, jc = j - ny / 2;
    return i < nx && j < ny && (ic * ic + jc * jc) < a.r2;
  }
  if (ALG == 1) return (i >= 1) && (i < nx - 2) && (j >= 1) && (j < ny - 2);
  return i < nx && j < ny && i >= nx / 2 - a.tox && i < nx / 2 + a.tox &&
         j >= ny / 2 - a.toy && j < ny / 2 + a.toy;
}

// Corners of cell (i, j): x = present, y = past, in the order (i,j),
// (i+1,j), (i+1,j+1), (i,j+1) (tipTracker.cu:140-174), clamped at the edge.
template <typename Real>
__device__ __forceinline__ void tip_corners(const TipArgs &a, const Real *past,
                                            const Real *present, int i, int j,
                                            Real x[4], Real y[4]) {
  const int nx = a.nx, ny = a.ny;
  const int s0 = i + nx * j;
  const int sx = (i < nx - 1) ? s0 + 1 : s0;
  const int sy = (j < ny - 1) ? s0 + nx : s0;
  const int sxy = ((j < ny - 1) && (i < nx - 1)) ? s0 + nx + 1 : s0;
  x[0] = present[s0];
  x[1] = present[sx];
  x[2] = present[sxy];
  x[3] = present[sy];
  y[0] = past[s0];
  y[1] = past[sx];
  y[2] = past[sxy];
  y[3] = past[sy];
}

constexpr int kTipRows = 4;  // FP32 closed form: cells per thread, 8 rows apart

// FP32 closed form: a cell is a candidate when the threshold lies within
// the corner range of both levels (a bilinear interpolant on the unit cell
// stays within its corner values, so no root of x = Uth, y = Uth lies
// inside any other cell). A block scans a 32x32 tile, gathers its
// candidates in shared memory and runs the FP64 intersection on them with
// full warps: GB300 issues FP64 at a small fraction of its FP32 rate and a
// warp pays for an FP64 instruction whatever its active lanes, so a
// candidate per warp would cost a whole warp's FP64 time each. Other
// forms (FP64 levels, Newton) keep one thread per cell.
template <typename Real, bool HOLES, int ALG, bool GRAD>
__global__ void __launch_bounds__(256)
    tip_kernel(const TipArgs a, const Real *__restrict__ past,
               const Real *__restrict__ present, int *count, yh_tip *vec,
               int cap, yh_sym_state *sym, unsigned int *done, uint8_t *plot) {
  grid_dep_wait();
  constexpr bool COMPACT = sizeof(Real) == 4 && ALG == 1;
  const int i = blockIdx.x * 32 + threadIdx.x;
  const int t = threadIdx.x + 32 * threadIdx.y;
  const float ptime =
      sym ? (float)(a.dt * (double)sym->step) : (float)a.ptime;
  if (COMPACT) {
    __shared__ int s_n;
    __shared__ short2 s_cell[256 * kTipRows];
    if (t == 0) s_n = 0;
    __syncthreads();
    const float th = (float)a.Uth, tol = 1e-5f;
#pragma unroll
    for (int m = 0; m < kTipRows; ++m) {
      const int j = blockIdx.y * 8 * kTipRows + threadIdx.y + 8 * m;
      if (!tip_active<HOLES, ALG>(a, i, j)) continue;
      Real x[4], y[4];
      tip_corners(a, past, present, i, j, x, y);
      const float xmn = fminf(fminf(x[0], x[1]), fminf(x[2], x[3]));
      const float xmx = fmaxf(fmaxf(x[0], x[1]), fmaxf(x[2], x[3]));
      const float ymn = fminf(fminf(y[0], y[1]), fminf(y[2], y[3]));
      const float ymx = fmaxf(fmaxf(y[0], y[1]), fmaxf(y[2], y[3]));
      if (th >= xmn - tol && th <= xmx + tol && th >= ymn - tol &&
          th <= ymx + tol) {
        const int k = atomicAdd(&s_n, 1);
        s_cell[k] = make_short2((short)(threadIdx.x), (short)(threadIdx.y + 8 * m));
      }
    }
    __syncthreads();
    const int n = s_n;
    for (int k = t; k < n; k += 256) {
      const int ci = blockIdx.x * 32 + s_cell[k].x;
      const int cj = blockIdx.y * 8 * kTipRows + s_cell[k].y;
      Real x[4], y[4];
      tip_corners(a, past, present, ci, cj, x, y);
      tip_cell_f32div<GRAD>(a, ci, cj, x[0], x[1], x[2], x[3], y[0], y[1],
                            y[2], y[3], !HOLES, ptime, present, count, vec,
                            cap, plot);
    }
  } else {
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (tip_active<HOLES, ALG>(a, i, j)) {
      Real x[4], y[4];
      tip_corners(a, past, present, i, j, x, y);
      if (ALG == 2)
        tip_cell_newton<GRAD>(a, i, j, x[0], x[1], x[2], x[3], y[0], y[1],
                              y[2], y[3], ptime, present, count, vec, cap,
                              plot);
      else
        tip_cell<GRAD>(a, i, j, x[0], x[1], x[2], x[3], y[0], y[1], y[2],
                       y[3], !HOLES, ptime, present, count, vec, cap, plot);
    }
  }
  if (sym == nullptr) return;
  // Last block to finish chooses the disc centre.
  __shared__ bool s_last;
  __syncthreads();
  if (t == 0) {
    __threadfence();
    const unsigned nb = gridDim.x * gridDim.y;
    s_last = atomicAdd(done, 1u) == nb - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (t == 0) *done = 0u;
  pick_centre_block(t, count, vec, cap, sym);
}

__global__ void pick_centre_kernel(const int *count, const yh_tip *vec,
                                   int cap, yh_sym_state *sym) {
  pick_centre_block(threadIdx.x, count, vec, cap, sym);
}

// With sym_pick != nullptr the tips are stamped dt*sym->step (so a captured
// graph stays valid as steps advance) and the last block picks the centre;
// otherwise they are stamped `ptime`. `done` is a zeroed counter. The
// algorithm (p.tipAlgorithm 1 closed form, 2 Newton) and the gradient
// (p.tipGrad) follow p; plot (may be null) gets the tips' cells marked.
template <typename Real>
cudaError_t launch_tips(const yh_param_var &p, const Real *past,
                        const Real *present, bool holes, double ptime,
                        int *count, yh_tip *vec, int cap,
                        yh_sym_state *sym_pick, unsigned int *done,
                        cudaStream_t s, uint8_t *plot) {
  if (p.tipAlgorithm != 1 && p.tipAlgorithm != 2) return cudaErrorNotSupported;
  TipArgs a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.r2 = p.tipOffsetX * p.tipOffsetY;
  a.tox = p.tipOffsetX;
  a.toy = p.tipOffsetY;
  a.Uth = p.Uth;
  a.invdx = p.invdx;
  a.invdy = p.invdy;
  a.dt = p.dt;
  a.ptime = ptime;
  const bool newton = p.tipAlgorithm == 2, grad = p.tipGrad;
  const int rows = (sizeof(Real) == 4 && !newton) ? 8 * kTipRows : 8;
  const dim3 block(32, 8);
  const dim3 grid((p.nx + 31) / 32, (p.ny + rows - 1) / rows);
#define YH_TIP(H, ALG, G)                                                   \
  if (holes == H && newton == (ALG == 2) && grad == G)                      \
    return launch_pdl(tip_kernel<Real, H, ALG, G>, grid, block, 0, s, a,     \
                      past, present, count, vec, cap, sym_pick, done, plot);
  YH_TIP(true, 1, false)
  YH_TIP(true, 1, true)
  YH_TIP(true, 2, false)
  YH_TIP(true, 2, true)
  YH_TIP(false, 1, false)
  YH_TIP(false, 1, true)
  YH_TIP(false, 2, false)
  YH_TIP(false, 2, true)
#undef YH_TIP
  return cudaErrorInvalidValue;
}

cudaError_t launch_pick_centre(const int *count, const yh_tip *vec, int cap,
                               yh_sym_state *sym, cudaStream_t s) {
  pick_centre_kernel<<<1, 256, 0, s>>>(count, vec, cap, sym);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Phase integrals + solve
// ---------------------------------------------------------------------------

template <typename Real>
struct PhaseArgs {
  int nx, ny, r2, R;  // R: largest integer with R*R < r2
  Real hx, hy, invdx, invdy;
  double hxhy;
};

// The comoving field computed by the last block of the phase launch from
// the c it has just solved for (the work of comoving_kernel, in FP32, for
// the FP32 BFECC), then phi += dt*c and step += 1 when `advance`.
struct PhaseTail {
  float *rows, *cols;  // null: no comoving field, no advance
  float hx, hy;
  double dt;
  int advance;
};

constexpr int kPhaseBX = 32, kPhaseBY = 8;
constexpr int kPhaseRows = 2;  // cells per thread, 8 rows apart: 32x16 tiles

// Phase-integral accumulators. FP32 fields: float-float pairs hi + lo kept
// exact by Knuth's TwoSum (The Art of Computer Programming vol. 2, 4.2.2),
// about 48 significant bits on the FP32 pipe. GB300 issues FP64 at a small
// fraction of its FP32 rate; a per-cell FP64 sum and shuffle tree made this
// launch FP64-bound. FP64 fields: plain doubles. Both store in 8 bytes.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

struct AccF {
  float hi, lo;
  __device__ __forceinline__ void set(float v) {
    hi = v;
    lo = 0.f;
  }
  __device__ __forceinline__ void add(const AccF &b) {
    float s, e;
    two_sum(hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, b.lo));
    two_sum(s, e, hi, lo);
  }
  __device__ __forceinline__ void add(float v) {
    AccF b;
    b.set(v);
    add(b);
  }
  __device__ __forceinline__ AccF down(int off, int width) const {
    AccF r;
    r.hi = __shfl_down_sync(0xffffffffu, hi, off, width);
    r.lo = __shfl_down_sync(0xffffffffu, lo, off, width);
    return r;
  }
  __device__ __forceinline__ double value() const {
    return (double)hi + (double)lo;
  }
  __device__ __forceinline__ void store(double *p) const {
    *reinterpret_cast<float2 *>(p) = make_float2(hi, lo);
  }
  __device__ __forceinline__ static AccF load(const double *p) {
    const float2 v = __ldcg(reinterpret_cast<const float2 *>(p));
    AccF r;
    r.hi = v.x;
    r.lo = v.y;
    return r;
  }
};

struct AccD {
  double v;
  __device__ __forceinline__ void set(double x) { v = x; }
  __device__ __forceinline__ void add(const AccD &b) { v += b.v; }
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ AccD down(int off, int width) const {
    AccD r;
    r.v = __shfl_down_sync(0xffffffffu, v, off, width);
    return r;
  }
  __device__ __forceinline__ double value() const { return v; }
  __device__ __forceinline__ void store(double *p) const { *p = v; }
  __device__ __forceinline__ static AccD load(const double *p) {
    AccD r;
    r.v = __ldcg(p);
    return r;
  }
};

template <typename Real>
struct AccOf {
  using T = AccD;
};
template <>
struct AccOf<float> {
  using T = AccF;
};

// v > 0 from the bits, with no floating-point compare: an FP64 compare
// issues on GB300's narrow FP64 pipe. Equal to v > 0 for every input,
// NaN included.
__device__ __forceinline__ bool adv_pos(double v) {
  const long long b = __double_as_longlong(v);
  return b > 0 && b <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool adv_pos(float v) {
  const int b = __float_as_int(v);
  return b > 0 && b <= 0x7f800000;
}

// 2nd-order one-sided derivative, upwinded by the sign of the comoving
// field (convFB2ndOX/Y, symmetryReduction.cu:242-262).
template <typename Real>
__device__ __forceinline__ Real fb2(Real c, Real p1, Real p2, Real m1, Real m2,
                                    bool pos, Real inv) {
  return pos ? (Real(-3) * c + Real(4) * p1 - p2) * inv
             : (Real(3) * c - Real(4) * m1 + m2) * inv;
}
// Negated 4th-order central derivative (convCentral2X/Y,
// symmetryReduction.cu:224-240).
template <typename Real>
__device__ __forceinline__ Real c4(Real p1, Real p2, Real m1, Real m2,
                                   Real inv) {
  return (p2 - Real(8) * p1 + Real(8) * m1 - m2) * inv * Real(1.0 / 6.0);
}

// The 12 integrands of cell (i, j) when it lies in the disc: templates
// (x, y, theta) against the slices (x, y, theta) and the tangent,
// summed over the fields (integralTrapz.cu:17-184 with the slices of
// symmetryReduction.cu:72-222).
template <int NF, typename Real, bool FROZEN, bool HOLES, typename AdvT>
__device__ __forceinline__ bool phase_cell(
    const PhaseArgs<Real> &a, const Fld<Real> &st, const Fld<Real> &tan,
    const Fld<Real> &tx, const Fld<Real> &ty, const Fld<Real> &tt,
    const AdvT *adv_rows, const AdvT *adv_cols,
    const uint8_t *__restrict__ solid, int i, int j, int cx, int cy,
    Real s[12]) {
  const int nx = a.nx, ny = a.ny;
  if (i < 0 || i >= nx || j < 0 || j >= ny) return false;
  const int ic = i - nx / 2 - cx, jc = j - ny / 2 - cy;
  if (ic * ic + jc * jc >= a.r2) return false;
  const int C = i + nx * j;
  const bool tissue = !HOLES || solid[C] != 0;
  const bool px = tissue && adv_pos(adv_rows[j]);
  const bool py = tissue && adv_pos(adv_cols[i]);
  const int row = nx * j;
  const int iE = mirror(i + 1, nx), iW = mirror(i - 1, nx);
  const int iEE = mirror(i + 2, nx), iWW = mirror(i - 2, nx);
  const int jN = nx * mirror(j + 1, ny), jS = nx * mirror(j - 1, ny);
  const int jNN = nx * mirror(j + 2, ny), jSS = nx * mirror(j - 2, ny);
  const Real x = (Real)i, y = (Real)j;
#pragma unroll
  for (int k = 0; k < 12; ++k) s[k] = Real(0);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const Real *__restrict__ g = st.f[f];
    const Real c = g[C];
    const Real e1 = g[row + iE], e2 = g[row + iEE];
    const Real w1 = g[row + iW], w2 = g[row + iWW];
    const Real n1 = g[i + jN], n2 = g[i + jNN];
    const Real s1 = g[i + jS], s2 = g[i + jSS];
    const Real dx = fb2(c, e1, e2, w1, w2, px, a.invdx);
    const Real dy = fb2(c, n1, n2, s1, s2, py, a.invdy);
    const Real dth = a.hx * x * dy - a.hy * y * dx;
    Real Tx, Ty, Tt;
    if (FROZEN) {
      Tx = tx.f[f][C];
      Ty = ty.f[f][C];
      Tt = tt.f[f][C];
    } else {
      Tx = c4(e1, e2, w1, w2, a.invdx);
      Ty = c4(n1, n2, s1, s2, a.invdy);
      Tt = a.hx * x * Ty - a.hy * y * Tx;
    }
    const Real vt = tan.f[f][C];
    const Real Tv[3] = {Tx, Ty, Tt};
    const Real Cv[4] = {dx, dy, dth, vt};
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q < 3 ? 3 * p + q : 9 + p] += Tv[p] * Cv[q];
  }
  return true;
}

// One block covers a 32x16 tile of the disc's bounding box, placed by the
// current disc centre read from `sym` (so a captured graph follows the
// tip). Per block: 12 partial sums (accumulator pairs); the last block to
// finish sums them in a fixed order, solves in FP64 and, with a tail, writes
// the comoving field.
template <int NF, typename Real, bool FROZEN, bool HOLES, typename AdvT>
__global__ void __launch_bounds__(kPhaseBX *kPhaseBY)
    phase_kernel(const PhaseArgs<Real> a, const Fld<Real> st,
                 const Fld<Real> tan, const Fld<Real> tx, const Fld<Real> ty,
                 const Fld<Real> tt, const AdvT *adv_rows,
                 const AdvT *adv_cols, const uint8_t *__restrict__ solid,
                 yh_sym_state *sym, double *partials, unsigned int *done,
                 const PhaseTail tail) {
  // adv_rows/adv_cols are not __restrict__: the tail rewrites them
  using Acc = typename AccOf<Real>::T;
  grid_dep_wait();
  const int nx = a.nx, ny = a.ny;
  // integer centre as slice_kernel/trapz_kernel round it
  // (symmetryReduction.cu:98-104): float arithmetic, round-half-even.
  const int cx = __float2int_rn(sym->centre[0] - (float)(nx / 2));
  const int cy = __float2int_rn(sym->centre[1] - (float)(ny / 2));
  // cos and sin of phi_adv = phi for the solve and the comoving field:
  // block 0 takes them off the last block's serial tail (the counter's
  // 256-byte slot holds them; the completion fence publishes them)
  double *rot = reinterpret_cast<double *>(done) + 1;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 &&
      threadIdx.y == 0) {
    double sn, cs;
    sincos(sym->phi[2], &sn, &cs);
    rot[0] = cs;
    rot[1] = sn;
  }
  const int i = nx / 2 + cx - a.R + (int)(blockIdx.x * kPhaseBX + threadIdx.x);
  const int j0 = ny / 2 + cy - a.R +
                 (int)(blockIdx.y * kPhaseBY * kPhaseRows + threadIdx.y);
  Acc acc[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k].set(Real(0));
#pragma unroll
  for (int m = 0; m < kPhaseRows; ++m) {
    Real s[12];
    if (phase_cell<NF, Real, FROZEN, HOLES, AdvT>(
            a, st, tan, tx, ty, tt, adv_rows, adv_cols, solid, i,
            j0 + m * kPhaseBY, cx, cy, s)) {
#pragma unroll
      for (int k = 0; k < 12; ++k) acc[k].add(s[k]);
    }
  }
  // block sum, transposed through shared memory: warp q (0-7) sums
  // integrals q and q + 8, 8 threads' values a lane, then a shuffle tree
  // (one tree per integral instead of twelve in every warp)
  constexpr int NT = kPhaseBX * kPhaseBY;
  __shared__ Acc s_a[12][NT];
  __shared__ bool s_last;
  const int lane = threadIdx.x;  // blockDim.x == 32
  const int warp = threadIdx.y;
  const int t = threadIdx.x + kPhaseBX * threadIdx.y;
#pragma unroll
  for (int k = 0; k < 12; ++k) s_a[k][t] = acc[k];
  __syncthreads();
  const unsigned nb = gridDim.x * gridDim.y;
  const unsigned bid = blockIdx.x + gridDim.x * blockIdx.y;
  for (int q = warp; q < 12; q += kPhaseBY) {
    Acc v = s_a[q][lane];
#pragma unroll
    for (int m = 1; m < NT / 32; ++m) v.add(s_a[q][lane + 32 * m]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v.add(v.down(off, 32));
    if (lane == 0) v.store(&partials[(size_t)bid * 12 + q]);
  }
  __syncthreads();
  if (t == 0) {
    __threadfence();
    s_last = atomicAdd(done, 1u) == nb - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // Last block: 12 groups of 16 lanes (warps 0-5), lane r sums the block
  // partials r, r+16, ... in order, then a 16-lane tree.
  __shared__ double s_I[12];
  __shared__ double s_c[3], s_cs, s_sn;
  __shared__ double s_phi[3], s_cold[3];
  if (t == 224) {  // warp 7 (no partial sums): the tail's other inputs
    s_cs = __ldcg(rot);
    s_sn = __ldcg(rot + 1);
    for (int kk = 0; kk < 3; ++kk) {
      s_phi[kk] = sym->phi[kk];
      s_cold[kk] = sym->c[kk];
    }
  }
  if (t < 192) {
    const int k = t >> 4, r = t & 15;
    Acc v;
    v.set(Real(0));
    // the same order (r, r + 16, ...), sixteen loads in flight at a time
    for (unsigned b0 = r; b0 < nb; b0 += 256) {
      Acc x[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const unsigned b = b0 + 16 * u;
        if (b < nb)
          x[u] = Acc::load(&partials[(size_t)b * 12 + k]);
        else
          x[u].set(Real(0));
      }
#pragma unroll
      for (int u = 0; u < 16; ++u) v.add(x[u]);
    }
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) v.add(v.down(off, 16));
    if (r == 0) s_I[k] = a.hxhy * v.value();
  }
  __syncthreads();
  if (t == 0) {
    double I[12];
    for (int kk = 0; kk < 12; ++kk) {
      I[kk] = s_I[kk];
      sym->integrals[kk] = I[kk];
    }
    // phi_adv = phi: one angle for the solve and the comoving field
    double c[3];
    const int stt = solve3_cofactor(I, s_cs, s_sn, c);
    sym->status = stt;
    if (stt != YH_OK) sym->nsingular += 1;
    for (int kk = 0; kk < 3; ++kk) {
      const double ck = stt == YH_OK ? c[kk] : s_cold[kk];
      s_c[kk] = ck;
      sym->c[kk] = ck;
      sym->c_adv[kk] = ck;
      sym->phi_adv[kk] = s_phi[kk];
    }
    *done = 0u;
  }
  if (tail.rows == nullptr) return;
  __syncthreads();
  // adv_x[j] = hy*y*ct - cx*cos(pt) + cy*sin(pt);
  // adv_y[i] = -hx*x*ct - cx*sin(pt) - cy*cos(pt)   (symmetryReduction.cu:55-56)
  const float fcx = (float)s_c[0], fcy = (float)s_c[1], fct = (float)s_c[2];
  const float fcs = (float)s_cs, fsn = (float)s_sn;
  const float r0 = fcy * fsn - fcx * fcs, c0 = -(fcx * fsn + fcy * fcs);
  const float hyct = tail.hy * fct, hxct = tail.hx * fct;
  for (int jj = t; jj < ny; jj += kPhaseBX * kPhaseBY)
    tail.rows[jj] = hyct * (float)jj + r0;
  for (int ii = t; ii < nx; ii += kPhaseBX * kPhaseBY)
    tail.cols[ii] = c0 - hxct * (float)ii;
  if (tail.advance && t == 0) {
    for (int kk = 0; kk < 3; ++kk) sym->phi[kk] = s_phi[kk] + s_c[kk] * tail.dt;
    sym->step += 1;
  }
}

static void phase_geometry(const yh_param_var &p, int *R, dim3 *grid) {
  const int r2 = p.tipOffsetX * p.tipOffsetY;
  int r = 0;
  while ((long long)(r + 1) * (r + 1) < r2) ++r;
  // the box never needs to exceed twice the grid
  const int bx = 2 * r + 1 < 2 * p.nx ? 2 * r + 1 : 2 * p.nx;
  const int by = 2 * r + 1 < 2 * p.ny ? 2 * r + 1 : 2 * p.ny;
  constexpr int TY = kPhaseBY * kPhaseRows;
  *R = r;
  *grid = dim3((bx + kPhaseBX - 1) / kPhaseBX, (by + TY - 1) / TY);
}

size_t phase_workspace_bytes(const yh_param_var &p) {
  int R;
  dim3 g;
  phase_geometry(p, &R, &g);
  // counter (256 B slot) + 12 accumulators of 8 bytes per block
  return 256 + (size_t)g.x * g.y * 12 * sizeof(double);
}

template <typename Real, typename AdvT>
static cudaError_t phase_dispatch(const yh_param_var &p, int nf,
                                  const Fld<Real> &st, const Fld<Real> &tan,
                                  const Fld<Real> &tx, const Fld<Real> &ty,
                                  const Fld<Real> &tt, const AdvT *adv_rows,
                                  const AdvT *adv_cols, const uint8_t *solid,
                                  yh_sym_state *sym, void *workspace,
                                  const PhaseTail &tail, cudaStream_t s) {
  PhaseArgs<Real> a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.r2 = p.tipOffsetX * p.tipOffsetY;
  dim3 grid;
  phase_geometry(p, &a.R, &grid);
  a.hx = (Real)p.hx;
  a.hy = (Real)p.hy;
  a.invdx = (Real)p.invdx;
  a.invdy = (Real)p.invdy;
  a.hxhy = p.hx * p.hy;
  unsigned int *done = reinterpret_cast<unsigned int *>(workspace);
  double *partials =
      reinterpret_cast<double *>(reinterpret_cast<char *>(workspace) + 256);
  const dim3 block(kPhaseBX, kPhaseBY);
  const bool frozen = tx.f[0] != nullptr;
  const bool holes = p.solidSwitch && solid;
#define YH_PH(NF, FZ, HO)                                                      \
  if (nf == NF && frozen == FZ && holes == HO)                                 \
    return launch_pdl(phase_kernel<NF, Real, FZ, HO, AdvT>, grid, block, 0, s, \
                      a, st, tan, tx, ty, tt, adv_rows, adv_cols, solid, sym,  \
                      partials, done, tail);
  YH_PH(2, false, false)
  YH_PH(2, false, true)
  YH_PH(2, true, false)
  YH_PH(2, true, true)
  YH_PH(3, false, false)
  YH_PH(3, false, true)
  YH_PH(3, true, false)
  YH_PH(3, true, true)
#undef YH_PH
  return cudaErrorInvalidValue;
}

template <typename Real>
cudaError_t launch_phase(const yh_param_var &p, int nf, const Fld<Real> &st,
                         const Fld<Real> &tan, const Fld<Real> &tx,
                         const Fld<Real> &ty, const Fld<Real> &tt,
                         const double *adv_rows, const double *adv_cols,
                         const uint8_t *solid, yh_sym_state *sym,
                         void *workspace, cudaStream_t s) {
  PhaseTail none = {};
  return phase_dispatch<Real, double>(p, nf, st, tan, tx, ty, tt, adv_rows,
                                      adv_cols, solid, sym, workspace, none, s);
}

cudaError_t launch_phase_comoving(const yh_param_var &p, int nf,
                                  const Fld<float> &st, const Fld<float> &tan,
                                  const Fld<float> &tx, const Fld<float> &ty,
                                  const Fld<float> &tt, float *adv_rows,
                                  float *adv_cols, const uint8_t *solid,
                                  yh_sym_state *sym, void *workspace,
                                  bool advance, cudaStream_t s) {
  PhaseTail tail;
  tail.rows = adv_rows;
  tail.cols = adv_cols;
  tail.hx = (float)p.hx;
  tail.hy = (float)p.hy;
  tail.dt = p.dt;
  tail.advance = advance ? 1 : 0;
  return phase_dispatch<float, float>(p, nf, st, tan, tx, ty, tt, adv_rows,
                                      adv_cols, solid, sym, workspace, tail, s);
}

// Template derivative fields over the whole grid (frozen template).
template <int NF, typename Real>
__global__ void template_kernel(const PhaseArgs<Real> a, const Fld<Real> st,
                                const Fld<Real> tx, const Fld<Real> ty,
                                const Fld<Real> tt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  if (i >= nx || j >= ny) return;
  const int C = i + nx * j, row = nx * j;
  const Real x = (Real)i, y = (Real)j;
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    const Real *g = st.f[f];
    const Real Tx = c4(g[row + mirror(i + 1, nx)], g[row + mirror(i + 2, nx)],
                       g[row + mirror(i - 1, nx)], g[row + mirror(i - 2, nx)],
                       a.invdx);
    const Real Ty = c4(g[i + nx * mirror(j + 1, ny)],
                       g[i + nx * mirror(j + 2, ny)],
                       g[i + nx * mirror(j - 1, ny)],
                       g[i + nx * mirror(j - 2, ny)], a.invdy);
    tx.f[f][C] = Tx;
    ty.f[f][C] = Ty;
    tt.f[f][C] = a.hx * x * Ty - a.hy * y * Tx;
  }
}

template <typename Real>
cudaError_t launch_template(const yh_param_var &p, int nf,
                            const Fld<Real> &st, const Fld<Real> &tx,
                            const Fld<Real> &ty, const Fld<Real> &tt,
                            cudaStream_t s) {
  PhaseArgs<Real> a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.hx = (Real)p.hx;
  a.hy = (Real)p.hy;
  a.invdx = (Real)p.invdx;
  a.invdy = (Real)p.invdy;
  const dim3 block(32, 8);
  const dim3 grid((p.nx + 31) / 32, (p.ny + 7) / 8);
  if (nf == 2)
    template_kernel<2, Real><<<grid, block, 0, s>>>(a, st, tx, ty, tt);
  else
    template_kernel<3, Real><<<grid, block, 0, s>>>(a, st, tx, ty, tt);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Comoving field and phi update
// ---------------------------------------------------------------------------

// adv_x[j] = hy*y*ct - cx*cos(pt) + cy*sin(pt);
// adv_y[i] = -hx*x*ct - cx*sin(pt) - cy*cos(pt)   (symmetryReduction.cu:55-56)
// from (c_adv, phi_adv); then, if `advance`, phi += dt*c and step += 1
// (main.cu:936-952).
__global__ void comoving_kernel(int nx, int ny, double hx, double hy,
                                double dt, yh_sym_state *sym,
                                double *adv_rows, double *adv_cols,
                                float *adv_rows_f, float *adv_cols_f,
                                int advance) {
  __shared__ double s_c[3], s_cs, s_sn;
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) s_c[k] = sym->c_adv[k];
    s_cs = cos(sym->phi_adv[2]);
    s_sn = sin(sym->phi_adv[2]);
  }
  __syncthreads();
  const double cx = s_c[0], cy = s_c[1], ct = s_c[2], cs = s_cs, sn = s_sn;
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    const double y = (double)j;
    const double v = hy * y * ct - cx * cs + cy * sn;
    adv_rows[j] = v;
    if (adv_rows_f) adv_rows_f[j] = (float)v;
  }
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    const double x = (double)i;
    const double v = -hx * x * ct - cx * sn - cy * cs;
    adv_cols[i] = v;
    if (adv_cols_f) adv_cols_f[i] = (float)v;
  }
  __syncthreads();
  if (advance && threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) sym->phi[k] = sym->phi[k] + sym->c[k] * dt;
    sym->step += 1;
  }
}

cudaError_t launch_comoving(const yh_param_var &p, yh_sym_state *sym,
                            double *adv_rows, double *adv_cols,
                            float *adv_rows_f, float *adv_cols_f,
                            bool advance, cudaStream_t s) {
  comoving_kernel<<<1, 256, 0, s>>>(p.nx, p.ny, p.hx, p.hy, p.dt, sym,
                                    adv_rows, adv_cols, adv_rows_f,
                                    adv_cols_f, advance ? 1 : 0);
  return cudaGetLastError();
}

__global__ void sym_advance_kernel(double dt, yh_sym_state *sym) {
  for (int k = 0; k < 3; ++k) sym->phi[k] = sym->phi[k] + sym->c[k] * dt;
  sym->step += 1;
}

cudaError_t launch_sym_advance(const yh_param_var &p, yh_sym_state *sym,
                               cudaStream_t s) {
  sym_advance_kernel<<<1, 1, 0, s>>>(p.dt, sym);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// BFECC
// ---------------------------------------------------------------------------

template <typename Real>
struct BfeccArgs {
  int nx, ny;
  Real dt, hx, hy, tc;
};

// Neighbour indices of the passes (advFDBFECC.cu:112-126), with "outside
// the domain" extended to "not tissue" when there are holes.
struct BIdx {
  int W, E, S, N, cW, W2, cE, E2, cS, S2, cN, N2;
};

template <bool HOLES>
__device__ __forceinline__ BIdx bfecc_idx(int i, int j, int nx, int ny,
                                          const uint8_t *solid, bool &sc) {
  const int C = i + nx * j;
  bool hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  sc = true;
  if (HOLES) {
    sc = solid[C] != 0;
    if (!sc) {
      BIdx r = {C, C, C, C, C, C, C, C, C, C, C, C};
      return r;
    }
    hw = hw && solid[C - 1];
    he = he && solid[C + 1];
    hs = hs && solid[C - nx];
    hn = hn && solid[C + nx];
  }
  BIdx r;
  r.W = hw ? C - 1 : (he ? C + 1 : C);
  r.E = he ? C + 1 : (hw ? C - 1 : C);
  r.S = hs ? C - nx : (hn ? C + nx : C);
  r.N = hn ? C + nx : (hs ? C - nx : C);
  r.cW = hw ? C : (he ? C + 1 : C);
  r.W2 = hw ? C - 1 : C;
  r.cE = he ? C : (hw ? C - 1 : C);
  r.E2 = he ? C + 1 : C;
  r.cS = hs ? C : (hn ? C + nx : C);
  r.S2 = hs ? C - nx : C;
  r.cN = hn ? C : (hs ? C - nx : C);
  r.N2 = hn ? C + nx : C;
  return r;
}

// cx = -adv.x, Rx = sign(cx)*cx*dt/hx (advFDBFECC.cu:30-34).
template <typename Real>
__device__ __forceinline__ void bfecc_ratios(const BfeccArgs<Real> &a, Real ax,
                                             Real ay, Real &cx, Real &cy,
                                             Real &Rx, Real &Ry) {
  cx = -ax;
  cy = -ay;
  const Real sx = cx > Real(0) ? Real(1) : (cx < Real(0) ? Real(-1) : Real(0));
  const Real sy = cy > Real(0) ? Real(1) : (cy < Real(0) ? Real(-1) : Real(0));
  Rx = sx * cx * a.dt / a.hx;
  Ry = sy * cy * a.dt / a.hy;
}

// ADV2D: the comoving field as full nx*ny arrays (adv_rows = adv.x,
// adv_cols = adv.y, the reference's layout); otherwise as the separable
// vectors adv_rows[ny], adv_cols[nx].
template <int PASS, int NF, typename Real, bool HOLES, bool ADV2D>
__global__ void __launch_bounds__(256)
    bfecc_pass(const BfeccArgs<Real> a, const Fld<Real> in, const Fld<Real> uf,
               const Fld<Real> ue, const Fld<Real> out,
               const Real *__restrict__ adv_rows,
               const Real *__restrict__ adv_cols,
               const uint8_t *__restrict__ solid) {
  grid_dep_wait();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int nx = a.nx, ny = a.ny;
  if (i >= nx || j >= ny) return;
  const int C = i + nx * j;
  bool sc;
  const BIdx n = bfecc_idx<HOLES>(i, j, nx, ny, solid, sc);
  Real cx, cy, Rx, Ry;
  const Real ax = ADV2D ? adv_rows[C] : adv_rows[j];
  const Real ay = ADV2D ? adv_cols[C] : adv_cols[i];
  bfecc_ratios(a, sc ? ax : Real(0), sc ? ay : Real(0), cx, cy, Rx, Ry);
#pragma unroll
  for (int f = 0; f < NF; ++f) {
    if (PASS == 1) {
      const Real *__restrict__ g = in.f[f];
      const Real FDx = cx > Real(0) ? g[C] - g[n.W] : g[C] - g[n.E];
      const Real FDy = cy > Real(0) ? g[C] - g[n.S] : g[C] - g[n.N];
      uf.f[f][C] = g[C] - a.tc * (Rx * FDx + Ry * FDy);
    } else if (PASS == 2) {
      const Real *__restrict__ q = uf.f[f];
      const Real FDx = cx > Real(0) ? q[n.cE] - q[n.E2] : q[n.cW] - q[n.W2];
      const Real FDy = cy > Real(0) ? q[n.cN] - q[n.N2] : q[n.cS] - q[n.S2];
      const Real ub = q[C] - a.tc * (Rx * FDx + Ry * FDy);
      const Real g = in.f[f][C];
      ue.f[f][C] = g - Real(0.5) * (ub - g);
    } else {
      const Real *__restrict__ q = ue.f[f];
      const Real FDx = cx > Real(0) ? q[C] - q[n.W] : q[C] - q[n.E];
      const Real FDy = cy > Real(0) ? q[C] - q[n.S] : q[C] - q[n.N];
      const Real r = q[C] - a.tc * (Rx * FDx + Ry * FDy);
      out.f[f][C] = sc ? r : Real(0);
    }
  }
}

// The three passes in one launch. A block owns a 32x16 tile of the output:
// pass 1 on the tile and a 2-cell ring (uf), pass 2 on the tile and a
// 1-cell ring (ue), pass 3 on the tile, all in shared memory; every pass
// reads one neighbour per axis, so the input tile with a 3-cell ring
// covers them. Each cell's arithmetic is bfecc_pass's, in the same order,
// so the result equals the three launches bit for bit; the ring cells are
// computed by two or three blocks (1.4x the pass-1 work of a lone pass).
constexpr int kFuseTX = 32, kFuseTY = 16;

// Offset in a region of row pitch P of the global neighbour index n of C.
__device__ __forceinline__ int bfecc_local(int n, int C, int nx, int P) {
  const int d = n - C;
  return d == 0 ? 0 : (d == -1 ? -1 : (d == 1 ? 1 : (d < 0 ? -P : P)));
}

// Offsets, in a region of row pitch P, of bfecc_idx's neighbours of (i, j)
// in the order W, E, S, N, cW, W2, cE, E2, cS, S2, cN, N2: constants for a
// cell off the grid's edges without holes (bfecc_idx gives the plain
// neighbours there), bfecc_idx itself otherwise.
template <bool HOLES>
__device__ __forceinline__ void fused_offsets(int i, int j, int nx, int ny,
                                              const uint8_t *solid, int P,
                                              int (&o)[12]) {
  if (!HOLES && i > 0 && i < nx - 1 && j > 0 && j < ny - 1) {
    o[0] = -1; o[1] = 1; o[2] = -P; o[3] = P;
    o[4] = 0; o[5] = -1; o[6] = 0; o[7] = 1;
    o[8] = 0; o[9] = -P; o[10] = 0; o[11] = P;
    return;
  }
  const int C = i + nx * j;
  bool sc;
  const BIdx n = bfecc_idx<HOLES>(i, j, nx, ny, solid, sc);
  const int g[12] = {n.W, n.E, n.S, n.N, n.cW, n.W2, n.cE, n.E2,
                     n.cS, n.S2, n.cN, n.N2};
#pragma unroll
  for (int q = 0; q < 12; ++q) o[q] = bfecc_local(g[q], C, nx, P);
}

template <int NF, bool HOLES>
__global__ void __launch_bounds__(256)
    bfecc_fused(const BfeccArgs<float> a, const Fld<float> in,
                const Fld<float> out, const float *__restrict__ adv_rows,
                const float *__restrict__ adv_cols,
                const uint8_t *__restrict__ solid) {
  grid_dep_wait();
  constexpr int GX = kFuseTX + 6, GY = kFuseTY + 6;  // input, ring 3
  constexpr int FX = kFuseTX + 4, FY = kFuseTY + 4;  // uf, ring 2
  constexpr int EX = kFuseTX + 2, EY = kFuseTY + 2;  // ue, ring 1
  __shared__ float s_g[NF][GY * GX];
  __shared__ float s_f[NF][FY * FX];
  __shared__ float s_e[NF][EY * EX];
  // bfecc_ratios splits by axis: cx, Rx depend on the row, cy, Ry on the
  // column, so each is computed once per tile row / column. Off-tissue
  // cells read their own value only (every difference is 0), so which
  // ratios they get does not change their bits.
  __shared__ float s_cx[GY], s_rx[GY], s_cy[GX], s_ry[GX];
  const int nx = a.nx, ny = a.ny;
  const int bi = blockIdx.x * kFuseTX, bj = blockIdx.y * kFuseTY;
  const int t = threadIdx.x + 32 * threadIdx.y;
  if (t < GY) {
    const int j = bj - 3 + t;
    float cx = 0.f, cy, Rx = 0.f, Ry;
    if (j >= 0 && j < ny) bfecc_ratios(a, adv_rows[j], 0.f, cx, cy, Rx, Ry);
    s_cx[t] = cx;
    s_rx[t] = Rx;
  } else if (t >= 64 && t < 64 + GX) {
    const int i = bi - 3 + (t - 64);
    float cx, cy = 0.f, Rx, Ry = 0.f;
    if (i >= 0 && i < nx) bfecc_ratios(a, 0.f, adv_cols[i], cx, cy, Rx, Ry);
    s_cy[t - 64] = cy;
    s_ry[t - 64] = Ry;
  }
  // input tile with a 3-cell ring (cells outside the grid are not read)
  for (int k = t; k < GX * GY; k += 256) {
    const int i = bi - 3 + k % GX, j = bj - 3 + k / GX;
    if (i >= 0 && i < nx && j >= 0 && j < ny)
#pragma unroll
      for (int f = 0; f < NF; ++f) s_g[f][k] = in.f[f][i + nx * j];
  }
  __syncthreads();
  // pass 1 on the tile and a 2-cell ring
  for (int k = t; k < FX * FY; k += 256) {
    const int li = k % FX, lj = k / FX;
    const int i = bi - 2 + li, j = bj - 2 + lj;
    if (i < 0 || i >= nx || j < 0 || j >= ny) continue;
    int o[12];
    fused_offsets<HOLES>(i, j, nx, ny, solid, GX, o);
    const float cx = s_cx[lj + 1], Rx = s_rx[lj + 1];
    const float cy = s_cy[li + 1], Ry = s_ry[li + 1];
    const int g0 = (lj + 1) * GX + (li + 1);
    const int oW = o[0], oE = o[1], oS = o[2], oN = o[3];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const float *g = s_g[f] + g0;
      const float FDx = cx > 0.f ? g[0] - g[oW] : g[0] - g[oE];
      const float FDy = cy > 0.f ? g[0] - g[oS] : g[0] - g[oN];
      s_f[f][k] = g[0] - a.tc * (Rx * FDx + Ry * FDy);
    }
  }
  __syncthreads();
  // pass 2 on the tile and a 1-cell ring
  for (int k = t; k < EX * EY; k += 256) {
    const int li = k % EX, lj = k / EX;
    const int i = bi - 1 + li, j = bj - 1 + lj;
    if (i < 0 || i >= nx || j < 0 || j >= ny) continue;
    int o[12];
    fused_offsets<HOLES>(i, j, nx, ny, solid, FX, o);
    const float cx = s_cx[lj + 2], Rx = s_rx[lj + 2];
    const float cy = s_cy[li + 2], Ry = s_ry[li + 2];
    const int f0 = (lj + 1) * FX + (li + 1);
    const int g0 = (lj + 2) * GX + (li + 2);
    const int ocW = o[4], oW2 = o[5], ocE = o[6], oE2 = o[7];
    const int ocS = o[8], oS2 = o[9], ocN = o[10], oN2 = o[11];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const float *q = s_f[f] + f0;
      const float FDx = cx > 0.f ? q[ocE] - q[oE2] : q[ocW] - q[oW2];
      const float FDy = cy > 0.f ? q[ocN] - q[oN2] : q[ocS] - q[oS2];
      const float ub = q[0] - a.tc * (Rx * FDx + Ry * FDy);
      const float g = s_g[f][g0];
      s_e[f][k] = g - 0.5f * (ub - g);
    }
  }
  __syncthreads();
  // pass 3 on the tile
  for (int k = t; k < kFuseTX * kFuseTY; k += 256) {
    const int li = k % kFuseTX, lj = k / kFuseTX;
    const int i = bi + li, j = bj + lj;
    if (i >= nx || j >= ny) continue;
    const int C = i + nx * j;
    const bool sc = !HOLES || solid[C] != 0;
    int o[12];
    fused_offsets<HOLES>(i, j, nx, ny, solid, EX, o);
    const float cx = s_cx[lj + 3], Rx = s_rx[lj + 3];
    const float cy = s_cy[li + 3], Ry = s_ry[li + 3];
    const int e0 = (lj + 1) * EX + (li + 1);
    const int oW = o[0], oE = o[1], oS = o[2], oN = o[3];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const float *q = s_e[f] + e0;
      const float FDx = cx > 0.f ? q[0] - q[oW] : q[0] - q[oE];
      const float FDy = cy > 0.f ? q[0] - q[oS] : q[0] - q[oN];
      const float r = q[0] - a.tc * (Rx * FDx + Ry * FDy);
      out.f[f][C] = sc ? r : 0.f;
    }
  }
}

template <int NF, typename Real, bool HOLES, bool ADV2D>
static cudaError_t bfecc_nf(const BfeccArgs<Real> &a, const Fld<Real> &in,
                            const Fld<Real> &out, const Real *ar,
                            const Real *ac, const uint8_t *solid,
                            const Fld<Real> &uf, const Fld<Real> &ue,
                            cudaStream_t s) {
  const dim3 block(32, 8);
  const dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8);
  cudaError_t e = launch_pdl(bfecc_pass<1, NF, Real, HOLES, ADV2D>, grid,
                             block, 0, s, a, in, uf, ue, out, ar, ac, solid);
  if (e == cudaSuccess)
    e = launch_pdl(bfecc_pass<2, NF, Real, HOLES, ADV2D>, grid, block, 0, s,
                   a, in, uf, ue, out, ar, ac, solid);
  if (e == cudaSuccess)
    e = launch_pdl(bfecc_pass<3, NF, Real, HOLES, ADV2D>, grid, block, 0, s,
                   a, in, uf, ue, out, ar, ac, solid);
  return e;
}

template <typename Real, bool ADV2D>
static cudaError_t bfecc_dispatch(const yh_param_var &p, int nf,
                                  const Fld<Real> &in, const Fld<Real> &out,
                                  const Real *ar, const Real *ac,
                                  const uint8_t *solid, const Fld<Real> &uf,
                                  const Fld<Real> &ue, cudaStream_t s) {
  BfeccArgs<Real> a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.dt = (Real)p.dt;
  a.hx = (Real)p.hx;
  a.hy = (Real)p.hy;
  a.tc = (Real)p.tc;
  const bool holes = p.solidSwitch && solid;
  if (nf == 2)
    return holes ? bfecc_nf<2, Real, true, ADV2D>(a, in, out, ar, ac, solid,
                                                  uf, ue, s)
                 : bfecc_nf<2, Real, false, ADV2D>(a, in, out, ar, ac, solid,
                                                   uf, ue, s);
  return holes ? bfecc_nf<3, Real, true, ADV2D>(a, in, out, ar, ac, solid, uf,
                                                ue, s)
               : bfecc_nf<3, Real, false, ADV2D>(a, in, out, ar, ac, solid,
                                                 uf, ue, s);
}

template <typename Real>
cudaError_t launch_bfecc(const yh_param_var &p, int nf, const Fld<Real> &in,
                         const Fld<Real> &out, const Real *adv_rows,
                         const Real *adv_cols, const uint8_t *solid,
                         const Fld<Real> &uf, const Fld<Real> &ue,
                         cudaStream_t s) {
  return bfecc_dispatch<Real, false>(p, nf, in, out, adv_rows, adv_cols,
                                     solid, uf, ue, s);
}

cudaError_t launch_bfecc_fused(const yh_param_var &p, int nf,
                               const Fld<float> &in, const Fld<float> &out,
                               const float *adv_rows, const float *adv_cols,
                               const uint8_t *solid, cudaStream_t s) {
  BfeccArgs<float> a;
  a.nx = p.nx;
  a.ny = p.ny;
  a.dt = (float)p.dt;
  a.hx = (float)p.hx;
  a.hy = (float)p.hy;
  a.tc = (float)p.tc;
  const bool holes = p.solidSwitch && solid;
  if (p.nx < 2 || p.ny < 2) return cudaErrorInvalidValue;
  // out must not alias in: a block's ring cells are other blocks' output
  for (int f = 0; f < nf; ++f)
    for (int g = 0; g < nf; ++g)
      if (in.f[f] == out.f[g]) return cudaErrorInvalidValue;
  const dim3 block(32, 8);
  const dim3 grid((p.nx + kFuseTX - 1) / kFuseTX, (p.ny + kFuseTY - 1) / kFuseTY);
#define YH_BF(NF, H)                                                          \
  if (nf == NF && holes == H)                                                 \
    return launch_pdl(bfecc_fused<NF, H>, grid, block, 0, s, a, in, out,      \
                      adv_rows, adv_cols, solid);
  YH_BF(2, false)
  YH_BF(2, true)
  YH_BF(3, false)
  YH_BF(3, true)
#undef YH_BF
  return cudaErrorInvalidValue;
}

template <typename Real>
cudaError_t launch_bfecc_2d(const yh_param_var &p, int nf,
                            const Fld<Real> &in, const Fld<Real> &out,
                            const Real *adv_x, const Real *adv_y,
                            const uint8_t *solid, const Fld<Real> &uf,
                            const Fld<Real> &ue, cudaStream_t s) {
  return bfecc_dispatch<Real, true>(p, nf, in, out, adv_x, adv_y, solid, uf,
                                    ue, s);
}

#define YH_INST(Real)                                                         \
  template cudaError_t launch_tips<Real>(                                     \
      const yh_param_var &, const Real *, const Real *, bool, double, int *,  \
      yh_tip *, int, yh_sym_state *, unsigned int *, cudaStream_t,            \
      uint8_t *);                                                            \
  template cudaError_t launch_phase<Real>(                                    \
      const yh_param_var &, int, const Fld<Real> &, const Fld<Real> &,        \
      const Fld<Real> &, const Fld<Real> &, const Fld<Real> &,                \
      const double *, const double *, const uint8_t *, yh_sym_state *,        \
      void *, cudaStream_t);                                                  \
  template cudaError_t launch_template<Real>(                                 \
      const yh_param_var &, int, const Fld<Real> &, const Fld<Real> &,        \
      const Fld<Real> &, const Fld<Real> &, cudaStream_t);                    \
  template cudaError_t launch_bfecc<Real>(                                    \
      const yh_param_var &, int, const Fld<Real> &, const Fld<Real> &,        \
      const Real *, const Real *, const uint8_t *, const Fld<Real> &,         \
      const Fld<Real> &, cudaStream_t);                                       \
  template cudaError_t launch_bfecc_2d<Real>(                                 \
      const yh_param_var &, int, const Fld<Real> &, const Fld<Real> &,        \
      const Real *, const Real *, const uint8_t *, const Fld<Real> &,         \
      const Fld<Real> &, cudaStream_t);
YH_INST(float)
YH_INST(double)
#undef YH_INST

}  // namespace yh
