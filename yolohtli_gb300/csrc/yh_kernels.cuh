// Launchers of the yolohtli_gb300 kernels (host-callable, C++).
#pragma once

#include <type_traits>
#include <utility>

#include "yh_common.cuh"

namespace yh {

// Launch with programmatic stream serialization: the kernel's blocks may be
// scheduled while the previous kernel on the stream drains. Every kernel
// launched this way calls grid_dep_wait() as its first statement, so it
// still starts its work only after its predecessor has completed, and the
// chain stays ordered.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block,
                              size_t smem, cudaStream_t s, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <typename Real>
inline bool aligned16(const Fld<Real> &x, int model) {
  const int nf = model == YH_MODEL_FK3V ? 3 : 2;
  for (int f = 0; f < nf; ++f)
    if (reinterpret_cast<uintptr_t>(x.f[f]) & 15) return false;
  return true;
}

// yh_rd.cu
// codes: optional per-cell hole codes of `solid` (launch_hole_codes), used
// by the FP32 float4 kernel; the scalar kernels read `solid`. reset:
// optional counter the launch sets to 0 (the symmetry-reduced step's tip
// count, so no memset node sits between its kernels).
template <typename Real>
cudaError_t launch_rd_step(const StepCoeffs<Real> &a, const Fld<Real> &in,
                           const Fld<Real> &out, const Fld<Real> &tan,
                           const uint8_t *solid, cudaStream_t s,
                           const uint8_t *codes = nullptr,
                           int *reset = nullptr);
cudaError_t launch_hole_codes(const uint8_t *solid, int nx, int ny,
                              uint8_t *codes, cudaStream_t s);
template <typename Real>
cudaError_t launch_stimulate(Real *u, const uint8_t *solid, int nx, int ny,
                             int i0, int j0, int i1, int j1, Real value,
                             cudaStream_t s);

// yh_rd_tb.cu
int rd_tb_max_steps();
cudaError_t launch_rd_tb(const StepCoeffs<float> &a, const Fld<float> &in,
                         const Fld<float> &out, const uint8_t *solid,
                         int nsteps, cudaStream_t s);

// yh_rd_2s.cu: two FK3V steps per launch (codes: hole codes or null)
bool rd_2s_supported(const StepCoeffs<float> &a, const Fld<float> &in,
                     const Fld<float> &out, bool holes, const uint8_t *codes);
// With err (a device flag), the tile inputs arrive by TMA bulk tensor copies
// where the rows allow it (nx % 4; with hole codes nx % 16); an expired
// wait sets *err. The same bits either way.
cudaError_t launch_rd_2s(const StepCoeffs<float> &a, const Fld<float> &in,
                         const Fld<float> &out, const uint8_t *codes,
                         int *err, cudaStream_t s);

// yh_rd_resident.cu
constexpr int kResMaxStims = 32;  // stimulus events per resident launch
struct ResidentPlan {
  bool ok;
  int nb, rq, rrem, rmax;  // blocks, rows per block (rq or rq+1), max rows
  int threads;             // compute threads per block (+ 64 or 128 receiving)
  size_t smem;             // dynamic shared memory per block
};
ResidentPlan resident_plan(const StepCoeffs<float> &a, int device);
// bytes of the tagged boundary-row buffers of a plan
size_t resident_halo_bytes(const ResidentPlan &pl, int nx);
// io: the state, updated in place; prev_u (may be null): receives u of the
// level before the last step. mute >= 0: that block publishes no boundary
// row, so its neighbours' bounded waits run out (the failure self-test).
cudaError_t launch_rd_resident(const StepCoeffs<float> &a, const Fld<float> &io,
                               float *prev_u, const uint8_t *solid,
                               int nsteps, int step0,
                               const yh_stim *stims, int nstims,
                               const ResidentPlan &pl,
                               unsigned long long *halo, int *error,
                               cudaStream_t s, int mute = -1);

// yh_sr.cu
// holes: the hole-domain branch of the reference (a disc around the grid
// centre, tipTracker.cu:47-122); it does not read the mask itself.
// p.tipAlgorithm (1 closed form, 2 Newton) and p.tipGrad select the kernel;
// plot (may be null) gets the cells of the tips marked.
template <typename Real>
cudaError_t launch_tips(const yh_param_var &p, const Real *past,
                        const Real *present, bool holes, double ptime,
                        int *count, yh_tip *vec, int cap,
                        yh_sym_state *sym_pick, unsigned int *done,
                        cudaStream_t s, uint8_t *plot = nullptr);

// yh_analysis.cu: tipAlgorithm 3 (filament cells), contours, space APD
template <typename Real>
cudaError_t launch_filament(const yh_param_var &p, const Real *past,
                            const Real *present, uint8_t *mark,
                            cudaStream_t s);
template <typename Real>
cudaError_t launch_contour(const yh_param_var &p, const Real *field1,
                           const Real *field2, const uint8_t *stim_area,
                           int mode, float time, int *count,
                           yh_contour_pt *vec, int cap, uint8_t *plot,
                           cudaStream_t s);
template <typename Real>
struct ApdFields {
  Real *apd1, *apd2, *sapd, *dapd, *back, *front;
  uint8_t *first;
};
template <typename Real>
cudaError_t launch_space_apd(const yh_param_var &p, int count,
                             const Real *uold, const Real *unew,
                             const ApdFields<Real> &f,
                             const uint8_t *stim_area, bool stimulate,
                             cudaStream_t s);
cudaError_t launch_pick_centre(const int *count, const yh_tip *vec, int cap,
                               yh_sym_state *sym, cudaStream_t s);

size_t phase_workspace_bytes(const yh_param_var &p);
template <typename Real>
cudaError_t launch_phase(const yh_param_var &p, int nf, const Fld<Real> &st,
                         const Fld<Real> &tan, const Fld<Real> &tx,
                         const Fld<Real> &ty, const Fld<Real> &tt,
                         const double *adv_rows, const double *adv_cols,
                         const uint8_t *solid, yh_sym_state *sym,
                         void *workspace, cudaStream_t s);
// The phase launch of the FP32 symmetry-reduced step: upwinds by the FP32
// comoving field adv_rows/adv_cols and, in its last block, rewrites that
// field from the new c (the comoving launch folded in); with `advance`
// also phi += dt*c, step += 1.
cudaError_t launch_phase_comoving(const yh_param_var &p, int nf,
                                  const Fld<float> &st, const Fld<float> &tan,
                                  const Fld<float> &tx, const Fld<float> &ty,
                                  const Fld<float> &tt, float *adv_rows,
                                  float *adv_cols, const uint8_t *solid,
                                  yh_sym_state *sym, void *workspace,
                                  bool advance, cudaStream_t s);
template <typename Real>
cudaError_t launch_template(const yh_param_var &p, int nf,
                            const Fld<Real> &st, const Fld<Real> &tx,
                            const Fld<Real> &ty, const Fld<Real> &tt,
                            cudaStream_t s);
cudaError_t launch_comoving(const yh_param_var &p, yh_sym_state *sym,
                            double *adv_rows, double *adv_cols,
                            float *adv_rows_f, float *adv_cols_f,
                            bool advance, cudaStream_t s);
template <typename Real>
cudaError_t launch_bfecc(const yh_param_var &p, int nf, const Fld<Real> &in,
                         const Fld<Real> &out, const Real *adv_rows,
                         const Real *adv_cols, const uint8_t *solid,
                         const Fld<Real> &uf, const Fld<Real> &ue,
                         cudaStream_t s);
// The three passes in one launch (FP32, separable comoving field): the
// same values, bit for bit; no uf/ue scratch in global memory.
cudaError_t launch_bfecc_fused(const yh_param_var &p, int nf,
                               const Fld<float> &in, const Fld<float> &out,
                               const float *adv_rows, const float *adv_cols,
                               const uint8_t *solid, cudaStream_t s);
// The same passes reading a full nx*ny comoving field (adv_x, adv_y), as
// the reference's advFDBFECC_kernel receives it.
template <typename Real>
cudaError_t launch_bfecc_2d(const yh_param_var &p, int nf,
                            const Fld<Real> &in, const Fld<Real> &out,
                            const Real *adv_x, const Real *adv_y,
                            const uint8_t *solid, const Fld<Real> &uf,
                            const Fld<Real> &ue, cudaStream_t s);

// FP64 3x3 solve of the drift/rotation system with partial pivoting.
// Row r: [I[3r] cos(pt) + I[3r+1] sin(pt), I[3r+1] cos(pt) - I[3r] sin(pt),
// I[3r+2]] . c = I[9+r]  (symmetryReduction.cu:390-396). Returns YH_OK, or
// YH_ESINGULAR when a pivot is below 1e-13 of the largest entry (the
// reference divides by unpivoted entries, symmetryReduction.cu:398-412).
// solve3 with cos(pt), sin(pt) given.
__host__ __device__ inline int solve3_cs(const double I[12], double cs,
                                         double sn, double c[3]) {
  double A[3][4];
  double amax = 0.0;
  for (int r = 0; r < 3; ++r) {
    A[r][0] = I[3 * r] * cs + I[3 * r + 1] * sn;
    A[r][1] = I[3 * r + 1] * cs - I[3 * r] * sn;
    A[r][2] = I[3 * r + 2];
    A[r][3] = I[9 + r];
    for (int k = 0; k < 3; ++k) amax = fmax(amax, fabs(A[r][k]));
  }
  if (!(amax > 0.0) || !isfinite(amax)) return YH_ESINGULAR;
  const double tol = 1e-13 * amax;
  for (int col = 0; col < 3; ++col) {
    int piv = col;
    for (int r = col + 1; r < 3; ++r)
      if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
    if (!(fabs(A[piv][col]) > tol)) return YH_ESINGULAR;
    if (piv != col)
      for (int k = 0; k < 4; ++k) {
        const double t = A[col][k];
        A[col][k] = A[piv][k];
        A[piv][k] = t;
      }
    for (int r = col + 1; r < 3; ++r) {
      const double m = A[r][col] / A[col][col];
      for (int k = col; k < 4; ++k) A[r][k] -= m * A[col][k];
    }
  }
  double x[3];
  for (int r = 2; r >= 0; --r) {
    double s = A[r][3];
    for (int k = r + 1; k < 3; ++k) s -= A[r][k] * x[k];
    x[r] = s / A[r][r];
  }
  for (int k = 0; k < 3; ++k) c[k] = x[k];
  return YH_OK;
}
__host__ __device__ inline int solve3(const double I[12], double pt,
                                      double c[3]) {
  return solve3_cs(I, cos(pt), sin(pt), c);
}
// The same system by cofactors (Cramer's rule): one reciprocal and a short
// chain of FMAs instead of the pivoted elimination's dependent divisions,
// for the FP32 engine's last block, where this chain is serial FP64 work.
// YH_ESINGULAR when |det| <= 1e-13 amax^3 (amax the largest entry), or the
// system is not finite.
__host__ __device__ inline int solve3_cofactor(const double I[12], double cs,
                                               double sn, double c[3]) {
  double A[3][3], b[3];
  double amax = 0.0;
  for (int r = 0; r < 3; ++r) {
    A[r][0] = I[3 * r] * cs + I[3 * r + 1] * sn;
    A[r][1] = I[3 * r + 1] * cs - I[3 * r] * sn;
    A[r][2] = I[3 * r + 2];
    b[r] = I[9 + r];
    for (int k = 0; k < 3; ++k) amax = fmax(amax, fabs(A[r][k]));
  }
  if (!(amax > 0.0) || !isfinite(amax)) return YH_ESINGULAR;
  // cofactors C[r][k] of A
  const double C00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
  const double C01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  const double C02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  const double C10 = A[0][2] * A[2][1] - A[0][1] * A[2][2];
  const double C11 = A[0][0] * A[2][2] - A[0][2] * A[2][0];
  const double C12 = A[0][1] * A[2][0] - A[0][0] * A[2][1];
  const double C20 = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  const double C21 = A[0][2] * A[1][0] - A[0][0] * A[1][2];
  const double C22 = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  const double det = A[0][0] * C00 + A[0][1] * C01 + A[0][2] * C02;
  if (!(fabs(det) > 1e-13 * amax * amax * amax) || !isfinite(det))
    return YH_ESINGULAR;
  const double inv = 1.0 / det;
  c[0] = (C00 * b[0] + C10 * b[1] + C20 * b[2]) * inv;
  c[1] = (C01 * b[0] + C11 * b[1] + C21 * b[2]) * inv;
  c[2] = (C02 * b[0] + C12 * b[1] + C22 * b[2]) * inv;
  return YH_OK;
}
cudaError_t launch_sym_advance(const yh_param_var &p, yh_sym_state *sym,
                               cudaStream_t s);

// yh_params.cu
template <typename Real>
StepCoeffs<Real> make_step_coeffs(const yh_param_var &p, int model,
                                  const yh_fk_params *fk);

}  // namespace yh
