// Launchers of the yolohtli_gb300 kernels (host-callable, C++).
#pragma once

#include <type_traits>

#include "yh_common.cuh"

namespace yh {

template <typename Real>
inline bool aligned16(const Fld<Real> &x, int model) {
  const int nf = model == YH_MODEL_FK3V ? 3 : 2;
  for (int f = 0; f < nf; ++f)
    if (reinterpret_cast<uintptr_t>(x.f[f]) & 15) return false;
  return true;
}

// yh_rd.cu
template <typename Real>
cudaError_t launch_rd_step(const StepCoeffs<Real> &a, const Fld<Real> &in,
                           const Fld<Real> &out, const Fld<Real> &tan,
                           const uint8_t *solid, cudaStream_t s);
template <typename Real>
cudaError_t launch_stimulate(Real *u, const uint8_t *solid, int nx, int ny,
                             int i0, int j0, int i1, int j1, Real value,
                             cudaStream_t s);

// yh_sr.cu
template <typename Real>
cudaError_t launch_tips(const yh_param_var &p, const Real *past,
                        const Real *present, const uint8_t *solid,
                        double ptime, int *count, yh_tip *vec, int cap,
                        yh_sym_state *sym_pick, unsigned int *done,
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
cudaError_t launch_sym_advance(const yh_param_var &p, yh_sym_state *sym,
                               cudaStream_t s);

// yh_params.cu
template <typename Real>
StepCoeffs<Real> make_step_coeffs(const yh_param_var &p, int model,
                                  const yh_fk_params *fk);

}  // namespace yh
