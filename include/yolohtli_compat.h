/*
 * yolohtli_gb300 — FP64 drop-in for the reference's own host entry points.
 *
 * libyolohtli_gb300.so also exports, with identical C++ signatures (and so
 * identical mangled symbols), the seven host wrappers of the reference's
 * hot path declared in its hostPrototypes.h:22-42 and the two of its
 * contour/APD analysis (hostPrototypes.h:46-51):
 *
 *   reactionDiffusion_wrapper   (reactionDiffusion.cu:568-577)
 *   tip_wrapper                 (tipTracker.cu:569-611), tipAlgorithm 1-3
 *   slice_wrapper               (symmetryReduction.cu:312-322)
 *   Cxy_field_wrapper           (symmetryReduction.cu:64-70)
 *   advFDBFECC_wrapper          (advFDBFECC.cu:355-362)
 *   solve_matrix                (symmetryReduction.cu:329-420)
 *   trapz_wrapper               (integralTrapz.cu:85-184)
 *   countour_wrapper            (spaceAPD.cu:257-276)
 *   sAPD_wrapper                (spaceAPD.cu:376-383)
 *
 * They take the reference's FP64 buffers (REAL = double) and run this
 * library's kernels instantiated in FP64, so a driver written against the
 * reference (its main.cu) links against this library instead of the
 * reference's kernel translation units. The reference passes its
 * parameters through process-global __constant__ symbols (main.cu:40-51)
 * that live in the caller's own device code; this library cannot read
 * them, so the driver hands over the same paramVar once more with
 * yh_compat_set_params() after its cudaMemcpyToSymbol block (main.cu:309-402).
 *
 * Semantics are the reference's, with these differences: every wrapper
 * rejects options off this path (RK2/RK4, lap4, anisotropy, Dirichlet,
 * slice scheme != 2) through yh_compat_last_error() instead of running
 * them; advFDBFECC_wrapper runs BFECC as three race-free passes (the
 * reference's single launch reads neighbours written in the same launch)
 * and leaves ub untouched; the tip and contour marks drop a mark whose
 * index falls outside the plot array and the contour kernel reads no value
 * past the end of field2 (the reference writes and reads there);
 * slice/trapz take the disc centre from
 * tipx/tipy when count == 0 or no tip was found (the reference then reads
 * tip_vector[-1]); solve_matrix pivots.
 *
 * The wrappers return void like the reference's; errors are kept in a
 * last-error slot instead of being dropped.
 */
#ifndef YOLOHTLI_GB300_COMPAT_H
#define YOLOHTLI_GB300_COMPAT_H

#include "yolohtli.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The parameters the compat wrappers use, layout-identical to paramVar. */
int yh_compat_set_params(const yh_param_var *p);

/* Status of the most recent compat wrapper call (YH_OK or YH_E*). */
int yh_compat_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* YOLOHTLI_GB300_COMPAT_H */
