/*
 * ORACLE — TEST INFRASTRUCTURE ONLY (see yh_oracle_impl.h for the rules and
 * the parity pin). Built by oracle/build_oracle.sh into
 * oracle/_build/liboracle.so; loaded through ctypes by oracle/oracle.py.
 *
 * This translation unit instantiates the field operators in FP64 (_f64) and
 * FP32 (_f32) and adds the FP64-only parts: the tip tracker, the 3x3 solve,
 * the disc-centre choice and the symmetry-reduced step sequence.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/yolohtli.h"

#define REAL double
#define ORC_SUFFIX _f64
#define ORC_TANH tanh
#include "yh_oracle_impl.h"
#undef REAL
#undef ORC_SUFFIX
#undef ORC_TANH

#define REAL float
#define ORC_SUFFIX _f32
#define ORC_TANH tanhf
#include "yh_oracle_impl.h"
#undef REAL
#undef ORC_SUFFIX
#undef ORC_TANH

int orc_abi_version(void) { return 1; }

/* ---------------------------------------------------------------------- */
/* Spiral tip, closed-form bilinear isoline intersection                   */
/* (spiralTip_kernel, tipTracker.cu:20-208; tipRecordPlane :210-241)       */
/* ---------------------------------------------------------------------- */

/* Appends a tip if (s, t) lies strictly inside the unit cell
 * (tipTracker.cu:215,233-236). s and t are the float2 the kernel stores. */
static void orc_record(int i, int j, float s, float t, double ptime,
                       yh_tip *out, int cap, int *n) {
  if ((s > 0.0 && s < 1.0) && (t > 0.0 && t < 1.0)) {
    if (*n < cap) {
      yh_tip d;
      d.x = (float)i + s;
      d.y = (float)j + t;
      d.vx = 0.0f;
      d.vy = 0.0f;
      d.t = (float)ptime;
      out[*n] = d;
    }
    ++*n;
  }
}

/* One cell's two candidate tips from the corner values x1..x4 (present)
 * and y1..y4 (past), ordered (i,j), (i+1,j), (i+1,j+1), (i,j+1)
 * (tipTracker.cu:140-174). `need_disc` applies the square-domain test
 * disc >= 0 (tipTracker.cu:185,197). */
static void orc_tip_cell(double Uth, int i, int j, double x1, double x2,
                         double x3, double x4, double y1, double y2, double y3,
                         double y4, int need_disc, double ptime, yh_tip *out,
                         int cap, int *n) {
  const double x3y1 = x3 * y1, x4y1 = x4 * y1, x3y2 = x3 * y2, x4y2 = x4 * y2;
  const double x1y3 = x1 * y3, x2y3 = x2 * y3, x1y4 = x1 * y4, x2y4 = x2 * y4;
  const double x2y1 = x2 * y1, x1y2 = x1 * y2, x4y3 = x4 * y3, x3y4 = x3 * y4;
  const double den1 =
      2.0 * (x3y1 - x4y1 - x3y2 + x4y2 - x1y3 + x2y3 + x1y4 - x2y4);
  const double den2 =
      2.0 * (x2y1 - x3y1 - x1y2 + x4y2 + x1y3 - x4y3 - x2y4 + x3y4);
  const double ctn1 = x1 - x2 + x3 - x4 - y1 + y2 - y3 + y4;
  const double ctn2 = x3y1 - 2.0 * x4y1 + x4y2 - x1y3 + 2.0 * x1y4 - x2y4;
  const double q = -ctn2 + Uth * ctn1;
  const double disc =
      sqrt(4.0 * (x3y1 - x3y2 - x4y1 + x4y2 - x1y3 + x1y4 + x2y3 - x2y4) *
               (x4y1 - x1y4 + Uth * (x1 - x4 - y1 + y4)) +
           q * q);
  const double px = ctn2 - Uth * ctn1;
  const double py =
      Uth * ctn1 - x3y1 + x4y2 + x1y3 - x2y4 + 2.0 * (x2y1 - x1y2);
  const int ok = !need_disc || disc >= 0.0;
  float s = (float)((px + disc) / den1), t = (float)((py + disc) / den2);
  if (ok) orc_record(i, j, s, t, ptime, out, cap, n);
  s = (float)((px - disc) / den1);
  t = (float)((py - disc) / den2);
  if (ok) orc_record(i, j, s, t, ptime, out, cap, n);
}

/* All tips between `past` (y) and `present` (x), square branch
 * i in [1,nx-3], j in [1,ny-3] (tipTracker.cu:126), or, with holes, the
 * disc of radius^2 tipOffsetX*tipOffsetY around the grid centre
 * (tipTracker.cu:47-57). Returns the number found (may exceed cap). */
int orc_tips(const yh_param_var *p, const double *past, const double *present,
             const uint8_t *solid, double ptime, yh_tip *out, int cap) {
  const int nx = p->nx, ny = p->ny;
  int n = 0;
  const int holes = p->solidSwitch && solid;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      if (holes) {
        int ic = i - nx / 2, jc = j - ny / 2;
        if (!(ic * ic + jc * jc < p->tipOffsetX * p->tipOffsetY)) continue;
      } else if (!((i >= 1) && (i < nx - 2) && (j >= 1) && (j < ny - 2))) {
        continue;
      }
      const int s0 = i + nx * j;
      const int sx = (i < nx - 1) ? s0 + 1 : s0;
      const int sy = (j < ny - 1) ? s0 + nx : s0;
      const int sxy = ((j < ny - 1) && (i < nx - 1)) ? s0 + nx + 1 : s0;
      orc_tip_cell(p->Uth, i, j, present[s0], present[sx], present[sxy],
                   present[sy], past[s0], past[sx], past[sxy], past[sy],
                   !holes, ptime, out, cap, &n);
    }
  return n;
}

/* Deterministic disc-centre choice: the tip nearest to the previous centre,
 * ties broken by (y, x); the previous centre if there is no tip. */
void orc_pick_centre(const yh_tip *tips, int n, float centre[2]) {
  int best = -1;
  double bd = 0.0;
  for (int k = 0; k < n; ++k) {
    double dx = (double)tips[k].x - centre[0];
    double dy = (double)tips[k].y - centre[1];
    double d = dx * dx + dy * dy;
    if (best < 0 || d < bd ||
        (d == bd && (tips[k].y < tips[best].y ||
                     (tips[k].y == tips[best].y && tips[k].x < tips[best].x)))) {
      best = k;
      bd = d;
    }
  }
  if (best >= 0) {
    centre[0] = tips[best].x;
    centre[1] = tips[best].y;
  }
}

/* ---------------------------------------------------------------------- */
/* 3x3 drift / rotation solve (symmetryReduction.cu:386-412)               */
/* ---------------------------------------------------------------------- */

/* Row r of the system is
 *   [I[3r] cos(pt) + I[3r+1] sin(pt),  I[3r+1] cos(pt) - I[3r] sin(pt),  I[3r+2]] . c = I[9+r].
 * The reference eliminates without pivoting: rows 2 and 3 are scaled by
 * a1/b1 and a1/C1 and row 1 subtracted, then row 3 is eliminated against
 * row 2 the same way, then back substitution. Restated here step by step. */
void orc_solve_ref(const double I[12], const double phi[3], double c[3]) {
  const double cs = cos(phi[2]), sn = sin(phi[2]);
  double r[3][4];
  for (int k = 0; k < 3; ++k) {
    r[k][0] = I[3 * k] * cs + I[3 * k + 1] * sn;
    r[k][1] = I[3 * k + 1] * cs - I[3 * k] * sn;
    r[k][2] = I[3 * k + 2];
    r[k][3] = I[9 + k];
  }
  /* eliminate column 0 from rows 1 and 2 */
  double s1 = r[0][0] / r[1][0];
  double b2p = s1 * r[1][1] - r[0][1];
  double b3p = s1 * r[1][2] - r[0][2];
  double d2p = s1 * r[1][3] - r[0][3];
  double s2 = r[0][0] / r[2][0];
  double c2p = s2 * r[2][1] - r[0][1];
  double c3p = s2 * r[2][2] - r[0][2];
  double d3p = s2 * r[2][3] - r[0][3];
  /* eliminate column 1 from the last row */
  double s3 = b2p / c2p;
  double c3pp = s3 * c3p - b3p;
  double d3pp = s3 * d3p - d2p;
  c[2] = d3pp / c3pp;
  c[1] = (d2p - b3p * c[2]) / b2p;
  c[0] = (r[0][3] - r[0][1] * c[1] - r[0][2] * c[2]) / r[0][0];
}

/* ---------------------------------------------------------------------- */
/* Symmetry-reduced step sequence (main.cu:894-954)                        */
/* ---------------------------------------------------------------------- */

typedef struct orc_sr {
  yh_param_var p;
  yh_fk_params fk;
  int model, nf, template_mode;
  double c[3], phi[3], c_adv[3], phi_adv[3];
  double I[12];
  float centre[2];
  int step;
  int ntips;
  const uint8_t *solid;
  double *S[3], *R[3], *tan[3];
  double *cx[3], *cy[3], *ct[3], *tx[3], *ty[3], *tt[3];
  double *uf, *ue, *advx, *advy;
  yh_tip *tips;
  int tipcap;
} orc_sr;

static double *orc_zeros(size_t n) { return (double *)calloc(n, sizeof(double)); }

orc_sr *orc_sr_create(const yh_param_var *p, int model, const yh_fk_params *fk,
                      const uint8_t *solid, const double *const *state,
                      int template_mode, const double *const *templ) {
  orc_sr *s = (orc_sr *)calloc(1, sizeof(orc_sr));
  const size_t n = (size_t)p->nx * p->ny;
  s->p = *p;
  if (fk) s->fk = *fk;
  s->model = model;
  s->nf = model == YH_MODEL_FK3V ? 3 : 2;
  s->template_mode = template_mode;
  s->solid = solid;
  s->centre[0] = p->tipx;
  s->centre[1] = p->tipy;
  for (int f = 0; f < s->nf; ++f) {
    s->S[f] = orc_zeros(n);
    memcpy(s->S[f], state[f], n * sizeof(double));
    s->R[f] = orc_zeros(n);
    s->tan[f] = orc_zeros(n);
    s->cx[f] = orc_zeros(n);
    s->cy[f] = orc_zeros(n);
    s->ct[f] = orc_zeros(n);
    s->tx[f] = orc_zeros(n);
    s->ty[f] = orc_zeros(n);
    s->tt[f] = orc_zeros(n);
  }
  s->uf = orc_zeros(n);
  s->ue = orc_zeros(n);
  s->advx = orc_zeros((size_t)p->ny);
  s->advy = orc_zeros((size_t)p->nx);
  s->tipcap = 4096;
  s->tips = (yh_tip *)calloc((size_t)s->tipcap, sizeof(yh_tip));
  if (template_mode == YH_TEMPLATE_FROZEN && templ) {
    /* Template derivatives of the given state over the whole grid: a disc
     * of radius covering everything. */
    yh_param_var q = *p;
    q.tipOffsetX = q.tipOffsetY = 4 * (p->nx + p->ny);
    float cc[2] = {(float)(p->nx / 2), (float)(p->ny / 2)};
    orc_slices_f64(&q, s->nf, templ, s->advx, s->advy, NULL, cc, NULL, NULL,
                   NULL, s->tx, s->ty, s->tt);
  }
  return s;
}

void orc_sr_destroy(orc_sr *s) {
  if (!s) return;
  for (int f = 0; f < 3; ++f) {
    free(s->S[f]); free(s->R[f]); free(s->tan[f]);
    free(s->cx[f]); free(s->cy[f]); free(s->ct[f]);
    free(s->tx[f]); free(s->ty[f]); free(s->tt[f]);
  }
  free(s->uf); free(s->ue); free(s->advx); free(s->advy); free(s->tips);
  free(s);
}

/* slice + 12 integrals + solve on the current S (main.cu:906-926). */
static void orc_sr_phase(orc_sr *s) {
  const int current = s->template_mode == YH_TEMPLATE_CURRENT;
  yh_param_var *p = &s->p;
  orc_comoving_f64(p, s->c_adv, s->phi_adv, s->advx, s->advy);
  orc_slices_f64(p, s->nf, (const double *const *)s->S, s->advx, s->advy,
                 s->solid, s->centre, s->cx, s->cy, s->ct,
                 current ? s->tx : NULL, current ? s->ty : NULL,
                 current ? s->tt : NULL);
  /* Template arrays cover the grid in frozen mode; the integrals keep only
   * the disc (integralTrapz.cu:50-57). */
  orc_integrals_f64(p, s->nf, (const double *const *)s->tx,
                    (const double *const *)s->ty, (const double *const *)s->tt,
                    (const double *const *)s->cx, (const double *const *)s->cy,
                    (const double *const *)s->ct, (const double *const *)s->tan,
                    s->centre, s->I);
  orc_solve_ref(s->I, s->phi, s->c);
  for (int k = 0; k < 3; ++k) {
    s->c_adv[k] = s->c[k];
    s->phi_adv[k] = s->phi[k];
  }
}

/* One symmetry-reduced step (main.cu:894-954, Euler branch of phi):
 * RD S->R with tangent; tips between S.u (x) and R.u (y) (main.cu:900 and
 * the argument order of tip_wrapper); centre choice (count>0); slices,
 * integrals and solve on S (twice at count==0, main.cu:910-926); comoving
 * field; BFECC R->S; phi += dt*c. */
void orc_sr_step(orc_sr *s) {
  yh_param_var *p = &s->p;
  orc_rd_step_f64(p, s->model, &s->fk, (const double *const *)s->S, s->R,
                  s->tan, s->solid);
  const double ptime = p->dt * (double)s->step;
  s->ntips = orc_tips(p, s->R[0], s->S[0], s->solid, ptime, s->tips, s->tipcap);
  if (s->step > 0)
    orc_pick_centre(s->tips, s->ntips < s->tipcap ? s->ntips : s->tipcap,
                    s->centre);
  if (s->step == 0) orc_sr_phase(s);
  orc_sr_phase(s);
  orc_comoving_f64(p, s->c_adv, s->phi_adv, s->advx, s->advy);
  orc_bfecc_f64(p, s->nf, (const double *const *)s->R, s->S, s->advx, s->advy,
                s->solid, s->uf, s->ue);
  for (int k = 0; k < 3; ++k) s->phi[k] += p->dt * s->c[k];
  s->step += 1;
}

void orc_sr_get(const orc_sr *s, double *const *state, double c[3],
                double phi[3], double I[12], float centre[2], int *step,
                int *ntips) {
  const size_t n = (size_t)s->p.nx * s->p.ny;
  if (state)
    for (int f = 0; f < s->nf; ++f)
      if (state[f]) memcpy(state[f], s->S[f], n * sizeof(double));
  if (c) memcpy(c, s->c, sizeof(s->c));
  if (phi) memcpy(phi, s->phi, sizeof(s->phi));
  if (I) memcpy(I, s->I, sizeof(s->I));
  if (centre) { centre[0] = s->centre[0]; centre[1] = s->centre[1]; }
  if (step) *step = s->step;
  if (ntips) *ntips = s->ntips;
}

/* Tangent of the last RD of the sequence (for checks). */
void orc_sr_get_tangent(const orc_sr *s, double *const *tan) {
  const size_t n = (size_t)s->p.nx * s->p.ny;
  for (int f = 0; f < s->nf; ++f)
    if (tan[f]) memcpy(tan[f], s->tan[f], n * sizeof(double));
}

/* ---------------------------------------------------------------------- */
/* Plain multi-step driver (main.cu:876-887), FP64 and FP32                */
/* ---------------------------------------------------------------------- */

#define ORC_RUN(SUF, T)                                                        \
  void orc_run##SUF(const yh_param_var *p, int model, const yh_fk_params *fk, \
                    T *const *state, T *const *scratch, const uint8_t *solid,  \
                    int nsteps, const yh_stim *stims, int nstims,              \
                    int step0) {                                               \
    const int nf = model == YH_MODEL_FK3V ? 3 : 2;                             \
    T *a[3] = {state[0], state[1], nf > 2 ? state[2] : NULL};                  \
    T *b[3] = {scratch[0], scratch[1], nf > 2 ? scratch[2] : NULL};            \
    for (int s = 0; s < nsteps; ++s) {                                         \
      for (int k = 0; k < nstims; ++k)                                         \
        if (stims[k].step == step0 + s)                                        \
          orc_stimulate_box##SUF(p, a[0], solid, stims[k].i0, stims[k].j0,     \
                                 stims[k].i1, stims[k].j1,                     \
                                 (T)stims[k].value);                           \
      orc_rd_step##SUF(p, model, fk, (const T *const *)a, b, NULL, solid);     \
      for (int f = 0; f < 3; ++f) {                                            \
        T *t = a[f];                                                           \
        a[f] = b[f];                                                           \
        b[f] = t;                                                              \
      }                                                                        \
    }                                                                          \
    if (nsteps % 2) {                                                          \
      const size_t n = (size_t)p->nx * p->ny;                                  \
      for (int f = 0; f < nf; ++f) memcpy(state[f], a[f], n * sizeof(T));      \
    }                                                                          \
  }
ORC_RUN(_f64, double)
ORC_RUN(_f32, float)
