/*
 * ORACLE — TEST INFRASTRUCTURE ONLY (the rules are in yh_oracle_impl.h).
 *
 * FP64 tangent-linear model of the adjoint solver's forward map
 * (yh_adjoint_* in include/yolohtli.h): forward-mode differentiation by
 * dual numbers (value, derivative) of the same discrete steps, so it shares
 * no code and no derivation with the reverse sweep it checks. Given a
 * direction (dD per cell, dtheta for the 13 FK3V parameters) it returns the
 * loss L and the directional derivative dL = <dL/dD, dD> + <dL/dtheta,
 * dtheta>, which the adjoint's two gradients must reproduce.
 *
 * The map (one step, every cell):
 *   r = dt D / h^2, du = sum over the 4 faces of (r_c + r_m)/2 (u_m - u_c),
 *   m the mirrored neighbour (no-flux edges, helper_functions.cu:69-79);
 *   H1 = H(u - u_c), H2 = H(u - u_v): steps, or (1 + tanh(x/eps))/2;
 *   sig = 1 / (1 + 2^(k2 (u - u_csi))), k2 = -2k / ln 2;
 *   jp = s_tr - v (1 - u)(u - u_c) s_td, jn = u s_to, s_X = tc dt / tau_X;
 *   u' = u + tc du - (H1 jp + (1 - H1) jn - w sig s_tsi);
 *   v' = H1 (v - v s_tvp) + (1 - H1)(v + (1 - v)(H2 s_tv1m + (1 - H2) s_tv2m));
 *   w' = H1 (w - w s_twp) + (1 - H1)(w + (1 - w) s_twm)
 * (Fenton & Karma 1998 with the tc-scaled Euler step of the solver). The
 * loss sums (u - target)^2 at the probe cells (px sp + sp/2, py sp + sp/2)
 * on the states after every `frame` steps.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/yolohtli.h"

typedef struct {
  double v, d;
} dl;

static inline dl mk(double v, double d) {
  dl r = {v, d};
  return r;
}
static inline dl cst(double v) { return mk(v, 0.0); }
static inline dl add(dl a, dl b) { return mk(a.v + b.v, a.d + b.d); }
static inline dl sub(dl a, dl b) { return mk(a.v - b.v, a.d - b.d); }
static inline dl mul(dl a, dl b) { return mk(a.v * b.v, a.d * b.v + a.v * b.d); }
static inline dl dvd(dl a, dl b) {
  return mk(a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v));
}
static inline dl dexp2(dl a) {
  const double e = exp2(a.v);
  return mk(e, e * log(2.0) * a.d);
}
static inline dl dtanh(dl a) {
  const double t = tanh(a.v);
  return mk(t, (1.0 - t * t) * a.d);
}

/* H(x): a step (derivative 0) or (1 + tanh(x/eps)) / 2 */
static inline dl heav(dl x, double eps) {
  if (eps > 0.0)
    return mul(cst(0.5), add(cst(1.0), dtanh(dvd(x, cst(eps)))));
  return cst(x.v >= 0.0 ? 1.0 : 0.0);
}

static inline int mir(int i, int n) {
  if (i < 0) return -i;
  if (i > n - 1) return 2 * (n - 1) - i;
  return i;
}

/* fk, dfk: the 13 parameters and their direction, yh_fk_params order.
 * D, dD: nx*ny. u0/v0/w0: initial state. target: frames x npy x npx.
 * Returns L in *loss and dL in *dloss. */
int orc_adj_tlm(const yh_param_var *p, const yh_fk_params *fk,
                const yh_fk_params *dfk, double eps, int nsteps, int frame,
                int sp, const float *D, const float *dD, const float *u0,
                const float *v0, const float *w0, const float *target,
                double *loss, double *dloss) {
  const int nx = p->nx, ny = p->ny, n = nx * ny;
  const int npx = nx / sp, npy = ny / sp;
  const double tcdt = p->tc * p->dt, tc = p->tc;
  const double rs = p->dt / (p->hx * p->hx);
  /* raw coefficients with their tangents */
  const double *f = &fk->tau_d, *df = &dfk->tau_d;
  dl s[9];
  for (int q = 0; q < 9; ++q)
    s[q] = mk(tcdt / f[q], -tcdt / (f[q] * f[q]) * df[q]);
  const dl s_td = s[0], s_tr = s[1], s_tsi = s[2], s_to = s[3], s_tvp = s[4],
           s_tv1m = s[5], s_tv2m = s[6], s_twp = s[7], s_twm = s[8];
  const dl u_c = mk(fk->u_c, dfk->u_c), u_v = mk(fk->u_v, dfk->u_v);
  const dl u_csi = mk(fk->u_csi, dfk->u_csi);
  const dl k2 = mk(-2.0 * fk->k / log(2.0), -2.0 * dfk->k / log(2.0));
  dl *r = malloc(sizeof(dl) * n);
  dl *x = malloc(sizeof(dl) * 3 * n), *y = malloc(sizeof(dl) * 3 * n);
  if (!r || !x || !y) {
    free(r);
    free(x);
    free(y);
    return -1;
  }
  for (int c = 0; c < n; ++c) {
    r[c] = mk(rs * (double)D[c], rs * (double)dD[c]);
    x[c] = cst(u0[c]);
    x[n + c] = cst(v0[c]);
    x[2 * n + c] = cst(w0[c]);
  }
  dl L = cst(0.0);
  for (int t = 0; t < nsteps; ++t) {
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int c = i + nx * j;
        const int m[4] = {mir(i - 1, nx) + nx * j, mir(i + 1, nx) + nx * j,
                          i + nx * mir(j - 1, ny), i + nx * mir(j + 1, ny)};
        const dl u = x[c], v = x[n + c], w = x[2 * n + c];
        dl du = cst(0.0);
        for (int q = 0; q < 4; ++q)
          du = add(du, mul(mul(cst(0.5), add(r[c], r[m[q]])), sub(x[m[q]], u)));
        const dl H1 = heav(sub(u, u_c), eps), H2 = heav(sub(u, u_v), eps);
        const dl one = cst(1.0), L1 = sub(one, H1);
        const dl sig = dvd(one, add(one, dexp2(mul(k2, sub(u, u_csi)))));
        const dl jp = sub(s_tr, mul(mul(mul(v, sub(one, u)), sub(u, u_c)), s_td));
        const dl jn = mul(u, s_to);
        const dl Jd = sub(add(mul(H1, jp), mul(L1, jn)), mul(mul(w, sig), s_tsi));
        y[c] = sub(add(u, mul(cst(tc), du)), Jd);
        const dl sv = add(mul(H2, s_tv1m), mul(sub(one, H2), s_tv2m));
        const dl vp = sub(v, mul(v, s_tvp)), vm = add(v, mul(sub(one, v), sv));
        y[n + c] = add(mul(H1, vp), mul(L1, vm));
        const dl wp = sub(w, mul(w, s_twp)), wm = add(w, mul(sub(one, w), s_twm));
        y[2 * n + c] = add(mul(H1, wp), mul(L1, wm));
      }
    dl *tmp = x;
    x = y;
    y = tmp;
    if ((t + 1) % frame == 0) {
      const float *tg = target + (size_t)((t + 1) / frame - 1) * npx * npy;
      for (int py = 0; py < npy; ++py)
        for (int px = 0; px < npx; ++px) {
          const dl d = sub(x[(px * sp + sp / 2) + nx * (py * sp + sp / 2)],
                           cst((double)tg[px + npx * py]));
          L = add(L, mul(d, d));
        }
    }
  }
  free(r);
  free(x);
  free(y);
  *loss = L.v;
  *dloss = L.d;
  return 0;
}
