/*
 * ORACLE — TEST INFRASTRUCTURE ONLY. Never linked into, loaded by or called
 * from the product library; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py use it, as the checker.
 *
 * A CPU restatement, in plain C, of the reference's algorithm for the 2D
 * monodomain hot path of Yolohtli. This file is included twice by
 * yh_oracle.c, once with REAL = double (suffix _f64, the oracle proper) and
 * once with REAL = float (suffix _f32, the FP32 transcription timed as the
 * CPU baseline). Each function cites the reference file:line it follows.
 *
 * Parity pin: the _f64 functions are checked against the reference's own
 * CUDA kernels, compiled unchanged for sm_103a and run headless (see
 * oracle/ref_build.sh, oracle/ref_harness.cpp), through the golden fixtures
 * in tests/golden/. FK3V has no reference counterpart: its oracle is a
 * restatement of Fenton & Karma, Chaos 8:20 (1998), eqs. (1)-(6).
 *
 * Semantics kept from the reference, on purpose:
 *  - mirror ghost cells coord_i(-1)=1, coord_i(nx)=nx-2 (helper_functions.cu:69-79);
 *  - hole coefficients (1,2,1)/(2,2,0)/(0,2,2)/(0,0,0) (reactionDiffusion.cu:162-169);
 *  - non-tissue cells set to 0 after the step (reactionDiffusion.cu:521-535);
 *  - BFECC index swaps at the domain edge (advFDBFECC.cu:112-126), but as
 *    three separate passes (the reference reads neighbours written in the
 *    same launch, a race);
 *  - slice disc centre rounding with __float2int_rn on floats
 *    (symmetryReduction.cu:98-107) and the corner origin x=i, y=j;
 *  - the integrals' effective weight hx*hy over the open disc
 *    (integralTrapz.cu:50-57,79).
 * Differences, on purpose (each one is a defect of the reference):
 *  - y = j instead of (i2d/nx)%nx (symmetryReduction.cu:46,110; equal when ny<=nx);
 *  - the disc centre is the tip nearest to the previous centre, not the
 *    last one pushed by an atomic (symmetryReduction.cu:102-103).
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define SFX(name) CAT(name, ORC_SUFFIX)

/* coord_i / coord_j (helper_functions.cu:69-79): mirror about the edge cell. */
static inline int SFX(orc_mirror)(int i, int n) {
  if (i < 0) return -i;
  if (i >= n) return 2 * (n - 1) - i;
  return i;
}

/* ---------------------------------------------------------------------- */
/* Reaction terms                                                          */
/* ---------------------------------------------------------------------- */

/* REF2V currents (reactionDiffusion.cu:131-141), mouse stimulus off. */
static inline void SFX(orc_ref2v_currents)(const yh_param_var *p, REAL u,
                                           REAL v, REAL *I_sum, REAL *I_v) {
  REAL mu = (REAL)p->mu, alpha = (REAL)p->alpha, eps = (REAL)p->eps;
  REAL delta = (REAL)p->delta, gamma = (REAL)p->gamma, beta = (REAL)p->beta;
  REAL theta = (REAL)p->theta;
  *I_sum = -(mu * u * ((REAL)1.0 - u) * (u - alpha) - u * v);
  *I_v = -(eps * (delta * (u - gamma) * (beta - u) - v - theta));
}

/* Fenton-Karma 3V (Chaos 8:20, 1998), eqs. (2)-(6):
 *   p = H(u - u_c), q = H(u - u_v)
 *   J_fi = -v p (1-u)(u-u_c)/tau_d
 *   J_so = u (1-p)/tau_0 + p/tau_r
 *   J_si = -w (1 + tanh(k(u-u_csi)))/(2 tau_si)
 *   dv/dt = (1-p)(1-v)/tau_v^-(u) - p v/tau_v^+,
 *           tau_v^-(u) = q tau_v1^- + (1-q) tau_v2^-
 *   dw/dt = (1-p)(1-w)/tau_w^- - p w/tau_w^+
 * Returns the ionic current J = J_fi + J_so + J_si and the gate rates. */
static inline void SFX(orc_fk3v_rates)(const yh_fk_params *fk, REAL u, REAL v,
                                       REAL w, REAL *J, REAL *dv, REAL *dw) {
  int p = u >= (REAL)fk->u_c;
  int q = u >= (REAL)fk->u_v;
  REAL jfi = p ? -v * ((REAL)1.0 - u) * (u - (REAL)fk->u_c) / (REAL)fk->tau_d
               : (REAL)0.0;
  REAL jso = p ? (REAL)1.0 / (REAL)fk->tau_r : u / (REAL)fk->tau_0;
  REAL jsi = -w * ((REAL)1.0 + ORC_TANH((REAL)fk->k * (u - (REAL)fk->u_csi))) /
             ((REAL)2.0 * (REAL)fk->tau_si);
  REAL tvm = q ? (REAL)fk->tau_v1_minus : (REAL)fk->tau_v2_minus;
  *J = jfi + jso + jsi;
  *dv = p ? -v / (REAL)fk->tau_v_plus : ((REAL)1.0 - v) / tvm;
  *dw = p ? -w / (REAL)fk->tau_w_plus : ((REAL)1.0 - w) / (REAL)fk->tau_w_minus;
}

/* ---------------------------------------------------------------------- */
/* Explicit Euler reaction-diffusion step                                  */
/* ---------------------------------------------------------------------- */

/* Hole coefficients of one axis (reactionDiffusion.cu:162-169):
 * (lo, centre, hi) weights for the neighbours lo (W or N), hi (E or S). */
static inline void SFX(orc_hole_coeffs)(int s_lo, int s_c, int s_hi,
                                        REAL *c_lo, REAL *c_c, REAL *c_hi) {
  *c_lo = (s_lo && s_hi) && (s_lo && s_c) ? (REAL)1.0
                                          : ((s_lo && s_c) ? (REAL)2.0 : (REAL)0.0);
  *c_c = s_c ? ((s_lo || s_hi) ? (REAL)2.0 : (REAL)0.0) : (REAL)0.0;
  *c_hi = (s_lo && s_hi) && (s_c && s_hi) ? (REAL)1.0
                                          : ((s_c && s_hi) ? (REAL)2.0 : (REAL)0.0);
}

/* One Euler step of the whole grid (reactionDiffusion.cu:100-199,498-561,
 * timeIntOrder=1, Neumann, lap4=0, no anisotropy). in/out/tan are nf field
 * pointers (u, v[, w]); tan may be NULL. For REF2V, v diffuses with rscale
 * only when gateDiff (reactionDiffusion.cu:175,192); FK3V v, w never diffuse.
 * The tangent is (rhs)/dt (reactionDiffusion.cu:529-530,551-552), written
 * whenever tan != NULL (the reference writes it only when gateDiff). */
void SFX(orc_rd_step)(const yh_param_var *p, int model, const yh_fk_params *fk,
                      const REAL *const *in, REAL *const *out, REAL *const *tan,
                      const uint8_t *solid) {
  const int nx = p->nx, ny = p->ny;
  const REAL rx = (REAL)p->rx, ry = (REAL)p->ry, dt = (REAL)p->dt;
  const REAL tc = (REAL)p->tc, rscale = (REAL)p->rscale;
  const int holes = p->solidSwitch && solid;
  const int nf = model == YH_MODEL_FK3V ? 3 : 2;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const int C = i + nx * j;
      const int S = i + nx * SFX(orc_mirror)(j - 1, ny);
      const int N = i + nx * SFX(orc_mirror)(j + 1, ny);
      const int W = SFX(orc_mirror)(i - 1, nx) + nx * j;
      const int E = SFX(orc_mirror)(i + 1, nx) + nx * j;
      const REAL *U = in[0], *V = in[1];
      const REAL u = U[C], v = V[C];
      REAL cxw = 1, cxc = 2, cxe = 1, cyn = 1, cyc = 2, cys = 1;
      int sc = 1;
      if (holes) {
        sc = solid[C] != 0;
        SFX(orc_hole_coeffs)(solid[W] != 0, sc, solid[E] != 0, &cxw, &cxc, &cxe);
        SFX(orc_hole_coeffs)(solid[N] != 0, sc, solid[S] != 0, &cyn, &cyc, &cys);
      }
      REAL du, rhs[3];
      if (holes)
        du = (cxw * U[W] - cxc * u + cxe * U[E]) * rx +
             (cyn * U[N] - cyc * u + cys * U[S]) * ry;
      else
        du = (U[W] - (REAL)2.0 * u + U[E]) * rx +
             (U[N] - (REAL)2.0 * u + U[S]) * ry;
      if (model == YH_MODEL_REF2V) {
        REAL I_sum, I_v, dv = 0;
        SFX(orc_ref2v_currents)(p, u, v, &I_sum, &I_v);
        if (p->gateDiff) {
          if (holes)
            dv = (cxw * V[W] - cxc * v + cxe * V[E]) * rx * rscale +
                 (cyn * V[N] - cyc * v + cys * V[S]) * ry * rscale;
          else
            dv = (V[W] - (REAL)2.0 * v + V[E]) * rx * rscale +
                 (V[N] - (REAL)2.0 * v + V[S]) * ry * rscale;
        }
        du -= dt * I_sum;
        dv -= dt * I_v;
        rhs[0] = du;
        rhs[1] = dv;
      } else {
        const REAL w = in[2][C];
        REAL J, gv, gw;
        SFX(orc_fk3v_rates)(fk, u, v, w, &J, &gv, &gw);
        du -= dt * J;
        rhs[0] = du;
        rhs[1] = dt * gv;
        rhs[2] = dt * gw;
      }
      for (int f = 0; f < nf; ++f) {
        const REAL x0 = in[f][C];
        out[f][C] = sc ? x0 + tc * rhs[f] : (REAL)0.0;
        if (tan && tan[f]) tan[f][C] = sc ? rhs[f] / dt : (REAL)0.0;
      }
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Stimulus                                                                */
/* ---------------------------------------------------------------------- */
void SFX(orc_stimulate_box)(const yh_param_var *p, REAL *u, const uint8_t *solid,
                            int i0, int j0, int i1, int j1, REAL value) {
  const int nx = p->nx, ny = p->ny;
  if (i0 < 0) i0 = 0;
  if (j0 < 0) j0 = 0;
  if (i1 > nx) i1 = nx;
  if (j1 > ny) j1 = ny;
  for (int j = j0; j < j1; ++j)
    for (int i = i0; i < i1; ++i) {
      const int C = i + nx * j;
      if (!(p->solidSwitch && solid) || solid[C]) u[C] = value;
    }
}

/* ---------------------------------------------------------------------- */
/* Comoving field (Cxy_field_kernel, symmetryReduction.cu:20-62)           */
/* ---------------------------------------------------------------------- */
/* adv.x depends on the row only, adv.y on the column only:
 * adv_x[j] = hy*y*ct - cx*cos(pt) + cy*sin(pt), adv_y[i] = -hx*x*ct - cx*sin(pt) - cy*cos(pt). */
void SFX(orc_comoving)(const yh_param_var *p, const double c[3],
                       const double phi[3], double *adv_x_rows,
                       double *adv_y_cols) {
  const double cs = cos(phi[2]), sn = sin(phi[2]);
  for (int j = 0; j < p->ny; ++j) {
    const double y = (double)j;
    adv_x_rows[j] = p->hy * y * c[2] - c[0] * cs + c[1] * sn;
  }
  for (int i = 0; i < p->nx; ++i) {
    const double x = (double)i;
    adv_y_cols[i] = -p->hx * x * c[2] - c[0] * sn - c[1] * cs;
  }
}

/* ---------------------------------------------------------------------- */
/* BFECC advection (advFDBFECC.cu:18-165, Neumann, square or holes)        */
/* ---------------------------------------------------------------------- */

/* Upwind ratios of a cell: cx = -adv.x, Rx = sign(cx)*cx*dt/hx
 * (advFDBFECC.cu:30-34). adv is 0 on non-tissue cells (symmetryReduction.cu:50-51). */
static inline void SFX(orc_bfecc_ratios)(const yh_param_var *p, double ax,
                                         double ay, REAL *cx, REAL *cy,
                                         REAL *Rx, REAL *Ry) {
  REAL x = (REAL)(-ax), y = (REAL)(-ay);
  REAL sx = x > 0 ? (REAL)1 : (x < 0 ? (REAL)-1 : (REAL)0);
  REAL sy = y > 0 ? (REAL)1 : (y < 0 ? (REAL)-1 : (REAL)0);
  *cx = x;
  *cy = y;
  *Rx = sx * x * (REAL)p->dt / (REAL)p->hx;
  *Ry = sy * y * (REAL)p->dt / (REAL)p->hy;
}

/* Neighbour indices of the BFECC passes (advFDBFECC.cu:112-126): the forward
 * neighbours W,E,S,N and the backward pairs (i2dW,W2), (i2dE,E2), ... The
 * hole variant replaces "outside the domain" by "not tissue" with the same
 * swaps, using the mask in the geometric sense (S = j-1, N = j+1). */
typedef struct {
  int W, E, S, N, cW, W2, cE, E2, cS, S2, cN, N2;
} SFX(orc_bfecc_idx);

static inline SFX(orc_bfecc_idx) SFX(orc_bfecc_neighbours)(
    const yh_param_var *p, const uint8_t *solid, int i, int j) {
  const int nx = p->nx, ny = p->ny, C = i + nx * j;
  int hw = i > 0, he = i < nx - 1, hs = j > 0, hn = j < ny - 1;
  if (p->solidSwitch && solid) {
    if (!solid[C]) {
      SFX(orc_bfecc_idx) r = {C, C, C, C, C, C, C, C, C, C, C, C};
      return r;
    }
    hw = hw && solid[C - 1];
    he = he && solid[C + 1];
    hs = hs && solid[C - nx];
    hn = hn && solid[C + nx];
  }
  SFX(orc_bfecc_idx) r;
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

/* Three race-free passes per field: uf = F(in); ue = in - (F^-1(uf) - in)/2;
 * out = F(ue), with F the first-order upwind step (advFDBFECC.cu:128-144).
 * uf and ue are scratch arrays of nx*ny. */
void SFX(orc_bfecc)(const yh_param_var *p, int nf, const REAL *const *in,
                    REAL *const *out, const double *adv_x_rows,
                    const double *adv_y_cols, const uint8_t *solid, REAL *uf,
                    REAL *ue) {
  const int nx = p->nx, ny = p->ny;
  const REAL tc = (REAL)p->tc;
  const int holes = p->solidSwitch && solid;
  for (int f = 0; f < nf; ++f) {
    const REAL *g = in[f];
    REAL *o = out[f];
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int C = i + nx * j;
        const int sc = !holes || solid[C];
        REAL cx, cy, Rx, Ry;
        SFX(orc_bfecc_ratios)(p, sc ? adv_x_rows[j] : 0.0,
                              sc ? adv_y_cols[i] : 0.0, &cx, &cy, &Rx, &Ry);
        SFX(orc_bfecc_idx) n = SFX(orc_bfecc_neighbours)(p, solid, i, j);
        REAL FDx = cx > 0 ? g[C] - g[n.W] : g[C] - g[n.E];
        REAL FDy = cy > 0 ? g[C] - g[n.S] : g[C] - g[n.N];
        uf[C] = g[C] - tc * (Rx * FDx + Ry * FDy);
      }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int C = i + nx * j;
        const int sc = !holes || solid[C];
        REAL cx, cy, Rx, Ry;
        SFX(orc_bfecc_ratios)(p, sc ? adv_x_rows[j] : 0.0,
                              sc ? adv_y_cols[i] : 0.0, &cx, &cy, &Rx, &Ry);
        SFX(orc_bfecc_idx) n = SFX(orc_bfecc_neighbours)(p, solid, i, j);
        REAL FDx = cx > 0 ? uf[n.cE] - uf[n.E2] : uf[n.cW] - uf[n.W2];
        REAL FDy = cy > 0 ? uf[n.cN] - uf[n.N2] : uf[n.cS] - uf[n.S2];
        REAL ub = uf[C] - tc * (Rx * FDx + Ry * FDy);
        ue[C] = g[C] - (REAL)0.5 * (ub - g[C]);
      }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int C = i + nx * j;
        const int sc = !holes || solid[C];
        REAL cx, cy, Rx, Ry;
        SFX(orc_bfecc_ratios)(p, sc ? adv_x_rows[j] : 0.0,
                              sc ? adv_y_cols[i] : 0.0, &cx, &cy, &Rx, &Ry);
        SFX(orc_bfecc_idx) n = SFX(orc_bfecc_neighbours)(p, solid, i, j);
        REAL FDx = cx > 0 ? ue[C] - ue[n.W] : ue[C] - ue[n.E];
        REAL FDy = cy > 0 ? ue[C] - ue[n.S] : ue[C] - ue[n.N];
        REAL r = ue[C] - tc * (Rx * FDx + Ry * FDy);
        o[C] = sc ? r : (REAL)0.0;
      }
  }
}

/* ---------------------------------------------------------------------- */
/* Slices and phase-condition integrals                                    */
/* ---------------------------------------------------------------------- */

/* Integer disc centre as slice_kernel / trapz_kernel round it: float
 * arithmetic, then round-half-even (symmetryReduction.cu:95-107). */
static inline void SFX(orc_disc_centre)(const yh_param_var *p,
                                        const float centre[2], int *cx,
                                        int *cy) {
  float fx = centre[0] - (float)(p->nx / 2);
  float fy = centre[1] - (float)(p->ny / 2);
  *cx = (int)nearbyintf(fx);
  *cy = (int)nearbyintf(fy);
}

static inline int SFX(orc_in_disc)(const yh_param_var *p, int i, int j, int cx,
                                   int cy) {
  int ic = i - p->nx / 2 - cx, jc = j - p->ny / 2 - cy;
  return ic * ic + jc * jc < p->tipOffsetX * p->tipOffsetY;
}

/* Current-state derivative of field f at cell (i,j) along x, 2nd-order
 * one-sided, upwinded by the sign of adv (convFB2ndOX/Y,
 * symmetryReduction.cu:242-262; invdx = 0.5/hx). */
static inline REAL SFX(orc_fb2x)(const yh_param_var *p, const REAL *f, int i,
                                 int j, double advx) {
  const int nx = p->nx, C = i + nx * j;
  const int E = SFX(orc_mirror)(i + 1, nx) + nx * j;
  const int W = SFX(orc_mirror)(i - 1, nx) + nx * j;
  const int EE = SFX(orc_mirror)(i + 2, nx) + nx * j;
  const int WW = SFX(orc_mirror)(i - 2, nx) + nx * j;
  const REAL inv = (REAL)p->invdx;
  return advx > 0.0 ? ((REAL)-3.0 * f[C] + (REAL)4.0 * f[E] - f[EE]) * inv
                    : ((REAL)3.0 * f[C] - (REAL)4.0 * f[W] + f[WW]) * inv;
}
static inline REAL SFX(orc_fb2y)(const yh_param_var *p, const REAL *f, int i,
                                 int j, double advy) {
  const int nx = p->nx, ny = p->ny, C = i + nx * j;
  const int N = i + nx * SFX(orc_mirror)(j + 1, ny);
  const int S = i + nx * SFX(orc_mirror)(j - 1, ny);
  const int NN = i + nx * SFX(orc_mirror)(j + 2, ny);
  const int SS = i + nx * SFX(orc_mirror)(j - 2, ny);
  const REAL inv = (REAL)p->invdy;
  return advy > 0.0 ? ((REAL)-3.0 * f[C] + (REAL)4.0 * f[N] - f[NN]) * inv
                    : ((REAL)3.0 * f[C] - (REAL)4.0 * f[S] + f[SS]) * inv;
}
/* Template derivative: the NEGATED 4th-order central difference
 * (convCentral2X/Y, symmetryReduction.cu:224-240). */
static inline REAL SFX(orc_c4x)(const yh_param_var *p, const REAL *f, int i,
                                int j) {
  const int nx = p->nx;
  const int E = SFX(orc_mirror)(i + 1, nx) + nx * j;
  const int W = SFX(orc_mirror)(i - 1, nx) + nx * j;
  const int EE = SFX(orc_mirror)(i + 2, nx) + nx * j;
  const int WW = SFX(orc_mirror)(i - 2, nx) + nx * j;
  return (f[EE] - (REAL)8.0 * f[E] + (REAL)8.0 * f[W] - f[WW]) *
         (REAL)p->invdx * (REAL)(1.0 / 6.0);
}
static inline REAL SFX(orc_c4y)(const yh_param_var *p, const REAL *f, int i,
                                int j) {
  const int nx = p->nx, ny = p->ny;
  const int N = i + nx * SFX(orc_mirror)(j + 1, ny);
  const int S = i + nx * SFX(orc_mirror)(j - 1, ny);
  const int NN = i + nx * SFX(orc_mirror)(j + 2, ny);
  const int SS = i + nx * SFX(orc_mirror)(j - 2, ny);
  return (f[NN] - (REAL)8.0 * f[N] + (REAL)8.0 * f[S] - f[SS]) *
         (REAL)p->invdy * (REAL)(1.0 / 6.0);
}

/* Slices of one state (slice_kernel scheme 2, symmetryReduction.cu:167-206):
 * cur_{x,y,t}[f] (upwinded) and, when tmpl_x != NULL, the template
 * tmpl_{x,y,t}[f] (negated 4th-order central), 0 outside the disc.
 * The theta derivative is hx*x*d_y - hy*y*d_x with x=i, y=j. Any output
 * pointer array may be NULL. */
void SFX(orc_slices)(const yh_param_var *p, int nf, const REAL *const *g,
                     const double *adv_x_rows, const double *adv_y_cols,
                     const uint8_t *solid, const float centre[2],
                     REAL *const *cur_x, REAL *const *cur_y, REAL *const *cur_t,
                     REAL *const *tmpl_x, REAL *const *tmpl_y,
                     REAL *const *tmpl_t) {
  const int nx = p->nx, ny = p->ny;
  int cx, cy;
  SFX(orc_disc_centre)(p, centre, &cx, &cy);
  const int holes = p->solidSwitch && solid;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const int C = i + nx * j;
      const int sc = SFX(orc_in_disc)(p, i, j, cx, cy);
      const REAL x = (REAL)i, y = (REAL)j;
      const double ax = (!holes || solid[C]) ? adv_x_rows[j] : 0.0;
      const double ay = (!holes || solid[C]) ? adv_y_cols[i] : 0.0;
      for (int f = 0; f < nf; ++f) {
        REAL dx = sc ? SFX(orc_fb2x)(p, g[f], i, j, ax) : (REAL)0.0;
        REAL dy = sc ? SFX(orc_fb2y)(p, g[f], i, j, ay) : (REAL)0.0;
        REAL dtt = sc ? (REAL)p->hx * x * dy - (REAL)p->hy * y * dx : (REAL)0.0;
        if (cur_x) cur_x[f][C] = dx;
        if (cur_y) cur_y[f][C] = dy;
        if (cur_t) cur_t[f][C] = dtt;
        if (tmpl_x) {
          REAL tx = sc ? SFX(orc_c4x)(p, g[f], i, j) : (REAL)0.0;
          REAL ty = sc ? SFX(orc_c4y)(p, g[f], i, j) : (REAL)0.0;
          REAL tt = sc ? (REAL)p->hx * x * ty - (REAL)p->hy * y * tx : (REAL)0.0;
          tmpl_x[f][C] = tx;
          if (tmpl_y) tmpl_y[f][C] = ty;
          if (tmpl_t) tmpl_t[f][C] = tt;
        }
      }
    }
}

/* The 12 phase integrals (integralTrapz.cu:17-82,97-179):
 *   I[3a+b] = hx*hy * sum_{disc} sum_f T_a[f] * C_b[f],  a,b in {x,y,t}
 *   I[9+a]  = hx*hy * sum_{disc} sum_f T_a[f] * tan[f]
 * summed in FP64 in index order. The template/current arrays are 0 outside
 * the disc, as slice_kernel leaves them. */
void SFX(orc_integrals)(const yh_param_var *p, int nf, const REAL *const *tx,
                        const REAL *const *ty, const REAL *const *tt,
                        const REAL *const *cxv, const REAL *const *cyv,
                        const REAL *const *ctv, const REAL *const *tan,
                        const float centre[2], double I[12]) {
  const int nx = p->nx, ny = p->ny;
  int cx, cy;
  SFX(orc_disc_centre)(p, centre, &cx, &cy);
  double acc[12];
  for (int k = 0; k < 12; ++k) acc[k] = 0.0;
  const REAL *const *T[3] = {tx, ty, tt};
  const REAL *const *Cc[4] = {cxv, cyv, ctv, tan};
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      if (!SFX(orc_in_disc)(p, i, j, cx, cy)) continue;
      const int C = i + nx * j;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) {
          double s = 0.0;
          for (int f = 0; f < nf; ++f)
            s += (double)T[a][f][C] * (double)Cc[b][f][C];
          const int k = b < 3 ? 3 * a + b : 9 + a;
          acc[k] += s;
        }
    }
  for (int k = 0; k < 12; ++k) I[k] = p->hx * p->hy * acc[k];
}

#undef SFX
#undef CAT
#undef CAT2
