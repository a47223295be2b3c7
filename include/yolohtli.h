/*
 * yolohtli_gb300 — C ABI of the GB300 (sm_103a) monodomain hot path.
 *
 * One shared library, libyolohtli_gb300.so, exports everything declared here.
 * Every entry point is `extern "C"`, takes plain pointers, sizes and POD structs,
 * returns an int status (YH_OK = 0, negative = YH_E*), never calls exit(), and
 * launches asynchronously on the cudaStream_t passed as `void *stream`
 * (NULL = the legacy default stream, as the reference uses).
 *
 * Two layers:
 *   1. Stateless operators on caller-owned device buffers. Each one replaces
 *      one host wrapper of the reference (hostPrototypes.h:22-42); the
 *      comment above each declaration names it.
 *   2. A solver handle that owns the buffers and runs whole protocols
 *      (plain steps, stimulus events, symmetry-reduced steps) inside CUDA
 *      graphs without host round trips.
 *
 * Fields are FP32 structure-of-arrays, row-major, idx = i + nx*j, exactly the
 * reference's I2D layout (typeDefinition.cuh:129). The reference stores
 * FP64 (typeDefinition.cuh:4); the FP64 drop-in for its own symbols is in
 * yolohtli_compat.h.
 *
 * Threading: a handle is not thread-safe; use one handle per host thread /
 * stream. Stateless operators are reentrant.
 */
#ifndef YOLOHTLI_GB300_H
#define YOLOHTLI_GB300_H

#include <stddef.h>
#include <stdint.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Status codes                                                         */
/* ------------------------------------------------------------------ */
enum {
  YH_OK = 0,
  YH_EINVAL = -1,        /* bad argument (null pointer, size, flag)          */
  YH_ECUDA = -2,         /* a CUDA runtime call failed                       */
  YH_ENOMEM = -3,        /* device or host allocation failed                 */
  YH_ESINGULAR = -4,     /* 3x3 drift/rotation system singular (see the solves) */
  YH_ENONFINITE = -5,    /* NaN or Inf in the state                          */
  YH_EOVERFLOW = -6,     /* tip buffer full; extra tips were dropped         */
  YH_EUNSUPPORTED = -7,  /* option off this path: RK2/RK4, lap4, anisotropy,
                            Dirichlet boundaries                             */
  YH_ENOTREADY = -8,     /* call order (e.g. yh_sr_step before yh_sr_begin)  */
  YH_ETIMEOUT = -9,      /* a bounded device-side wait gave up (resident
                            solver); the state is not valid                  */
  YH_ECORRUPT = -10      /* checkpoint file: bad magic, version, byte order,
                            sizes or checksum, or a short file               */
};

enum { YH_MODEL_REF2V = 0,   /* the reference's 2-variable cubic model
                                (reactionDiffusion.cu:131-141)               */
       YH_MODEL_FK3V = 1 };  /* Fenton-Karma 3-variable model (1998)        */

enum { YH_TEMPLATE_CURRENT = 0,  /* template re-taken from the state every step,
                                    as the reference does (symmetryReduction.cu:184-205) */
       YH_TEMPLATE_FROZEN = 1 }; /* template derivatives taken once from a given state */

/* ------------------------------------------------------------------ */
/* ABI structs                                                          */
/* ------------------------------------------------------------------ */

/* CUDA's int2/float2 are 8-byte aligned; these mirror them in plain C. */
typedef struct yh_int2 { int x, y; } __attribute__((aligned(8))) yh_int2;
typedef struct yh_float2 { float x, y; } __attribute__((aligned(8))) yh_float2;

/* Field-for-field the reference's paramVar (typeDefinition.cuh:35-125):
 * same order, same types (REAL = double), so a reference driver can hand its
 * `param` to this library unchanged. The fields this path reads are:
 * nx, ny, hx, hy, dt, rx, ry, rscale, tc, invdx, invdy, alpha..theta, Uth,
 * tipOffsetX/Y, tipx/tipy, solidSwitch, neumannBC, gateDiff, anisotropy,
 * lap4, timeIntOrder, tipAlgorithm. */
typedef struct yh_param_var {
  bool animate;
  bool saveEveryIt;
  bool plotTip;
  bool recordTip;
  bool plotContour;
  bool recordContour;
  bool stimulate;
  bool apdContour;
  bool plotTimeSeries;
  bool recordTimeSeries;
  bool reduceSym;
  bool reduceSymStart;
  bool clock, counterclock;
  bool firstIterTip, firstIterContour;
  bool firstFPS;

  bool solidSwitch;
  bool neumannBC;
  bool gateDiff;
  bool anisotropy;
  bool tipGrad;
  int lap4;
  int contourMode;
  int timeIntOrder;
  int tipAlgorithm;

  bool load;
  bool save;

  int nx;
  int ny;
  int memSize;
  double Lx, Ly, hx, hy;
  double dt;
  double diff_par, diff_per;
  double Dxx, Dyy, Dxy;
  double rx, ry, rxy, rbx, rby;
  double rscale;
  double invdx, invdy;
  double sample;
  int count;
  double physicalTime, physicalTimeLim;
  int startRecTime;
  double stimPeriod;
  double stimDuration;
  double stimMag;
  bool fibThreshold;
  bool fibTerminated;
  int leapShocks;
  int eSize;
  yh_int2 point;
  int nc;
  double rdomTrapz, rdomStim, rdomAPD;
  double stcx, stcy;
  yh_float2 pointStim;
  int savePackage;
  float tiempo;
  double degrad;
  double boundaryVal;
  double qx4, qy4, fx4, fy4;

  int itPerFrame;
  int tipOffsetX;
  int tipOffsetY;
  float minVarColor;
  float maxVarColor;

  int wnx;
  int wny;
  float uMax;
  float uMin;
  float vMax;
  float vMin;

  float tipx;
  float tipy;

  double contourThresh1, contourThresh2, contourThresh3;
  double Uth;
  double tc;
  double alpha;
  double beta;
  double gamma;
  double delta;
  double eps;
  double mu;
  double theta;
} yh_param_var;

/* Fenton-Karma (1998) parameters, times in ms, potentials dimensionless.
 * Not in the reference (it has only the 2-variable model). */
typedef struct yh_fk_params {
  double tau_d, tau_r, tau_si, tau_0;
  double tau_v_plus, tau_v1_minus, tau_v2_minus;
  double tau_w_plus, tau_w_minus;
  double u_c, u_v, u_csi, k;
} yh_fk_params;

/* A tip point: the reference's vec5dyn (typeDefinition.cuh:19-20). */
typedef struct yh_tip { float x, y, vx, vy, t; } yh_tip;

/* Device pointers of one FP32 state: the reference's stateVar
 * (typeDefinition.cuh:7-9) plus the third FK variable w (NULL for REF2V). */
typedef struct yh_fields { float *u, *v, *w; } yh_fields;

/* Symmetry-reduction state, kept in DEVICE memory by the operators below.
 * c and phi are the reference's REAL3 c, phi (main.cu:60); integrals is its
 * `REAL *integrals` (main.cu:220), in the same order I0..I11
 * (integralTrapz.cu:97-179). */
typedef struct yh_sym_state {
  double c[3];          /* cx, cy, ctheta of the last solve                 */
  double phi[3];        /* phi_x, phi_y, phi_theta (integrated frame)       */
  double c_adv[3];      /* c used for the advection field of the last BFECC */
  double phi_adv[3];    /* phi used for the same                            */
  double integrals[12];
  float centre[2];      /* disc centre of the phase integrals (cells)       */
  int step;             /* steps taken (the reference's param.count)        */
  int status;           /* YH_OK or YH_ESINGULAR from the last solve        */
  int ntips;            /* tips found by the last tip pass                  */
  int nsingular;        /* solves that found the system singular (and kept
                           the previous c) since the state was zeroed      */
} yh_sym_state;

/* A contour point: the reference's float3 of contour_vector
 * (spaceAPD.cu:18-153): position (cells) and time. */
typedef struct yh_contour_pt { float x, y, t; } yh_contour_pt;

/* Per-cell fields of the space-APD tracker (sAPD_kernel, spaceAPD.cu:278):
 * device arrays of nx*ny; apd1, apd2, back, front and first carry the
 * tracker's state from call to call (start them at 0). */
typedef struct yh_apd_fields {
  float *apd1, *apd2, *sapd, *dapd, *back, *front;
  uint8_t *first;
} yh_apd_fields;

/* A stimulus event of a protocol: u = value on tissue cells of the box
 * [i0,i1) x [j0,j1), applied before step `step` is taken. */
typedef struct yh_stim { int step; int i0, j0, i1, j1; float value; } yh_stim;

/* ------------------------------------------------------------------ */
/* Parameter helpers                                                    */
/* ------------------------------------------------------------------ */

/* The reference's defaults (saveFiles.cu:105-231) for an nx x ny grid, with
 * derived coefficients as main.cu:148-158 computes them (dt not halved). */
int yh_param_defaults(yh_param_var *p, int nx, int ny);
/* Recompute rx, ry, invdx, invdy, ... from dt, hx, hy, Dxx, Dyy. */
int yh_param_derive(yh_param_var *p);
/* Fenton-Karma BR-fit parameter set. */
int yh_fk_defaults(yh_fk_params *fk);
const char *yh_status_string(int status);
const char *yh_version(void);
/* sizeof of an ABI struct by name ("yh_param_var", "yh_fk_params",
 * "yh_tip", "yh_fields", "yh_sym_state", "yh_stim"); 0 if unknown. */
size_t yh_sizeof(const char *type_name);

/* ------------------------------------------------------------------ */
/* Layer 1: stateless operators on caller-owned device buffers         */
/* ------------------------------------------------------------------ */

/* One explicit Euler reaction-diffusion step, out <- in, with the 5-point
 * mirror (no-flux) Laplacian, hole coefficients when p->solidSwitch, and the
 * state tangent vel_tan = (out - in)/dt when vel_tan.u != NULL.
 * Replaces reactionDiffusion_wrapper (hostPrototypes.h:22-25,
 * reactionDiffusion.cu:568-577). `solid` is nx*ny bytes, nonzero = tissue. */
int yh_reaction_diffusion(const yh_param_var *p, int model,
                          const yh_fk_params *fk, yh_fields out, yh_fields in,
                          yh_fields vel_tan, const uint8_t *solid,
                          void *stream);

/* Spiral-tip detection between the time levels g_past and g_present (u
 * fields) at time `physical_time`: p->tipAlgorithm 1, the closed-form
 * bilinear isoline intersection (spiralTip_kernel, tipTracker.cu:20-208),
 * or 2, Newton's method on the same bilinear interpolants in the 2*tipOffset
 * window around the grid centre (spiralTipNewton_kernel,
 * tipTracker.cu:244-432); with p->tipGrad each tip carries the gradient of
 * g_present (gradient, tipTracker.cu:519-566) in vx, vy. Resets *tip_count
 * to 0, then appends every tip. Replaces tip_wrapper (hostPrototypes.h:26-28,
 * tipTracker.cu:569-611); tipAlgorithm 3 is yh_filament_mark. tip_count and
 * tip_vector are device pointers; at most `capacity` tips are stored,
 * *tip_count keeps the full number found. */
int yh_spiral_tip(const yh_param_var *p, const float *g_past,
                  const float *g_present, double physical_time,
                  int *tip_count, yh_tip *tip_vector, int capacity,
                  const uint8_t *solid, void *stream);

/* Chooses the disc centre of the phase integrals from the tips found: the
 * tip nearest to the previous centre (sym->centre); unchanged if no tip.
 * The reference takes the last tip pushed (symmetryReduction.cu:102-103),
 * whose order is not deterministic. */
int yh_pick_centre(const int *tip_count, const yh_tip *tip_vector,
                   int capacity, yh_sym_state *sym, void *stream);

/* Workspace bytes needed by yh_phase_integrals for this grid (any disc
 * radius). The workspace holds a completion counter that must be zero before
 * the first call; every call leaves it at zero again. */
size_t yh_phase_integrals_workspace(int nx, int ny);

/* Fused slice + phase-condition integrals + FP64 3x3 solve:
 *  - current-state derivatives (2nd-order one-sided, upwinded by the sign of
 *    the comoving field adv_x_rows[j], adv_y_cols[i], 0 off tissue),
 *  - template derivatives (negated 4th-order central of `state` when
 *    templ_x.u == NULL, else the stored template fields templ_x/y/t),
 *  - the 12 integrals over the open disc of radius^2 tipOffsetX*tipOffsetY
 *    around sym->centre, summed per thread, warp and block as float-float
 *    pairs (~48 significant bits, no FP64 instruction per cell), the block
 *    sums added in a fixed order, FP64 from the 12 integrals on,
 *  - the FP64 3x3 solve by cofactors, rotated by sym->phi[2] (YH_ESINGULAR
 *    when |det| <= 1e-13 amax^3, c then kept): sym->c, sym->integrals,
 *    sym->status; then sym->c_adv = c, sym->phi_adv = phi.
 * Replaces slice_wrapper + trapz_wrapper + solve_matrix
 * (hostPrototypes.h:30-33,39-42; symmetryReduction.cu:72-222,329-420;
 * integralTrapz.cu:17-184). `workspace`: device memory of at least
 * yh_phase_integrals_workspace(nx, ny) bytes. */
int yh_phase_integrals(const yh_param_var *p, int model, yh_fields state,
                       yh_fields vel_tan, yh_fields templ_x,
                       yh_fields templ_y, yh_fields templ_t,
                       const double *adv_x_rows, const double *adv_y_cols,
                       const uint8_t *solid, yh_sym_state *sym,
                       void *workspace, void *stream);

/* yh_phase_integrals without the workspace argument, for callers that may
 * not allocate device memory themselves: a host application whose device
 * memory is owned by its own pool, or a caller in a section where a
 * cudaMalloc (which can synchronize the device) is not allowed. No
 * counterpart in the reference (its trapz_wrapper allocates and frees
 * scratch on every call, integralTrapz.cu:89-92,181-182).
 * The scratch is a fixed array of yh_phase_integrals_noalloc_limit() bytes
 * (384 KiB + 256 B) compiled into the library: every GPU that loads the
 * library holds it until the process exits. A disc needing more than 4096
 * blocks of partial sums is rejected with YH_EINVAL. The first call on each
 * device looks up the array's device address, so make it before capturing
 * a stream into a CUDA graph. All calls share the one array and it keeps
 * the last call's partial sums: calls that may overlap on the GPU (on
 * different streams) race and give wrong results; serialize them. Never
 * calls cudaMalloc or cudaFree. The looked-up address is kept for the
 * life of the process: after cudaDeviceReset (or anything else that tears
 * down and recreates the device's context) the library must be reloaded
 * before this entry point is called again. */
int yh_phase_integrals_noalloc(const yh_param_var *p, int model,
                               yh_fields state, yh_fields vel_tan,
                               yh_fields templ_x, yh_fields templ_y,
                               yh_fields templ_t, const double *adv_x_rows,
                               const double *adv_y_cols, const uint8_t *solid,
                               yh_sym_state *sym, void *stream);
size_t yh_phase_integrals_noalloc_limit(void);

/* Template derivative fields (negated 4th-order central, as the reference's
 * convCentral2X/Y, symmetryReduction.cu:224-240) of a state over the whole
 * grid; used to freeze a template. */
int yh_template_slices(const yh_param_var *p, int model, yh_fields state,
                       yh_fields templ_x, yh_fields templ_y,
                       yh_fields templ_t, void *stream);

/* The comoving field of (sym->c_adv, sym->phi_adv). It is separable:
 * adv.x = hy*j*ct - cx*cos(pt) + cy*sin(pt) depends on the row j only and
 * adv.y = -hx*i*ct - cx*sin(pt) - cy*cos(pt) on the column i only, so it is
 * written as adv_x_rows[ny] and adv_y_cols[nx] in FP64 (and FP32 copies when
 * the _f32 pointers are not NULL). With advance_phi != 0 it then applies
 * phi += dt*c, step += 1 (main.cu:936-952).
 * Replaces Cxy_field_wrapper (hostPrototypes.h:34-35,
 * symmetryReduction.cu:20-70). */
int yh_comoving_field(const yh_param_var *p, yh_sym_state *sym,
                      double *adv_x_rows, double *adv_y_cols,
                      float *adv_x_rows_f32, float *adv_y_cols_f32,
                      int advance_phi, void *stream);

/* BFECC advection out <- in by the comoving field (FP32 row/column vectors
 * of yh_comoving_field): the three race-free passes in one launch (tiles in
 * shared memory), or, when out aliases in, as three launches through the
 * caller's scratch fields uf and ue. Both give the same bits.
 * Replaces advFDBFECC_wrapper (hostPrototypes.h:36-38, advFDBFECC.cu:18-362). */
int yh_advect_bfecc(const yh_param_var *p, int model, yh_fields out,
                    yh_fields in, const float *adv_x_rows_f32,
                    const float *adv_y_cols_f32, const uint8_t *solid,
                    yh_fields uf, yh_fields ue, void *stream);
/* The three launches always (uf and ue hold the passes' results). */
int yh_advect_bfecc_3pass(const yh_param_var *p, int model, yh_fields out,
                          yh_fields in, const float *adv_x_rows_f32,
                          const float *adv_y_cols_f32, const uint8_t *solid,
                          yh_fields uf, yh_fields ue, void *stream);

/* phi += dt * c and step += 1 on the device (main.cu:935-952). */
int yh_sym_advance(const yh_param_var *p, yh_sym_state *sym, void *stream);

/* u = value on tissue cells of [i0,i1) x [j0,j1). */
int yh_stimulate_box(const yh_param_var *p, float *u, const uint8_t *solid,
                     int i0, int j0, int i1, int j1, float value,
                     void *stream);

/* FP64 instances of three operators above: the same kernel templates
 * compiled for double, on FP64 device buffers (REAL = double, the
 * reference's storage, typeDefinition.cuh:4). They separate rounding from
 * discretisation: a run of these against the FP64 oracle isolates the
 * discrete map, a run of the FP32 operators against them isolates FP32
 * rounding. Not a fast path (GB300 issues FP64 at a small fraction of its
 * FP32 rate). Arguments and status codes as the FP32 operators. */
typedef struct yh_fields64 { double *u, *v, *w; } yh_fields64;
int yh_reaction_diffusion_f64(const yh_param_var *p, int model,
                              const yh_fk_params *fk, yh_fields64 out,
                              yh_fields64 in, yh_fields64 vel_tan,
                              const uint8_t *solid, void *stream);
int yh_spiral_tip_f64(const yh_param_var *p, const double *g_past,
                      const double *g_present, double physical_time,
                      int *tip_count, yh_tip *tip_vector, int capacity,
                      const uint8_t *solid, void *stream);
int yh_stimulate_box_f64(const yh_param_var *p, double *u,
                         const uint8_t *solid, int i0, int j0, int i1, int j1,
                         double value, void *stream);

/* ------------------------------------------------------------------ */
/* Layer 2: solver handle                                               */
/* ------------------------------------------------------------------ */
typedef struct yh_solver yh_solver;

/* Copies the parameters, uploads the hole mask (NULL = no holes) and
 * allocates the device state. The state starts at zero. */
int yh_create(const yh_param_var *p, int model, const yh_fk_params *fk,
              const uint8_t *solid_host, void *stream, yh_solver **out);
int yh_destroy(yh_solver *h);
int yh_synchronize(yh_solver *h);

/* Copies into / out of the current state; the pointers may be host (pinned
 * or pageable) or device memory. NULL pointers are skipped. */
int yh_set_state(yh_solver *h, const float *u, const float *v, const float *w);
int yh_get_state(yh_solver *h, float *u, float *v, float *w);
/* Device pointers of the current state (valid until the next step). */
int yh_state_device(yh_solver *h, yh_fields *cur);

/* Steps per kernel launch of the plain solver (temporal blocking depth);
 * 1 = one launch per step. Values are clamped to what the model allows
 * (1..8; always 1 for REF2V with gateDiff, whose v diffuses too). */
int yh_set_time_block(yh_solver *h, int steps_per_launch);
int yh_get_time_block(yh_solver *h, int *steps_per_launch);

/* How yh_run advances the plain solver:
 *  STEP      one launch per step (graph-replayed);
 *  BLOCKED   steps_per_launch steps per launch (temporal blocking in
 *            registers and shared memory);
 *  RESIDENT  the whole run in one cooperative launch: each SM keeps its
 *            stripe of the state in shared memory for all steps, stimulus
 *            events are applied in the kernel; only for grids that fit
 *            (about 1.7M cells on a GB300). A bounded wait between blocks
 *            that gives up makes yh_synchronize / yh_get_state return
 *            YH_ETIMEOUT.
 * BLOCKED and RESIDENT need a model where only u diffuses (FK3V, or REF2V
 * without gateDiff); YH_EUNSUPPORTED otherwise. */
enum { YH_ENGINE_STEP = 0, YH_ENGINE_BLOCKED = 1, YH_ENGINE_RESIDENT = 2 };
int yh_set_engine(yh_solver *h, int engine, int steps_per_launch);
/* Failure self-test of the bounded device-side waits: a 128^2 FK3V grid on
 * the resident engine, first with one block publishing none of its
 * boundary rows (its neighbours' waits run out after their 1 s bound; the
 * launch ends with every block returned and *muted_status = YH_ETIMEOUT),
 * then normally on the same context (*after_status = YH_OK). Returns
 * YH_EUNSUPPORTED where the resident engine does not run. */
int yh_selftest_resident_timeout(int *muted_status, int *after_status);
int yh_get_engine(yh_solver *h, int *engine, int *steps_per_launch);

/* Autotuner: times probe_steps plain steps from the current state for each
 * engine and depth the model allows, restores the state and counters, and
 * keeps the fastest (returned in *engine, *steps_per_launch). */
int yh_autotune(yh_solver *h, int probe_steps, int *engine,
                int *steps_per_launch);

/* nsteps plain explicit steps with the stimulus events of `stims` whose step
 * lies in [h.step, h.step + nsteps), captured and replayed as a CUDA graph. */
int yh_run(yh_solver *h, int nsteps, const yh_stim *stims, int nstims);

/* Tip detection between the current state and the previous time level
 * (plain mode: x = new u, y = old u, main.cu:963). */
int yh_track_tips(yh_solver *h);
int yh_get_tips(yh_solver *h, yh_tip *out, int capacity, int *n);

/* Symmetry reduction (main.cu:894-954). template_mode YH_TEMPLATE_FROZEN
 * takes the template from the host state (tu, tv, tw); CURRENT ignores it. */
int yh_sr_begin(yh_solver *h, int template_mode, const float *tu,
                const float *tv, const float *tw);
/* nsteps symmetry-reduced steps. Returns YH_ESINGULAR when a solve during
 * these steps found the drift/rotation system singular (the frame then kept
 * its previous c and is not a valid comoving frame; the steps were taken);
 * yh_get_sym's nsingular counts such solves since yh_sr_begin. Reads that
 * count back once per call (one stream synchronisation). */
int yh_sr_step(yh_solver *h, int nsteps);
/* yh_sr_step in two halves, for several handles driven from one thread (a
 * sweep over parameters on several streams): yh_sr_enqueue enqueues the
 * steps on the handle's stream and returns without waiting;
 * yh_sr_status waits for the stream and returns YH_ESINGULAR when a
 * solve since the last status read (by either call) found the system
 * singular. */
int yh_sr_enqueue(yh_solver *h, int nsteps);
int yh_sr_status(yh_solver *h);
int yh_get_sym(yh_solver *h, yh_sym_state *out);

/* Steps taken so far, the clock that stimulus events are matched against.
 * yh_set_step moves that clock (step >= 0) and leaves the state as it is. */
int yh_get_step(yh_solver *h, int *step);
int yh_set_step(yh_solver *h, int step);

/* Kernel launches this handle has performed so far (graph replays count
 * every kernel node they run). */
int yh_get_launch_count(yh_solver *h, long long *n);

/* Counts the state values (every field, every cell) that are NaN or Inf, in
 * one launch; *bad_values (may be NULL) gets the count. YH_ENONFINITE when
 * it is not zero. */
int yh_check_finite(yh_solver *h, long long *bad_values);

/* Checkpoint and resume of a plain run (the file format is under layer 4).
 * Save writes the state, the step count, the parameters and the mask.
 * Load restores the state and the step count into a handle created for the
 * same problem. It returns YH_EINVAL when the file's grid, model, step
 * coefficients (rx, ry, rscale, dt, tc, gateDiff, the REF2V constants),
 * FK3V parameters or mask differ from the handle's. Neither the previous
 * time level (tip tracking) nor a symmetry-reduction state is part of a
 * checkpoint: a symmetry-reduced run resumes with a new yh_sr_begin. */
int yh_save_checkpoint(yh_solver *h, const char *path);
int yh_load_checkpoint(yh_solver *h, const char *path);
/* 1 when two (parameters, model, FK3V parameters) describe the same problem
 * for a resume (grid, model, step coefficients, FK3V parameters: the rule
 * yh_load_checkpoint applies before the mask), else 0. Host only. */
int yh_checkpoint_same_problem(const yh_param_var *a, int model_a,
                               const yh_fk_params *fk_a,
                               const yh_param_var *b, int model_b,
                               const yh_fk_params *fk_b);

/* tipAlgorithm 3 (abouzarTip_kernel / abubuFilament,
 * tipTracker.cu:434-517): marks (sets to 1, never clears) the cells whose
 * 2x2 corners straddle both u = Uth and u_present = u_past. mark: nx*ny
 * device bytes. */
int yh_filament_mark(const yh_param_var *p, const float *past,
                     const float *present, uint8_t *mark, void *stream);

/* Contour points of field2 (countour_wrapper / countour_kernel,
 * spaceAPD.cu:18-276): mode 1 its zero level with sub-cell positions (the
 * space-APD contour), mode 2 the level contourThresh2 where field1 <
 * contourThresh1, mode 3 the levels 2*contourThresh2 and contourThresh2 -
 * contourThresh3 in a band around contourThresh2 where field1 <
 * contourThresh1; stim_area (nx*ny bytes) masks as the reference does.
 * Resets *count (and plot, when given) first; at most `capacity` points are
 * stored. All pointers are device pointers. */
int yh_contour(const yh_param_var *p, const float *field1, const float *field2,
               const uint8_t *stim_area, int mode, float time, int *count,
               yh_contour_pt *vec, int capacity, uint8_t *plot, void *stream);

/* One step of the space-APD tracker (sAPD_wrapper / sAPD_kernel,
 * spaceAPD.cu:278-383) between uold and unew at step `count` (times are
 * dt * count): upstroke/downstroke times through u = 0.15, two successive
 * APDs, sapd = sign(APD1 - APD2); with `stimulate` only inside stim_area,
 * and dapd = APD2 there. */
int yh_space_apd(const yh_param_var *p, int count, const float *uold,
                 const float *unew, yh_apd_fields f, const uint8_t *stim_area,
                 int stimulate, void *stream);

/* ------------------------------------------------------------------ */
/* Layer 3: batched solver (many independent grids, one launch per step)  */
/* ------------------------------------------------------------------ */
/* No reference counterpart: the reference solves one grid per process and
 * keeps its parameters in process-global __constant__ symbols
 * (main.cu:40-51), which rules out batching. Each instance of a batch has
 * its own grid size, parameters (D through rx/ry, the FK3V time constants),
 * hole mask and stimulus events. Three schedules advance them (the
 * autotuner picks one): groups small enough to stay in the L2, each group
 * by all the run's steps with one or two steps per launch; one launch
 * sequence per instance (the single-grid kernels); or the wavefront engine,
 * one persistent launch per run. Graphs and internal streams fork from and
 * join the caller's stream. FK3V in FP32, the same cell update as the
 * single-grid solver (same bits under every schedule); nx % 4 == 0. */
typedef struct yh_batch yh_batch;

/* A stimulus event of one instance of a batch. */
typedef struct yh_batch_stim {
  int instance;
  yh_stim s;
} yh_batch_stim;

/* count instances: params[k] (nx % 4 == 0, the options of yh_create), fk[k]
 * and masks[k] (1 byte per cell, nonzero = tissue; NULL: no holes, used
 * when params[k].solidSwitch). State starts at zero. */
int yh_batch_create(int count, const yh_param_var *params,
                    const yh_fk_params *fk, const uint8_t *const *masks,
                    void *stream, yh_batch **out);
int yh_batch_destroy(yh_batch *b);
/* YH_ETIMEOUT if a depth-2 launch's bounded TMA wait gave up. */
int yh_batch_synchronize(yh_batch *b);
/* State of instance k (host or device pointers, nx*ny floats each). */
int yh_batch_set_state(yh_batch *b, int k, const float *u, const float *v,
                       const float *w);
int yh_batch_get_state(yh_batch *b, int k, float *u, float *v, float *w);
/* Device pointers of instance k's current state (valid until the next step). */
int yh_batch_state_device(yh_batch *b, int k, yh_fields *cur);
/* nsteps steps of every instance with the events whose step lies in
 * [step, step + nsteps); events of one instance and step apply in the
 * order given. */
int yh_batch_run(yh_batch *b, int nsteps, const yh_batch_stim *stims,
                 int nstims);
/* yh_batch_run with the states in host memory: instance k's state is
 * copied in from u_in[k], v_in[k], w_in[k] before its first step and its
 * result out to u_out[k], v_out[k], w_out[k] after its last (any of the six
 * arrays, or any entry, may be NULL: that field is not copied), and the
 * call returns when the outputs are written. Under the per-instance
 * schedule (yh_batch_set_schedule with group_cells 0) every instance's
 * copies run on its own stream beside the other instances' steps (pinned
 * host memory lets them overlap); the other schedules copy on the caller's
 * stream before and after the run. */
int yh_batch_run_host(yh_batch *b, int nsteps, const yh_batch_stim *stims,
                      int nstims, const float *const *u_in,
                      const float *const *v_in, const float *const *w_in,
                      float *const *u_out, float *const *v_out,
                      float *const *w_out);
/* Schedule of later runs: groups of about group_cells cells (largest
 * instances first) on `streams` internal streams (1-64). The default is
 * 1,048,576 cells on 2 streams. group_cells 0: every instance runs its own
 * sequence of single-grid launches (the step engine's kernels, one or, at
 * depth 2, two steps per launch, the instance's coefficients in the kernel
 * parameters, 64-step graphs per instance), the instances spread over the
 * streams so that large and small ones run together. */
int yh_batch_set_schedule(yh_batch *b, long long group_cells, int streams);
/* Steps per launch: 1 (the default) or 2 (64 x 16 tiles, inputs staged by
 * TMA bulk tensor copies, the same bits; YH_EUNSUPPORTED unless every
 * instance's rows allow it: nx % 16 == 0 for instances with holes). */
int yh_batch_set_depth(yh_batch *b, int depth);
/* The wavefront engine: one persistent launch per run segment (a run is one
 * segment unless an instance has more than 4 events in it). Each instance
 * goes to a cluster of `cluster` CTAs (1, 2 or 4; one CTA per SM, the
 * instance's columns split into that many bands), which advances it up to K
 * steps per pass with its rows in shared-memory rings: level k of a pass
 * computes step k on row p - 2k at wavefront position p, neighbouring bands
 * exchange their edge columns through distributed shared memory. K is as
 * large as the rings allow (at most (R - 3) / 2 for R ring rows, R <= 128),
 * capped at max_levels when max_levels > 0. Instances go to the clusters
 * longest first, each to the least loaded. The same bits as one launch per
 * step; the state is updated in place. YH_EUNSUPPORTED where an instance
 * has fewer quads (nx / 4) than `cluster` or its rings would hold fewer
 * than 8 rows (nx / cluster above ~1,690 cells). cluster 0 returns to the
 * grouped launches; yh_batch_set_depth and yh_batch_set_schedule do too. */
int yh_batch_set_wave(yh_batch *b, int cluster, int max_levels);
/* The wavefront engine's shape (*cluster 0: grouped launches) and the
 * clusters of its launch. */
int yh_batch_get_wave(yh_batch *b, int *cluster, int *max_levels,
                      int *clusters);
/* The schedule autotuner: times probe_steps steps (rounded up to even, no
 * events) of every schedule of groups of 256 K, 512 K, 1 M or 2 M cells
 * on 2, 3 or 4 streams at depth 1 and (where supported) 2, of one launch
 * sequence per instance on 6, 8 or 12 streams at depth 1 and 2, and of the
 * wavefront engine
 * with 1, 2 and 4 CTAs per instance, on the current state, keeps the
 * fastest and restores the state and the step count. The choice is
 * returned in *group_cells, *streams and *depth (any may be NULL): one
 * sequence per instance reports *group_cells 0 and *depth 1 or 2, the
 * wavefront engine *depth 0, *streams = CTAs per instance and *group_cells
 * 0. */
int yh_batch_autotune(yh_batch *b, int probe_steps, long long *group_cells,
                      int *streams, int *depth);
int yh_batch_get_step(yh_batch *b, int *step);
/* Moves the batch's step clock (step >= 0); the states are unchanged. */
int yh_batch_set_step(yh_batch *b, int step);
int yh_batch_get_launch_count(yh_batch *b, long long *n);

/* ------------------------------------------------------------------ */
/* Layer 5: adjoint (gradients of a probe loss: D(x, y), FK parameters) */
/* ------------------------------------------------------------------ */
/* No reference counterpart (the reference has constant D and no
 * gradients). FK3V with a per-cell diffusion coefficient D (nx*ny floats,
 * cm^2/ms): du_i = dt/h^2 sum over the 4 faces of (D_i + D_m)/2 (u_m - u_i),
 * m the mirrored neighbour (no-flux edges as the reference's mirror
 * ghosts), then the FK3V Euler update in exact arithmetic. The loss sums
 * (u - target)^2 over a lattice of probes (every probe_spacing cells, at
 * the cell centres of the lattice squares) on the states after every
 * frame_steps steps. One run takes nsteps forward steps keeping a
 * checkpoint every checkpoint_steps, then recomputes each segment and
 * sweeps it backwards (the recompute of the next segment runs on a second
 * stream of the handle beside the sweep; the forward pass keeps the last
 * segment): memory is the checkpoints plus two segments. fp64
 * runs the same in FP64 (for gradient checks). hx must equal hy. smooth:
 * 0 keeps FK3V's switches H(u - u_c), H(u - u_v) as steps (the model of
 * the other engines; its derivative exists almost everywhere but grows with
 * the horizon and leaves out the threshold-crossing times); smooth > 0
 * replaces them by (1 + tanh(x / smooth)) / 2 in this solver's forward and
 * reverse steps. */
typedef struct yh_adjoint yh_adjoint;
int yh_adjoint_create(const yh_param_var *p, const yh_fk_params *fk,
                      int nsteps, int frame_steps, int probe_spacing,
                      int checkpoint_steps, int fp64, double smooth,
                      void *stream, yh_adjoint **out);
/* `batch` independent instances (1-4096) with the same grid, steps, probes
 * and FK parameters and their own D, initial state and target, advanced by
 * one launch per step. Every per-instance array below is then the
 * instances' arrays one after another (D, u0, v0, w0, grad_D: batch x nx*ny;
 * target, probes: batch x frames x probes; loss: batch doubles; grad_fk:
 * batch structs). checkpoint_steps = 1 keeps every state (no recompute:
 * 3 nx ny nsteps batch values). yh_adjoint_create is batch 1. */
int yh_adjoint_create_batch(const yh_param_var *p, const yh_fk_params *fk,
                            int batch, int nsteps, int frame_steps,
                            int probe_spacing, int checkpoint_steps, int fp64,
                            double smooth, void *stream, yh_adjoint **out);
int yh_adjoint_batch(yh_adjoint *h, int *batch);
int yh_adjoint_destroy(yh_adjoint *h);
/* Frames (nsteps / frame_steps) and probes (nx / spacing, ny / spacing). */
int yh_adjoint_probes(yh_adjoint *h, int *frames, int *probes_x,
                      int *probes_y);
/* target: frames x probes_y x probes_x floats, host or device. */
int yh_adjoint_set_target(yh_adjoint *h, const float *target);
/* A forward run from (u0, v0, w0) with D that writes the probe values of
 * every frame (the shape of a target) to `probes` (device). */
int yh_adjoint_record(yh_adjoint *h, const float *D, const float *u0,
                      const float *v0, const float *w0, float *probes);
/* Loss (host) and, when grad_D is not NULL, dLoss/dD (device, nx*ny) from
 * the initial state (u0, v0, w0) and D, all device arrays. */
int yh_adjoint_run(yh_adjoint *h, const float *D, const float *u0,
                   const float *v0, const float *w0, double *loss,
                   float *grad_D);
/* yh_adjoint_run that also returns dLoss/d(FK parameter) for each of the
 * 13 fields of yh_fk_params in grad_fk (host): the sum over steps and
 * cells of the adjoint state times the derivative of the pointwise update
 * with respect to the parameter. With smooth = 0 the thresholds u_c, u_v
 * enter only where they are not switches (u_c in the fast current). */
int yh_adjoint_run_fk(yh_adjoint *h, const float *D, const float *u0,
                      const float *v0, const float *w0, double *loss,
                      float *grad_D, yh_fk_params *grad_fk);
/* New FK parameters for the following runs (checked as at create). */
int yh_adjoint_set_fk(yh_adjoint *h, const yh_fk_params *fk);

/* ------------------------------------------------------------------ */
/* Layer 4: the reference's interchange files                           */
/* ------------------------------------------------------------------ */
/* Line for line the files the reference writes for its MATLAB
 * post-processing (same labels, order and printf conversions: the output of
 * the same data is byte-identical). Host code, no GPU. Each returns YH_OK
 * or YH_EINVAL (argument, open or write error). */

/* dataparamcsv.csv: printParameters (printFunctions.cu:266-403). ic_path and
 * results_path fill the two path lines (NULL: "NA", as the reference writes
 * when it neither loads nor saves). */
int yh_write_param_csv(const char *path, const yh_param_var *p,
                       const char *ic_path, const char *results_path);
/* Reads it back as loadParamValues does (saveFiles.cu:540-711): the second
 * field of every line from the third on, as a float, into the fields the
 * writer wrote; count and physicalTime reset, animate set. */
int yh_read_param_csv(const char *path, yh_param_var *p);
/* raw_data.dat: "u v" per cell, row-major (print2D2column,
 * printFunctions.cu:58-78); the reader is loadData (saveFiles.cu:507-537). */
int yh_write_raw_data(const char *path, const yh_param_var *p, const float *u,
                      const float *v);
int yh_read_raw_data(const char *path, const yh_param_var *p, float *u,
                     float *v);
/* raw_data<count>.dat of the symmetry-reduced saves: the window of
 * 2*tipOffset+2 cells around (tipx, tipy) (print2DSubWindow,
 * printFunctions.cu:80-103); YH_EINVAL when it leaves the grid. */
int yh_write_raw_window(const char *path, const yh_param_var *p,
                        const float *u, const float *v);
/* dataTip.dat ("x y vx vy t" per tip) and dataTipSize.dat (the count, only
 * when n > 0), truncated when append == 0 (printTip,
 * printFunctions.cu:149-197). */
int yh_write_tips(const char *tip_path, const char *size_path,
                  const yh_tip *tips, int n, int append);
/* c_phi_list_sym.dat: "cx cy ctheta phix phiy phitheta" per entry, c and phi
 * n x 3 (printSym, printFunctions.cu:249-264). */
int yh_write_sym_list(const char *path, const double *c, const double *phi,
                      int n);

/* This library's own binary checkpoint. The reference's only state file,
 * raw_data.dat, keeps 6 decimals, and its reload path is dead. Host code,
 * no GPU. All integers are little-endian. Layout:
 *   a 64-byte header:
 *     bytes 0-7    magic "YHCKPT\0\0"
 *     8-11         format version, uint32 (1)
 *     12-15        byte-order mark, uint32 0x01020304
 *     16-35        nx, ny, model, nfields, mask flag, int32 each
 *     36-39        sizeof(yh_param_var), int32
 *     40-47        step, int64
 *     48-55        payload bytes, uint64
 *     56-63        FNV-1a 64-bit hash of the payload, uint64
 *   the payload:
 *     the yh_param_var, the yh_fk_params, the mask (nx*ny bytes, only when
 *     the flag is 1; nonzero = tissue), then nfields float32 arrays of nx*ny
 *     cells (u, v and, for FK3V, w).
 * Every function returns YH_EINVAL for an argument error or an open or write
 * error, and YH_ECORRUPT for a file that fails a check of the format, its
 * sizes or its hash. */
typedef struct yh_checkpoint_header {
  int nx, ny, model, nfields, has_mask;
  long long step;
} yh_checkpoint_header;

/* mask may be NULL: no mask is stored. w is ignored for REF2V. The file is
 * written as path + ".tmp", flushed to the disk (fsync) and renamed over
 * path, so an interrupted write leaves an existing checkpoint at path
 * unchanged. */
int yh_write_checkpoint(const char *path, const yh_param_var *p, int model,
                        const yh_fk_params *fk, const uint8_t *mask,
                        long long step, const float *u, const float *v,
                        const float *w);
/* Reads and checks only the header: the sizes the caller needs before
 * yh_read_checkpoint. */
int yh_read_checkpoint_header(const char *path, yh_checkpoint_header *out);
/* Reads the whole file and checks its hash. Any output may be NULL to skip
 * it. The arrays hold nx*ny elements, as the header gives. The mask is set
 * to 1 (all tissue) when the file holds none. The payload is streamed into
 * the outputs before the hash is compared: on YH_ECORRUPT (or any error)
 * they hold whatever had been read, so pass buffers whose contents may be
 * lost, not a live state. */
int yh_read_checkpoint(const char *path, yh_param_var *p, int *model,
                       yh_fk_params *fk, uint8_t *mask, long long *step,
                       float *u, float *v, float *w);

#ifdef __cplusplus
}
#endif

#endif /* YOLOHTLI_GB300_H */
