// The reference's interchange files (include/yolohtli.h, layer 4), so that
// its MATLAB post-processing reads this library's results unchanged:
//   dataparamcsv.csv   parameters, written by printParameters
//                      (printFunctions.cu:266-403) and read back by
//                      loadParamValues (saveFiles.cu:540-711)
//   raw_data.dat       u, v per cell, row-major (print2D2column,
//                      printFunctions.cu:58-78; read by loadData,
//                      saveFiles.cu:507-537); the window around the last tip
//                      of the symmetry-reduced saves (print2DSubWindow,
//                      printFunctions.cu:80-103)
//   dataTip.dat        tips, one per line, and dataTipSize.dat, the number
//                      of tips per save (printTip, printFunctions.cu:149-197)
//   c_phi_list_sym.dat c and phi per step (printSym, printFunctions.cu:249-264)
// The line formats (labels, order, printf conversions and the float/double
// casts behind them) are the reference's, so the files match its own output
// byte for byte; everything else (the API, validation, error returns
// instead of exit()) is this library's.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <string>
#include <vector>

#include "../../include/yolohtli.h"

namespace {

inline double f(double x) { return (double)(float)x; }  // the (float) casts

}  // namespace

extern "C" int yh_write_param_csv(const char *path, const yh_param_var *p,
                                  const char *ic_path,
                                  const char *results_path) {
  if (!path || !p) return YH_EINVAL;
  FILE *o = fopen(path, "w");
  if (!o) return YH_EINVAL;
  fprintf(o, "Initial condition path:,%s\n", ic_path ? ic_path : "NA");
  fprintf(o, "Results file path:,%s\n", results_path ? results_path : "NA");
  const struct {
    const char *label;
    int value;
  } flags[] = {
      {"Save every sampling period:,%d\n", p->saveEveryIt},
      {"plot tip on screen:,%d\n", p->plotTip},
      {"Save tip in to data file:,%d\n", p->recordTip},
      {"Plot contours on screen:,%d\n", p->plotContour},
      {"Save contours to data file:,%d\n", p->recordContour},
      {"Pacing stimulus:,%d\n", p->stimulate},
      {"Plot time series:,%d\n", p->plotTimeSeries},
      {"Record time series:,%d\n", p->recordTimeSeries},
      {"Reduce symmetry:,%d\n", p->reduceSym},
      {"Solid boundary:,%d\n", p->solidSwitch},
      {"Neumann BCs:,%d\n", p->neumannBC},
      {"Gate diffusion:,%d\n", p->gateDiff},
  };
  for (const auto &x : flags) fprintf(o, x.label, x.value ? 1 : 0);
  fprintf(o, "Tip trajectory algorithm:, %d\n", p->tipAlgorithm);
  fprintf(o, "Anisotropic tisue:,%d\n", p->anisotropy ? 1 : 0);
  fprintf(o, "Tip gradient:,%d\n", p->tipGrad ? 1 : 0);
  fprintf(o, "Contour mode (space APD or refractory):,%d\n", p->contourMode);
  fprintf(o, "Laplacian order:,%d\n", p->lap4 ? 1 : 0);
  fprintf(o, "Scheme order for time integration (Euler or RK4):,%d\n",
          p->timeIntOrder);
  fprintf(o, "Conduction block clock:,%d\n", p->clock ? 1 : 0);
  fprintf(o, "Conduction block counterclock:,%d\n", p->counterclock ? 1 : 0);
  fprintf(o, "# grid points X =,%d\n", p->nx);
  fprintf(o, "# grid points Y =,%d\n", p->ny);
  fprintf(o, "Physical Lx length,%f\n", f(p->Lx));
  fprintf(o, "Physical Ly length,%f\n", f(p->Ly));
  fprintf(o, "Physical dx,%f\n", f(p->hx));
  fprintf(o, "Physical dy,%f\n", f(p->hy));
  // the symmetry-reduced driver halves dt (main.cu); the file keeps the
  // full step
  fprintf(o, "Time step:,%f\n", p->reduceSym ? 2.0 * (float)p->dt : p->dt);
  const struct {
    const char *label;
    double value;
  } reals[] = {
      {"Diffusion parallel component:,%f\n", p->diff_par},
      {"Diffusion perpendicular component:,%f\n", p->diff_per},
      {"Initial fiber angle:,%f\n", p->degrad},
      {"Diffusion Dxx:,%f\n", p->Dxx},
      {"Diffusion Dyy:,%f\n", p->Dyy},
      {"Diffusion Dxy:,%f\n", p->Dxy},
      {"rxy (2*Dxy*dt/(4*dx*dy)):,%f\n", p->rxy},
      {"rbx (hx*Dxy/(Dxx*dy)):,%f\n", p->rbx},
      {"rby (hy*Dxy/(Dyy*dx)):,%f\n", p->rby},
      {"rx (Dxx*dt/(dx*dx)):,%f\n", p->rx},
      {"ry (Dyy*dt/(dy*dy)):,%f\n", p->ry},
      {"Gate r-scale:,%f\n", p->rscale},
      {"invdx (1/(2*hx)),%f\n", p->invdx},
      {"invdy (1/(2*hy)),%f\n", p->invdy},
      {"qx4 (dt*hx*hx*Dyy/12):,%f\n", p->qx4},
      {"qy4 (dt*hy*hx*Dxx/12):,%f\n", p->qy4},
      {"fx4 (dt*hx*hx/12):,%f\n", p->fx4},
      {"fy4 (dt*hy*hy/12):,%f\n", p->fy4},
      {"Physical time limit:,%f\n", p->physicalTimeLim},
      {"Start recording time:,%f\n", (double)p->startRecTime},
  };
  for (const auto &x : reals) fprintf(o, x.label, f(x.value));
  fprintf(o, "Number of electrodes,%d\n", p->eSize);
  fprintf(o, "Electrode position x:,%f\n", f(p->point.x));
  fprintf(o, "Electrode position y:,%f\n", f(p->point.y));
  fprintf(o, "Stimulus period (ms):,%f\n", p->stimPeriod);
  fprintf(o, "Stimulus magnitude:,%f\n", f(p->stimMag));
  fprintf(o, "Stimulus duration (ms):,%f\n", f(p->stimDuration));
  fprintf(o, "Voltage threshold for fibrillation:,%f\n", f(p->fibThreshold ? 1 : 0));
  fprintf(o, "Fibrillation terminated by pacing:,%d\n", p->fibTerminated ? 1 : 0);
  fprintf(o, "Number of LEAP shocks applied:,%d\n", p->leapShocks);
  fprintf(o, "Number of points in circles:,%d\n", p->nc);
  fprintf(o, "Stimulus position x:,%f\n", f(p->stcx));
  fprintf(o, "Stimulus position y:,%f\n", f(p->stcy));
  fprintf(o, "Stimulus area radius:,%f\n", f(p->rdomStim));
  fprintf(o, "APD area radius:,%f\n", f(p->rdomAPD));
  fprintf(o, "Tip offset x,%d\n", p->tipOffsetX);
  fprintf(o, "Tip offset y,%d\n", p->tipOffsetY);
  fprintf(o, "Integral area radius:,%f\n", f(p->rdomTrapz));
  fprintf(o, "Dirichlet BC value:,%f\n", f(p->boundaryVal));
  fprintf(o, "Iterations per frame:,%d\n", p->itPerFrame);
  fprintf(o, "Sampling period (ms):,%f\n", p->sample);
  fprintf(o, "Min signal range,%f\n", f(p->minVarColor));
  fprintf(o, "Max signal range,%f\n", f(p->maxVarColor));
  fprintf(o, "Secondary window size x,%d\n", p->wnx);
  fprintf(o, "Secondary window size y,%d\n", p->wny);
  fprintf(o, "Secondary window min signal 1,%f\n", f(p->uMin));
  fprintf(o, "Secondary window max signal 1,%f\n", f(p->uMax));
  fprintf(o, "Secondary window min signal 2,%f\n", f(p->vMin));
  fprintf(o, "Secondary window max signal 2,%f\n", f(p->vMax));
  fprintf(o, "Last tip point X,%f\n", f(p->tipx));
  fprintf(o, "Last tip point Y,%f\n", f(p->tipy));
  const struct {
    const char *label;
    double value;
  } tail[] = {
      {"Contour threshold 1:,%f\n", p->contourThresh1},
      {"Contour threshold 2:,%f\n", p->contourThresh2},
      {"Contour threshold 3:,%f\n", p->contourThresh3},
      {"Filament voltage threshold:,%f\n", p->Uth},
      {"time scale (tc):,%f\n", p->tc},
      {"alpha:,%f\n", p->alpha},
      {"beta:,%f\n", p->beta},
      {"gamma:,%f\n", p->gamma},
      {"delta:,%f\n", p->delta},
      {"epsilon:,%f\n", p->eps},
      {"mu:,%f\n", p->mu},
      {"theta:,%f\n", p->theta},
  };
  for (const auto &x : tail) fprintf(o, x.label, f(x.value));
  const int bad = ferror(o);
  fclose(o);
  return bad ? YH_EINVAL : YH_OK;
}

extern "C" int yh_read_param_csv(const char *path, yh_param_var *p) {
  if (!path || !p) return YH_EINVAL;
  FILE *in = fopen(path, "r");
  if (!in) return YH_EINVAL;
  // the second comma-separated field of every line, as a float
  std::vector<float> v;
  char line[512];
  while (fgets(line, sizeof(line), in)) {
    const char *c = strchr(line, ',');
    v.push_back(c ? strtof(c + 1, nullptr) : 0.f);
  }
  fclose(in);
  constexpr int kLines = 91;  // the lines printParameters writes
  if ((int)v.size() < kLines) return YH_EINVAL;
  int i = 2;  // the two path lines come first
  auto next = [&]() { return v[i++]; };
  p->animate = true;
  p->saveEveryIt = (int)next();
  p->plotTip = (int)next();
  p->recordTip = (int)next();
  p->plotContour = (int)next();
  p->recordContour = (int)next();
  p->stimulate = (int)next();
  p->plotTimeSeries = (int)next();
  p->recordTimeSeries = (int)next();
  p->reduceSym = (int)next();
  p->reduceSymStart = p->reduceSym;
  p->solidSwitch = (int)next();
  p->neumannBC = (int)next();
  p->gateDiff = (int)next();
  p->tipAlgorithm = (int)next();
  p->anisotropy = (int)next();
  p->tipGrad = (int)next();
  p->contourMode = (int)next();
  p->lap4 = (int)next();
  p->timeIntOrder = (int)next();
  p->clock = (int)next();
  p->counterclock = (int)next();
  p->nx = (int)next();
  p->ny = (int)next();
  p->Lx = next();
  p->Ly = next();
  p->hx = next();
  p->hy = next();
  p->dt = next();
  p->diff_par = next();
  p->diff_per = next();
  p->degrad = next();
  p->Dxx = next();
  p->Dyy = next();
  p->Dxy = next();
  p->rxy = next();
  p->rbx = next();
  p->rby = next();
  p->rx = next();
  p->ry = next();
  p->rscale = next();
  p->invdx = next();
  p->invdy = next();
  p->qx4 = next();
  p->qy4 = next();
  p->fx4 = next();
  p->fy4 = next();
  p->count = 0;
  p->physicalTime = 0.0;
  p->physicalTimeLim = next();
  p->startRecTime = (int)next();
  p->eSize = (int)next();
  // The reference fills the electrode position with make_int2(values[++i],
  // values[++i]) (saveFiles.cu:660), whose argument order C++ leaves open;
  // its GCC build takes y from the first of the two lines, so a written
  // (x, y) reads back as (y, x). This reader does the same.
  p->point.y = (int)next();
  p->point.x = (int)next();
  p->stimPeriod = next();
  p->stimMag = next();
  p->stimDuration = next();
  p->fibThreshold = next() != 0.f;
  p->fibTerminated = next() != 0.f;
  p->leapShocks = (int)next();
  p->nc = (int)next();
  p->stcx = next();
  p->stcy = next();
  p->rdomStim = next();
  p->rdomAPD = next();
  p->tipOffsetX = (int)next();
  p->tipOffsetY = (int)next();
  p->rdomTrapz = next();
  p->boundaryVal = next();
  p->itPerFrame = (int)next();
  p->sample = next();
  p->minVarColor = next();
  p->maxVarColor = next();
  p->wnx = (int)next();
  p->wny = (int)next();
  p->uMin = next();
  p->uMax = next();
  p->vMin = next();
  p->vMax = next();
  p->tipx = next();
  p->tipy = next();
  p->contourThresh1 = next();
  p->contourThresh2 = next();
  p->contourThresh3 = next();
  p->Uth = next();
  p->tc = next();
  p->alpha = next();
  p->beta = next();
  p->gamma = next();
  p->delta = next();
  p->eps = next();
  p->mu = next();
  p->theta = next();
  return YH_OK;
}

extern "C" int yh_write_raw_data(const char *path, const yh_param_var *p,
                                 const float *u, const float *v) {
  if (!path || !p || !u || !v || p->nx <= 0 || p->ny <= 0) return YH_EINVAL;
  FILE *o = fopen(path, "w");
  if (!o) return YH_EINVAL;
  const size_t n = (size_t)p->nx * p->ny;
  for (size_t k = 0; k < n; ++k) fprintf(o, "%f %f\n", (double)u[k], (double)v[k]);
  const int bad = ferror(o);
  fclose(o);
  return bad ? YH_EINVAL : YH_OK;
}

extern "C" int yh_write_raw_window(const char *path, const yh_param_var *p,
                                   const float *u, const float *v) {
  if (!path || !p || !u || !v) return YH_EINVAL;
  const int x0 = (int)floorf(p->tipx) - p->tipOffsetX - 1;
  const int x1 = (int)floorf(p->tipx) + p->tipOffsetX + 1;
  const int y0 = (int)floorf(p->tipy) - p->tipOffsetY - 1;
  const int y1 = (int)floorf(p->tipy) + p->tipOffsetY + 1;
  // the reference reads outside the grid here; this library refuses
  if (x0 < 0 || y0 < 0 || x1 > p->nx || y1 > p->ny) return YH_EINVAL;
  FILE *o = fopen(path, "w");
  if (!o) return YH_EINVAL;
  for (int j = y0; j < y1; ++j)
    for (int i = x0; i < x1; ++i) {
      const size_t k = (size_t)i + (size_t)p->nx * j;
      fprintf(o, "%f %f\n", (double)u[k], (double)v[k]);
    }
  const int bad = ferror(o);
  fclose(o);
  return bad ? YH_EINVAL : YH_OK;
}

extern "C" int yh_read_raw_data(const char *path, const yh_param_var *p,
                                float *u, float *v) {
  if (!path || !p || !u || !v || p->nx <= 0 || p->ny <= 0) return YH_EINVAL;
  FILE *in = fopen(path, "r");
  if (!in) return YH_EINVAL;
  const size_t n = (size_t)p->nx * p->ny;
  for (size_t k = 0; k < n; ++k)
    if (fscanf(in, "%f %f", &u[k], &v[k]) != 2) {
      fclose(in);
      return YH_EINVAL;
    }
  fclose(in);
  return YH_OK;
}

extern "C" int yh_write_tips(const char *tip_path, const char *size_path,
                             const yh_tip *tips, int n, int append) {
  if (!tip_path || !size_path || n < 0 || (n && !tips)) return YH_EINVAL;
  FILE *a = fopen(tip_path, append ? "a" : "w");
  FILE *b = fopen(size_path, append ? "a" : "w");
  if (!a || !b) {
    if (a) fclose(a);
    if (b) fclose(b);
    return YH_EINVAL;
  }
  for (int k = 0; k < n; ++k)
    fprintf(a, "%f %f %f %f %f\n", (double)tips[k].x, (double)tips[k].y,
            (double)tips[k].vx, (double)tips[k].vy, (double)tips[k].t);
  if (n > 0) fprintf(b, "%d\n", n);  // a save without tips adds no line
  const int bad = ferror(a) || ferror(b);
  fclose(a);
  fclose(b);
  return bad ? YH_EINVAL : YH_OK;
}

extern "C" int yh_write_sym_list(const char *path, const double *c,
                                 const double *phi, int n) {
  if (!path || n < 0 || (n && (!c || !phi))) return YH_EINVAL;
  FILE *o = fopen(path, "w");
  if (!o) return YH_EINVAL;
  for (int k = 0; k < n; ++k)
    fprintf(o, "%f %f %f %f %f %f\n", c[3 * k], c[3 * k + 1], c[3 * k + 2],
            phi[3 * k], phi[3 * k + 1], phi[3 * k + 2]);
  const int bad = ferror(o);
  fclose(o);
  return bad ? YH_EINVAL : YH_OK;
}

// ---------------------------------------------------------------------------
// Binary checkpoint (this library's format; the header file gives the byte
// layout). The header is packed field by field at fixed offsets, so struct
// padding never reaches the file; the payload is streamed through a 1 MiB
// buffer with its FNV-1a 64-bit hash computed on the way.
// ---------------------------------------------------------------------------
namespace {

constexpr char kMagic[8] = {'Y', 'H', 'C', 'K', 'P', 'T', 0, 0};
constexpr uint32_t kVersion = 1;
constexpr uint32_t kByteOrder = 0x01020304u;
constexpr size_t kHeaderBytes = 64;
constexpr size_t kChunk = 1 << 20;

struct Fnv1a64 {  // FNV-1a, 64-bit offset basis and prime
  uint64_t h = 0xcbf29ce484222325ull;
  void add(const void *data, size_t n) {
    const uint8_t *b = (const uint8_t *)data;
    for (size_t k = 0; k < n; ++k) {
      h ^= b[k];
      h *= 0x100000001b3ull;
    }
  }
};

struct Header {
  int32_t nx, ny, model, nfields, has_mask, param_bytes;
  int64_t step;
  uint64_t payload, hash;
};

inline int nfields_of(int model) { return model == YH_MODEL_FK3V ? 3 : 2; }

inline uint64_t payload_bytes(int nx, int ny, int nf, int has_mask) {
  const uint64_t n = (uint64_t)nx * (uint64_t)ny;
  return sizeof(yh_param_var) + sizeof(yh_fk_params) +
         (has_mask ? n : 0) + (uint64_t)nf * n * sizeof(float);
}

template <typename T>
inline void put(uint8_t *b, size_t off, T x) { memcpy(b + off, &x, sizeof(T)); }
template <typename T>
inline T get(const uint8_t *b, size_t off) {
  T x;
  memcpy(&x, b + off, sizeof(T));
  return x;
}

void pack(const Header &h, uint8_t *b) {
  memset(b, 0, kHeaderBytes);
  memcpy(b, kMagic, 8);
  put<uint32_t>(b, 8, kVersion);
  put<uint32_t>(b, 12, kByteOrder);
  put<int32_t>(b, 16, h.nx);
  put<int32_t>(b, 20, h.ny);
  put<int32_t>(b, 24, h.model);
  put<int32_t>(b, 28, h.nfields);
  put<int32_t>(b, 32, h.has_mask);
  put<int32_t>(b, 36, h.param_bytes);
  put<int64_t>(b, 40, h.step);
  put<uint64_t>(b, 48, h.payload);
  put<uint64_t>(b, 56, h.hash);
}

// YH_ECORRUPT unless every header field is one this library writes.
int unpack(const uint8_t *b, Header *h) {
  if (memcmp(b, kMagic, 8) != 0) return YH_ECORRUPT;
  if (get<uint32_t>(b, 8) != kVersion) return YH_ECORRUPT;
  if (get<uint32_t>(b, 12) != kByteOrder) return YH_ECORRUPT;
  h->nx = get<int32_t>(b, 16);
  h->ny = get<int32_t>(b, 20);
  h->model = get<int32_t>(b, 24);
  h->nfields = get<int32_t>(b, 28);
  h->has_mask = get<int32_t>(b, 32);
  h->param_bytes = get<int32_t>(b, 36);
  h->step = get<int64_t>(b, 40);
  h->payload = get<uint64_t>(b, 48);
  h->hash = get<uint64_t>(b, 56);
  if (h->nx < 1 || h->ny < 1 ||
      (int64_t)h->nx * h->ny > (int64_t)(1LL << 31) - 1)
    return YH_ECORRUPT;
  if (h->model != YH_MODEL_REF2V && h->model != YH_MODEL_FK3V)
    return YH_ECORRUPT;
  if (h->nfields != nfields_of(h->model)) return YH_ECORRUPT;
  if (h->has_mask != 0 && h->has_mask != 1) return YH_ECORRUPT;
  if (h->param_bytes != (int32_t)sizeof(yh_param_var)) return YH_ECORRUPT;
  if (h->step < 0) return YH_ECORRUPT;
  if (h->payload != payload_bytes(h->nx, h->ny, h->nfields, h->has_mask))
    return YH_ECORRUPT;
  return YH_OK;
}

// Opens path and reads and checks its header; *in is open on success.
int open_checkpoint(const char *path, FILE **in, Header *h) {
  *in = fopen(path, "rb");
  if (!*in) return YH_EINVAL;
  uint8_t b[kHeaderBytes];
  int rc = fread(b, 1, kHeaderBytes, *in) == kHeaderBytes ? unpack(b, h)
                                                          : YH_ECORRUPT;
  if (rc) {
    fclose(*in);
    *in = nullptr;
  }
  return rc;
}

// Reads n payload bytes into dst (NULL: read and hash, keep nothing).
bool read_hashed(FILE *in, void *dst, uint64_t n, Fnv1a64 *hash,
                 std::vector<uint8_t> *buf) {
  uint8_t *d = (uint8_t *)dst;
  while (n > 0) {
    const size_t m = (size_t)(n < kChunk ? n : kChunk);
    uint8_t *to = d ? d : buf->data();
    if (fread(to, 1, m, in) != m) return false;
    hash->add(to, m);
    if (d) d += m;
    n -= m;
  }
  return true;
}

}  // namespace

extern "C" int yh_write_checkpoint(const char *path, const yh_param_var *p,
                                   int model, const yh_fk_params *fk,
                                   const uint8_t *mask, long long step,
                                   const float *u, const float *v,
                                   const float *w) {
  if (!path || !p || !u || !v || step < 0) return YH_EINVAL;
  if (model != YH_MODEL_REF2V && model != YH_MODEL_FK3V) return YH_EINVAL;
  if (model == YH_MODEL_FK3V && (!fk || !w)) return YH_EINVAL;
  if (p->nx < 1 || p->ny < 1 ||
      (long long)p->nx * p->ny > (1LL << 31) - 1)
    return YH_EINVAL;
  Header h;
  h.nx = p->nx;
  h.ny = p->ny;
  h.model = model;
  h.nfields = nfields_of(model);
  h.has_mask = mask ? 1 : 0;
  h.param_bytes = (int32_t)sizeof(yh_param_var);
  h.step = step;
  h.payload = payload_bytes(h.nx, h.ny, h.nfields, h.has_mask);
  yh_fk_params fk0;
  memset(&fk0, 0, sizeof(fk0));
  if (fk) fk0 = *fk;
  const size_t n = (size_t)h.nx * h.ny;
  struct Part { const void *data; size_t bytes; };
  const Part parts[6] = {{p, sizeof(yh_param_var)},
                         {&fk0, sizeof(fk0)},
                         {mask, mask ? n : 0},
                         {u, n * sizeof(float)},
                         {v, n * sizeof(float)},
                         {w, h.nfields > 2 ? n * sizeof(float) : 0}};
  Fnv1a64 hash;
  for (const Part &q : parts) hash.add(q.data, q.bytes);
  h.hash = hash.h;
  uint8_t b[kHeaderBytes];
  pack(h, b);
  // Written to path.tmp, flushed to the disk, then renamed over path: an
  // interrupted save (a crash, a kill, a full disk) leaves the previous
  // checkpoint at `path` intact.
  std::string tmp = std::string(path) + ".tmp";
  FILE *o = fopen(tmp.c_str(), "wb");
  if (!o) return YH_EINVAL;
  bool ok = fwrite(b, 1, kHeaderBytes, o) == kHeaderBytes;
  for (const Part &q : parts)
    if (ok && q.bytes) ok = fwrite(q.data, 1, q.bytes, o) == q.bytes;
  ok = ok && fflush(o) == 0 && fsync(fileno(o)) == 0;
  ok = (fclose(o) == 0) && ok;
  ok = ok && rename(tmp.c_str(), path) == 0;
  if (!ok) remove(tmp.c_str());
  return ok ? YH_OK : YH_EINVAL;
}

extern "C" int yh_read_checkpoint_header(const char *path,
                                         yh_checkpoint_header *out) {
  if (!path || !out) return YH_EINVAL;
  FILE *in;
  Header h;
  const int rc = open_checkpoint(path, &in, &h);
  if (rc) return rc;
  fclose(in);
  out->nx = h.nx;
  out->ny = h.ny;
  out->model = h.model;
  out->nfields = h.nfields;
  out->has_mask = h.has_mask;
  out->step = h.step;
  return YH_OK;
}

extern "C" int yh_read_checkpoint(const char *path, yh_param_var *p,
                                  int *model, yh_fk_params *fk, uint8_t *mask,
                                  long long *step, float *u, float *v,
                                  float *w) {
  if (!path) return YH_EINVAL;
  FILE *in;
  Header h;
  int rc = open_checkpoint(path, &in, &h);
  if (rc) return rc;
  std::vector<uint8_t> buf(kChunk);
  yh_param_var pv;
  const size_t n = (size_t)h.nx * h.ny;
  Fnv1a64 hash;
  bool ok = read_hashed(in, &pv, sizeof(pv), &hash, &buf) &&
            read_hashed(in, fk, sizeof(yh_fk_params), &hash, &buf) &&
            (!h.has_mask || read_hashed(in, mask, n, &hash, &buf)) &&
            read_hashed(in, u, n * sizeof(float), &hash, &buf) &&
            read_hashed(in, v, n * sizeof(float), &hash, &buf) &&
            (h.nfields < 3 || read_hashed(in, w, n * sizeof(float), &hash, &buf));
  // nothing may follow the payload
  ok = ok && fgetc(in) == EOF;
  fclose(in);
  if (!ok || hash.h != h.hash || pv.nx != h.nx || pv.ny != h.ny)
    return YH_ECORRUPT;
  if (p) *p = pv;
  if (model) *model = h.model;
  if (step) *step = h.step;
  if (mask && !h.has_mask) memset(mask, 1, n);
  return YH_OK;
}
