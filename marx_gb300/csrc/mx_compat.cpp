// libmarx_gb300_compat: MARX's stage API over Marx_Photon_Type (the
// reference's array-of-structures photon list), traced by libmarx_gb300.
//
// Each stage call prunes the batch, gathers the attributes of the photons
// in sorted_index into the engine's structure-of-arrays columns (host
// staging, one copy to the device per column), runs the stage through
// mx_trace, and scatters the results back into the attributes.  The stage
// order, the history bits and the pruning are the reference's
// (marx/src/marx.c:240-273, hrma.c:1161-1175, diffract.c:974-990,
// acis-i.c:96-112, acis-s.c:180-195, hrc-i.c:119-131, hrc-s.c:236-250,
// photon.c:40-118).
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dlfcn.h>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/marx_gb300.h"
#include "../../include/marx_gb300_compat.h"

// The reference's parameter-file library, linked by the calling program
// (pfile.h:82-85).  Weak: the library loads without it, and *_init then
// reports that no parameter file can be read.
extern "C" {
int pf_get_string(Param_File_Type *, char *, char *, unsigned int) __attribute__((weak));
int pf_get_double(Param_File_Type *, char *, double *) __attribute__((weak));
int pf_get_integer(Param_File_Type *, char *, int *) __attribute__((weak));
int pf_get_boolean(Param_File_Type *, char *, int *) __attribute__((weak));
}

// Globals of the reference's mirror module that its other modules read:
// the aperture area behind a source's photon rate (source.c:260-264) and
// the cap position the SAOSAC source places its rays at (s-saosac.c:224).
// marx_mirror_init sets both; a program linking this library instead of
// those modules gets them from here.
extern "C" {
__attribute__((visibility("default"))) double Marx_Mirror_Geometric_Area = 1.0;
__attribute__((visibility("default"))) double _Marx_HRMA_Cap_Position = 10079.5;
}

namespace {

// The MARX type ids the *_init functions return (marx.h:364-376).
constexpr int MIRROR_HRMA = 2;
constexpr int DET_ID[5] = {0, 4, 3, 2, 1};   // by MX_DETECTOR_*: NONE, ACIS-I, ACIS-S, HRC-I, HRC-S

struct Dev {
  void *ptr = nullptr;
  size_t bytes = 0;
  bool ensure(size_t need) {
    if (need <= bytes) return true;
    if (ptr) cudaFree(ptr);
    ptr = nullptr; bytes = 0;
    if (cudaMalloc(&ptr, need) != cudaSuccess) { ptr = nullptr; return false; }
    bytes = need;
    return true;
  }
  void release() { if (ptr) cudaFree(ptr); ptr = nullptr; bytes = 0; }
};

struct State {
  std::mutex mu;
  mx_config cfg;
  bool cfg_init = false;
  int mirror = -1, grating = -1, detector = -1, dither = -1;   // types once initialised
  mx_context *ctx = nullptr;
  bool dirty = true;
  double ctx_source_distance = 0.0;
  uint64_t seed = 0;
  const double *U = nullptr, *N = nullptr;
  unsigned int var_n = 0;
  std::string err;
  Dev dev;                            // every device column in one allocation
  std::vector<char> host;             // the staged columns
};

State &S() {
  static State s;
  return s;
}

void ensure_cfg(State &s) {
  if (!s.cfg_init) { mx_config_default(&s.cfg); s.cfg_init = true; }
}

int error(State &s, const char *fmt, ...) {
  char b[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(b, sizeof b, fmt, ap);
  va_end(ap);
  s.err = b;
  fprintf(stderr, "***MARX (gb300 compat) error: %s\n", b);
  return -1;
}

// A parameter through the caller's parameter-file library, as text for
// mx_config_read_params.
int pf_reader(void *user, const char *name, char type, char *value, size_t len) {
  Param_File_Type *pf = (Param_File_Type *) user;
  char *nm = const_cast<char *>(name);
  switch (type) {
    case 'r': {
      double d;
      if (pf_get_double(pf, nm, &d) != 0) return -1;
      snprintf(value, len, "%.17g", d);
      return 0;
    }
    case 'i': {
      int i;
      if (pf_get_integer(pf, nm, &i) != 0) return -1;
      snprintf(value, len, "%d", i);
      return 0;
    }
    case 'b': {
      int b;
      if (pf_get_boolean(pf, nm, &b) != 0) return -1;
      snprintf(value, len, "%s", b ? "yes" : "no");
      return 0;
    }
    default:
      return pf_get_string(pf, nm, value, (unsigned int) len) == 0 ? 0 : -1;
  }
}

int read_group(State &s, Param_File_Type *pf, uint32_t group, const char *who) {
  if (!pf_get_string || !pf_get_double || !pf_get_integer || !pf_get_boolean)
    return error(s, "%s: the program links no parameter-file library (pf_get_*)", who);
  if (!pf) return error(s, "%s: null parameter file", who);
  ensure_cfg(s);
  mx_config c = s.cfg;
  if (mx_config_read_params(&c, group, pf_reader, pf, 1) != MX_OK)
    return error(s, "%s: %s", who, mx_last_error(nullptr));
  s.cfg = c;
  s.dirty = true;
  return 0;
}

// The table pack: MARX_GB300_PACK, else caldb/marx_tables.mxpack in the
// package directory above the library's own.
std::string pack_path() {
  if (const char *e = getenv("MARX_GB300_PACK")) return e;
  Dl_info info;
  if (dladdr((void *) &pack_path, &info) && info.dli_fname) {
    std::string lib(info.dli_fname);
    size_t a = lib.rfind('/');
    std::string dir = a == std::string::npos ? "." : lib.substr(0, a);
    size_t b = dir.rfind('/');
    std::string pkg = b == std::string::npos ? ".." : dir.substr(0, b);
    return pkg + "/caldb/marx_tables.mxpack";
  }
  return "marx_gb300/caldb/marx_tables.mxpack";
}

// The engine context for the current configuration and batch.
int context(State &s, const Marx_Photon_Type *pt) {
  ensure_cfg(s);
  if (s.ctx && (s.dirty || s.ctx_source_distance != pt->source_distance)) {
    mx_config c = s.cfg;
    c.source_distance = pt->source_distance;
    if (mx_configure(s.ctx, &c) != MX_OK) return error(s, "configuring the engine: %s", mx_last_error(s.ctx));
  } else if (!s.ctx) {
    mx_config c = s.cfg;
    c.source_distance = pt->source_distance;
    s.ctx = mx_create(pack_path().c_str(), &c);
    if (!s.ctx) return error(s, "creating the engine: %s", mx_last_error(nullptr));
  }
  s.dirty = false;
  s.ctx_source_distance = pt->source_distance;
  if (mx_set_start_time(s.ctx, pt->start_time) != MX_OK) return error(s, "setting the batch start time");
  return 0;
}

// Column byte offsets of one staged batch of n photons (every column padded
// to 256 bytes).
struct Layout {
  size_t energy, x, p, t, flags, tag, shell, order, ccd, ypix, zpix, dith, sup, pha, upix, vpix, region, pi, U, N,
      total;
  Layout(size_t n, bool var) {
    size_t o = 0;
    auto put = [&](size_t bytes) { size_t a = o; o = (o + bytes + 255) & ~(size_t) 255; return a; };
    energy = put(8 * n); x = put(24 * n); p = put(24 * n); t = put(8 * n); flags = put(4 * n); tag = put(4 * n);
    shell = put(n); order = put(n); ccd = put(n); ypix = put(4 * n); zpix = put(4 * n); dith = put(12 * n);
    sup = put(4 * n); pha = put(2 * n); upix = put(4 * n); vpix = put(4 * n); region = put(n); pi = put(4 * n);
    U = var ? put(8 * (size_t) MX_NUM_U * n) : 0;
    N = var ? put(8 * (size_t) MX_NUM_N * n) : 0;
    total = o;
  }
};

template <class T> T *at(std::vector<char> &h, size_t off) { return (T *) (h.data() + off); }

// One stage over the photons of sorted_index.
int run_stage(State &s, Marx_Photon_Type *pt, uint32_t stage, const char *who) {
  if (context(s, pt)) return -1;
  const size_t n = pt->num_sorted;
  if (n == 0) return 0;
  const bool var = s.U != nullptr;
  const unsigned int *idx = pt->sorted_index;
  Marx_Photon_Attr_Type *A = pt->attributes;
  if (var)
    for (size_t k = 0; k < n; k++)
      if (idx[k] >= s.var_n)
        return error(s, "%s: photon %u has no pre-drawn variates (%u given)", who, idx[k], s.var_n);
  if (stage == MX_STAGE_DETECT)
    for (size_t k = 0; k < n; k++) {
      const Marx_Dither_Type &d = A[idx[k]].dither_state;
      if (d.dy != 0.f || d.dz != 0.f || d.dtheta != 0.f)
        return error(s, "%s: detector motion (DitherModel FILE) is not supported by this library", who);
    }
  Layout L(n, var);
  s.host.resize(L.total);
  std::vector<char> &h = s.host;
  double *E = at<double>(h, L.energy), *X = at<double>(h, L.x), *P = at<double>(h, L.p), *T = at<double>(h, L.t);
  uint32_t *F = at<uint32_t>(h, L.flags), *G = at<uint32_t>(h, L.tag);
  int8_t *SH = at<int8_t>(h, L.shell), *OR = at<int8_t>(h, L.order), *CC = at<int8_t>(h, L.ccd);
  float *YP = at<float>(h, L.ypix), *ZP = at<float>(h, L.zpix), *DI = at<float>(h, L.dith);
  int8_t *SU = at<int8_t>(h, L.sup);
  int16_t *PH = at<int16_t>(h, L.pha);
  float *UP = at<float>(h, L.upix), *VP = at<float>(h, L.vpix), *PI = at<float>(h, L.pi);
  uint8_t *RG = at<uint8_t>(h, L.region);
  for (size_t k = 0; k < n; k++) {
    const Marx_Photon_Attr_Type &a = A[idx[k]];
    E[k] = a.energy;
    X[k] = a.x.x; X[n + k] = a.x.y; X[2 * n + k] = a.x.z;
    P[k] = a.p.x; P[n + k] = a.p.y; P[2 * n + k] = a.p.z;
    T[k] = a.arrival_time; F[k] = a.flags; G[k] = a.tag;
    SH[k] = (int8_t) a.mirror_shell; OR[k] = a.order; CC[k] = a.ccd_num;
    YP[k] = a.y_pixel; ZP[k] = a.z_pixel;
    DI[k] = a.dither_state.ra; DI[n + k] = a.dither_state.dec; DI[2 * n + k] = a.dither_state.roll;
    for (int j = 0; j < 4; j++) SU[j * n + k] = a.support_orders[j];
    PH[k] = a.pulse_height; UP[k] = a.u_pixel; VP[k] = a.v_pixel; RG[k] = (uint8_t) a.detector_region;
    PI[k] = a.pi;
  }
  if (var) {
    double *u = at<double>(h, L.U), *v = at<double>(h, L.N);
    for (int j = 0; j < MX_NUM_U; j++)
      for (size_t k = 0; k < n; k++) u[j * n + k] = s.U[(size_t) j * s.var_n + idx[k]];
    for (int j = 0; j < MX_NUM_N; j++)
      for (size_t k = 0; k < n; k++) v[j * n + k] = s.N[(size_t) j * s.var_n + idx[k]];
  }
  if (!s.dev.ensure(L.total)) return error(s, "%s: cannot allocate %zu bytes of device memory", who, L.total);
  cudaStream_t st = (cudaStream_t) mx_stream(s.ctx);
  char *d = (char *) s.dev.ptr;
  if (cudaMemcpyAsync(d, h.data(), L.total, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return error(s, "%s: copying the photons to the device", who);
  mx_photons ph;
  memset(&ph, 0, sizeof ph);
  ph.n = (uint32_t) n;
  ph.energy = (double *) (d + L.energy); ph.x = (double *) (d + L.x); ph.p = (double *) (d + L.p);
  ph.arrival_time = (double *) (d + L.t); ph.flags = (uint32_t *) (d + L.flags); ph.tag = (uint32_t *) (d + L.tag);
  ph.mirror_shell = (int8_t *) (d + L.shell); ph.order = (int8_t *) (d + L.order); ph.ccd_num = (int8_t *) (d + L.ccd);
  ph.y_pixel = (float *) (d + L.ypix); ph.z_pixel = (float *) (d + L.zpix); ph.dither_state = (float *) (d + L.dith);
  ph.support_orders = (int8_t *) (d + L.sup); ph.pulse_height = (int16_t *) (d + L.pha);
  ph.u_pixel = (float *) (d + L.upix); ph.v_pixel = (float *) (d + L.vpix);
  ph.detector_region = (uint8_t *) (d + L.region); ph.pi = (float *) (d + L.pi);
  mx_variates mv = {var ? (const double *) (d + L.U) : nullptr, var ? (const double *) (d + L.N) : nullptr};
  if (mx_trace(s.ctx, &ph, stage, &mv, s.seed, st) != MX_OK)
    return error(s, "%s: %s", who, mx_last_error(s.ctx));
  // the outputs: every column before the variates
  if (cudaMemcpyAsync(h.data(), d, L.pi + 4 * n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return error(s, "%s: copying the photons back: %s", who, cudaGetErrorString(cudaGetLastError()));
  for (size_t k = 0; k < n; k++) {
    Marx_Photon_Attr_Type &a = A[idx[k]];
    a.x.x = X[k]; a.x.y = X[n + k]; a.x.z = X[2 * n + k];
    a.p.x = P[k]; a.p.y = P[n + k]; a.p.z = P[2 * n + k];
    a.flags = F[k];
    a.mirror_shell = (unsigned int) SH[k]; a.order = OR[k]; a.ccd_num = CC[k];
    a.y_pixel = YP[k]; a.z_pixel = ZP[k];
    a.dither_state.ra = DI[k]; a.dither_state.dec = DI[n + k]; a.dither_state.roll = DI[2 * n + k];
    for (int j = 0; j < 4; j++) a.support_orders[j] = SU[j * n + k];
    a.pulse_height = PH[k]; a.u_pixel = UP[k]; a.v_pixel = VP[k]; a.detector_region = (signed char) RG[k];
    a.pi = PI[k];
  }
  return 0;
}

}  // namespace

extern "C" {

void marx_prune_photons(Marx_Photon_Type *pt) {
  if (!pt) return;
  unsigned int m = 0;
  for (unsigned int i = 0; i < pt->num_sorted; i++) {
    const unsigned int k = pt->sorted_index[i];
    const Marx_Photon_Attr_Type &a = pt->attributes[k];
    if (a.flags & BAD_PHOTON_MASK) continue;
    if (pt->sorted_energies) pt->sorted_energies[m] = a.energy;
    pt->sorted_index[m++] = k;
  }
  pt->num_sorted = m;
}

Marx_Photon_Type *marx_alloc_photon_type(unsigned int num) {
  Marx_Photon_Type *pt = (Marx_Photon_Type *) calloc(1, sizeof(Marx_Photon_Type));
  if (!pt) return nullptr;
  pt->attributes = (Marx_Photon_Attr_Type *) calloc(num ? num : 1, sizeof(Marx_Photon_Attr_Type));
  pt->sorted_energies = (double *) calloc(num ? num : 1, sizeof(double));
  pt->sorted_index = (unsigned int *) calloc(num ? num : 1, sizeof(unsigned int));
  if (!pt->attributes || !pt->sorted_energies || !pt->sorted_index) {
    marx_dealloc_photon_type(pt);
    error(S(), "marx_alloc_photon_type: out of memory for %u photons", num);
    return nullptr;
  }
  pt->max_n_photons = num;
  return pt;
}

int marx_dealloc_photon_type(Marx_Photon_Type *pt) {
  if (!pt) return -1;
  free(pt->attributes);
  free(pt->sorted_energies);
  free(pt->sorted_index);
  free(pt);
  return 0;
}

int marx_mirror_init(Param_File_Type *pf) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.mirror = -1;
  if (read_group(s, pf, MX_PARAMS_MIRROR, "marx_mirror_init")) return -1;
  int seed;
  if (pf_get_integer(pf, (char *) "RandomSeed", &seed) == 0 && seed >= 0) s.seed = (uint64_t) seed;
  double area = 0.0;
  if (mx_geometric_area(pack_path().c_str(), &s.cfg, &area) != MX_OK)
    return error(s, "marx_mirror_init: %s", mx_last_error(nullptr));
  Marx_Mirror_Geometric_Area = area;
  _Marx_HRMA_Cap_Position = s.cfg.hrma_cap_x;
  s.mirror = MIRROR_HRMA;
  return s.mirror;
}

int marx_grating_init(Param_File_Type *pf) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.grating = -1;
  if (read_group(s, pf, MX_PARAMS_GRATING, "marx_grating_init")) return -1;
  s.grating = s.cfg.grating;
  return s.grating;
}

int marx_detector_init(Param_File_Type *pf) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.detector = -1;
  if (read_group(s, pf, MX_PARAMS_DETECTOR, "marx_detector_init")) return -1;
  s.detector = DET_ID[s.cfg.detector];
  return s.detector;
}

int marx_gb300_compat_dither_init(Param_File_Type *pf) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.dither = -1;
  if (read_group(s, pf, MX_PARAMS_DITHER, "marx_gb300_compat_dither_init")) return -1;
  if (s.cfg.dither == MX_DITHER_FILE)
    return error(s, "marx_gb300_compat_dither_init: DitherModel FILE is not supported by this library");
  s.dither = s.cfg.dither;
  return 0;
}

int marx_mirror_reflect(Marx_Photon_Type *pt, int verbose) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.mirror != MIRROR_HRMA) return error(s, "Mirror not initialized.");
  if (!pt) return error(s, "marx_mirror_reflect: null photon list");
  if (pt->history & MARX_MIRROR_SHELL_OK) return 0;   // been here already
  pt->history |= MARX_MIRROR_SHELL_OK;
  if (verbose > 0) fprintf(stderr, "Reflecting from HRMA\n");
  marx_prune_photons(pt);
  return run_stage(s, pt, MX_STAGE_MIRROR, "marx_mirror_reflect");
}

int marx_grating_diffract(Marx_Photon_Type *pt, int verbose) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.grating < 0) return error(s, "Grating not initialized.");
  if (!pt) return error(s, "marx_grating_diffract: null photon list");
  if (s.grating == MX_GRATING_NONE) return 0;
  if (pt->history & MARX_ORDER_OK) return 0;
  pt->history |= MARX_ORDER_OK;
  if (s.grating == MX_GRATING_LETG) {
    if (s.cfg.leg_fine_orders) pt->history |= MARX_ORDER1_OK;
    if (s.cfg.leg_coarse_orders) pt->history |= MARX_ORDER2_OK | MARX_ORDER3_OK | MARX_ORDER4_OK;
  }
  if (verbose > 0) fprintf(stderr, "Diffracting from %s.\n", s.grating == MX_GRATING_HETG ? "HETG" : "LETG");
  marx_prune_photons(pt);
  return run_stage(s, pt, MX_STAGE_GRATING, "marx_grating_diffract");
}

int marx_detect(Marx_Photon_Type *pt, int verbose) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.detector < 0) return error(s, "Detector not initialized.");
  if (!pt) return error(s, "marx_detect: null photon list");
  const int k = s.cfg.detector;
  if (k == MX_DETECTOR_NONE) return 0;
  if (pt->history & MARX_DET_NUM_OK) return 0;
  if (k == MX_DETECTOR_ACIS_I || k == MX_DETECTOR_ACIS_S)
    pt->history |= MARX_DET_PIXEL_OK | MARX_DET_NUM_OK | MARX_PULSEHEIGHT_OK | MARX_PI_OK;
  else
    pt->history |= MARX_DET_REGION_OK | MARX_PULSEHEIGHT_OK | MARX_DET_PIXEL_OK | MARX_DET_NUM_OK;
  if (k == MX_DETECTOR_HRC_S) pt->history |= MARX_DET_UV_PIXEL_OK;
  static const char *names[5] = {"NONE", "ACIS-I", "ACIS-S", "HRC-I", "HRC-S"};
  if (verbose > 0) fprintf(stderr, "Detecting with %s\n", names[k]);
  marx_prune_photons(pt);
  return run_stage(s, pt, MX_STAGE_DETECT, "marx_detect");
}

int marx_gb300_compat_dither_photons(Marx_Photon_Type *pt, unsigned int *num_dithered) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.dither < 0) return error(s, "marx_gb300_compat_dither_photons: dither not initialized");
  if (!pt) return error(s, "marx_gb300_compat_dither_photons: null photon list");
  if (num_dithered) *num_dithered = pt->n_photons;
  if (s.dither == MX_DITHER_NONE || pt->n_photons == 0) return 0;
  // every photon of the batch in attribute order, as _marx_dither_photons
  // walks them: a temporary sorted_index over all of them
  std::vector<unsigned int> all(pt->n_photons);
  for (unsigned int i = 0; i < pt->n_photons; i++) all[i] = i;
  unsigned int *keep_idx = pt->sorted_index, keep_num = pt->num_sorted;
  pt->sorted_index = all.data();
  pt->num_sorted = pt->n_photons;
  int r = run_stage(s, pt, MX_STAGE_DITHER, "marx_gb300_compat_dither_photons");
  pt->sorted_index = keep_idx;
  pt->num_sorted = keep_num;
  return r;
}

void marx_gb300_compat_set_seed(uint64_t seed) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  s.seed = seed;
}

int marx_gb300_compat_set_variates(const double *U, const double *N, unsigned int n) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if ((U == nullptr) != (N == nullptr)) return error(s, "marx_gb300_compat_set_variates: give both U and N or neither");
  s.U = U; s.N = N; s.var_n = U ? n : 0;
  return 0;
}

const char *marx_gb300_compat_last_error(void) { return S().err.c_str(); }

void marx_gb300_compat_shutdown(void) {
  State &s = S();
  std::lock_guard<std::mutex> lk(s.mu);
  if (s.ctx) mx_destroy(s.ctx);
  s.ctx = nullptr;
  s.dev.release();
  s.dirty = true;
}

}  // extern "C"
