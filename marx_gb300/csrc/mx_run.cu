// mx_run_marx: marx's main loop (marx/src/marx.c:545-608) driven by the
// engine.  A parameter file with command-line overrides configures the
// engine (mx_config_read_par) and the run: the source (SourceType,
// SourceRA/SourceDec, SourceDistance, the spectrum), NumRays and dNumRays
// or ExposureTime, RandomSeed, OutputDir, OutputVectors and DumpToRayFile.
// Each iteration creates up to dNumRays photons on the device
// (marx_create_photons, source.c:268-385: energies and directions by the
// source model, Poisson arrival times with mean 1 / (flux x geometric
// area), tags), traces them (aspect dither, mirror, grating, detector as
// process_photons, marx.c:240-273) and appends them to the output
// directory (marx_write_photons) or the ray file; the run ends with the
// marx.par and obs.par that marx2fits reads beside the column files
// (marx.c:475-503, :999-1196).
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "mx_context.h"
#include "mx_device.cuh"

using namespace mx;

namespace {

// Source-domain draw of a photon's arrival-time spacing (the models use
// draws 0 .. 7).
constexpr uint32_t TIME_DRAW = 16;
constexpr int TIME_ITEMS = 4, TIME_THREADS = 256, TIME_TILE = TIME_ITEMS * TIME_THREADS;

// Exponential spacings mt (-log(1 - u)) of photons first_tag .. first_tag
// + n - 1 (JDMexpn_random times the mean time, source.c:320-330), summed
// within each 1024-photon tile; the tile's total goes to sums.
__global__ void __launch_bounds__(TIME_THREADS) mx_time_tiles(double *t, uint32_t n, uint64_t seed, uint32_t first_tag,
                                                              double mt, double *sums) {
  __shared__ double warp_tot[TIME_THREADS / 32];
  const uint32_t base = blockIdx.x * TIME_TILE + threadIdx.x * TIME_ITEMS;
  double v[TIME_ITEMS], run = 0.0;
#pragma unroll
  for (int j = 0; j < TIME_ITEMS; j++) {
    const uint32_t i = base + j;
    const double u = i < n ? source_uniform(seed, first_tag + i, TIME_DRAW) : 0.0;
    run += i < n ? mt * -log1p(-u) : 0.0;
    v[j] = run;
  }
  // exclusive scan of the threads' totals across the block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double x = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  double before = x - run;
  for (int w = 0; w < warp; w++) before += warp_tot[w];
#pragma unroll
  for (int j = 0; j < TIME_ITEMS; j++)
    if (base + j < n) t[base + j] = before + v[j];
  if (threadIdx.x == TIME_THREADS - 1) sums[blockIdx.x] = before + run;
}

// Exclusive running sum of the tile totals (one block).
__global__ void __launch_bounds__(1024) mx_time_offsets(double *sums, uint32_t ntile) {
  __shared__ double part[1024];
  __shared__ double carry;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (uint32_t b0 = 0; b0 < ntile; b0 += 1024) {
    const uint32_t k = b0 + threadIdx.x;
    const double v = k < ntile ? sums[k] : 0.0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {   // inclusive Hillis-Steele scan
      const double y = threadIdx.x >= (unsigned) o ? part[threadIdx.x - o] : 0.0;
      __syncthreads();
      part[threadIdx.x] += y;
      __syncthreads();
    }
    if (k < ntile) sums[k] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(TIME_THREADS) mx_time_add(double *t, uint32_t n, const double *sums) {
  const double off = sums[blockIdx.x];
  for (int j = 0; j < TIME_ITEMS; j++) {
    const uint32_t i = blockIdx.x * TIME_TILE + j * TIME_THREADS + threadIdx.x;
    if (i < n) t[i] += off;
  }
}

std::string lower(std::string s) {
  for (char &c : s) c = (char) tolower((unsigned char) c);
  return s;
}

// ---------------------------------------------------- parameter lines --
// A .par file's lines (pfile stops reading at a blank line).
std::vector<std::string> par_lines(const std::string &text) {
  std::vector<std::string> out;
  size_t a = 0;
  while (a <= text.size()) {
    size_t b = text.find('\n', a);
    if (b == std::string::npos) b = text.size();
    std::string ln = text.substr(a, b - a);
    if (!ln.empty() && ln.back() == '\r') ln.pop_back();
    bool blank = ln.find_first_not_of(" \t") == std::string::npos;
    if (!blank) out.push_back(ln);
    a = b + 1;
  }
  return out;
}

// The value field (the fourth) of a parameter line: [start, end).
bool value_span(const std::string &ln, size_t &a, size_t &b) {
  size_t pos = 0;
  for (int k = 0; k < 3; k++) {
    pos = ln.find(',', pos);
    if (pos == std::string::npos) return false;
    pos++;
  }
  a = pos;
  if (a < ln.size() && ln[a] == '"') {
    b = ln.find('"', a + 1);
    b = b == std::string::npos ? ln.size() : b + 1;
  } else {
    b = ln.find(',', a);
    if (b == std::string::npos) b = ln.size();
  }
  return true;
}

// Set parameter `name` (compared without case, as pfile does) to value,
// quoted for string and file parameters; a parameter the file lacks is
// appended as a hidden one of type `kind`.
void par_set(std::vector<std::string> &lines, const std::string &name, const std::string &value, char kind) {
  for (std::string &ln : lines) {
    if (ln.empty() || ln[0] == '#' || std::count(ln.begin(), ln.end(), ',') < 3) continue;
    size_t c = ln.find(',');
    std::string nm = ln.substr(0, c);
    nm.erase(0, nm.find_first_not_of(" \t"));
    nm.erase(nm.find_last_not_of(" \t") + 1);
    if (lower(nm) != lower(name)) continue;
    size_t c2 = ln.find(',', c + 1);
    std::string ty = ln.substr(c + 1, c2 - c - 1);
    ty.erase(0, ty.find_first_not_of(" \t"));
    const bool quoted = !ty.empty() && (ty[0] == 's' || ty[0] == 'f');
    size_t a, b;
    if (!value_span(ln, a, b)) return;
    ln = ln.substr(0, a) + (quoted ? "\"" + value + "\"" : value) + ln.substr(b);
    return;
  }
  const bool quoted = kind == 's' || kind == 'f';
  lines.push_back(name + "," + kind + ",h," + (quoted ? "\"" + value + "\"" : value) + ",,,\"\"");
}

std::string fmt(double v) {
  char b[64];
  snprintf(b, sizeof b, "%.17g", v);
  return b;
}

bool write_text(const std::string &path, const std::vector<std::string> &lines) {
  FILE *f = fopen(path.c_str(), "w");
  if (!f) return false;
  for (const std::string &ln : lines) fprintf(f, "%s\n", ln.c_str());
  return fclose(f) == 0;
}

// OutputVectors letters (compute_write_mask, marx.c:899-975).
bool write_mask_of(const std::string &v, uint32_t &mask, std::string &err) {
  mask = MX_OUT_DET_UV;
  for (char ch : v) {
    switch (ch) {
      case '#': mask |= MX_OUT_TAG; break;
      case 'E': mask |= MX_OUT_ENERGY; break;
      case 'T': mask |= MX_OUT_TIME; break;
      case 'X': case 'Y': case 'Z': mask |= MX_OUT_X; break;
      case '1': case '2': case '3': mask |= MX_OUT_P; break;
      case 'P': mask |= MX_OUT_PHA; break;
      case 'x': case 'y': mask |= MX_OUT_DET_PIXEL; break;
      case 'M': mask |= MX_OUT_SHELL; break;
      case 'O': mask |= MX_OUT_ORDER; break;
      case 'a': mask |= MX_OUT_ORDER1; break;
      case 'b': mask |= MX_OUT_ORDER2; break;
      case 'c': mask |= MX_OUT_ORDER3; break;
      case 'd': mask |= MX_OUT_ORDER4; break;
      case 'D': mask |= MX_OUT_DET_NUM; break;
      case 'S': mask |= MX_OUT_SKY_DITHER | MX_OUT_DET_DITHER; break;
      case 'r': mask |= MX_OUT_DET_REGION; break;
      case 'B': mask |= MX_OUT_PI; break;
      default: err = std::string("Output vector '") + ch + "' not understood."; return false;
    }
  }
  return true;
}

// The two numeric columns of a FILE spectrum (JDMread_column_ddata: lines
// of whitespace-separated numbers; '#' comments and other lines skipped).
bool read_spectrum(const std::string &path, std::vector<double> &e, std::vector<double> &f, std::string &err) {
  FILE *fp = fopen(path.c_str(), "r");
  if (!fp) { err = "cannot open spectrum file " + path; return false; }
  char line[4096];
  while (fgets(line, sizeof line, fp)) {
    const char *s = line;
    while (*s == ' ' || *s == '\t') s++;
    if (*s == '#' || *s == '\n' || *s == 0) continue;
    char *end;
    double a = strtod(s, &end);
    if (end == s) continue;
    const char *s2 = end;
    double b = strtod(s2, &end);
    if (end == s2) continue;
    e.push_back(a);
    f.push_back(b);
  }
  fclose(fp);
  if (e.empty()) { err = "Error reading spectrum from " + path; return false; }
  return true;
}

struct Run {
  ParSet P;
  std::string err;
  const std::string *raw(const char *name) const { return P.find(name); }
  bool str(const char *name, std::string &out) {
    const std::string *v = P.find(name);
    if (!v) { err = std::string("parameter ") + name + " is missing"; return false; }
    out = *v;
    return true;
  }
  bool num(const char *name, double &out) {
    std::string v;
    if (!str(name, v)) return false;
    char *end;
    out = strtod(v.c_str(), &end);
    if (v.empty() || *end) { err = std::string("parameter ") + name + ": not a number '" + v + "'"; return false; }
    return true;
  }
  bool integer(const char *name, long &out) {
    double d;
    if (!num(name, d)) return false;
    if (d != std::floor(d)) { err = std::string("parameter ") + name + ": not an integer"; return false; }
    out = (long) d;
    return true;
  }
  bool boolean(const char *name, bool &out) {
    std::string v;
    if (!str(name, v)) return false;
    v = lower(v);
    out = v == "yes" || v == "y" || v == "1" || v == "true";
    return true;
  }
};

// One device column set for up to cap photons (every column of mx_photons).
struct DevList {
  DevBuf buf;
  mx_photons ph{};
  cudaError_t ensure(uint32_t cap) {
    const size_t n = cap;
    const size_t bytes[19] = {8 * n, 24 * n, 24 * n, 8 * n, 4 * n, 4 * n, n, n, n, 4 * n, 4 * n, 12 * n,
                              4 * n, 2 * n, 4 * n, 4 * n, n, 4 * n, 12 * n};
    size_t off[19], tot = 0;
    for (int k = 0; k < 19; k++) { off[k] = tot; tot += (bytes[k] + 255) & ~(size_t) 255; }
    cudaError_t e = buf.ensure(tot);
    if (e != cudaSuccess) return e;
    char *b = (char *) buf.ptr;
    ph.energy = (double *) (b + off[0]); ph.x = (double *) (b + off[1]); ph.p = (double *) (b + off[2]);
    ph.arrival_time = (double *) (b + off[3]); ph.flags = (uint32_t *) (b + off[4]); ph.tag = (uint32_t *) (b + off[5]);
    ph.mirror_shell = (int8_t *) (b + off[6]); ph.order = (int8_t *) (b + off[7]); ph.ccd_num = (int8_t *) (b + off[8]);
    ph.y_pixel = (float *) (b + off[9]); ph.z_pixel = (float *) (b + off[10]); ph.dither_state = (float *) (b + off[11]);
    ph.support_orders = (int8_t *) (b + off[12]); ph.pulse_height = (int16_t *) (b + off[13]);
    ph.u_pixel = (float *) (b + off[14]); ph.v_pixel = (float *) (b + off[15]);
    ph.detector_region = (uint8_t *) (b + off[16]); ph.pi = (float *) (b + off[17]);
    ph.det_dither = (float *) (b + off[18]);
    return cudaSuccess;
  }
};

// Host copies of the columns the writer reads, laid out as mx_photons with
// a component stride of n.
struct HostList {
  std::vector<double> energy, x, p, t;
  std::vector<uint32_t> flags, tag;
  std::vector<int8_t> shell, order, ccd, sup;
  std::vector<float> ypix, zpix, dith, upix, vpix, pi, ddith;
  std::vector<int16_t> pha;
  std::vector<uint8_t> region;
  mx_photons ph{};
  void resize(uint32_t n) {
    energy.resize(n); x.resize(3 * (size_t) n); p.resize(3 * (size_t) n); t.resize(n); flags.resize(n); tag.resize(n);
    shell.resize(n); order.resize(n); ccd.resize(n); sup.resize(4 * (size_t) n); ypix.resize(n); zpix.resize(n);
    dith.resize(3 * (size_t) n); upix.resize(n); vpix.resize(n); pi.resize(n); ddith.resize(3 * (size_t) n);
    pha.resize(n); region.resize(n);
    ph.n = n; ph.stride = n;
    ph.energy = energy.data(); ph.x = x.data(); ph.p = p.data(); ph.arrival_time = t.data(); ph.flags = flags.data();
    ph.tag = tag.data(); ph.mirror_shell = shell.data(); ph.order = order.data(); ph.ccd_num = ccd.data();
    ph.y_pixel = ypix.data(); ph.z_pixel = zpix.data(); ph.dither_state = dith.data();
    ph.support_orders = sup.data(); ph.pulse_height = pha.data(); ph.u_pixel = upix.data(); ph.v_pixel = vpix.data();
    ph.detector_region = region.data(); ph.pi = pi.data(); ph.det_dither = ddith.data();
  }
};

// n photons of a device list whose columns are laid out for cap photons
// (stride cap) into a host list of n (stride n).
cudaError_t copy_out(const mx_photons &d, uint32_t cap, uint32_t n, HostList &h, cudaStream_t st) {
  h.resize(n);
  struct Col { const void *src; void *dst; size_t elem; int comps; };
  const Col cols[19] = {
      {d.energy, h.ph.energy, 8, 1}, {d.x, h.ph.x, 8, 3}, {d.p, h.ph.p, 8, 3}, {d.arrival_time, h.ph.arrival_time, 8, 1},
      {d.flags, h.ph.flags, 4, 1}, {d.tag, h.ph.tag, 4, 1}, {d.mirror_shell, h.ph.mirror_shell, 1, 1},
      {d.order, h.ph.order, 1, 1}, {d.ccd_num, h.ph.ccd_num, 1, 1}, {d.y_pixel, h.ph.y_pixel, 4, 1},
      {d.z_pixel, h.ph.z_pixel, 4, 1}, {d.dither_state, h.ph.dither_state, 4, 3},
      {d.support_orders, h.ph.support_orders, 1, 4}, {d.pulse_height, h.ph.pulse_height, 2, 1},
      {d.u_pixel, h.ph.u_pixel, 4, 1}, {d.v_pixel, h.ph.v_pixel, 4, 1}, {d.detector_region, h.ph.detector_region, 1, 1},
      {d.pi, h.ph.pi, 4, 1}, {d.det_dither, h.ph.det_dither, 4, 3}};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 19 && e == cudaSuccess; k++)
    e = cudaMemcpy2DAsync(cols[k].dst, (size_t) n * cols[k].elem, cols[k].src, (size_t) cap * cols[k].elem,
                          (size_t) n * cols[k].elem, cols[k].comps, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

// n photons of a host list (stride n) into a device list laid out for cap
// photons (stride cap): the columns a trace reads.
cudaError_t copy_in(const HostList &h, uint32_t n, const mx_photons &d, uint32_t cap, cudaStream_t st) {
  struct Col { const void *src; void *dst; size_t elem; int comps; };
  const Col cols[12] = {
      {h.ph.energy, d.energy, 8, 1}, {h.ph.x, d.x, 8, 3}, {h.ph.p, d.p, 8, 3}, {h.ph.arrival_time, d.arrival_time, 8, 1},
      {h.ph.flags, d.flags, 4, 1}, {h.ph.tag, d.tag, 4, 1}, {h.ph.mirror_shell, d.mirror_shell, 1, 1},
      {h.ph.order, d.order, 1, 1}, {h.ph.ccd_num, d.ccd_num, 1, 1}, {h.ph.y_pixel, d.y_pixel, 4, 1},
      {h.ph.z_pixel, d.z_pixel, 4, 1}, {h.ph.dither_state, d.dither_state, 4, 3}};
  const size_t hs = h.ph.stride;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 12 && e == cudaSuccess; k++)
    e = cudaMemcpy2DAsync(cols[k].dst, (size_t) cap * cols[k].elem, cols[k].src, hs * cols[k].elem,
                          (size_t) n * cols[k].elem, cols[k].comps, cudaMemcpyHostToDevice, st);
  return e;
}

const char *source_names[] = {"POINT", "GAUSS", "BETA", "DISK", "LINE"};

}  // namespace

extern "C" int mx_run_marx(const char *pack_path, const char *par_path, const char *const *overrides, int n_overrides,
                           mx_run_stats *stats) {
  if (!pack_path || !par_path) return mx_fail(nullptr, MX_EINVAL, "mx_run_marx: null argument");
  Run R;
  std::string err;
  if (!load_par(par_path, overrides, n_overrides, R.P, err)) return mx_fail(nullptr, MX_EINVAL, "mx_run_marx: " + err);
  auto bad = [&](const std::string &m) { return mx_fail(nullptr, MX_EINVAL, "mx_run_marx: " + m); };
  mx_config cfg;
  mx_config_default(&cfg);
  int r = mx_config_read_params(&cfg, MX_PARAMS_ALL, par_reader, &R.P, 0);
  if (r) return r;

  // run parameters (marx.c:789-805, source.c:77-88, spectrum.c:118-274)
  long num_rays = 0, drays = 0, seed_par = -1;
  double exposure = 0.0, ra = 0.0, dec = 0.0, distance = 0.0;
  std::string out_dir, vectors, src_name, spec_type;
  bool dump = false;
  if (!R.integer("NumRays", num_rays) || !R.integer("dNumRays", drays) || !R.num("ExposureTime", exposure) ||
      !R.str("OutputDir", out_dir) || !R.str("OutputVectors", vectors) || !R.str("SourceType", src_name) ||
      !R.num("SourceRA", ra) || !R.num("SourceDEC", dec) || !R.str("SpectrumType", spec_type))
    return bad(R.err);
  if (R.raw("RandomSeed")) R.integer("RandomSeed", seed_par);
  if (R.raw("SourceDistance") && !R.num("SourceDistance", distance)) return bad(R.err);
  if (R.raw("DumpToRayFile") && !R.boolean("DumpToRayFile", dump)) return bad(R.err);
  if (drays <= 0 || drays > (1l << 30)) return bad("dNumRays must lie in 1 .. 2^30");
  if (exposure <= 0.0 && num_rays == 0) return bad("NumRays is 0 and no ExposureTime");
  uint32_t write_mask = 0;
  if (!write_mask_of(vectors, write_mask, err)) return bad(err);
  cfg.source_distance = distance * 1000.0;   // m -> mm (source.c:401)

  mx_source src;
  memset(&src, 0, sizeof src);
  const bool saosac = src_name == "SAOSAC";
  std::string saosac_file;
  if (saosac && !R.str("SAOSACFile", saosac_file)) return bad(R.err);
  int kind = saosac ? 0 : -1;
  for (int k = 0; k < 5; k++)
    if (src_name == source_names[k]) kind = k;
  if (kind < 0)
    return bad("SourceType " + src_name + " is not supported here (POINT, GAUSS, BETA, DISK, LINE, SAOSAC)");
  src.kind = kind;
  const char *model_pars[5][2] = {{nullptr, nullptr}, {"S-GaussSigma", nullptr}, {"S-BetaCoreRadius", "S-BetaBeta"},
                                  {"S-DiskTheta0", "S-DiskTheta1"}, {"S-LinePhi", "S-LineTheta"}};
  for (int k = 0; k < 2; k++)
    if (model_pars[kind][k] && !R.num(model_pars[kind][k], src.param[k])) return bad(R.err);
  if (mx_source_direction(&cfg, ra, dec, src.p) != MX_OK) return bad("source direction");
  double flux = 0.0;
  std::vector<double> spec_e, spec_f;
  if (!R.num("SourceFlux", flux)) return bad(R.err);
  if (saosac) {
    // the rays carry their energies; the spectrum's total flux is 0, so
    // photons of a file without RT_TIME get zero times (source.c:315-337)
    flux = 0.0;
  } else if (spec_type == "FLAT") {
    if (!R.num("MinEnergy", src.energy_min) || !R.num("MaxEnergy", src.energy_max)) return bad(R.err);
    if (flux <= 0.0) return bad("SourceFlux for FLAT spectrum must be positive");
    if (src.energy_max - src.energy_min < 0.0 || src.energy_max <= 0.0) return bad("bad MinEnergy, MaxEnergy");
  } else if (spec_type == "FILE") {
    std::string file;
    if (!R.str("SpectrumFile", file)) return bad(R.err);
    if (!read_spectrum(file, spec_e, spec_f, err)) return bad(err);
    double tot = 0.0;   // compute_cumulated_vector's total (spectrum.c:40-97)
    for (size_t i = 1; i < spec_e.size(); i++) tot += spec_f[i] * (spec_e[i] - spec_e[i - 1]);
    if (flux <= 0.0) flux = tot;
    if (!(flux > 0.0) || !std::isfinite(flux)) return bad("The flux must be positive and finite");
    src.spectrum_n = (uint32_t) spec_e.size();
    src.spectrum_energy = spec_e.data();
    src.spectrum_flux = spec_f.data();
  } else
    return bad("SpectrumType " + spec_type + " is not supported (FLAT, FILE)");
  const uint64_t seed = seed_par >= 0 ? (uint64_t) seed_par : (uint64_t) time(nullptr);

  mx_context *c = mx_create(pack_path, &cfg);
  if (!c) return MX_EPACK;
  struct Closer { mx_context *c; ~Closer() { mx_destroy(c); } } closer{c};
  // errors past this point are reported with no context (it is destroyed
  // on return): the context's message moves to mx_last_error(NULL)
  auto ctx_fail = [&](int code) { return mx_fail(nullptr, code, "mx_run_marx: " + c->err); };
  const double mt = flux > 0.0 ? 1.0 / flux / c->hm.geom_area_cm2 : 0.0;   // compute_mean_time (source.c:260-264)
  mx_saosac *sa = nullptr;
  if (saosac && !(sa = mx_saosac_open(saosac_file.c_str(), cfg.hrma_cap_x)))
    return mx_fail(nullptr, MX_EINVAL, std::string("mx_run_marx: ") + mx_last_error(nullptr));
  struct SaCloser { mx_saosac *s; ~SaCloser() { mx_saosac_close(s); } } sa_closer{sa};
  HostList hin;
  cudaStream_t st = c->stream;
  const uint32_t cap = (uint32_t) drays;
  DevList dev;
  DevBuf sums;
  cudaError_t e = dev.ensure(cap);
  const uint32_t ntile = (cap + TIME_TILE - 1) / TIME_TILE;
  if (e == cudaSuccess) e = sums.ensure((size_t) ntile * sizeof(double));
  if (e != cudaSuccess) return mx_cuda_fail(nullptr, e, "mx_run_marx: allocating the photon columns");
  HostList host;
  std::vector<double> times(cap);
  const uint32_t history = mx_output_history(&cfg, MX_STAGE_ALL);
  mkdir(out_dir.c_str(), 0777);
  const std::string ray_file = R.raw("RayFile") ? *R.raw("RayFile") : std::string("marx.rays");

  uint64_t collected = 0, detected = 0;
  uint32_t tag_start = 0, iterations = 0;
  double total_time = 0.0, start_time = 0.0;
  const uint64_t to_collect = num_rays > 0 ? (uint64_t) num_rays : 0, to_detect = num_rays < 0 ? (uint64_t) -num_rays : 0;
  uint32_t per_iter = cap;
  if (exposure <= 0.0) per_iter = (uint32_t) std::min<uint64_t>(cap, num_rays > 0 ? to_collect : to_detect);
  bool first = true;
  while (true) {
    double left = 0.0;
    if (exposure > 0.0) {
      left = exposure - total_time;
      if (left <= 0.0) break;
    } else if (num_rays > 0) {
      if (collected >= to_collect) break;
    } else if (detected >= to_detect)
      break;
    mx_photons d = dev.ph;
    d.n = per_iter;
    d.stride = cap;
    uint32_t n = per_iter;
    if (saosac) {
      // the next rows of the ray file (saosac_create_photons), copied to
      // the device; the mirror stage is skipped (its history bit is set)
      hin.resize(per_iter);
      std::fill(hin.ccd.begin(), hin.ccd.end(), (int8_t) -1);
      if ((r = mx_saosac_read(sa, &hin.ph, per_iter, nullptr, seed, tag_start, &n)) != MX_OK)
        return mx_fail(nullptr, r, std::string("mx_run_marx: ") + mx_last_error(nullptr));
      if (n == 0) break;
      if (!mx_saosac_has_time(sa))   // marx_create_photons gives them Poisson times of mean 0 and clears the flags
        for (uint32_t i = 0; i < n; i++) { hin.t[i] = 0.0; hin.flags[i] = 0u; }
      std::copy(hin.t.begin(), hin.t.begin() + n, times.begin());
      if ((e = copy_in(hin, n, d, cap, st)) != cudaSuccess) return mx_cuda_fail(nullptr, e, "mx_run_marx: rays");
    } else {
      if ((r = mx_generate_source(c, &src, tag_start, seed, &d, st)) != MX_OK) return ctx_fail(r);
      mx_time_tiles<<<(per_iter + TIME_TILE - 1) / TIME_TILE, TIME_THREADS, 0, st>>>(d.arrival_time, per_iter, seed,
                                                                                   tag_start, mt, (double *) sums.ptr);
      mx_time_offsets<<<1, 1024, 0, st>>>((double *) sums.ptr, (per_iter + TIME_TILE - 1) / TIME_TILE);
      mx_time_add<<<(per_iter + TIME_TILE - 1) / TIME_TILE, TIME_THREADS, 0, st>>>(d.arrival_time, per_iter,
                                                                                 (const double *) sums.ptr);
      c->launches += 3;
      e = cudaMemcpyAsync(times.data(), d.arrival_time, (size_t) per_iter * 8, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e != cudaSuccess) return mx_cuda_fail(nullptr, e, "mx_run_marx: photon times");
      if (exposure > 0.0)   // the first photon at or past the time left ends the batch (source.c:327-333)
        for (uint32_t i = 0; i < per_iter; i++)
          if (times[i] >= left) { n = i + 1; break; }
    }
    d.n = n;
    if ((r = mx_set_start_time(c, start_time)) != MX_OK) return ctx_fail(r);
    // the ray file holds the dithered rays; SAOSAC rays have passed the mirror
    const uint32_t stages = dump ? MX_STAGE_DITHER : saosac ? (MX_STAGE_ALL & ~MX_STAGE_MIRROR) : MX_STAGE_ALL;
    if ((r = mx_trace_tables(c, c->T, &d, stages, nullptr, nullptr, seed, st, !saosac)) != MX_OK) return ctx_fail(r);
    if ((e = copy_out(d, cap, n, host, st)) != cudaSuccess)
      return mx_cuda_fail(nullptr, e, "mx_run_marx: copying photons out");
    if (dump) {
      if ((r = mx_write_rayfile(&host.ph, history & (MX_OUT_ENERGY | MX_OUT_TIME | MX_OUT_X | MX_OUT_P | MX_OUT_TAG |
                                                     MX_OUT_SKY_DITHER),
                                ray_file.c_str(), first ? 0 : 1, total_time)) != MX_OK)
        return mx_fail(nullptr, r, std::string("mx_run_marx: ") + mx_write_error());
    } else if ((r = mx_write_photons(&host.ph, history, write_mask, cfg.dither != MX_DITHER_NONE, out_dir.c_str(),
                                     first ? 0 : 1, total_time)) != MX_OK)
      return mx_fail(nullptr, r, std::string("mx_run_marx: ") + mx_write_error());
    first = false;
    uint32_t good = 0;
    for (uint32_t i = 0; i < n; i++) good += (host.flags[i] & MX_BAD_PHOTON_MASK) == 0;
    collected += n;
    detected += good;
    const double batch_time = times[n - 1];
    total_time += batch_time;
    start_time = total_time;   // pt->start_time += pt->total_time (source.c:285)
    tag_start += n;
    iterations++;
    if (n != per_iter) break;
  }

  // marx.par (the parameter file with the overrides) and obs.par
  // (write_obs_par, marx.c:999-1196) beside the column files
  {
    FILE *f = fopen(par_path, "r");
    std::string text;
    if (f) {
      char b[4096];
      size_t k;
      while ((k = fread(b, 1, sizeof b, f)) > 0) text.append(b, k);
      fclose(f);
    }
    std::vector<std::string> lines = par_lines(text);
    for (int k = 0; k < n_overrides; k++) {
      const char *o = overrides[k], *eq = strchr(o, '=');
      par_set(lines, std::string(o, eq - o), std::string(eq + 1), 's');
    }
    if (!write_text(out_dir + "/marx.par", lines)) return mx_fail(nullptr, MX_EINVAL, "mx_run_marx: writing marx.par");
    static const char *det_names[5] = {"NONE", "ACIS-I", "ACIS-S", "HRC-I", "HRC-S"};
    static const char *tmpl[5] = {"generic_obs", "acis_i_obs", "acis_s_obs", "hrc_i_obs", "hrc_s_obs"};
    const std::string det = det_names[cfg.detector], grat = cfg.grating == 1 ? "HETG" : cfg.grating == 2 ? "LETG" : "NONE";
    size_t cnt = 0;
    const int32_t *w = c->pack.get<int32_t>(std::string("obs/") + tmpl[cfg.detector], &cnt, err);
    if (w && cnt >= 1 && (size_t) w[0] <= 4 * (cnt - 1)) {
      std::vector<std::string> obs = par_lines(std::string((const char *) (w + 1), (size_t) w[0]));
      auto norm = [](double a) { a = std::fmod(a, 360.0); return a < 0 ? a + 360.0 : a; };
      const std::string datamode = det.rfind("ACIS", 0) == 0 ? "GRADED" : (grat != "NONE" ? "SPECTROSCOPIC" : "IMAGING");
      par_set(obs, "ra_nom", fmt(norm(cfg.ra_nom)), 'r');
      par_set(obs, "roll_nom", fmt(norm(cfg.roll_nom)), 'r');
      par_set(obs, "dec_nom", fmt(cfg.dec_nom), 'r');
      par_set(obs, "ra_pnt", fmt(norm(cfg.ra_nom)), 'r');
      par_set(obs, "roll_pnt", fmt(norm(cfg.roll_nom)), 'r');
      par_set(obs, "dec_pnt", fmt(cfg.dec_nom), 'r');
      par_set(obs, "foc_len", fmt(cfg.focal_length), 'r');
      par_set(obs, "datamode", datamode, 's');
      par_set(obs, "detnam", det, 's');
      par_set(obs, "grating", grat, 's');
      par_set(obs, "object", src_name, 's');
      par_set(obs, "title", src_name, 's');
      par_set(obs, "tstart", fmt(0.0), 'r');
      par_set(obs, "tstop", fmt(total_time), 'r');
      par_set(obs, "sim_x", fmt(cfg.det_offset[0]), 'r');
      par_set(obs, "sim_y", fmt(cfg.det_offset[1]), 'r');
      par_set(obs, "sim_z", fmt(cfg.det_offset[2]), 'r');
      par_set(obs, "defocus", fmt(cfg.det_offset[0]), 'r');
      for (const char *k : {"DY_AVG", "DZ_AVG", "DTH_AVG"}) par_set(obs, k, fmt(0.0), 'r');
      for (const char *k : {"LIVETIME", "ONTIME", "EXPOSURE", "TELAPSE"}) par_set(obs, k, fmt(total_time), 'r');
      if (!write_text(out_dir + "/obs.par", obs)) return mx_fail(nullptr, MX_EINVAL, "mx_run_marx: writing obs.par");
    }
  }
  if (stats) {
    stats->collected = collected;
    stats->detected = detected;
    stats->total_time = total_time;
    stats->iterations = iterations;
    stats->reserved = 0;
  }
  return MX_OK;
}
