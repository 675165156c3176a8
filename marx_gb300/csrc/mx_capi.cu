// Trace kernels and the C ABI of libmarx_gb300 (include/marx_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "mx_device.cuh"
#include "mx_host.h"
#include "mx_kernels.cuh"
#include "mx_context.h"

using namespace mx;

thread_local std::string g_create_err;

int mx_fail(mx_context *c, int code, const std::string &msg) {
  if (c) c->err = msg; else g_create_err = msg;
  return code;
}
int mx_cuda_fail(mx_context *c, cudaError_t e, const char *what) {
  return mx_fail(c, MX_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
static int fail(mx_context *c, int code, const std::string &msg) { return mx_fail(c, code, msg); }
static int cuda_fail(mx_context *c, cudaError_t e, const char *what) { return mx_cuda_fail(c, e, what); }

// ------------------------------------------------------------ uploading --
template <class T> static size_t put(std::vector<char> &blob, const std::vector<T> &v) {
  size_t off = (blob.size() + 255) & ~(size_t) 255;
  blob.resize(off + v.size() * sizeof(T));
  memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
  return off;
}

static int upload_model(mx_context *c) {
  HostModel &M = c->hm;
  std::vector<char> blob;
  size_t o_sh = put(blob, M.shells), o_opt = put(blob, M.optc), o_fh = put(blob, M.fold_hdr),
         o_fe = put(blob, M.fold_ealpha), o_ft = put(blob, M.fold_theta), o_gr = put(blob, M.gratings),
         o_sl = put(blob, M.optc_slope), o_fi = put(blob, M.fold_inv_de),
         o_ge = put(blob, M.geff_energy), o_gc = put(blob, M.geff_cum), o_ok = put(blob, M.order_k),
         o_se = put(blob, M.sectors), o_ch = put(blob, M.chips);
  if (M.support_energy.empty()) { M.support_energy.push_back(0.f); M.support_cum.push_back(0.f); M.support_k.push_back(0.0); }
  size_t o_pe = put(blob, M.support_energy), o_pc = put(blob, M.support_cum), o_pk = put(blob, M.support_k);
  size_t o_ht = put(blob, M.hrc_tab), o_hs = put(blob, M.hrc_slope);
  size_t o_fm = put(blob, M.fef_map), o_fr = put(blob, M.fef), o_ff = put(blob, M.fef_f), o_fs = put(blob, M.fef_slope);
  size_t o_co = put(blob, M.contam);
  cudaError_t e = c->tables.ensure(blob.size());
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating device tables");
  e = cudaMemcpy(c->tables.ptr, blob.data(), blob.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(c, e, "uploading device tables");
  char *b = (char *) c->tables.ptr;
  c->T = M.T;
  c->T.shells = (const MxShellDev *) (b + o_sh);
  c->T.optc = (const float *) (b + o_opt);
  c->T.fold_hdr = (const double *) (b + o_fh);
  c->T.fold_ealpha = (const double *) (b + o_fe);
  c->T.fold_theta = (const float *) (b + o_ft);
  c->T.optc_slope = (const double *) (b + o_sl);
  c->T.fold_inv_de = (const double *) (b + o_fi);
  c->T.gratings = (const MxGratingDev *) (b + o_gr);
  c->T.geff_energy = (const float *) (b + o_ge);
  c->T.geff_cum = (const float *) (b + o_gc);
  c->T.order_k = (const double *) (b + o_ok);
  c->T.sectors = (const double *) (b + o_se);
  c->T.chips = (const MxChipDev *) (b + o_ch);
  c->T.support_energy = (const float *) (b + o_pe);
  c->T.support_cum = (const float *) (b + o_pc);
  c->T.support_k = (const double *) (b + o_pk);
  c->T.hrc_tab = (const float *) (b + o_ht);
  c->T.hrc_slope = (const double *) (b + o_hs);
  c->T.fef_map = (const int32_t *) (b + o_fm);
  c->T.fef = (const MxFefDev *) (b + o_fr);
  c->T.fef_f = (const float *) (b + o_ff);
  c->T.fef_slope = (const double *) (b + o_fs);
  c->T.contam = (const MxContamDev *) (b + o_co);
  c->T.asp_t = (const double *) c->asp.ptr;
  c->T.asp_v = c->asp.ptr ? (const double *) c->asp.ptr + ((c->asp_n + 1 + 7) & ~7u) : nullptr;
  c->T.asp_n = c->asp_n;
  c->T.asp_record_only = c->asp_record_only;
  c->shared_bytes = trace_shared_bytes(c->T);
  if (c->shared_bytes > 200 * 1024) return fail(c, MX_ERANGE, "tables exceed the shared-memory budget");
  return MX_OK;
}

static int configure(mx_context *c, const mx_config *cfg) {
  std::string err;
  if (!build_model(c->pack, *cfg, c->hm, err)) return fail(c, MX_EINVAL, err);
  c->cfg = *cfg;
  c->events_ready = false;
  int r = upload_model(c);
  if (r) return r;
  for (int s = 0; s < 2; s++) {
    cudaError_t e = trace_occupancy(s == 1, (int) c->shared_bytes, &c->trace_blocks[s]);
    if (e != cudaSuccess) return cuda_fail(c, e, "querying occupancy");
    if (c->trace_blocks[s] < 1) return fail(c, MX_ERANGE, "trace kernel cannot be resident");
  }
  cudaError_t e = wave_occupancy((int) c->shared_bytes, &c->wave_blocks);
  if (e != cudaSuccess) return cuda_fail(c, e, "querying occupancy");
  if (c->wave_blocks < 1) return fail(c, MX_ERANGE, "wavefront kernels cannot be resident");
  return MX_OK;
}

// ------------------------------------------------------------------ ABI --
extern "C" {

void mx_config_default(mx_config *c) {
  memset(c, 0, sizeof(*c));
  static const double xo[4] = {-3.277664, -0.257891, 0.733315, -0.541755};
  static const double bp[4] = {0.303427, 0.0951899, 0.178899, 0.151085};
  static const double bh[4] = {0.0051428, 0.0713614, 0.0101367, 0.0239287};
  static const double sp[4] = {2.8420331, 1.7305226, 1.0077613, 2.1199425};
  static const double sh[4] = {3.2451338, 2.4618956, 2.9027099, 2.0209803};
  static const double th[4] = {4.755, 4.755, -5.205, -5.205};
  static const double pe[4] = {0.400195, 0.400195, 0.200081, 0.200081};
  static const double dpp[4] = {162e-6, 162e-6, 146e-6, 146e-6};
  c->hrma_cap_x = 10079.771554;
  for (int i = 0; i < 4; i++) {
    c->shell_xoffset[i] = xo[i]; c->blur_p[i] = bp[i]; c->blur_h[i] = bh[i];
    c->scat_p[i] = sp[i]; c->scat_h[i] = sh[i]; c->shutters[i] = 0xF;
    c->hetg_theta[i] = th[i]; c->hetg_dtheta[i] = 1.5; c->hetg_period[i] = pe[i];
    c->hetg_dpp[i] = dpp[i]; c->hetg_vig[i] = 1.0;
  }
  c->hrma_vig = 1.0;
  c->use_blur = c->use_wfold = c->use_struts = c->use_scale_factors = 1;
  c->grating = MX_GRATING_HETG; c->use_sector_files = 1;
  c->meg_rowland = c->heg_rowland = 8632.48;
  c->dither = MX_DITHER_INTERNAL;
  c->dither_amp[0] = 16.0; c->dither_amp[1] = 16.0; c->dither_amp[2] = 0.0;
  c->dither_period[0] = 1414.2; c->dither_period[1] = 2000.0; c->dither_period[2] = 1e5;
  c->roll_nom = 237.36968458476;
  c->aspect_blur = 0.07;
  c->detector = MX_DETECTOR_ACIS_S;
  c->acis_exposure_time = 3.2; c->acis_frame_transfer_time = 0.041;
  c->focal_length = 10065.5;
  for (int i = 0; i < 4; i++) {
    c->letg_theta[i] = 0.07; c->letg_dtheta[i] = 0.617; c->letg_period[i] = 0.991216;
    c->letg_dpp[i] = 78e-6; c->letg_vig[i] = 1.0;
  }
  c->leg_rowland = 8637.0;
  c->letg_acis_dtheta = -0.0867;
  c->leg_fine_orders = 19; c->leg_coarse_orders = 121;
  c->leg_fine_period = 25.4; c->leg_fine_bar_height = 2.5; c->leg_fine_bar_width = 2.5;
  c->leg_coarse_period = 2000.0; c->leg_coarse_bar_height = 26.0; c->leg_coarse_bar_width = 68.0;
  static const double bi[13] = {13.8994, 64.1124, 64.5285, 15.7528, 4.25636, 61.35, 64.178, 0.0,
                                10.8269, 73.3361, 63.9927, 0.0, 256.0};
  static const double bs[13] = {13.900, 64.110, 64.530, 15.750, 4.2560, 67.420, 64.110, 0.0,
                                10.820, 53.030, 63.880, 0.0, 256.000};
  for (int k = 0; k < 13; k++) { c->hrc_i_blur[k] = bi[k]; c->hrc_s_blur[k] = bs[k]; }
  c->hrc_hesf = 1; c->hesf_n = 2;
  c->hesf_offset_x = 26.3; c->hesf_offset_z = -5.359;
  c->hesf_gap_y1 = 28.7; c->hesf_gap_y2 = 36.7;
  c->hesf_length = 294.0; c->hesf_cr_width = 15.7;
  c->hesf_height[0] = 22.3; c->hesf_height[1] = 50.0;
  c->hesf_theta[0] = 4.5; c->hesf_theta[1] = 7.0;
  c->ra_nom = 250.2134679741175; c->dec_nom = -53.75743813458669;
}

mx_context *mx_create(const char *pack_path, const mx_config *cfg) {
  if (!pack_path || !cfg) { g_create_err = "mx_create: null argument"; return nullptr; }
  mx_context *c = new mx_context();
  std::string err;
  if (!c->pack.load(pack_path, err)) { g_create_err = err; delete c; return nullptr; }
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **) &c->d_overrun, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(c->d_overrun, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc((void **) &c->d_event_bad, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(c->d_event_bad, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) { g_create_err = std::string("CUDA: ") + cudaGetErrorString(e); mx_destroy(c); return nullptr; }
  if (configure(c, cfg) != MX_OK) { g_create_err = c->err; mx_destroy(c); return nullptr; }
  return c;
}

int mx_configure(mx_context *c, const mx_config *cfg) {
  if (!c || !cfg) return fail(c, MX_EINVAL, "mx_configure: null argument");
  cudaStreamSynchronize(c->stream);
  return configure(c, cfg);
}

int mx_set_start_time(mx_context *c, double start_time) {
  if (!c) return MX_EINVAL;
  c->cfg.start_time = start_time;
  c->T.start_time = start_time;
  c->hm.T.start_time = start_time;
  return MX_OK;
}

int mx_geometric_area(const char *pack_path, const mx_config *cfg, double *cm2) {
  if (!pack_path || !cfg || !cm2) { g_create_err = "mx_geometric_area: null argument"; return MX_EINVAL; }
  Pack pk;
  HostModel hm;
  std::string err;
  if (!pk.load(pack_path, err)) { g_create_err = err; return MX_EPACK; }
  if (!build_model(pk, *cfg, hm, err)) { g_create_err = err; return MX_EINVAL; }
  *cm2 = hm.geom_area_cm2;
  return MX_OK;
}

int mx_validate_config(const char *pack_path, const mx_config *cfg) {
  if (!pack_path || !cfg) { g_create_err = "mx_validate_config: null argument"; return MX_EINVAL; }
  Pack pk;
  HostModel hm;
  std::string err;
  if (!pk.load(pack_path, err)) { g_create_err = err; return MX_EPACK; }
  if (!build_model(pk, *cfg, hm, err)) { g_create_err = err; return MX_EINVAL; }
  return MX_OK;
}

void mx_destroy(mx_context *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->tables.release();
  for (auto &b : c->io) b.release();
  c->scan.release();
  c->wave.release();
  c->spec.release();
  c->asp.release();
  c->ev_tab.release();
  c->ev_scan.release();
  c->ev_io.release();
  for (int k = 0; k < MX_PIPE_STREAMS; k++) {
    c->pipe_wave[k].release();
    if (c->pipe[k]) cudaStreamDestroy(c->pipe[k]);
  }
  if (c->pipe_in) cudaStreamDestroy(c->pipe_in);
  if (c->pipe_out) cudaStreamDestroy(c->pipe_out);
  for (auto &row : c->pipe_ev)
    for (auto &ev : row)
      if (ev) cudaEventDestroy(ev);
  for (auto &ev : c->split_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->d_overrun) cudaFree(c->d_overrun);
  if (c->d_event_bad) cudaFree(c->d_event_bad);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *mx_last_error(const mx_context *c) { return c ? c->err.c_str() : g_create_err.c_str(); }

void *mx_stream(mx_context *c) { return c ? (void *) c->stream : nullptr; }

int mx_set_aspect_solution(mx_context *c, const double *rows, uint32_t n, double ra_nom, double dec_nom,
                           double roll_nom, double tstart, int record_only) {
  if (!c) return MX_EINVAL;
  if (n && !rows) return fail(c, MX_EINVAL, "mx_set_aspect_solution: null rows");
  cudaStreamSynchronize(c->stream);
  if (n == 0) {
    c->asp.release();
    c->asp_n = 0;
  } else {
    // times, padded to a multiple of 8 doubles, then the rows of 8 values
    const size_t nt = ((size_t) n + 1 + 7) & ~(size_t) 7;
    std::vector<double> h(nt + 8 * ((size_t) n + 1), 0.0);
    int r = mx_aspsol_convert(rows, n, ra_nom, dec_nom, roll_nom, tstart, h.data(), h.data() + nt);
    if (r) return fail(c, r, "mx_set_aspect_solution: bad arguments");
    for (uint32_t i = 2; i <= n; i++)   // row 1 carries TSTART twice over
      if (!(h[i] >= h[i - 1])) return fail(c, MX_EINVAL, "mx_set_aspect_solution: times decrease");
    cudaError_t e = c->asp.ensure(h.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(c->asp.ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, e, "uploading the aspect solution");
    c->asp_n = n;
  }
  c->asp_record_only = record_only ? 1 : 0;
  c->T.asp_t = (const double *) c->asp.ptr;
  c->T.asp_v = c->asp.ptr ? (const double *) c->asp.ptr + (((size_t) c->asp_n + 1 + 7) & ~(size_t) 7) : nullptr;
  c->T.asp_n = c->asp_n;
  c->T.asp_record_only = c->asp_record_only;
  return MX_OK;
}

int mx_table_bytes(const mx_context *c, size_t *shared_bytes, size_t *global_bytes) {
  if (!c) return MX_EINVAL;
  if (shared_bytes) *shared_bytes = c->shared_bytes;
  if (global_bytes) *global_bytes = c->tables.bytes;
  return MX_OK;
}

uint64_t mx_launch_count(const mx_context *c) { return c ? c->launches : 0; }

int mx_set_trace_mode(mx_context *c, int mode) {
  if (!c || mode < MX_MODE_AUTO || mode > MX_MODE_WAVEFRONT) return fail(c, MX_EINVAL, "mx_set_trace_mode: bad mode");
  c->mode = mode;
  return MX_OK;
}

// Photons i0 .. i0 + m of a list, in place (the 3-vector columns keep the
// list's component stride).
static mx_photons slice_photons(const mx_photons *ph, size_t i0, size_t m) {
  mx_photons d = *ph;
  d.n = (uint32_t) m;
  d.stride = ph->stride ? ph->stride : ph->n;
  auto at = [&](auto *&col) {
    if (col) col += i0;
  };
  at(d.energy); at(d.x); at(d.p); at(d.arrival_time); at(d.flags); at(d.tag); at(d.mirror_shell); at(d.order);
  at(d.ccd_num); at(d.reserved8); at(d.y_pixel); at(d.z_pixel); at(d.dither_state); at(d.support_orders);
  at(d.pulse_height); at(d.u_pixel); at(d.v_pixel); at(d.detector_region); at(d.pi); at(d.det_dither);
  return d;
}

static int pipe_streams(mx_context *c) {
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < MX_PIPE_STREAMS && e == cudaSuccess; s++)
    if (!c->pipe[s]) e = cudaStreamCreateWithFlags(&c->pipe[s], cudaStreamNonBlocking);
  for (int q = 0; q < 1 + MX_PIPE_STREAMS && e == cudaSuccess; q++)
    if (!c->split_ev[q]) e = cudaEventCreateWithFlags(&c->split_ev[q], cudaEventDisableTiming);
  return e == cudaSuccess ? MX_OK : cuda_fail(c, e, "creating the trace streams");
}

// A device trace that takes the wavefront kernels with Philox draws, from
// MX_SPLIT_MIN_PHOTONS photons, runs as MX_PIPE_STREAMS consecutive parts
// traced at once on the context's pipeline streams (each with its own
// queues), forked from and joined back into the caller's stream: the launch,
// ramp and tail of one part's kernels overlap the other's work.  Photons
// are independent and draw by tag (a part without a tag column counts from
// its first photon's index), so the results equal the one-pass trace's.
int mx_trace_tables(mx_context *c, const MxTables &T, const mx_photons *ph, uint32_t stages, const double *U,
                    const double *N, uint64_t seed, cudaStream_t st, bool fresh) {
  const bool wave = ph && (stages & MX_STAGE_MIRROR) &&
                    (c->mode == MX_MODE_WAVEFRONT || (c->mode == MX_MODE_AUTO && ph->n >= MX_WAVEFRONT_MIN_PHOTONS));
  if (!wave || U || N || ph->n < MX_SPLIT_MIN_PHOTONS)
    return mx_trace_queues(c, T, ph, stages, U, N, seed, st, fresh, c->wave);
  TraceIO io;   // the argument checks, before anything is queued
  int r = mx_trace_io(c, T, ph, stages, U, N, seed, fresh, io, "mx_trace");
  if (r) return r;
  if ((r = pipe_streams(c))) return r;
  cudaError_t e = cudaEventRecord(c->split_ev[0], st);
  const size_t n = ph->n, part = ((n + MX_PIPE_STREAMS - 1) / MX_PIPE_STREAMS + 255) & ~(size_t) 255;
  for (int s = 0; s < MX_PIPE_STREAMS && e == cudaSuccess; s++) {
    const size_t i0 = std::min(n, s * part), m = std::min(part, n - i0);
    if ((e = cudaStreamWaitEvent(c->pipe[s], c->split_ev[0], 0)) != cudaSuccess) break;
    if (m) {
      const mx_photons d = slice_photons(ph, i0, m);
      if ((r = mx_trace_queues(c, T, &d, stages, U, N, seed, c->pipe[s], fresh, c->pipe_wave[s], true, (uint32_t) i0)))
        return r;
    }
    if ((e = cudaEventRecord(c->split_ev[1 + s], c->pipe[s])) == cudaSuccess)
      e = cudaStreamWaitEvent(st, c->split_ev[1 + s], 0);
  }
  return e == cudaSuccess ? MX_OK : cuda_fail(c, e, "trace");
}

}  // extern "C"

int mx_trace_io(mx_context *c, const MxTables &T, const mx_photons *ph, uint32_t stages, const double *U,
                const double *N, uint64_t seed, bool fresh, TraceIO &io, const char *who) {
  const std::string w(who);
  if (!ph) return fail(c, MX_EINVAL, w + ": null photon list");
  if (!ph->energy || !ph->p) return fail(c, MX_EINVAL, w + ": energy and p are required");
  if ((U == nullptr) != (N == nullptr)) return fail(c, MX_EINVAL, w + ": give both U and N or neither");
  if ((stages & MX_STAGE_DETECT) && T.nchips && (!ph->x)) return fail(c, MX_EINVAL, w + ": x is required");
  if ((stages & (MX_STAGE_DITHER | MX_STAGE_DETECT)) && T.dither_file && T.asp_n == 0)
    return fail(c, MX_EINVAL, w + ": DitherModel FILE needs mx_set_aspect_solution");
  memset(&io, 0, sizeof(io));
  io.energy = ph->energy; io.x = ph->x; io.p = ph->p; io.t = ph->arrival_time; io.flags = ph->flags;
  io.tag = ph->tag; io.shell = ph->mirror_shell; io.order = ph->order; io.ccd = ph->ccd_num;
  io.ypix = ph->y_pixel; io.zpix = ph->z_pixel; io.dith = ph->dither_state;
  io.support = ph->support_orders; io.pha = ph->pulse_height; io.upix = ph->u_pixel; io.vpix = ph->v_pixel;
  io.region = ph->detector_region;
  io.pi = ph->pi;
  io.ddith = ph->det_dither;
  io.U = U; io.N = N; io.n = ph->n; io.seed = seed; io.stages = stages; io.fresh = fresh ? 1 : 0;
  io.stride = ph->stride ? ph->stride : ph->n;
  if (io.stride < io.n) return fail(c, MX_EINVAL, w + ": stride below n");
  io.overrun = c->d_overrun;
  return MX_OK;
}

int mx_trace_queues(mx_context *c, const MxTables &T, const mx_photons *ph, uint32_t stages, const double *U,
                    const double *N, uint64_t seed, cudaStream_t st, bool fresh, DevBuf &queues, bool force_wave,
                    uint32_t tag0) {
  if (!ph) return fail(c, MX_EINVAL, "mx_trace: null photon list");
  if (ph->n == 0) return MX_OK;
  TraceIO io;
  int r = mx_trace_io(c, T, ph, stages, U, N, seed, fresh, io, "mx_trace");
  if (r) return r;
  io.tag0 = tag0;
  int slots = U != nullptr;
  bool wave = (stages & MX_STAGE_MIRROR) &&
              (c->mode == MX_MODE_WAVEFRONT || (c->mode == MX_MODE_AUTO && (force_wave || ph->n >= MX_WAVEFRONT_MIN_PHOTONS)));
  cudaError_t e;
  if (wave) {
    size_t qbytes = (size_t) ph->n * sizeof(MxRec);
    e = queues.ensure(2 * qbytes + 256);
    if (e != cudaSuccess) return cuda_fail(c, e, "allocating wavefront queues");
    WaveBufs w;
    w.q1 = (MxRec *) queues.ptr;
    w.q2 = (MxRec *) ((char *) queues.ptr + qbytes);
    w.counts = (unsigned int *) ((char *) queues.ptr + 2 * qbytes);
    e = launch_wavefront(T, io, w, c->num_sms * c->wave_blocks, (int) c->shared_bytes, st);
    c->launches += wave_kernels(T, stages);
  } else {
    e = launch_trace(T, io, c->num_sms * c->trace_blocks[slots ? 0 : 1], (int) c->shared_bytes, slots != 0, st);
    c->launches++;
  }
  if (e == cudaSuccess && (stages & MX_STAGE_DETECT) && (T.acis_fef || T.acis_qe)) {
    e = launch_acis_fef(T, io, c->num_sms * 8, st);
    c->launches++;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "launching the trace kernels");
  return MX_OK;
}

extern "C" {

int mx_trace(mx_context *c, const mx_photons *ph, uint32_t stages, const mx_variates *var, uint64_t seed,
             void *stream) {
  if (!c) return MX_EINVAL;
  return mx_trace_tables(c, c->T, ph, stages, var ? var->U : nullptr, var ? var->N : nullptr, seed,
                         (cudaStream_t) stream, false);
}

// The host columns of mx_trace_host: pointer, element size, components,
// copied in, copied out.
struct HostCol { const void *host; size_t elem; int comps; bool in, out; };
static int host_columns(const mx_photons *h, HostCol cols[19]) {
  const HostCol c[19] = {
      {h->energy, 8, 1, true, false},     {h->x, 8, 3, false, true},         {h->p, 8, 3, true, true},
      {h->arrival_time, 8, 1, true, false}, {h->flags, 4, 1, true, true},   {h->tag, 4, 1, true, false},
      {h->mirror_shell, 1, 1, false, true}, {h->order, 1, 1, false, true},   {h->ccd_num, 1, 1, false, true},
      {h->y_pixel, 4, 1, false, true},    {h->z_pixel, 4, 1, false, true},   {h->dither_state, 4, 3, false, true},
      {h->support_orders, 1, 4, false, true}, {h->pulse_height, 2, 1, false, true}, {h->u_pixel, 4, 1, false, true},
      {h->v_pixel, 4, 1, false, true},    {h->detector_region, 1, 1, false, true}, {h->pi, 4, 1, false, true},
      {h->det_dither, 4, 3, false, true}};
  for (int k = 0; k < 19; k++) cols[k] = c[k];
  return 19;
}

// Chunk boundaries of a pipelined mx_trace_host over n >= MX_PIPE_MIN_PHOTONS
// photons: chunk j is start[j] .. start[j + 1]; returns the number of chunks.
// The nominal chunk is a 1/nch share (nch = n / 2^19 within 4..MX_PIPE_CHUNKS);
// the first two chunks are a quarter and a half of it and so are the last
// two, so that the first kernels start after a short copy in and the step
// ends with a short copy out.  Every boundary but n is a multiple of 256.
// With u a quarter chunk (n <= 4 nch u) the middle takes at most nch - 1
// chunks, so there are at most nch + 3 <= MX_PIPE_MAX_CHUNKS.
static int pipe_chunks(size_t n, size_t start[MX_PIPE_MAX_CHUNKS + 1]) {
  const size_t nch = std::max<size_t>(4, std::min<size_t>(MX_PIPE_CHUNKS, n >> 19));
  const size_t u = ((n + 4 * nch - 1) / (4 * nch) + 255) & ~(size_t) 255;
  const size_t last = (n - u) & ~(size_t) 255, before = last - 2 * u;
  const size_t r = before - 3 * u, mid = (r + 4 * u - 1) / (4 * u);
  const size_t each = ((r + mid - 1) / mid + 255) & ~(size_t) 255;
  int k = 0;
  start[k++] = 0;
  start[k++] = u;
  for (size_t i0 = 3 * u; i0 < before; i0 += each) start[k++] = i0;
  start[k++] = before;
  start[k++] = last;
  start[k] = n;
  return k;
}

// mx_trace_host for a large list: MX_PIPE_CHUNKS chunks of consecutive
// photons.  The copies in run back to back on one stream and the copies out
// on another (the two directions of the host link at once); chunk j is
// traced on compute stream j % MX_PIPE_STREAMS with its own wavefront
// queues as soon as its copy is in, so the kernels of neighbouring chunks
// fill each other's tails and no copy waits behind a trace.  Photons are independent and draw by tag, so the results equal
// the single-pass trace's.  Multi-component columns keep the list's own
// component stride on the device; a chunk's pre-drawn variates are packed
// slot-major for its own length.
static int trace_host_pipelined(mx_context *c, const mx_photons *h, uint32_t stages, const mx_variates *hv,
                                uint64_t seed) {
  const size_t n = h->n;
  HostCol cols[19];
  const int NC = host_columns(h, cols);
  if (int r = pipe_streams(c)) return r;
  cudaError_t e = cudaSuccess;
  char *dev[19];
  for (int k = 0; k < NC; k++) {
    dev[k] = nullptr;
    if (!cols[k].host) continue;
    if ((e = c->io[k].ensure(n * cols[k].elem * cols[k].comps)) != cudaSuccess)
      return cuda_fail(c, e, "allocating staging buffers");
    dev[k] = (char *) c->io[k].ptr;
  }
  const bool slots = hv && hv->U && hv->N;
  if (slots && ((e = c->io[NC].ensure(n * MX_NUM_U * 8)) != cudaSuccess ||
                (e = c->io[NC + 1].ensure(n * MX_NUM_N * 8)) != cudaSuccess))
    return cuda_fail(c, e, "allocating variate buffers");
  if (!c->pipe_in && (e = cudaStreamCreateWithFlags(&c->pipe_in, cudaStreamNonBlocking)) != cudaSuccess)
    return cuda_fail(c, e, "creating the copy streams");
  if (!c->pipe_out && (e = cudaStreamCreateWithFlags(&c->pipe_out, cudaStreamNonBlocking)) != cudaSuccess)
    return cuda_fail(c, e, "creating the copy streams");
  for (int j = 0; j < MX_PIPE_MAX_CHUNKS && e == cudaSuccess; j++)
    for (int q = 0; q < 2 && e == cudaSuccess; q++)
      if (!c->pipe_ev[q][j]) e = cudaEventCreateWithFlags(&c->pipe_ev[q][j], cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(c, e, "creating the chunk events");
  // the staging buffers and queues were last used on the context's stream
  // or by an earlier call: every stream of this call waits for it first
  cudaEvent_t ready;
  if ((e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming)) != cudaSuccess) return cuda_fail(c, e, "event");
  cudaEventRecord(ready, c->stream);
  for (int s = 0; s < MX_PIPE_STREAMS; s++) cudaStreamWaitEvent(c->pipe[s], ready, 0);
  cudaStreamWaitEvent(c->pipe_in, ready, 0);
  cudaStreamWaitEvent(c->pipe_out, ready, 0);
  cudaEventDestroy(ready);
  size_t start[MX_PIPE_MAX_CHUNKS + 1];
  const int nch = pipe_chunks(n, start);
  // chunk j's copies in on pipe_in, marked done by pipe_ev[0][j]
  auto copy_in = [&](int j) -> int {
    const size_t i0 = start[j], m = start[j + 1] - start[j];
    for (int k = 0; k < NC && e == cudaSuccess; k++) {
      if (!cols[k].host || !cols[k].in) continue;
      const size_t el = cols[k].elem;
      e = cudaMemcpy2DAsync(dev[k] + i0 * el, n * el, (const char *) cols[k].host + i0 * el, n * el, m * el,
                            cols[k].comps, cudaMemcpyHostToDevice, c->pipe_in);
    }
    if (slots && e == cudaSuccess) {
      double *u = (double *) c->io[NC].ptr + i0 * MX_NUM_U, *v = (double *) c->io[NC + 1].ptr + i0 * MX_NUM_N;
      e = cudaMemcpy2DAsync(u, m * 8, hv->U + i0, n * 8, m * 8, MX_NUM_U, cudaMemcpyHostToDevice, c->pipe_in);
      if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(v, m * 8, hv->N + i0, n * 8, m * 8, MX_NUM_N, cudaMemcpyHostToDevice, c->pipe_in);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->pipe_ev[0][j], c->pipe_in);
    return e == cudaSuccess ? MX_OK : cuda_fail(c, e, "copying photons to the device");
  };
  // chunk j traced on compute stream j % MX_PIPE_STREAMS (with its own
  // queues) once its copy is in, marked done by pipe_ev[1][j]
  auto trace = [&](int j) -> int {
    const size_t i0 = start[j], m = start[j + 1] - start[j];
    cudaStream_t st = c->pipe[j % MX_PIPE_STREAMS];
    if ((e = cudaStreamWaitEvent(st, c->pipe_ev[0][j], 0)) != cudaSuccess) return cuda_fail(c, e, "trace");
    const double *dU = nullptr, *dN = nullptr;
    if (slots) {
      dU = (double *) c->io[NC].ptr + i0 * MX_NUM_U;
      dN = (double *) c->io[NC + 1].ptr + i0 * MX_NUM_N;
    }
    mx_photons d;
    memset(&d, 0, sizeof(d));
    d.n = (uint32_t) m;
    d.stride = (uint32_t) n;
    auto at = [&](int k) { return dev[k] ? (void *) (dev[k] + i0 * cols[k].elem) : nullptr; };
    d.energy = (double *) at(0); d.x = (double *) at(1); d.p = (double *) at(2);
    d.arrival_time = (double *) at(3); d.flags = (uint32_t *) at(4); d.tag = (uint32_t *) at(5);
    d.mirror_shell = (int8_t *) at(6); d.order = (int8_t *) at(7); d.ccd_num = (int8_t *) at(8);
    d.y_pixel = (float *) at(9); d.z_pixel = (float *) at(10); d.dither_state = (float *) at(11);
    d.support_orders = (int8_t *) at(12); d.pulse_height = (int16_t *) at(13); d.u_pixel = (float *) at(14);
    d.v_pixel = (float *) at(15); d.detector_region = (uint8_t *) at(16); d.pi = (float *) at(17);
    d.det_dither = (float *) at(18);
    int r = mx_trace_queues(c, c->T, &d, stages, dU, dN, seed, st, true, c->pipe_wave[j % MX_PIPE_STREAMS], true,
                            (uint32_t) i0);
    if (r) return r;
    if ((e = cudaEventRecord(c->pipe_ev[1][j], st)) != cudaSuccess) return cuda_fail(c, e, "trace");
    return MX_OK;
  };
  // chunk j's copies out on pipe_out (in chunk order) after its trace
  auto copy_out = [&](int j) -> int {
    const size_t i0 = start[j], m = start[j + 1] - start[j];
    e = cudaStreamWaitEvent(c->pipe_out, c->pipe_ev[1][j], 0);
    for (int k = 0; k < NC && e == cudaSuccess; k++) {
      if (!cols[k].host || !cols[k].out) continue;
      const size_t el = cols[k].elem;
      e = cudaMemcpy2DAsync((char *) cols[k].host + i0 * el, n * el, dev[k] + i0 * el, n * el, m * el,
                            cols[k].comps, cudaMemcpyDeviceToHost, c->pipe_out);
    }
    return e == cudaSuccess ? MX_OK : cuda_fail(c, e, "copying photons to the host");
  };
  // issued chunk by chunk, so that the first kernels are queued as soon as
  // their copies are (the streams and events order the work, not the calls)
  for (int j = 0; j < nch; j++) {
    int r = copy_in(j);
    if (!r) r = trace(j);
    if (!r) r = copy_out(j);
    if (r) return r;
  }
  for (int s = 0; s < MX_PIPE_STREAMS && e == cudaSuccess; s++) e = cudaStreamSynchronize(c->pipe[s]);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->pipe_in);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->pipe_out);
  if (e != cudaSuccess) return cuda_fail(c, e, "trace");
  return MX_OK;
}

int mx_trace_host(mx_context *c, const mx_photons *h, uint32_t stages, const mx_variates *hv, uint64_t seed) {
  if (!c) return MX_EINVAL;
  if (!h) return fail(c, MX_EINVAL, "mx_trace_host: null photon list");
  size_t n = h->n;
  if (n == 0) return MX_OK;
  if (!h->energy || !h->p) return fail(c, MX_EINVAL, "mx_trace_host: energy and p are required");
  if (h->stride && h->stride != h->n) return fail(c, MX_EINVAL, "mx_trace_host: host lists must be contiguous (stride 0 or n)");
  struct Col { const void *host; size_t elem; int comps; bool in, out; };
  const int NC = 19;
  const Col cols[NC] = {
      {h->energy, 8, 1, true, false},     {h->x, 8, 3, false, true},         {h->p, 8, 3, true, true},
      {h->arrival_time, 8, 1, true, false}, {h->flags, 4, 1, true, true},   {h->tag, 4, 1, true, false},
      {h->mirror_shell, 1, 1, false, true}, {h->order, 1, 1, false, true},   {h->ccd_num, 1, 1, false, true},
      {h->y_pixel, 4, 1, false, true},    {h->z_pixel, 4, 1, false, true},   {h->dither_state, 4, 3, false, true},
      {h->support_orders, 1, 4, false, true}, {h->pulse_height, 2, 1, false, true}, {h->u_pixel, 4, 1, false, true},
      {h->v_pixel, 4, 1, false, true},    {h->detector_region, 1, 1, false, true}, {h->pi, 4, 1, false, true},
      {h->det_dither, 4, 3, false, true}};
  if (n >= MX_PIPE_MIN_PHOTONS && (stages & MX_STAGE_MIRROR)) return trace_host_pipelined(c, h, stages, hv, seed);
  void *dev[NC];
  cudaStream_t st = c->stream;
  cudaError_t e;
  for (int k = 0; k < NC; k++) {
    dev[k] = nullptr;
    if (!cols[k].host) continue;
    size_t bytes = n * cols[k].elem * cols[k].comps;
    if ((e = c->io[k].ensure(bytes)) != cudaSuccess) return cuda_fail(c, e, "allocating staging buffers");
    dev[k] = c->io[k].ptr;
    if (cols[k].in && (e = cudaMemcpyAsync(dev[k], cols[k].host, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return cuda_fail(c, e, "copying photons to the device");
  }
  const double *dU = nullptr, *dN = nullptr;
  if (hv && hv->U && hv->N) {
    if ((e = c->io[NC].ensure(n * MX_NUM_U * 8)) != cudaSuccess || (e = c->io[NC + 1].ensure(n * MX_NUM_N * 8)) != cudaSuccess)
      return cuda_fail(c, e, "allocating variate buffers");
    cudaMemcpyAsync(c->io[NC].ptr, hv->U, n * MX_NUM_U * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(c->io[NC + 1].ptr, hv->N, n * MX_NUM_N * 8, cudaMemcpyHostToDevice, st);
    dU = (const double *) c->io[NC].ptr; dN = (const double *) c->io[NC + 1].ptr;
  }
  mx_photons d;
  memset(&d, 0, sizeof(d));
  d.n = h->n;
  d.energy = (double *) dev[0]; d.x = (double *) dev[1]; d.p = (double *) dev[2];
  d.arrival_time = (double *) dev[3]; d.flags = (uint32_t *) dev[4]; d.tag = (uint32_t *) dev[5];
  d.mirror_shell = (int8_t *) dev[6]; d.order = (int8_t *) dev[7]; d.ccd_num = (int8_t *) dev[8];
  d.y_pixel = (float *) dev[9]; d.z_pixel = (float *) dev[10]; d.dither_state = (float *) dev[11];
  d.support_orders = (int8_t *) dev[12]; d.pulse_height = (int16_t *) dev[13]; d.u_pixel = (float *) dev[14];
  d.v_pixel = (float *) dev[15]; d.detector_region = (uint8_t *) dev[16]; d.pi = (float *) dev[17];
  d.det_dither = (float *) dev[18];
  int r = mx_trace_tables(c, c->T, &d, stages, dU, dN, seed, st, true);
  if (r) return r;
  for (int k = 0; k < NC; k++) {
    if (!cols[k].host || !cols[k].out) continue;
    size_t bytes = n * cols[k].elem * cols[k].comps;
    if ((e = cudaMemcpyAsync((void *) cols[k].host, dev[k], bytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return cuda_fail(c, e, "copying photons to the host");
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(c, e, "trace");
  return MX_OK;
}

int mx_compact(mx_context *c, const uint32_t *flags, uint32_t n, uint32_t *idx_out, uint32_t *count_out,
               void *stream) {
  if (!c || !flags || !idx_out || !count_out) return fail(c, MX_EINVAL, "mx_compact: null argument");
  if (n == 0) { *count_out = 0; return MX_OK; }
  uint32_t nblk = (n + MX_COMPACT_TILE - 1) / MX_COMPACT_TILE;
  cudaError_t e = c->scan.ensure((size_t) (nblk + 1) * sizeof(uint32_t));
  if (e != cudaSuccess) return cuda_fail(c, e, "allocating compaction scratch");
  cudaStream_t st = (cudaStream_t) stream;
  e = launch_compact(flags, n, idx_out, (uint32_t *) c->scan.ptr, nblk, st);
  c->launches += 3;
  if (e != cudaSuccess) return cuda_fail(c, e, "launching compaction");
  e = cudaMemcpyAsync(count_out, (uint32_t *) c->scan.ptr + nblk, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(c, e, "compaction");
  return MX_OK;
}

int mx_overrun_count(mx_context *c, unsigned long long *count, int reset) {
  if (!c || !count) return MX_EINVAL;
  cudaError_t e = cudaMemcpy(count, c->d_overrun, sizeof(*count), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(c->d_overrun, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) return cuda_fail(c, e, "reading the overrun counter");
  return MX_OK;
}

int mx_probe_fp64(double *tflops, double *ms) {
  return probe_fp64(tflops, ms) == cudaSuccess ? MX_OK : MX_ECUDA;
}

int mx_math_check(int fn, const double *x, double *y, size_t n) {
  if (fn < 0 || fn > 8 || (n && (!x || !y))) return MX_EINVAL;
  if (n > ((size_t) 1 << 32)) return MX_ERANGE;
  return math_check(fn, x, y, n) == cudaSuccess ? MX_OK : MX_ECUDA;
}

}  // extern "C"
