// Trace, compaction and probe kernels.
#include <cuda_runtime.h>

#include "mx_device.cuh"
#include "mx_kernels.cuh"
#include "mx_wave.cuh"

using namespace mx;

// Shared-memory staging per block: shell geometry, gratings, chips, then
// the optical-constant and correction-factor tables (the per-photon binary
// searches run on these).
size_t trace_shared_bytes(const MxTables &T) { return tables_shared_bytes(T); }

// The detector part of the dither state the dither stage recorded (dy, dz,
// dtheta of Marx_Dither_Type): the aspect solution's at the photon's time,
// zero with the INTERNAL model.  Taken again from the table here instead of
// being carried through the trace.
__device__ __forceinline__ void store_det_dither(const MxTables &T, const TraceIO &io, size_t n, uint32_t i, double t,
                                                 uint32_t flags) {
  if (!io.ddith || !((io.stages & MX_STAGE_DITHER) && T.dither)) return;
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (T.dither_file && !(flags & MX_PHOTON_ASPECT_END)) aspsol_state(T, T.start_time + t, s);
  io.ddith[i] = s[3]; io.ddith[n + i] = s[4]; io.ddith[2 * n + i] = s[5];
}

// Fused dither -> mirror -> grating -> detector trace, one photon per
// thread, grid-stride over the photon list with a resident grid.
__global__ void __launch_bounds__(MX_TRACE_BLOCK) mx_trace_kernel(MxTables T, TraceIO io) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);

  const size_t n = io.stride;   // component stride of the 3-vector columns
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < io.n; i += stride) {
    Ph q;
    q.e = io.energy[i];
    q.t = io.t ? io.t[i] : 0.0;
    q.p = mk(io.p[i], io.p[n + i], io.p[2 * n + i]);
    q.flags = io.flags ? io.flags[i] : 0u;
    q.set = 0;
    for (int k = 0; k < 4; k++) q.sup[k] = (!io.fresh && io.support) ? io.support[k * n + i] : 0;
    if (io.fresh) {
      q.x = mk(0.0, 0.0, 0.0);
      q.shell = 0; q.order = 0; q.ccd = -1; q.ypix = 0.f; q.zpix = 0.f;
      q.dith[0] = q.dith[1] = q.dith[2] = 0.f;
      clear_extra(io, i);
    } else {
      q.x = io.x ? mk(io.x[i], io.x[n + i], io.x[2 * n + i]) : mk(0.0, 0.0, 0.0);
      q.shell = io.shell ? io.shell[i] : 0;
      q.order = io.order ? io.order[i] : 0;
      q.ccd = io.ccd ? io.ccd[i] : -1;
      q.ypix = io.ypix ? io.ypix[i] : 0.f;
      q.zpix = io.zpix ? io.zpix[i] : 0.f;
      for (int k = 0; k < 3; k++) q.dith[k] = io.dith ? io.dith[k * n + i] : 0.f;
    }
    Rng r;
    r.U = io.U; r.N = io.N; r.seed = io.seed; r.n = io.n; r.i = i;
    r.tag = io.tag ? io.tag[i] : io.tag0 + i;
    r.upos = r.uend = r.npos = r.nend = 0;
    r.overrun = false;
    trace_photon(T, sh, optc, slope, gr, ch, io.stages, q, r);
    if (r.overrun) {
      q.flags |= MX_PHOTON_VARIATE_OVERRUN;
      atomicAdd(io.overrun, 1ull);
    }
    if (io.x) { io.x[i] = q.x.x; io.x[n + i] = q.x.y; io.x[2 * n + i] = q.x.z; }
    io.p[i] = q.p.x; io.p[n + i] = q.p.y; io.p[2 * n + i] = q.p.z;
    if (io.flags) io.flags[i] = q.flags;
    if (io.shell) io.shell[i] = (int8_t) q.shell;
    if (io.order) io.order[i] = (int8_t) q.order;
    if (io.ccd) io.ccd[i] = (int8_t) q.ccd;
    if (io.ypix) io.ypix[i] = q.ypix;
    if (io.zpix) io.zpix[i] = q.zpix;
    if (io.dith) for (int k = 0; k < 3; k++) io.dith[k * n + i] = q.dith[k];
    store_det_dither(T, io, n, i, q.t, q.flags);
    store_extra(io, i, q);
  }
}

// The ACIS response pass over every photon the trace put on a chip
// (_marx_acis_apply_qe_and_pha, acis-s.c:136-172): with DetIdeal = no the
// QE x contamination acceptance, with an FEF the pulse height and PI, then
// the frame-transfer streak of those detected, as _marx_acis_s_detect and
// _marx_acis_i_detect order them (acis-s.c:230-236).  The trace leaves
// these steps to this pass when the tables carry either.
// Photon i is on a chip and still to be detected.
__device__ __forceinline__ bool acis_pending(const TraceIO &io, uint32_t i) {
  const int ccd = io.ccd[i];
  const uint32_t f0 = io.flags ? io.flags[i] : 0u;
  return ccd >= 0 && ccd <= 9 && !(f0 & (MX_BAD_PHOTON_MASK | MX_PHOTON_VARIATE_OVERRUN));
}

// Back from the detector frame of a photon with DitherModel FILE (kept out
// of line: the frame's search and rotation are not on the common path).
__device__ __noinline__ void leave_dithered_frame(const MxTables &T, double t, D3 &x, D3 &p) {
  const DetFrame f = det_frame(T, t);
  det_leave(T, f, x, p);
}

__device__ void acis_response(const MxTables &T, const TraceIO &io, uint32_t i, uint64_t seed, D3 off) {
  const size_t n = io.stride;
  const int ccd = io.ccd[i];
  Ph q;
  q.e = io.energy[i];
  q.t = io.t ? io.t[i] : 0.0;
  q.flags = io.flags ? io.flags[i] : 0u;
  q.ypix = io.ypix[i];
  q.zpix = io.zpix[i];
  Rng r;
  r.U = io.U; r.N = io.N; r.seed = seed; r.n = io.n; r.i = i;
  r.tag = io.tag ? io.tag[i] : io.tag0 + i;
  r.overrun = false;
  r.window(MX_U_DETECT, 2, MX_N_DETECT, 2);
  if (T.acis_qe && !acis_qe_accept(T, ccd, q, r)) {
    if (io.flags) io.flags[i] = q.flags | MX_PHOTON_UNDETECTED;
    return;
  }
  const int ub = r.upos, nb = r.npos;
  int16_t pha = -1;
  float pi = 0.0f;
  bool ok = true;
  if (T.acis_fef) {
    r.window(MX_U_FEF, r.U ? 8 : 64, MX_N_FEF, r.N ? 4 : 64);
    ok = acis_fef(T, ccd, q.ypix, q.zpix, q.e, r, pha, pi);
  }
  if (r.overrun) {
    q.flags |= MX_PHOTON_VARIATE_OVERRUN;
    atomicAdd(io.overrun, 1ull);
  } else if (!ok) {
    pha = -1; pi = 0.0f;
    q.flags |= MX_PHOTON_UNDETECTED;
  } else {
    r.window(ub, MX_U_DETECT + 2 - ub, nb, MX_N_DETECT + 2 - nb);   // the ACIS window, after the QE draw
    D3 x = mk(0, 0, 0), p = mk(0, 0, 0);
    acis_streak(T, T.chips[ccd], q, x, p, r);
    if (q.flags & MX_PHOTON_ACIS_STREAKED) {
      if (T.dither_file) leave_dithered_frame(T, q.t, x, p);
      else x = x + off;
      if (io.x) { io.x[i] = x.x; io.x[n + i] = x.y; io.x[2 * n + i] = x.z; }
      io.p[i] = p.x; io.p[n + i] = p.y; io.p[2 * n + i] = p.z;
      io.zpix[i] = q.zpix;
    }
  }
  if (T.acis_fef) {
    if (io.pha) io.pha[i] = pha;
    if (io.pi) io.pi[i] = pi;
  }
  if (io.flags) io.flags[i] = q.flags;
}

// A fifth or less of the photons reach a chip, and each costs several
// hundred FP64 operations here, so each block first gathers the indices of
// pending photons from successive 256-photon tiles into shared memory and
// works on them 256 at a time, every lane busy.
__global__ void __launch_bounds__(256) mx_acis_fef_kernel(MxTables T, TraceIO io, const uint64_t *seedp) {
  __shared__ uint32_t list[512];
  __shared__ int count;
  const uint64_t seed = seedp ? *seedp : io.seed;
  const D3 off = mk(T.det_offset[0], T.det_offset[1], T.det_offset[2]);
  if (threadIdx.x == 0) count = 0;
  __syncthreads();
  for (uint32_t base = blockIdx.x * 256u; base < io.n; base += gridDim.x * 256u) {
    const uint32_t i = base + threadIdx.x;
    if (i < io.n && acis_pending(io, i)) list[atomicAdd(&count, 1)] = i;   // count stays below 512
    __syncthreads();
    const int c = count;
    if (c >= 256) {
      acis_response(T, io, list[c - 256 + threadIdx.x], seed, off);
      __syncthreads();
      if (threadIdx.x == 0) count = c - 256;
    }
    __syncthreads();
  }
  const int c = count;
  if ((int) threadIdx.x < c) acis_response(T, io, list[threadIdx.x], seed, off);
}

cudaError_t launch_acis_fef(const MxTables &T, const TraceIO &io, int grid, cudaStream_t st, const uint64_t *seed_dev) {
  if (!io.ccd || !io.ypix || !io.zpix || io.n == 0) return cudaSuccess;
  uint32_t need = (io.n + 255) / 256;
  if ((uint32_t) grid > need) grid = (int) need;
  if (grid < 1) grid = 1;
  mx_acis_fef_kernel<<<grid, 256, 0, st>>>(T, io, seed_dev);
  return cudaGetLastError();
}

// ------------------------------------------------------------ wavefront --
// The same trace as mx_trace_kernel split where photons are lost, so that
// lost photons stop occupying SIMT lanes: phase A runs every photon up to
// the paraboloid intersection (the photons between the shells are lost
// there) and appends the rest to queue 1; phase T draws the paraboloid's
// normal blur and reflectivity test and moves the photons it reflects to
// queue 2; phase B finishes that reflection, intersects the hyperboloid and
// applies its reflectivity test, appending survivors to queue 1 again;
// phase C finishes the hyperboloid reflection and runs the detector, or,
// with a grating, the grating up to its order choice, appending the photons
// given an order to queue 2 for phase D (diffraction and detector).
// Appends are warp-aggregated (one atomic per warp); the order of records
// in a queue does not affect any photon's result.

__global__ void __launch_bounds__(MX_WAVE_BLOCK, MX_WAVE_MIN_BLOCKS) mx_wave_a(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const size_t n = io.stride;   // component stride of the 3-vector columns
  const uint32_t lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = warp * 32; base < io.n; base += nwarps * 32) {
    const uint32_t i = base + lane;
    bool keep = false;
    MxRec rec;
    if (i < io.n) {
      Ph q;
      q.e = io.energy[i];
      q.t = io.t ? io.t[i] : 0.0;
      q.p = mk(io.p[i], io.p[n + i], io.p[2 * n + i]);
      q.flags = io.flags ? io.flags[i] : 0u;
      q.set = 0;
      if (io.fresh) {
        q.x = mk(0.0, 0.0, 0.0); q.shell = 0;
        q.dith[0] = q.dith[1] = q.dith[2] = 0.f;
        clear_extra(io, i);
        if (io.order) io.order[i] = 0;
        if (io.ccd) io.ccd[i] = -1;
        if (io.ypix) io.ypix[i] = 0.f;
        if (io.zpix) io.zpix[i] = 0.f;
      } else {
        q.x = io.x ? mk(io.x[i], io.x[n + i], io.x[2 * n + i]) : mk(0.0, 0.0, 0.0);
        q.shell = io.shell ? io.shell[i] : 0;
        for (int k = 0; k < 3; k++) q.dith[k] = io.dith ? io.dith[k * n + i] : 0.f;
      }
      Rng r;
      r.U = io.U; r.N = io.N; r.seed = io.seed; r.n = io.n; r.i = i;
      r.tag = io.tag ? io.tag[i] : io.tag0 + i;
      r.upos = r.uend = r.npos = r.nend = 0;
      r.overrun = false;
      if ((io.stages & MX_STAGE_DITHER) && T.dither) dither_stage(T, q, r);
      if (io.dith) for (int k = 0; k < 3; k++) io.dith[k * n + i] = q.dith[k];
      store_det_dither(T, io, n, i, q.t, q.flags);
      MirrorState m;
      if (!(q.flags & MX_BAD_PHOTON_MASK) && mirror_front(T, sh, optc, slope, q, r, m)) {
        keep = true;
        to_rec(rec, q, m, r, i);
      } else
        store_core(io, i, q, r.overrun);
    }
    append(keep, rec, w.q1, &w.counts[0]);
  }
}

// One queue-to-queue phase: records of `in` (count at *in_count) through
// `step`; survivors are appended to `out`, the rest stored.
template <typename Step>
__device__ __forceinline__ void wave_pass(const TraceIO &io, const MxRec *in, const unsigned int *in_count, MxRec *out,
                                          unsigned int *out_count, Step step) {
  const uint32_t count = *(volatile const unsigned int *) in_count;
  const uint32_t lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = warp * 32; base < count; base += nwarps * 32) {
    const uint32_t k = base + lane;
    bool keep = false;
    MxRec rec;
    if (k < count) {
      rec = in[k];
      Ph q; MirrorState m; Rng r;
      from_rec(rec, q, m, r, io);
      if (step(q, r, m)) {
        keep = true;
        to_rec(rec, q, m, r, rec.i);
      } else
        store_core(io, rec.i, q, r.overrun);
    }
    append(keep, rec, out, out_count);
  }
}

__global__ void __launch_bounds__(MX_WAVE_BLOCK, MX_WAVE_MIN_BLOCKS) mx_wave_t(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  wave_pass(io, w.q1, &w.counts[0], w.q2, &w.counts[1],
            [&](Ph &q, Rng &r, MirrorState &m) { return mirror_ptest(T, sh, q, r, m); });
}

__global__ void __launch_bounds__(MX_WAVE_BLOCK, MX_WAVE_MIN_BLOCKS) mx_wave_b(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  wave_pass(io, w.q2, &w.counts[1], w.q1, &w.counts[2],
            [&](Ph &q, Rng &r, MirrorState &m) { return mirror_middle(T, sh, q, r, m); });
}

// The end of a photon's trace in phases C and D: the detector (when the
// photon is still good), then its output columns.
__device__ __forceinline__ void finish_photon(const MxTables &T, const MxChipDev *ch, const TraceIO &io, uint32_t i,
                                              Ph &q, Rng &r) {
  const int unset = 0x7fff;
  if (!r.overrun && (io.stages & MX_STAGE_DETECT) && T.nchips && !(q.flags & MX_BAD_PHOTON_MASK))
    any_detect_stage(T, ch + T.chip_off, T.nchips, q, r);
  store_core(io, i, q, r.overrun);
  store_extra(io, i, q);
  if (q.order != unset && io.order) io.order[i] = (int8_t) q.order;
  if (q.ccd != unset) {
    if (io.ccd) io.ccd[i] = (int8_t) q.ccd;
    if (q.ccd >= 0) {
      if (io.ypix) io.ypix[i] = q.ypix;
      if (io.zpix) io.zpix[i] = q.zpix;
    }
  }
}

__device__ __forceinline__ void load_supports(const MxTables &T, const TraceIO &io, uint32_t i, Ph &q) {
  if (T.grating == MX_GRATING_LETG)   // supports skipped by this photon keep their values
    for (int s = 0; s < 4; s++) q.sup[s] = io.support ? io.support[s * (size_t) io.stride + i] : 0;
}

// Phase C: the hyperboloid's reflection and the post-collimator struts, then
// with a grating its vignetting, Rowland torus and order choice, sending the
// photons given an order to phase D; every other photon runs the detector
// (without a grating) and is stored here.
__global__ void __launch_bounds__(MX_WAVE_BLOCK, MX_WAVE_MIN_BLOCKS) mx_wave_c(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const uint32_t count = *(volatile unsigned int *) &w.counts[2];
  const bool grating = (io.stages & MX_STAGE_GRATING) && T.grating;
  const uint32_t lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = warp * 32; base < count; base += nwarps * 32) {
    const uint32_t k = base + lane;
    bool to_d = false;
    MxRec rec;
    if (k < count) {
      rec = w.q1[k];
      const uint32_t i = rec.i;
      Ph q; MirrorState m; Rng r;
      from_rec(rec, q, m, r, io);
      const int unset = 0x7fff;
      q.order = unset; q.ccd = unset;
      load_supports(T, io, i, q);
      mirror_back(T, sh, q, r, m);
      if (!r.overrun && grating && !(q.flags & MX_BAD_PHOTON_MASK)) {
        D3 gx, gp;
        const int chosen = grating_front(T, gr, T.grating, q, r, gx, gp);
        if (chosen >= 0) {
          to_d = true;
          to_rec_d(rec, gx, gp, q, r, i, chosen);
        }
      }
      if (!to_d) finish_photon(T, ch, io, i, q, r);
    }
    if (grating) append(to_d, rec, w.q2, &w.counts[3]);
  }
}

// Phase D (with a grating): the diffraction into the chosen order (and the
// LETG's supports), the detector and the output columns.
__global__ void __launch_bounds__(MX_WAVE_BLOCK, MX_WAVE_MIN_BLOCKS) mx_wave_d(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const uint32_t count = *(volatile unsigned int *) &w.counts[3];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    const MxRec rec = w.q2[k];
    const uint32_t i = rec.i;
    Ph q;
    q.e = rec.e; q.t = rec.t; q.flags = rec.flags; q.shell = rec.shell; q.set = 0;
    const int unset = 0x7fff;
    q.ccd = unset;
    load_supports(T, io, i, q);
    Rng r;
    r.U = io.U; r.N = io.N; r.seed = io.seed; r.n = io.n; r.i = i; r.tag = rec.tag;
    if (T.grating == MX_GRATING_LETG) r.window(MX_U_LETG, 6, MX_N_LETG, 10);
    else r.window(MX_U_GRATING, 2, MX_N_GRATING, 2);
    r.upos = rec.upos; r.npos = rec.npos; r.overrun = rec.overrun != 0;
    const int chosen = (int) rec.pdn;
    q.order = chosen - gr[(T.grating == MX_GRATING_LETG ? 4 : 0) + q.shell].max_order;
    grating_back(T, gr, T.grating, q, r, mk(rec.x[0], rec.x[1], rec.x[2]), mk(rec.p[0], rec.p[1], rec.p[2]), chosen);
    finish_photon(T, ch, io, i, q, r);
  }
}

cudaError_t wave_occupancy(int shared_bytes, int *blocks_per_sm) {
  const void *f[5] = {(const void *) mx_wave_a, (const void *) mx_wave_t, (const void *) mx_wave_b,
                      (const void *) mx_wave_c, (const void *) mx_wave_d};
  int best = 1 << 30;
  for (int k = 0; k < 5; k++) {
    int b = 0;
    cudaError_t e = cudaFuncSetAttribute(f[k], cudaFuncAttributeMaxDynamicSharedMemorySize, shared_bytes);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f[k], MX_WAVE_BLOCK, shared_bytes);
    if (e != cudaSuccess) return e;
    if (b < best) best = b;
  }
  *blocks_per_sm = best;
  return cudaSuccess;
}

cudaError_t launch_wavefront(const MxTables &T, const TraceIO &io, const WaveBufs &w, int grid, int shared_bytes,
                             cudaStream_t st) {
  uint32_t need = (io.n + MX_WAVE_BLOCK - 1) / MX_WAVE_BLOCK;
  int ga = (uint32_t) grid > need ? (int) need : grid;
  if (ga < 1) ga = 1;
  cudaError_t e = cudaMemsetAsync(w.counts, 0, 4 * sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  mx_wave_a<<<ga, MX_WAVE_BLOCK, shared_bytes, st>>>(T, io, w);
  mx_wave_t<<<ga, MX_WAVE_BLOCK, shared_bytes, st>>>(T, io, w);
  mx_wave_b<<<ga, MX_WAVE_BLOCK, shared_bytes, st>>>(T, io, w);
  mx_wave_c<<<ga, MX_WAVE_BLOCK, shared_bytes, st>>>(T, io, w);
  if (wave_kernels(T, io.stages) == 5) mx_wave_d<<<ga, MX_WAVE_BLOCK, shared_bytes, st>>>(T, io, w);
  return cudaGetLastError();
}

cudaError_t trace_occupancy(bool philox, int shared_bytes, int *blocks_per_sm) {
  (void) philox;
  cudaError_t e = cudaFuncSetAttribute(mx_trace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, shared_bytes);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, mx_trace_kernel, MX_TRACE_BLOCK, shared_bytes);
}

cudaError_t launch_trace(const MxTables &T, const TraceIO &io, int grid, int shared_bytes, bool slots,
                         cudaStream_t st) {
  (void) slots;
  uint32_t need = (io.n + MX_TRACE_BLOCK - 1) / MX_TRACE_BLOCK;
  if ((uint32_t) grid > need) grid = (int) need;
  if (grid < 1) grid = 1;
  mx_trace_kernel<<<grid, MX_TRACE_BLOCK, shared_bytes, st>>>(T, io);
  return cudaGetLastError();
}

// ------------------------------------------------------------ compaction --
// marx_prune_photons (photon.c:40) as a three-pass stream compaction:
// per-tile survivor counts, an exclusive scan of the counts, then a
// warp-ballot / block-prefix scatter that keeps ascending index order.
__global__ void __launch_bounds__(MX_COMPACT_THREADS) mx_compact_count(const uint32_t *flags, uint32_t n,
                                                                       uint32_t *counts) {
  __shared__ uint32_t warp_tot[MX_COMPACT_THREADS / 32];
  uint32_t base = blockIdx.x * MX_COMPACT_TILE, c = 0;
  for (int j = 0; j < MX_COMPACT_ITEMS; j++) {
    uint32_t e = base + j * MX_COMPACT_THREADS + threadIdx.x;
    c += (e < n && (flags[e] & MX_BAD_PHOTON_MASK) == 0) ? 1u : 0u;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t s = 0;
    for (int w = 0; w < MX_COMPACT_THREADS / 32; w++) s += warp_tot[w];
    counts[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(1024) mx_compact_scan(uint32_t *counts, uint32_t nblk) {
  __shared__ uint32_t part[1024];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < nblk; base += 1024) {
    uint32_t k = base + threadIdx.x;
    uint32_t v = k < nblk ? counts[k] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {   // inclusive Hillis-Steele scan
      uint32_t t = threadIdx.x >= (unsigned) o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (k < nblk) counts[k] = carry + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[nblk] = carry;
}

__global__ void __launch_bounds__(MX_COMPACT_THREADS) mx_compact_scatter(const uint32_t *flags, uint32_t n,
                                                                         const uint32_t *offsets, uint32_t *idx) {
  __shared__ uint32_t warp_tot[MX_COMPACT_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t run = offsets[blockIdx.x];
  uint32_t base = blockIdx.x * MX_COMPACT_TILE;
  for (int j = 0; j < MX_COMPACT_ITEMS; j++) {
    uint32_t e = base + j * MX_COMPACT_THREADS + threadIdx.x;
    bool good = e < n && (flags[e] & MX_BAD_PHOTON_MASK) == 0;
    uint32_t ball = __ballot_sync(0xffffffffu, good);
    if (lane == 0) warp_tot[warp] = __popc(ball);
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int w = 0; w < MX_COMPACT_THREADS / 32; w++) {
      uint32_t t = warp_tot[w];
      before += (w < warp) ? t : 0;
      total += t;
    }
    if (good) idx[run + before + __popc(ball & ((1u << lane) - 1u))] = e;
    run += total;
    __syncthreads();
  }
}

cudaError_t launch_compact(const uint32_t *flags, uint32_t n, uint32_t *idx_out, uint32_t *scan, uint32_t nblk,
                           cudaStream_t st) {
  mx_compact_count<<<nblk, MX_COMPACT_THREADS, 0, st>>>(flags, n, scan);
  mx_compact_scan<<<1, 1024, 0, st>>>(scan, nblk);
  mx_compact_scatter<<<nblk, MX_COMPACT_THREADS, 0, st>>>(flags, n, scan, idx_out);
  return cudaGetLastError();
}

// ---------------------------------------------------- arithmetic check --
// The trace's own arithmetic helpers evaluated on the device, so that a
// test can hold them to their error bounds: fn 0 rcp_fast (y = 1/x),
// 1 sincospi_fast (y[2i], y[2i+1] = sin, cos of pi x), 2 d2f_rn
// (y = the float nearest x), 3 sine_to_float with amp 1, amp_exp 0
// (y = (float) sin x), 4 f2d of d2f_trunc (y = x truncated to float),
// 5 the Fresnel numerator and denominator in double-float and in double,
// 6 (double) (unsigned) x on the integer pipe, 7 sqrt_fast, 8 quarter_of.
__global__ void __launch_bounds__(256) mx_math_kernel(int fn, const double *x, double *y, size_t n) {
  const size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = fn == 5 ? 0.0 : x[i];
  if (fn == 0) y[i] = mx::rcp_fast(v);
  else if (fn == 1) {
    double sn, cs;
    mx::sincospi_fast(v, &sn, &cs);
    y[2 * i] = sn;
    y[2 * i + 1] = cs;
  } else if (fn == 2) y[i] = (double) mx::d2f_rn(v);
  else if (fn == 3) y[i] = (double) mx::sine_to_float(1.0, 0, v);
  else if (fn == 4) y[i] = mx::f2d(mx::d2f_trunc(v));
  else if (fn == 6) y[i] = mx::u2d(mx::trunc_to_unsigned(v));
  else if (fn == 7) y[i] = mx::sqrt_fast(v);
  else if (fn == 8) y[i] = mx::quarter_of(v);
  else {
    // x: n triples (cos, beta, delta); y: n quadruples, the double-float
    // numerator and denominator, then the double-precision ones
#ifdef __CUDA_ARCH__
    const double c = x[3 * i], b = x[3 * i + 1], d = x[3 * i + 2];
    mx::F2 fn, fd;
    mx::reflectivity_df(c, mx::d2f_trunc(b), mx::d2f_trunc(d), fn, fd);
    double num, den;
    mx::reflectivity_parts(c, b, d, num, den);
    y[4 * i] = mx::df_to(fn); y[4 * i + 1] = mx::df_to(fd);
    y[4 * i + 2] = num; y[4 * i + 3] = den;
#endif
  }
}

cudaError_t math_check(int fn, const double *x, double *y, size_t n) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = (unsigned) ((n + 255) / 256);
  mx_math_kernel<<<blocks, 256>>>(fn, x, y, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e;
}

// ----------------------------------------------------------- FP64 probe --
// Dependent-free DFMA chains: 8 accumulators per thread, so the FP64 pipe
// rather than latency bounds the rate.
__global__ void __launch_bounds__(256) mx_fp64_probe(double *out, int iters, double a, double b) {
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; k++) acc[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) acc[k] = fma(acc[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += acc[k];
  if (s == 1234.5) out[0] = s;   // keeps the chains live
}

cudaError_t probe_fp64(double *tflops, double *ms_out) {
  int dev, sms;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  double *out;
  if ((e = cudaMalloc(&out, sizeof(double))) != cudaSuccess) return e;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, iters = 1 << 14;
  mx_fp64_probe<<<blocks, 256>>>(out, 256, 0.999999, 1e-9);   // warm-up
  cudaEventRecord(a);
  mx_fp64_probe<<<blocks, 256>>>(out, iters, 0.999999, 1e-9);
  cudaEventRecord(b);
  e = cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return e;
  double flops = 2.0 * 8.0 * iters * (double) blocks * 256.0;
  *tflops = flops / (ms * 1e-3) / 1e12;
  if (ms_out) *ms_out = ms;
  return cudaGetLastError();
}
