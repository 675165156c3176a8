// Trace, compaction and probe kernels.
#include <cuda_runtime.h>

#include "mx_device.cuh"
#include "mx_kernels.cuh"

using namespace mx;

__host__ __device__ static inline size_t align16(size_t x) { return (x + 15) & ~(size_t) 15; }

// Shared-memory staging per block: shell geometry, gratings, chips, then
// the optical-constant and correction-factor tables (the per-photon binary
// searches run on these).
size_t trace_shared_bytes(const MxTables &T) {
  return align16(4 * sizeof(MxShellDev)) + align16(4 * sizeof(MxGratingDev)) +
         align16(MX_MAX_CHIPS * sizeof(MxChipDev)) + align16((size_t) T.optc_len * sizeof(float)) +
         align16((size_t) T.slope_len * sizeof(double));
}

__device__ __forceinline__ void copy_words(uint32_t *dst, const uint32_t *src, size_t words) {
  for (size_t k = threadIdx.x; k < words; k += blockDim.x) dst[k] = __ldg(src + k);
}

// Fused dither -> mirror -> grating -> detector trace, one photon per
// thread, grid-stride over the photon list with a resident grid.
__device__ __forceinline__ void stage_tables(const MxTables &T, MxShellDev *&sh, MxGratingDev *&gr, MxChipDev *&ch,
                                             float *&optc, double *&slope);

__global__ void __launch_bounds__(MX_TRACE_BLOCK) mx_trace_kernel(MxTables T, TraceIO io) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);

  const size_t n = io.n;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < io.n; i += stride) {
    Ph q;
    q.e = io.energy[i];
    q.t = io.t ? io.t[i] : 0.0;
    q.p = mk(io.p[i], io.p[n + i], io.p[2 * n + i]);
    q.flags = io.flags ? io.flags[i] : 0u;
    if (io.fresh) {
      q.x = mk(0.0, 0.0, 0.0);
      q.shell = 0; q.order = 0; q.ccd = -1; q.ypix = 0.f; q.zpix = 0.f;
      q.dith[0] = q.dith[1] = q.dith[2] = 0.f;
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
    r.tag = io.tag ? io.tag[i] : i;
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
  }
}

// ------------------------------------------------------------ wavefront --
// The same trace as mx_trace_kernel split at the two conic intersections,
// so that photons lost on the way (between the shells, absorbed by the
// paraboloid) stop occupying SIMT lanes: phase A runs every photon up to
// the paraboloid intersection and appends survivors to queue 1; phase B
// reflects them, intersects the hyperboloid and appends to queue 2; phase
// C reflects from the hyperboloid and runs the grating and the detector.
// Appends are warp-aggregated (one atomic per warp); the order of records
// in a queue does not affect any photon's result.

// Shared-memory layout: shells | gratings | chips | optical-constant and
// correction tables (float) | their interval slopes (double).
__device__ __forceinline__ void stage_tables(const MxTables &T, MxShellDev *&sh, MxGratingDev *&gr, MxChipDev *&ch,
                                             float *&optc, double *&slope) {
  extern __shared__ __align__(16) unsigned char smem[];
  size_t o_gr = align16(4 * sizeof(MxShellDev));
  size_t o_ch = o_gr + align16(4 * sizeof(MxGratingDev));
  size_t o_op = o_ch + align16(MX_MAX_CHIPS * sizeof(MxChipDev));
  size_t o_sl = o_op + align16((size_t) T.optc_len * sizeof(float));
  sh = (MxShellDev *) smem;
  gr = (MxGratingDev *) (smem + o_gr);
  ch = (MxChipDev *) (smem + o_ch);
  optc = (float *) (smem + o_op);
  slope = (double *) (smem + o_sl);
  copy_words((uint32_t *) slope, (const uint32_t *) T.optc_slope, (size_t) T.slope_len * 2);
  copy_words((uint32_t *) sh, (const uint32_t *) T.shells, 4 * sizeof(MxShellDev) / 4);
  copy_words((uint32_t *) gr, (const uint32_t *) T.gratings, 4 * sizeof(MxGratingDev) / 4);
  copy_words((uint32_t *) ch, (const uint32_t *) T.chips, MX_MAX_CHIPS * sizeof(MxChipDev) / 4);
  copy_words((uint32_t *) optc, (const uint32_t *) T.optc, (size_t) T.optc_len);
  __syncthreads();
}

__device__ __forceinline__ void append(bool keep, const MxRec &r, MxRec *q, unsigned int *cnt) {
  const unsigned lane = threadIdx.x & 31;
  unsigned mask = __ballot_sync(0xffffffffu, keep);
  if (mask == 0) return;
  int leader = __ffs(mask) - 1;
  unsigned base = 0;
  if ((int) lane == leader) base = atomicAdd(cnt, (unsigned) __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (keep) q[base + __popc(mask & ((1u << lane) - 1u))] = r;
}

__device__ __forceinline__ void to_rec(MxRec &r, const Ph &q, const MirrorState &m, const Rng &rng, uint32_t i) {
  r.x[0] = m.x.x; r.x[1] = m.x.y; r.x[2] = m.x.z;
  r.p[0] = m.p.x; r.p[1] = m.p.y; r.p[2] = m.p.z;
  r.n[0] = m.n.x; r.n[1] = m.n.y; r.n[2] = m.n.z;
  r.e = q.e; r.t = q.t; r.corr = m.corr; r.beta = m.beta; r.delta = m.delta;
  r.i = i; r.tag = rng.tag; r.flags = q.flags;
  r.shell = (uint8_t) q.shell; r.upos = (uint8_t) rng.upos; r.npos = (uint8_t) rng.npos; r.pad0 = 0;
}

__device__ __forceinline__ void from_rec(const MxRec &r, Ph &q, MirrorState &m, Rng &rng, const TraceIO &io) {
  m.x = mk(r.x[0], r.x[1], r.x[2]); m.p = mk(r.p[0], r.p[1], r.p[2]); m.n = mk(r.n[0], r.n[1], r.n[2]);
  m.corr = r.corr; m.beta = r.beta; m.delta = r.delta;
  q.e = r.e; q.t = r.t; q.flags = r.flags; q.shell = r.shell;
  q.x = m.x; q.p = m.p;
  rng.U = io.U; rng.N = io.N; rng.seed = io.seed; rng.n = io.n; rng.i = r.i; rng.tag = r.tag;
  rng.upos = r.upos; rng.uend = MX_U_MIRROR + 12; rng.npos = r.npos; rng.nend = MX_N_MIRROR + 2;
  rng.overrun = false;
}

// x, p, flags and shell of a photon whose trace ends in this phase.
__device__ __forceinline__ void store_core(const TraceIO &io, uint32_t i, const Ph &q, bool overrun) {
  const size_t n = io.n;
  uint32_t f = q.flags;
  if (overrun) { f |= MX_PHOTON_VARIATE_OVERRUN; atomicAdd(io.overrun, 1ull); }
  if (io.x) { io.x[i] = q.x.x; io.x[n + i] = q.x.y; io.x[2 * n + i] = q.x.z; }
  io.p[i] = q.p.x; io.p[n + i] = q.p.y; io.p[2 * n + i] = q.p.z;
  if (io.flags) io.flags[i] = f;
  if (io.shell) io.shell[i] = (int8_t) q.shell;
}

__global__ void __launch_bounds__(MX_TRACE_BLOCK, 3) mx_wave_a(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const size_t n = io.n;
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
      if (io.fresh) {
        q.x = mk(0.0, 0.0, 0.0); q.shell = 0;
        q.dith[0] = q.dith[1] = q.dith[2] = 0.f;
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
      r.tag = io.tag ? io.tag[i] : i;
      r.upos = r.uend = r.npos = r.nend = 0;
      r.overrun = false;
      if ((io.stages & MX_STAGE_DITHER) && T.dither) dither_stage(T, q, r);
      if (io.dith) for (int k = 0; k < 3; k++) io.dith[k * n + i] = q.dith[k];
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

__global__ void __launch_bounds__(MX_TRACE_BLOCK, 3) mx_wave_b(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const uint32_t count = *(volatile unsigned int *) &w.counts[0];
  const uint32_t lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = warp * 32; base < count; base += nwarps * 32) {
    const uint32_t k = base + lane;
    bool keep = false;
    MxRec rec;
    if (k < count) {
      rec = w.q1[k];
      Ph q; MirrorState m; Rng r;
      from_rec(rec, q, m, r, io);
      if (mirror_middle(T, sh, q, r, m)) {
        keep = true;
        to_rec(rec, q, m, r, rec.i);
      } else
        store_core(io, rec.i, q, r.overrun);
    }
    append(keep, rec, w.q2, &w.counts[1]);
  }
}

__global__ void __launch_bounds__(MX_TRACE_BLOCK) mx_wave_c(MxTables T, TraceIO io, WaveBufs w) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  const uint32_t count = *(volatile unsigned int *) &w.counts[1];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    const MxRec rec = w.q2[k];
    const uint32_t i = rec.i;
    Ph q; MirrorState m; Rng r;
    from_rec(rec, q, m, r, io);
    const int unset = 0x7fff;
    q.order = unset; q.ccd = unset;
    mirror_back(T, sh, q, r, m);
    if (!r.overrun && (io.stages & MX_STAGE_GRATING) && T.grating && !(q.flags & MX_BAD_PHOTON_MASK))
      grating_stage(T, gr, q, r);
    if (!r.overrun && (io.stages & MX_STAGE_DETECT) && T.nchips && !(q.flags & MX_BAD_PHOTON_MASK))
      detect_stage(T, ch + T.chip_off, T.nchips, q, r);
    store_core(io, i, q, r.overrun);
    if (q.order != unset && io.order) io.order[i] = (int8_t) q.order;
    if (q.ccd != unset) {
      if (io.ccd) io.ccd[i] = (int8_t) q.ccd;
      if (q.ccd >= 0) {
        if (io.ypix) io.ypix[i] = q.ypix;
        if (io.zpix) io.zpix[i] = q.zpix;
      }
    }
  }
}

cudaError_t wave_occupancy(int shared_bytes, int *blocks_per_sm) {
  int b[3];
  const void *f[3] = {(const void *) mx_wave_a, (const void *) mx_wave_b, (const void *) mx_wave_c};
  for (int k = 0; k < 3; k++) {
    cudaError_t e = cudaFuncSetAttribute(f[k], cudaFuncAttributeMaxDynamicSharedMemorySize, shared_bytes);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b[k], f[k], MX_TRACE_BLOCK, shared_bytes);
    if (e != cudaSuccess) return e;
  }
  *blocks_per_sm = b[0] < b[1] ? (b[0] < b[2] ? b[0] : b[2]) : (b[1] < b[2] ? b[1] : b[2]);
  return cudaSuccess;
}

cudaError_t launch_wavefront(const MxTables &T, const TraceIO &io, const WaveBufs &w, int grid, int shared_bytes,
                             cudaStream_t st) {
  uint32_t need = (io.n + MX_TRACE_BLOCK - 1) / MX_TRACE_BLOCK;
  int ga = (uint32_t) grid > need ? (int) need : grid;
  if (ga < 1) ga = 1;
  cudaError_t e = cudaMemsetAsync(w.counts, 0, 2 * sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  mx_wave_a<<<ga, MX_TRACE_BLOCK, shared_bytes, st>>>(T, io, w);
  mx_wave_b<<<ga, MX_TRACE_BLOCK, shared_bytes, st>>>(T, io, w);
  mx_wave_c<<<ga, MX_TRACE_BLOCK, shared_bytes, st>>>(T, io, w);
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
