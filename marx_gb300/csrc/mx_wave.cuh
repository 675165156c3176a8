// Device helpers shared by the wavefront and batched kernels: staging of
// the model tables in shared memory, warp-aggregated queue appends and the
// record format between phases.
#pragma once
#include <cuda_runtime.h>

#include "mx_device.cuh"
#include "mx_kernels.cuh"

using namespace mx;

__host__ __device__ static inline size_t align16(size_t x) { return (x + 15) & ~(size_t) 15; }

// Bytes of dynamic shared memory stage_tables fills.
__host__ __device__ static inline size_t tables_shared_bytes(const MxTables &T) {
  (void) T;
  return align16(4 * sizeof(MxShellDev)) + align16(MX_MAX_GRATINGS * sizeof(MxGratingDev)) +
         align16(MX_MAX_CHIPS * sizeof(MxChipDev));
}

__device__ __forceinline__ void copy_words(uint32_t *dst, const uint32_t *src, size_t words) {
  for (size_t k = threadIdx.x; k < words; k += blockDim.x) dst[k] = __ldg(src + k);
}

// Shared-memory layout: shells | gratings | chips | optical-constant and
// correction tables (float) | their interval slopes (double).
__device__ __forceinline__ void stage_tables(const MxTables &T, MxShellDev *&sh, MxGratingDev *&gr, MxChipDev *&ch,
                                             float *&optc, double *&slope) {
  extern __shared__ __align__(16) unsigned char smem[];
  size_t o_gr = align16(4 * sizeof(MxShellDev));
  size_t o_ch = o_gr + align16(MX_MAX_GRATINGS * sizeof(MxGratingDev));
  sh = (MxShellDev *) smem;
  gr = (MxGratingDev *) (smem + o_gr);
  ch = (MxChipDev *) (smem + o_ch);
  optc = (float *) T.optc;
  slope = (double *) T.optc_slope;
  copy_words((uint32_t *) sh, (const uint32_t *) T.shells, 4 * sizeof(MxShellDev) / 4);
  copy_words((uint32_t *) gr, (const uint32_t *) T.gratings, MX_MAX_GRATINGS * sizeof(MxGratingDev) / 4);
  copy_words((uint32_t *) ch, (const uint32_t *) T.chips, MX_MAX_CHIPS * sizeof(MxChipDev) / 4);
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
  r.shell = (uint8_t) q.shell; r.upos = (uint8_t) rng.upos; r.npos = (uint8_t) rng.npos;
  r.overrun = rng.overrun ? 1 : 0;
  r.pdn = m.pdn;
}

__device__ __forceinline__ void from_rec(const MxRec &r, Ph &q, MirrorState &m, Rng &rng, const TraceIO &io) {
  m.x = mk(r.x[0], r.x[1], r.x[2]); m.p = mk(r.p[0], r.p[1], r.p[2]); m.n = mk(r.n[0], r.n[1], r.n[2]);
  m.corr = r.corr; m.beta = r.beta; m.delta = r.delta; m.pdn = r.pdn;
  q.e = r.e; q.t = r.t; q.flags = r.flags; q.shell = r.shell; q.set = 0;
  q.x = m.x; q.p = m.p;
  rng.U = io.U; rng.N = io.N; rng.seed = io.seed; rng.n = io.n; rng.i = r.i; rng.tag = r.tag;
  rng.upos = r.upos; rng.uend = MX_U_MIRROR + 12; rng.npos = r.npos; rng.nend = MX_N_MIRROR + 2;
  rng.overrun = r.overrun != 0;
}

// The photons a grating diffracts, between phases C and D: at the Rowland
// torus in the grating's frame (x, p), with the chosen order index in the
// record's pdn field (n, corr, beta and delta are unused here).
__device__ __forceinline__ void to_rec_d(MxRec &r, D3 x, D3 p, const Ph &q, const Rng &rng, uint32_t i, int chosen) {
  r.x[0] = x.x; r.x[1] = x.y; r.x[2] = x.z;
  r.p[0] = p.x; r.p[1] = p.y; r.p[2] = p.z;
  r.e = q.e; r.t = q.t;
  r.i = i; r.tag = rng.tag; r.flags = q.flags;
  r.shell = (uint8_t) q.shell; r.upos = (uint8_t) rng.upos; r.npos = (uint8_t) rng.npos;
  r.overrun = rng.overrun ? 1 : 0;
  r.pdn = (double) chosen;
}

// x, p, flags and shell of a photon whose trace ends in this phase.
__device__ __forceinline__ void store_core(const TraceIO &io, uint32_t i, const Ph &q, bool overrun) {
  const size_t n = io.stride;   // component stride of the 3-vector columns
  uint32_t f = q.flags;
  if (overrun) { f |= MX_PHOTON_VARIATE_OVERRUN; atomicAdd(io.overrun, 1ull); }
  if (io.x) { io.x[i] = q.x.x; io.x[n + i] = q.x.y; io.x[2 * n + i] = q.x.z; }
  io.p[i] = q.p.x; io.p[n + i] = q.p.y; io.p[2 * n + i] = q.p.z;
  if (io.flags) io.flags[i] = f;
  if (io.shell) io.shell[i] = (int8_t) q.shell;
}


// The LETG and HRC outputs of a photon whose trace ends in this phase: only
// the columns its stages set (the reference leaves the others as they are).
__device__ __forceinline__ void store_extra(const TraceIO &io, uint32_t i, const Ph &q) {
  const size_t n = io.stride;
  if ((q.set & MX_SET_SUPPORT) && io.support)
    for (int k = 0; k < 4; k++) io.support[k * n + i] = q.sup[k];
  if ((q.set & MX_SET_HRC) && io.pha) io.pha[i] = q.pha;
  if ((q.set & MX_SET_REGION) && io.region) io.region[i] = q.region;
  if ((q.set & MX_SET_PI) && io.pi) io.pi[i] = q.pi;
  if (q.set & MX_SET_UV) {
    if (io.upix) io.upix[i] = q.upix;
    if (io.vpix) io.vpix[i] = q.vpix;
  }
}

// Zero the LETG and HRC output columns of photon i (fresh lists).
__device__ __forceinline__ void clear_extra(const TraceIO &io, uint32_t i) {
  const size_t n = io.stride;
  if (io.support) for (int k = 0; k < 4; k++) io.support[k * n + i] = 0;
  if (io.pha) io.pha[i] = 0;
  if (io.region) io.region[i] = 0;
  if (io.pi) io.pi[i] = 0.f;
  if (io.upix) io.upix[i] = 0.f;
  if (io.vpix) io.vpix[i] = 0.f;
}
