// Kernel launch interface shared by the C ABI translation unit.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "mx_model.h"

#define MX_TRACE_BLOCK 256
#define MX_WAVE_BLOCK 256         // threads per block of the wavefront kernels
#define MX_WAVE_MIN_BLOCKS 2     // resident blocks per SM they are compiled for: up to 128 registers, no spills (256 x 3 with 80 registers and 256 x 4, 128 x 5 and 128 x 7 measured no faster)
#define MX_WAVE_KERNELS 4        // kernels of one wavefront trace without a grating (5 with one)
#define MX_COMPACT_THREADS 256
#define MX_COMPACT_ITEMS 16
#define MX_COMPACT_TILE (MX_COMPACT_THREADS * MX_COMPACT_ITEMS)

struct TraceIO {
  double *energy, *x, *p, *t;
  uint32_t *flags, *tag;
  int8_t *shell, *order, *ccd;
  float *ypix, *zpix, *dith;
  float *ddith;                 // detector dither dy, dz, dtheta (3 components), or null
  int8_t *support;              // 4 components (stride): LETG support orders
  int16_t *pha;                 // HRC pulse height
  float *upix, *vpix;           // HRC-S u, v pixels
  uint8_t *region;              // HRC-S shield region
  float *pi;                    // ACIS PI energy (FEF)
  const double *U, *N;          // pre-drawn variates (slot-major) or null
  uint32_t n, stages;
  uint32_t stride;              // component stride of x, p and dither_state (>= n)
  uint32_t tag0;                // generator counter of photon 0 when tag is null (photon i: tag0 + i)
  uint64_t seed;
  int32_t fresh;                // 1: output columns start from their defaults instead of being read
  unsigned long long *overrun;  // count of photons that ran out of variate slots
};

// One photon between wavefront phases (128 bytes, written and read whole).
struct __align__(16) MxRec {
  double x[3], p[3], n[3];      // state at the last conic intersection: incoming direction, blurred normal
  double e, t, corr;
  float beta, delta;
  uint32_t i, tag, flags;       // photon index in the list, generator counter, flags
 uint8_t shell, upos, npos, overrun;   // overrun: a stage already ran past its variate slots
  double pdn;                   // p.n with the blurred normal (reflectivity test passed)
};

// Wavefront scratch: two record queues of n entries and their fill counts.
// Phase A appends to q1, the paraboloid test moves survivors to q2, phase B
// appends to q1 again (its first use is over), phase C reads it and, with a
// grating, appends the photons given an order to q2 for phase D.
struct WaveBufs {
  MxRec *q1, *q2;
  unsigned int *counts;         // [0]: first q1 fill, [1]: q2 fill, [2]: second q1 fill, [3]: second q2 fill
};
// Kernels of one wavefront trace: a, t, b, c and, with a grating stage, d.
__host__ __device__ inline int wave_kernels(const MxTables &T, uint32_t stages) {
  return (T.grating && (stages & MX_STAGE_GRATING)) ? 5 : 4;
}

size_t trace_shared_bytes(const MxTables &T);
cudaError_t wave_occupancy(int shared_bytes, int *blocks_per_sm);
cudaError_t launch_wavefront(const MxTables &T, const TraceIO &io, const WaveBufs &w, int grid, int shared_bytes,
                             cudaStream_t st);
cudaError_t trace_occupancy(bool philox, int shared_bytes, int *blocks_per_sm);
// The ACIS FEF pass over the photons the trace put on a chip (a no-op
// without the chip and pixel columns); seed_dev: the Philox seed in device
// memory instead of io.seed (a captured graph whose seed changes per run).
cudaError_t launch_acis_fef(const MxTables &T, const TraceIO &io, int grid, cudaStream_t st,
                            const uint64_t *seed_dev = nullptr);
cudaError_t launch_trace(const MxTables &T, const TraceIO &io, int grid, int shared_bytes, bool slots,
                         cudaStream_t st);
cudaError_t launch_compact(const uint32_t *flags, uint32_t n, uint32_t *idx_out, uint32_t *scan, uint32_t nblk,
                           cudaStream_t st);
cudaError_t probe_fp64(double *tflops, double *ms);
cudaError_t math_check(int fn, const double *x, double *y, size_t n);
