// Kernel launch interface shared by the C ABI translation unit.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "mx_model.h"

#define MX_TRACE_BLOCK 256
#define MX_COMPACT_THREADS 256
#define MX_COMPACT_ITEMS 16
#define MX_COMPACT_TILE (MX_COMPACT_THREADS * MX_COMPACT_ITEMS)

struct TraceIO {
  double *energy, *x, *p, *t;
  uint32_t *flags, *tag;
  int8_t *shell, *order, *ccd;
  float *ypix, *zpix, *dith;
  const double *U, *N;          // pre-drawn variates (slot-major) or null
  uint32_t n, stages;
  uint64_t seed;
  int32_t fresh;                // 1: output columns start from their defaults instead of being read
  unsigned long long *overrun;  // count of photons that ran out of variate slots
};

size_t trace_shared_bytes(const MxTables &T);
cudaError_t trace_occupancy(bool philox, int shared_bytes, int *blocks_per_sm);
cudaError_t launch_trace(const MxTables &T, const TraceIO &io, int grid, int shared_bytes, bool slots,
                         cudaStream_t st);
cudaError_t launch_compact(const uint32_t *flags, uint32_t n, uint32_t *idx_out, uint32_t *scan, uint32_t nblk,
                           cudaStream_t st);
cudaError_t probe_fp64(double *tflops, double *ms);
