// The context object behind the C ABI's opaque mx_context, shared by the
// translation units that implement the ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/marx_gb300.h"
#include "mx_host.h"
#include "mx_kernels.cuh"

struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr; bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, need);
    if (e == cudaSuccess) bytes = need;
    return e;
  }
  void release() { if (ptr) cudaFree(ptr); ptr = nullptr; bytes = 0; }
};

#define MX_PIPE_STREAMS 2
#define MX_PIPE_CHUNKS 16           // nominal chunks: about 2^19 photons each, 4 to 16
#define MX_PIPE_MAX_CHUNKS (MX_PIPE_CHUNKS + 4)   // with the shorter chunks at both ends
#define MX_PIPE_MIN_PHOTONS (1u << 19)
#define MX_SPLIT_MIN_PHOTONS (1u << 18)   // a device trace from here runs in MX_PIPE_STREAMS parts at once

struct mx_context {
  int device = 0;
  int num_sms = 0;
  std::string err;
  mx_config cfg;
  mx::Pack pack;
  mx::HostModel hm;
  MxTables T;              // launch copy with device pointers
  DevBuf tables;           // every table in one allocation
  size_t shared_bytes = 0;
  int trace_blocks[2] = {0, 0};   // resident blocks per SM for the slot / Philox kernels
  cudaStream_t stream = nullptr;
  DevBuf io[22];           // staging for mx_trace_host: 19 columns, U, N
  DevBuf scan;             // compaction block counts
  DevBuf wave;             // wavefront record queues
  DevBuf spec;             // FILE spectrum of the last mx_generate_source call
  int wave_blocks = 0;     // resident blocks per SM for the wavefront kernels
  int mode = MX_MODE_AUTO;
  unsigned long long *d_overrun = nullptr;
  unsigned long long launches = 0;
  // event coordinates (mx_events.cu): tables built on first use per configuration
  bool events_ready = false;
  alignas(16) char ev_geom[2048];   // the launch copy of the facet geometry
  DevBuf ev_tab, ev_scan, ev_io;
  unsigned long long *d_event_bad = nullptr;
  // mx_trace_host on large lists: chunks traced on MX_PIPE_STREAMS streams,
  // copied in on pipe_in and out on pipe_out; pipe_ev[0][j] marks chunk j
  // copied in, pipe_ev[1][j] traced
  cudaStream_t pipe[MX_PIPE_STREAMS] = {};
  DevBuf pipe_wave[MX_PIPE_STREAMS];
  cudaStream_t pipe_in = nullptr, pipe_out = nullptr;
  cudaEvent_t pipe_ev[2][MX_PIPE_MAX_CHUNKS] = {};
  // a device trace cut in parts on the pipe streams: the fork from the
  // caller's stream, then each part's end
  cudaEvent_t split_ev[1 + MX_PIPE_STREAMS] = {};
  // DitherModel FILE: the converted aspect solution (mx_set_aspect_solution)
  DevBuf asp;
  uint32_t asp_n = 0;
  int asp_record_only = 0;
};


// Record an error on the context (or as the creation error when c is null)
// and return code.
int mx_fail(mx_context *c, int code, const std::string &msg);
int mx_cuda_fail(mx_context *c, cudaError_t e, const char *what);
extern thread_local std::string g_create_err;

// mx_trace with an explicit copy of the launch tables (a batch traces each
// source with its own grating and detector choice).  fresh: the output
// columns start from their defaults instead of being read.
extern "C" __attribute__((visibility("hidden"))) int mx_trace_tables(mx_context *c, const MxTables &T, const mx_photons *ph, uint32_t stages,
                               const double *U, const double *N, uint64_t seed, cudaStream_t st, bool fresh);
// The same with the wavefront queues in `queues` instead of the context's
// own; force_wave: the wavefront kernels whatever the list's length (the
// chunks of a list that one pass would trace with them); tag0: the
// generator counter of the list's photon 0 when it has no tag column (a
// chunk starting at photon i0 of a longer list passes i0, so that photon i
// draws as photon i0 + i of the whole list).
__attribute__((visibility("hidden"))) int mx_trace_queues(mx_context *c, const MxTables &T, const mx_photons *ph,
                                                          uint32_t stages, const double *U, const double *N,
                                                          uint64_t seed, cudaStream_t st, bool fresh, DevBuf &queues,
                                                          bool force_wave = false, uint32_t tag0 = 0);

// The checks every trace entry point makes on its arguments, and the kernel
// view of the photon list built from them (who: the entry point's name for
// the messages).  MX_OK, or MX_EINVAL with the reason on the context.
__attribute__((visibility("hidden"))) int mx_trace_io(mx_context *c, const MxTables &T, const mx_photons *ph,
                                                      uint32_t stages, const double *U, const double *N, uint64_t seed,
                                                      bool fresh, TraceIO &io, const char *who);

// The rows of an ASPSOL table converted as the reference's reader converts
// them (mx_source.cpp): out is (n + 1) x 8, row 0 the reader's zero start
// state; times go to out_t (n + 1).
int mx_aspsol_convert(const double *rows, uint32_t n, double ra_nom, double dec_nom, double roll_nom, double tstart,
                      double *out_t, double *out_v);
