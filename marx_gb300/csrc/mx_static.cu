// mx_trace_static: the wavefront trace with its survivor queues in a device
// array compiled into the library, so the call itself allocates nothing.
//
// Who needs it: a caller that cannot allocate device memory when it traces,
// for example a host whose GPU memory is entirely reserved by another
// allocator (a framework's caching pool), or a latency-critical loop that
// must not enter the CUDA allocator (cudaMalloc and cudaFree may
// synchronise the device).  mx_trace allocates its queues on first use and
// grows them; this entry point uses the fixed array below instead.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "mx_context.h"

// Two queues of MX_STATIC_MAX_PHOTONS records and the queue counters.  The
// array lives as long as the library is loaded, on every GPU that loads it.
static __device__ __align__(256) unsigned char g_static_scratch[2 * (size_t) MX_STATIC_MAX_PHOTONS * sizeof(MxRec) + 256];

static std::mutex g_static_mu;
static void *g_static_addr[64];   // the array's device address, per device ordinal

// Looked up once per device, with that device current.  Host code cannot
// use g_static_scratch itself: on the host it names a stand-in, not device
// memory.
static int static_scratch(mx_context *c, void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_trace_static");
  if (dev < 0 || dev >= 64) return mx_fail(c, MX_ERANGE, "mx_trace_static: device ordinal above 63");
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return mx_cuda_fail(c, e, "mx_trace_static: locating the static scratch array");
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return MX_OK;
}

extern "C" int mx_trace_static(mx_context *c, const mx_photons *ph, uint32_t stages, const mx_variates *var,
                               uint64_t seed, void *stream) {
  if (!c || !ph) return mx_fail(c, MX_EINVAL, "mx_trace_static: null argument");
  if (ph->n > MX_STATIC_MAX_PHOTONS)
    return mx_fail(c, MX_ERANGE, "mx_trace_static: " + std::to_string(ph->n) + " photons exceed the static scratch (" +
                                     std::to_string(MX_STATIC_MAX_PHOTONS) + "); use mx_trace or smaller lists");
  if (!(stages & MX_STAGE_MIRROR)) return mx_fail(c, MX_EINVAL, "mx_trace_static: stages must include the mirror");
  if (ph->n == 0) return MX_OK;
  if (!ph->x) return mx_fail(c, MX_EINVAL, "mx_trace_static: x is required");
  // the context's tables, overrun counter and launch shape belong to its
  // device; the static array is looked up on the current one
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_trace_static");
  if (dev != c->device)
    return mx_fail(c, MX_EINVAL, "mx_trace_static: the current device (" + std::to_string(dev) +
                                     ") is not the context's (" + std::to_string(c->device) + ")");
  // the same argument checks and photon view as mx_trace
  TraceIO io;
  int r = mx_trace_io(c, c->T, ph, stages, var ? var->U : nullptr, var ? var->N : nullptr, seed, false, io,
                      "mx_trace_static");
  if (r) return r;
  void *scratch = nullptr;
  r = static_scratch(c, &scratch);
  if (r) return r;
  // Every call shares the array, so the queue counters are cleared on the
  // stream before the kernels run (launch_wavefront does it); calls that
  // overlap on the GPU would race on the queues.
  const size_t qbytes = (size_t) MX_STATIC_MAX_PHOTONS * sizeof(MxRec);
  WaveBufs w;
  w.q1 = (MxRec *) scratch;
  w.q2 = (MxRec *) ((char *) scratch + qbytes);
  w.counts = (unsigned int *) ((char *) scratch + 2 * qbytes);
  e = launch_wavefront(c->T, io, w, c->num_sms * c->wave_blocks, (int) c->shared_bytes, (cudaStream_t) stream);
  c->launches += wave_kernels(c->T, stages);
  if (e == cudaSuccess && (stages & MX_STAGE_DETECT) && (c->T.acis_fef || c->T.acis_qe)) {
    e = launch_acis_fef(c->T, io, c->num_sms * 8, (cudaStream_t) stream);
    c->launches++;
  }
  return e == cudaSuccess ? MX_OK : mx_cuda_fail(c, e, "mx_trace_static: launching the trace kernels");
}
