// Point-source generation and the batched form: many sources traced by one
// persistent cooperative kernel replayed from a CUDA graph, its launch
// shape chosen by a timing autotuner.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "mx_context.h"
#include "mx_wave.cuh"

namespace cg = cooperative_groups;

// One source as the kernels read it.
struct MxSourceDev {
  double p[3], pn[3];       // direction of travel; the normal to it in the x-y plane (source.c:206-209)
  double emin, de;          // FLAT: energy = emin + de * u
  double a, b, c;           // GAUSS: a = sigma; BETA: a = core radius, b = 1 / (1 - alpha);
                            // DISK: a = theta1, b = (theta0/theta1)^2, c = 1 - b; LINE: a = theta, b, c = cos, sin phi
  double axis[3], cos_al, sin_al;   // LINE: rotation from -x to p (JDMv_find_rotation_axis)
  int32_t kind, spec_off;   // MX_SOURCE_*; FILE spectrum rows [spec_off, spec_off + spec_n) of the table
  int32_t spec_n;           // 0: FLAT
  int32_t grating;          // 1: HETG
  int32_t chip_off, nchips; // chips[chip_off .. chip_off + nchips)
  int32_t img_off, img_nx;  // IMAGE: cumulative distribution rows [img_off, img_off + nx * ny) of the table
  int32_t img_ny, pad[3];   //        (a, b: radians per pixel along x and y; axis, cos_al, sin_al: the rotation)
};
static_assert(sizeof(MxSourceDev) % 16 == 0, "source record size");

#define MX_BATCH_MAX_SOURCES 4096

struct BatchIO {
  TraceIO io;                   // the batch's photon list (n = all photons), fresh outputs
  const MxSourceDev *src;
  const uint32_t *start;        // nsrc + 1 offsets
  int32_t nsrc, tile;
  MxRec *q1, *q2;
  unsigned int *ctr;            // [0] q1 entries [1] q2 entries [2..4] work counters of phases A, B, C
                                // [5] q1 entries of phase B (q1 reused) [6] work counter of phase T
                                // [7] q2 entries of phase C (q2 reused) [8] work counter of phase D
  const uint64_t *seed;         // device scalar, written before each graph launch
  const double *spec;           // FILE spectra of the sources (energies then cumulative flux, per source)
};

// JDMinterpolate_d (dinterpo.c:52-82) of the inverse cumulative spectrum:
// energies at spec[0..n), normalised cumulative flux at spec[n..2n).
__device__ double interp_d(double x, const double *xp, const double *yp, unsigned n) {
  if (n == 1) return __ldg(yp);
  unsigned n1 = bsearch_d(x, xp, n), n0 = n1 - 1;
  if (n1 < n && x == __ldg(xp + n1)) return __ldg(yp + n1);
  if (n1 == n) { n1--; n0--; }
  if (n1 == 0) n0 = 1;
  double x0 = __ldg(xp + n0), x1 = __ldg(xp + n1);
  if (x1 == x0) return __ldg(yp + n1);
  double y0 = __ldg(yp + n0), y1 = __ldg(yp + n1);
  return MX_DADD(y0, MX_DMUL(MX_DDIV(MX_DADD(y1, -y0), MX_DADD(x1, -x0)), MX_DADD(x, -x0)));
}

// JDMbinary_search_f (finterpo.c:37-57) over single-precision values held in
// the double table: the same bisection and comparisons.
__device__ __forceinline__ unsigned bsearch_cdf(float x, const double *xp, unsigned n) {
  unsigned n0 = 0, n1 = n;
  while (n1 > n0 + 1) {
    unsigned n2 = (n0 + n1) / 2;
    const float v = (float) __ldg(xp + n2);
    if (v >= x) {
      if (v == x) return n2;
      n1 = n2;
    } else
      n0 = n2;
  }
  if (x >= (float) __ldg(xp + n0)) return n1;
  return n0;
}

// The create_photons function of the source's model for one photon:
// point_create_photons (s-point.c:59), gauss_create_photons
// (s-gauss.c:76-130), beta_create_photons (s-beta.c:74-120),
// disk_create_photons (s-disk.c:63-105), line_create_photons
// (s-line.c:64-100), with flat_energy or file_energy (spectrum.c:138-190)
// first.  Source-domain draw 0 is the energy; the model's draws follow in
// the reference's order.  GAUSS, BETA and DISK rotate the source's fixed
// normal by each photon's own azimuth (the reference carries the rotated
// normal from one photon to the next; each photon's azimuth is uniform
// either way).
__device__ __forceinline__ void generate_photon(const MxSourceDev &S, const double *spec, uint64_t seed, uint32_t tag,
                                                Ph &q) {
  if (S.spec_n > 0) {
    const double *e = spec + S.spec_off, *cum = e + S.spec_n;
    q.e = interp_d(source_uniform(seed, tag, 0), cum, e, (unsigned) S.spec_n);
  } else
    q.e = MX_DADD(S.emin, MX_DMUL(S.de, source_uniform(seed, tag, 0)));   // rounded as written, no contraction
  const D3 p = mk(S.p[0], S.p[1], S.p[2]);
  if (S.kind == MX_SOURCE_POINT) q.p = p;
  else if (S.kind == MX_SOURCE_IMAGE) {
    // image_create_photons (s-image.c:290-350): a pixel by the image's
    // cumulative distribution, a uniform position in it, about the centre
    const unsigned n = (unsigned) S.img_nx * (unsigned) S.img_ny;
    const unsigned ofs = bsearch_cdf((float) source_uniform(seed, tag, 1), spec + S.img_off, n);
    double y = (double) (ofs / (unsigned) S.img_nx);
    double x = (double) (ofs % (unsigned) S.img_nx);
    y = MX_DADD(y, MX_DADD(MX_DMUL(-0.5, (double) S.img_ny), MX_DADD(source_uniform(seed, tag, 2), -0.5)));
    x = MX_DADD(x, MX_DADD(MX_DMUL(-0.5, (double) S.img_nx), MX_DADD(source_uniform(seed, tag, 3), -0.5)));
    y = MX_DMUL(y, S.b);
    x = MX_DMUL(x, S.a);
    double sy, cy, sx, cx;
    sincos(y, &sy, &cy);
    sincos(x, &sx, &cx);
    q.p = rotate_unit(mk(-cy * cx, cy * sx, -sy), mk(S.axis[0], S.axis[1], S.axis[2]), S.cos_al, S.sin_al);
  }
  else if (S.kind == MX_SOURCE_LINE) {
    double theta = S.a * (-1.0 + 2.0 * source_uniform(seed, tag, 1));
    double st, ct;
    sincos(theta, &st, &ct);
    double sin_theta = -st;
    D3 p0 = mk(-ct, sin_theta * S.b, sin_theta * S.c);
    q.p = rotate_unit(p0, mk(S.axis[0], S.axis[1], S.axis[2]), S.cos_al, S.sin_al);
  } else {
    double sphi, cphi;
    sincos(2.0 * PI * source_uniform(seed, tag, 1), &sphi, &cphi);
    D3 normal = rotate_unit(mk(S.pn[0], S.pn[1], S.pn[2]), p, cphi, sphi);
    double ang;
    if (S.kind == MX_SOURCE_DISK)
      ang = S.a * sqrt(S.b + S.c * source_uniform(seed, tag, 2));
    else {
      double rnd = source_uniform(seed, tag, 2);
      for (uint32_t k = 3; rnd == 0.0 && k < 8; k++) rnd = source_uniform(seed, tag, k);
      ang = S.kind == MX_SOURCE_GAUSS ? S.a * sqrt(-log(rnd)) : S.a * sqrt(pow(rnd, S.b) - 1.0);
    }
    double sa, ca;
    sincos(ang, &sa, &ca);
    q.p = rotate_unit(p, normal, ca, sa);
  }
  q.t = 0.0;
  q.x = mk(0.0, 0.0, 0.0);
  q.flags = 0u;
  q.shell = 0; q.order = 0; q.ccd = -1; q.ypix = q.zpix = 0.f;
  q.dith[0] = q.dith[1] = q.dith[2] = 0.f;
  q.set = 0;
  for (int k = 0; k < 4; k++) q.sup[k] = 0;
}

__global__ void __launch_bounds__(256) mx_generate_kernel(MxSourceDev S, const double *spec, uint32_t first_tag,
                                                           uint64_t seed, double *energy, double *p, double *t,
                                                           uint32_t *flags, uint32_t *tag, uint32_t n, uint32_t stride) {
  const size_t nn = stride;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    Ph q;
    generate_photon(S, spec, seed, first_tag + k, q);
    energy[k] = q.e;
    p[k] = q.p.x; p[nn + k] = q.p.y; p[2 * nn + k] = q.p.z;
    if (t) t[k] = 0.0;
    if (flags) flags[k] = 0u;
    if (tag) tag[k] = first_tag + k;
  }
}

// A warp's claim of `tile` consecutive work items from a global counter.
__device__ __forceinline__ uint32_t claim(unsigned int *ctr, int tile) {
  unsigned base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(ctr, (unsigned) tile);
  return __shfl_sync(0xffffffffu, base, 0);
}

__device__ __forceinline__ int source_of(uint32_t i, const uint32_t *start, int nsrc) {
  int lo = 0, hi = nsrc;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (start[mid] <= i) lo = mid; else hi = mid;
  }
  return lo;
}

// The end of a photon in phases C and D: the source's detector (when the
// photon is still good), then the output columns.
__device__ __forceinline__ void batch_finish(const MxTables &T, const MxChipDev *ch, const MxSourceDev &S,
                                             const TraceIO &io, uint32_t i, Ph &q, Rng &r) {
  const int unset = 0x7fff;
  if (!r.overrun && S.nchips && !(q.flags & MX_BAD_PHOTON_MASK)) detect_stage(T, ch + S.chip_off, S.nchips, q, r);
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

// The whole batch in one persistent cooperative launch.  The five phases
// of the wavefront trace (A, T, B, C and the gratings' D) are separated by
// grid-wide barriers; inside a
// phase warps claim tiles of work from a counter, so uneven sources and
// uneven survivor counts spread over every SM.  Every thread reaches every
// barrier: the claim loops end for a whole warp at once and nothing
// returns early.  Compiled for three resident blocks of 256 threads per SM
// (80 registers; about 250 bytes per thread spill to local memory): the
// autotuner picks three blocks per SM then, 2 % faster than two blocks of
// 128 registers on the 256-source batch.
__global__ void __launch_bounds__(256, 3) mx_batch_kernel(MxTables T, BatchIO b) {
  MxShellDev *sh; MxGratingDev *gr; MxChipDev *ch; float *optc; double *slope;
  stage_tables(T, sh, gr, ch, optc, slope);
  extern __shared__ __align__(16) unsigned char smem[];
  MxSourceDev *ssrc = (MxSourceDev *) (smem + tables_shared_bytes(T));
  uint32_t *sstart = (uint32_t *) (ssrc + b.nsrc);
  copy_words((uint32_t *) ssrc, (const uint32_t *) b.src, (size_t) b.nsrc * sizeof(MxSourceDev) / 4);
  copy_words(sstart, b.start, (size_t) b.nsrc + 1);
  __syncthreads();

  cg::grid_group grid = cg::this_grid();
  const uint64_t seed = *b.seed;
  TraceIO io = b.io;
  io.seed = seed;
  const size_t n = io.stride;   // component stride of the 3-vector columns
  const uint32_t lane = threadIdx.x & 31;

  // Phase A: generation, dither, aperture, paraboloid intersection.
  for (;;) {
    const uint32_t base = claim(&b.ctr[2], b.tile);
    if (base >= io.n) break;
    const uint32_t end = min(base + (uint32_t) b.tile, io.n);
    for (uint32_t j = base; j < end; j += 32) {
      const uint32_t i = j + lane;
      bool keep = false;
      MxRec rec;
      if (i < end) {
        const int s = source_of(i, sstart, b.nsrc);
        Ph q;
        generate_photon(ssrc[s], b.spec, seed, i, q);
        clear_extra(io, i);
        io.energy[i] = q.e;
        if (io.t) io.t[i] = 0.0;
        if (io.tag) io.tag[i] = i;
        if (io.order) io.order[i] = 0;
        if (io.ccd) io.ccd[i] = -1;
        if (io.ypix) io.ypix[i] = 0.f;
        if (io.zpix) io.zpix[i] = 0.f;
        Rng r;
        r.U = nullptr; r.N = nullptr; r.seed = seed; r.n = io.n; r.i = i; r.tag = i;
        r.upos = r.uend = r.npos = r.nend = 0;
        r.overrun = false;
        if (T.dither) dither_stage(T, q, r);
        if (io.dith) for (int k = 0; k < 3; k++) io.dith[k * n + i] = q.dith[k];
        MirrorState m;
        if (mirror_front(T, sh, optc, slope, q, r, m)) {
          keep = true;
          to_rec(rec, q, m, r, i);
        } else
          store_core(io, i, q, r.overrun);
      }
      append(keep, rec, b.q1, &b.ctr[0]);
    }
  }
  grid.sync();

  // Phase T: the paraboloid's normal blur and reflectivity test.
  const uint32_t nt = __ldcg(&b.ctr[0]);
  for (;;) {
    const uint32_t base = claim(&b.ctr[6], b.tile);
    if (base >= nt) break;
    const uint32_t end = min(base + (uint32_t) b.tile, nt);
    for (uint32_t j = base; j < end; j += 32) {
      const uint32_t k = j + lane;
      bool keep = false;
      MxRec rec;
      if (k < end) {
        rec = b.q1[k];
        Ph q; MirrorState m; Rng r;
        from_rec(rec, q, m, r, io);
        if (mirror_ptest(T, sh, q, r, m)) {
          keep = true;
          to_rec(rec, q, m, r, rec.i);
        } else
          store_core(io, rec.i, q, r.overrun);
      }
      append(keep, rec, b.q2, &b.ctr[1]);
    }
  }
  grid.sync();

  // Phase B: the rest of the paraboloid reflection, hyperboloid
  // intersection and reflectivity test (q1 is free again).
  const uint32_t nb = __ldcg(&b.ctr[1]);
  for (;;) {
    const uint32_t base = claim(&b.ctr[3], b.tile);
    if (base >= nb) break;
    const uint32_t end = min(base + (uint32_t) b.tile, nb);
    for (uint32_t j = base; j < end; j += 32) {
      const uint32_t k = j + lane;
      bool keep = false;
      MxRec rec;
      if (k < end) {
        rec = b.q2[k];
        Ph q; MirrorState m; Rng r;
        from_rec(rec, q, m, r, io);
        if (mirror_middle(T, sh, q, r, m)) {
          keep = true;
          to_rec(rec, q, m, r, rec.i);
        } else
          store_core(io, rec.i, q, r.overrun);
      }
      append(keep, rec, b.q1, &b.ctr[5]);
    }
  }
  grid.sync();

  // Phase C: hyperboloid reflection, the source's grating up to its order
  // choice; the photons given an order go on to phase D (q2 is free again),
  // the others run the detector (without a grating) and are stored.
  const uint32_t nc = __ldcg(&b.ctr[5]);
  for (;;) {
    const uint32_t base = claim(&b.ctr[4], b.tile);
    if (base >= nc) break;
    const uint32_t end = min(base + (uint32_t) b.tile, nc);
    for (uint32_t j = base; j < end; j += 32) {
      const uint32_t k = j + lane;
      bool to_d = false;
      MxRec rec;
      if (k < end) {
        rec = b.q1[k];
        const MxSourceDev &S = ssrc[source_of(rec.i, sstart, b.nsrc)];
        const uint32_t i = rec.i;
        Ph q; MirrorState m; Rng r;
        from_rec(rec, q, m, r, io);
        const int unset = 0x7fff;
        q.order = unset; q.ccd = unset;
        mirror_back(T, sh, q, r, m);
        if (!r.overrun && S.grating && !(q.flags & MX_BAD_PHOTON_MASK)) {
          D3 gx, gp;
          const int chosen = grating_front(T, gr, S.grating, q, r, gx, gp);
          if (chosen >= 0) {
            to_d = true;
            to_rec_d(rec, gx, gp, q, r, i, chosen);
          }
        }
        if (!to_d) batch_finish(T, ch, S, io, i, q, r);
      }
      append(to_d, rec, b.q2, &b.ctr[7]);
    }
  }
  grid.sync();

  // Phase D: the diffraction into the chosen order, the detector, the
  // output columns.
  const uint32_t nd = __ldcg(&b.ctr[7]);
  for (;;) {
    const uint32_t base = claim(&b.ctr[8], b.tile);
    if (base >= nd) break;
    const uint32_t end = min(base + (uint32_t) b.tile, nd);
    for (uint32_t k = base + lane; k < end; k += 32) {
      const MxRec rec = b.q2[k];
      const uint32_t i = rec.i;
      const MxSourceDev &S = ssrc[source_of(i, sstart, b.nsrc)];
      Ph q;
      q.e = rec.e; q.t = rec.t; q.flags = rec.flags; q.shell = rec.shell; q.set = 0;
      q.ccd = 0x7fff;
      Rng r;
      r.U = nullptr; r.N = nullptr; r.seed = seed; r.n = io.n; r.i = i; r.tag = rec.tag;
      if (S.grating == MX_GRATING_LETG) r.window(MX_U_LETG, 6, MX_N_LETG, 10);
      else r.window(MX_U_GRATING, 2, MX_N_GRATING, 2);
      r.upos = rec.upos; r.npos = rec.npos; r.overrun = rec.overrun != 0;
      const int chosen = (int) rec.pdn;
      q.order = chosen - gr[(S.grating == MX_GRATING_LETG ? 4 : 0) + q.shell].max_order;
      grating_back(T, gr, S.grating, q, r, mk(rec.x[0], rec.x[1], rec.x[2]), mk(rec.p[0], rec.p[1], rec.p[2]), chosen);
      batch_finish(T, ch, S, io, i, q, r);
    }
  }
}

// ------------------------------------------------------------------ host --
struct mx_batch {
  mx_context *ctx = nullptr;
  std::vector<mx_source> src;
  std::vector<MxSourceDev> dsrc;
  std::vector<double> spec;     // FILE spectra of the sources (host copy)
  DevBuf d_spec;
  std::vector<uint32_t> start;
  uint64_t total = 0;
  DevBuf d_src;                 // sources then starts
  DevBuf cols[12];              // photon list columns
  DevBuf queues;                // two record queues
  DevBuf ctr;                   // 9 counters, the seed at byte 64
  uint64_t *h_seed = nullptr;   // pinned, copied into the graph's seed slot
  mx_batch_params params;
  bool have_params = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  size_t shared_bytes = 0;
  std::string key;
};

static mx_photons batch_view(mx_batch *b) {
  mx_photons d;
  memset(&d, 0, sizeof(d));
  d.n = (uint32_t) b->total;
  d.energy = (double *) b->cols[0].ptr; d.x = (double *) b->cols[1].ptr; d.p = (double *) b->cols[2].ptr;
  d.arrival_time = (double *) b->cols[3].ptr; d.flags = (uint32_t *) b->cols[4].ptr; d.tag = (uint32_t *) b->cols[5].ptr;
  d.mirror_shell = (int8_t *) b->cols[6].ptr; d.order = (int8_t *) b->cols[7].ptr; d.ccd_num = (int8_t *) b->cols[8].ptr;
  d.y_pixel = (float *) b->cols[9].ptr; d.z_pixel = (float *) b->cols[10].ptr; d.dither_state = (float *) b->cols[11].ptr;
  return d;
}

static int batch_max_blocks(mx_batch *b, int block, int *blocks) {
  cudaError_t e = cudaFuncSetAttribute(mx_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) b->shared_bytes);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, mx_batch_kernel, block, b->shared_bytes);
  if (e != cudaSuccess) return mx_cuda_fail(b->ctx, e, "batch occupancy");
  return MX_OK;
}

static void drop_graph(mx_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr; b->graph = nullptr;
}

// Capture counter reset, seed upload and the cooperative kernel as a graph.
static int build_graph(mx_batch *b) {
  mx_context *c = b->ctx;
  drop_graph(b);
  int maxb = 0;
  int r = batch_max_blocks(b, b->params.block, &maxb);
  if (r) return r;
  if (maxb < 1) return mx_fail(c, MX_ERANGE, "batch kernel cannot be resident");
  int per_sm = std::min(std::max(1, b->params.blocks_per_sm), maxb);
  mx_photons d = batch_view(b);
  BatchIO io;
  memset(&io, 0, sizeof(io));
  io.io.energy = d.energy; io.io.x = d.x; io.io.p = d.p; io.io.t = d.arrival_time; io.io.flags = d.flags;
  io.io.tag = d.tag; io.io.shell = d.mirror_shell; io.io.order = d.order; io.io.ccd = d.ccd_num;
  io.io.ypix = d.y_pixel; io.io.zpix = d.z_pixel; io.io.dith = d.dither_state;
  io.io.support = d.support_orders; io.io.pha = d.pulse_height; io.io.upix = d.u_pixel; io.io.vpix = d.v_pixel;
  io.io.region = d.detector_region;
  io.io.pi = d.pi;
  io.io.U = nullptr; io.io.N = nullptr; io.io.n = d.n; io.io.stride = d.n; io.io.stages = MX_STAGE_ALL; io.io.fresh = 1;
  io.io.overrun = c->d_overrun;
  io.src = (const MxSourceDev *) b->d_src.ptr;
  io.start = (const uint32_t *) ((const char *) b->d_src.ptr + b->dsrc.size() * sizeof(MxSourceDev));
  io.nsrc = (int32_t) b->dsrc.size();
  io.tile = b->params.tile;
  size_t qbytes = (size_t) b->total * sizeof(MxRec);
  io.q1 = (MxRec *) b->queues.ptr;
  io.q2 = (MxRec *) ((char *) b->queues.ptr + qbytes);
  io.ctr = (unsigned int *) b->ctr.ptr;
  io.spec = (const double *) b->d_spec.ptr;
  io.seed = (const uint64_t *) ((char *) b->ctr.ptr + 64);
  MxTables T = c->T;

  cudaStream_t st;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "batch capture stream");
  e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->ctr.ptr, 0, 9 * sizeof(unsigned int), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync((char *) b->ctr.ptr + 64, b->h_seed, sizeof(uint64_t), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3(c->num_sms * per_sm);
    lc.blockDim = dim3(b->params.block);
    lc.dynamicSmemBytes = b->shared_bytes;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    e = cudaLaunchKernelEx(&lc, mx_batch_kernel, T, io);
  }
  // with an FEF: the pulse heights and streaks of the photons on a chip
  if (e == cudaSuccess && (T.acis_fef || T.acis_qe)) e = launch_acis_fef(T, io.io, c->num_sms * 8, st, io.seed);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(st, &g);
  cudaStreamDestroy(st);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    b->exec = nullptr;
    return mx_cuda_fail(c, e, "capturing the batch graph");
  }
  b->graph = g;
  return MX_OK;
}

static std::string batch_key(mx_batch *b) {
  // FNV-1a over the configuration, the source table and the device
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void *p, size_t nbytes) {
    const unsigned char *q = (const unsigned char *) p;
    for (size_t k = 0; k < nbytes; k++) { h ^= q[k]; h *= 1099511628211ull; }
  };
  mix(&b->ctx->cfg, sizeof(mx_config));
  mix(b->src.data(), b->src.size() * sizeof(mx_source));
  mix(&b->ctx->num_sms, sizeof(int));
  char buf[32];
  snprintf(buf, sizeof(buf), "%016llx", (unsigned long long) h);
  return buf;
}

// ------------------------------------------------------ source set-up --
static double src_len(const double a[3]) {   // JDMv_length (vector.c:77)
  double x = fabs(a[0]), y = fabs(a[1]), z = fabs(a[2]), t;
  if (z < x) { t = z; z = x; x = t; }
  if (z < y) { t = z; z = y; y = t; }
  if (z == 0.0) return 0.0;
  x = x / z; y = y / z;
  return z * sqrt(1.0 + x * x + y * y);
}

// The per-source constants of the source models' set-up (select_source,
// source.c:136-232; gauss/beta/disk/line select functions; the spectrum
// set-up of spectrum.c:145-274).  FILE spectra are appended to spec as
// energies then normalised cumulative flux (compute_cumulated_vector,
// spectrum.c:40-97).
static bool source_dev(const mx_source &q, MxSourceDev &S, std::vector<double> &spec, std::string &err) {
  const double PI_ = 3.14159265358979323846264338327950288;
  memset(&S, 0, sizeof(S));
  for (int k = 0; k < 3; k++) S.p[k] = q.p[k];
  if (!(q.p[0] < 0.0)) { err = "source direction must travel toward the mirror (p.x < 0)"; return false; }
  // the normal to the unnegated direction u = -p in the x-y plane
  double u[3] = {-q.p[0], -q.p[1], -q.p[2]};
  double pn[3] = {-u[1] / u[0], 1.0, 0.0};
  double l = src_len(pn);
  if (l != 0.0) { pn[0] = pn[0] / l; pn[1] = pn[1] / l; pn[2] = pn[2] / l; }
  for (int k = 0; k < 3; k++) S.pn[k] = pn[k];
  S.kind = q.kind;
  if (q.spectrum_n > 0) {
    if (!q.spectrum_energy || !q.spectrum_flux) { err = "FILE spectrum arrays missing"; return false; }
    const unsigned n = q.spectrum_n;
    std::vector<double> cum(n);
    double tot = 0.0, prev = q.spectrum_energy[0];
    for (unsigned i = 0; i < n; i++) {
      double x = q.spectrum_energy[i];
      if (x - prev < 0.0) { err = "Your file spectrum appears corrupt.  Perhaps you are using a wavelength grid"; return false; }
      tot += q.spectrum_flux[i] * (x - prev);
      cum[i] = tot;
      prev = x;
    }
    if (tot == 0.0) { err = "Your file spectrum seems to have zero flux in it"; return false; }
    for (unsigned i = 0; i < n; i++) cum[i] = cum[i] / tot;
    S.spec_off = (int32_t) spec.size();
    S.spec_n = (int32_t) n;
    spec.insert(spec.end(), q.spectrum_energy, q.spectrum_energy + n);
    spec.insert(spec.end(), cum.begin(), cum.end());
  } else {
    if (!(q.energy_max >= q.energy_min) || !(q.energy_min > 0)) { err = "need 0 < energy_min <= energy_max"; return false; }
    S.emin = q.energy_min; S.de = q.energy_max - q.energy_min;
  }
  const double arcsec = 1.0 / 3600.0 * PI_ / 180.0;
  switch (q.kind) {
    case MX_SOURCE_POINT: break;
    case MX_SOURCE_GAUSS: S.a = q.param[0] * arcsec; break;
    case MX_SOURCE_BETA: {
      double alpha = 3 * q.param[1] - 0.5;
      if ((alpha <= 1.0) || (q.param[0] <= 0.0)) { err = "Beta parameters out of range.  Must be greater than 1/2."; return false; }
      S.a = q.param[0] * (1.0 / 3600.0) * (PI_ / 180.0);
      S.b = 1.0 / (1.0 - alpha);
      break;
    }
    case MX_SOURCE_DISK: {
      double th = q.param[1] * arcsec, th0 = q.param[0] * arcsec;
      double x0 = th0 / th;
      x0 = x0 * x0;
      S.a = th; S.b = x0; S.c = 1.0 - x0;
      break;
    }
    case MX_SOURCE_LINE: {
      double phi = q.param[0] * (PI_ / 180.0);
      S.a = q.param[1] * arcsec;
      S.b = cos(phi); S.c = sin(phi);
      // JDMv_find_rotation_axis ((-1, 0, 0), p) (vector.c:289-330)
      double a[3] = {-1.0, 0.0, 0.0};
      double th = a[0] * q.p[0] + a[1] * q.p[1] + a[2] * q.p[2];
      if (fabs(th) > 1.0) th = th > 1.0 ? 1.0 : -1.0;
      th = acos(th);
      double cc[3] = {a[1] * q.p[2] - a[2] * q.p[1], a[2] * q.p[0] - a[0] * q.p[2], a[0] * q.p[1] - a[1] * q.p[0]};
      double len = src_len(cc);
      if (len > 0.0) { for (int k = 0; k < 3; k++) S.axis[k] = cc[k] / len; }
      else { S.axis[0] = -a[1]; S.axis[1] = -a[0]; S.axis[2] = 0.0; }
      S.cos_al = cos(th); S.sin_al = sin(th);
      break;
    }
    case MX_SOURCE_IMAGE: {
      // read_image (s-image.c:46-148): a float image, its running double sum
      // stored back as float, then each entry divided by the total
      if (!q.image || q.image_nx == 0 || q.image_ny == 0) { err = "IMAGE source without an image"; return false; }
      const size_t n = (size_t) q.image_nx * q.image_ny;
      if (n > (size_t) 1 << 30) { err = "image too large"; return false; }
      std::vector<float> cdf(n);
      double sum = 0;
      for (size_t i = 0; i < n; i++) {
        sum += (double) q.image[i];
        cdf[i] = (float) sum;
      }
      if (!(sum > 0.0)) { err = "IMAGE source with no positive flux"; return false; }
      S.img_off = (int32_t) spec.size();
      S.img_nx = (int32_t) q.image_nx;
      S.img_ny = (int32_t) q.image_ny;
      for (size_t i = 0; i < n; i++) spec.push_back((double) (float) (cdf[i] / sum));
      // open_image_fits_file (s-image.c:190-232): 0.5 arcsec when no scale is given
      double s1 = fabs(q.param[0]), s2 = fabs(q.param[1]);
      if (s1 == 0.0 || s2 == 0.0) s1 = s2 = 0.5 / 3600.0;
      S.a = s1 * PI_ / 180.0;
      S.b = s2 * PI_ / 180.0;
      // the rotation of (-1, 0, 0) into p (s-image.c:297-318)
      double th = -1.0 * q.p[0] + 0.0 * q.p[1] + 0.0 * q.p[2];
      if (fabs(th) > 1.0) th = th < 0 ? -1.0 : 1.0;
      th = acos(th);
      double nrm[3] = {0.0 * q.p[2] - 0.0 * q.p[1], 0.0 * q.p[0] - -1.0 * q.p[2], -1.0 * q.p[1] - 0.0 * q.p[0]};
      if (th != 0.0) {
        double l = src_len(nrm);
        if (l != 0.0) for (int k = 0; k < 3; k++) nrm[k] = nrm[k] / l;
      }
      for (int k = 0; k < 3; k++) S.axis[k] = nrm[k];
      S.cos_al = cos(th); S.sin_al = sin(th);
      break;
    }
    default: err = "unknown source model"; return false;
  }
  return true;
}

static std::mutex g_tune_mu;
static std::map<std::string, mx_batch_params> g_tune_cache;

extern "C" {

int mx_generate_source(mx_context *c, const mx_source *s, uint32_t first_tag, uint64_t seed, const mx_photons *d,
                       void *stream) {
  if (!c || !s || !d) return mx_fail(c, MX_EINVAL, "mx_generate_source: null argument");
  if (d->n == 0) return MX_OK;
  if (!d->energy || !d->p) return mx_fail(c, MX_EINVAL, "mx_generate_source: energy and p are required");
  MxSourceDev S;
  std::vector<double> spec;
  std::string err;
  if (!source_dev(*s, S, spec, err)) return mx_fail(c, MX_EINVAL, "mx_generate_source: " + err);
  const double *dspec = nullptr;
  if (!spec.empty()) {
    cudaError_t e = c->spec.ensure(spec.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(c->spec.ptr, spec.data(), spec.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_generate_source: uploading the spectrum");
    dspec = (const double *) c->spec.ptr;
  }
  int grid = std::max(1, std::min((int) ((d->n + 255) / 256), c->num_sms * 8));
  uint32_t stride = d->stride ? d->stride : d->n;
  if (stride < d->n) return mx_fail(c, MX_EINVAL, "mx_generate_source: stride below n");
  mx_generate_kernel<<<grid, 256, 0, (cudaStream_t) stream>>>(S, dspec, first_tag, seed, d->energy, d->p,
                                                              d->arrival_time, d->flags, d->tag, d->n, stride);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MX_OK : mx_cuda_fail(c, e, "launching photon generation");
}

mx_batch *mx_batch_create(mx_context *c, const mx_source *sources, int nsrc) {
  if (!c || !sources || nsrc <= 0) { g_create_err = "mx_batch_create: need a context and at least one source"; return nullptr; }
  if (nsrc > MX_BATCH_MAX_SOURCES) { g_create_err = "mx_batch_create: too many sources"; return nullptr; }
  mx_batch *b = new mx_batch();
  b->ctx = c;
  b->src.assign(sources, sources + nsrc);
  b->start.push_back(0);
  uint64_t tot = 0;
  for (int s = 0; s < nsrc; s++) {
    const mx_source &q = sources[s];
    MxSourceDev S;
    std::string err;
    if ((q.grating != MX_GRATING_NONE && q.grating != MX_GRATING_HETG) ||
        (q.detector != MX_DETECTOR_ACIS_I && q.detector != MX_DETECTOR_ACIS_S) || !source_dev(q, S, b->spec, err)) {
      g_create_err = "mx_batch_create: source " + std::to_string(s) + " is malformed" + (err.empty() ? "" : ": " + err);
      delete b;
      return nullptr;
    }
    S.grating = q.grating == MX_GRATING_HETG;
    S.chip_off = q.detector == MX_DETECTOR_ACIS_S ? 4 : 0;
    S.nchips = q.detector == MX_DETECTOR_ACIS_S ? 6 : 4;
    b->dsrc.push_back(S);
    tot += q.num_photons;
    b->start.push_back((uint32_t) tot);
  }
  if (tot >= (1ull << 31)) { g_create_err = "mx_batch_create: more than 2^31 photons"; delete b; return nullptr; }
  if (c->cfg.acis_exposure_time <= 0) { g_create_err = "mx_batch_create: ACIS_Exposure_Time must be > 0"; delete b; return nullptr; }
  b->total = tot;
  b->shared_bytes = tables_shared_bytes(c->T) + align16((size_t) nsrc * sizeof(MxSourceDev)) + align16((size_t) (nsrc + 1) * 4);
  const size_t elem[12] = {8, 24, 24, 8, 4, 4, 1, 1, 1, 4, 4, 12};
  cudaError_t e = b->d_src.ensure(b->dsrc.size() * sizeof(MxSourceDev) + b->start.size() * 4);
  for (int k = 0; k < 12 && e == cudaSuccess; k++) e = b->cols[k].ensure(std::max<size_t>(16, tot * elem[k]));
  if (e == cudaSuccess) e = b->queues.ensure(std::max<size_t>(256, 2 * tot * sizeof(MxRec)));
  if (e == cudaSuccess) e = b->ctr.ensure(128);
  if (e == cudaSuccess) e = b->d_spec.ensure(std::max<size_t>(16, b->spec.size() * sizeof(double)));
  if (e == cudaSuccess && !b->spec.empty())
    e = cudaMemcpy(b->d_spec.ptr, b->spec.data(), b->spec.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMallocHost((void **) &b->h_seed, sizeof(uint64_t));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_src.ptr, b->dsrc.data(), b->dsrc.size() * sizeof(MxSourceDev), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy((char *) b->d_src.ptr + b->dsrc.size() * sizeof(MxSourceDev), b->start.data(), b->start.size() * 4,
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    g_create_err = std::string("mx_batch_create: ") + cudaGetErrorString(e);
    mx_batch_destroy(b);
    return nullptr;
  }
  *b->h_seed = 0;
  b->key = batch_key(b);
  int maxb = 0;
  if (batch_max_blocks(b, 256, &maxb) != MX_OK || maxb < 1) {
    g_create_err = "mx_batch_create: the batch kernel cannot be resident (" + c->err + ")";
    mx_batch_destroy(b);
    return nullptr;
  }
  b->params.block = 256; b->params.tile = 256; b->params.blocks_per_sm = maxb; b->params.reserved = 0;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(b->key);
    if (it != g_tune_cache.end()) { b->params = it->second; b->have_params = true; }
  }
  return b;
}

void mx_batch_destroy(mx_batch *b) {
  if (!b) return;
  if (b->done) cudaEventSynchronize(b->done);
  drop_graph(b);
  b->d_src.release();
  for (auto &col : b->cols) col.release();
  b->queues.release();
  b->ctr.release();
  b->d_spec.release();
  if (b->h_seed) cudaFreeHost(b->h_seed);
  if (b->done) cudaEventDestroy(b->done);
  delete b;
}

int mx_batch_set_params(mx_batch *b, const mx_batch_params *p) {
  if (!b || !p) return MX_EINVAL;
  // warps claim tiles on their own, so any whole number of warps up to the
  // kernel's bound of 256 threads works
  if (p->block < 32 || p->block > 256 || (p->block % 32) != 0 || p->tile < 32 || (p->tile % 32) != 0 ||
      p->blocks_per_sm < 1)
    return mx_fail(b->ctx, MX_EINVAL, "mx_batch_set_params: block must be 32 to 256 threads in whole warps, "
                                      "tile a positive multiple of 32");
  int maxb = 0;
  int r = batch_max_blocks(b, p->block, &maxb);
  if (r) return r;
  if (p->blocks_per_sm > maxb) return mx_fail(b->ctx, MX_ERANGE, "mx_batch_set_params: more blocks per SM than fit");
  b->params = *p;
  drop_graph(b);
  return MX_OK;
}

int mx_batch_get_params(const mx_batch *b, mx_batch_params *p) {
  if (!b || !p) return MX_EINVAL;
  *p = b->params;
  return MX_OK;
}

int mx_batch_run(mx_batch *b, uint64_t seed, void *stream) {
  if (!b) return MX_EINVAL;
  if (b->total == 0) return MX_OK;
  if (!b->exec) {
    int r = build_graph(b);
    if (r) return r;
  }
  // the previous run has read the pinned seed before it is overwritten
  cudaError_t e = cudaEventSynchronize(b->done);
  if (e != cudaSuccess) return mx_cuda_fail(b->ctx, e, "batch");
  *b->h_seed = seed;
  e = cudaGraphLaunch(b->exec, (cudaStream_t) stream);
  if (e == cudaSuccess) e = cudaEventRecord(b->done, (cudaStream_t) stream);
  b->ctx->launches += (b->ctx->T.acis_fef || b->ctx->T.acis_qe) ? 2 : 1;
  return e == cudaSuccess ? MX_OK : mx_cuda_fail(b->ctx, e, "launching the batch graph");
}

int mx_batch_run_sequential(mx_batch *b, uint64_t seed, void *stream) {
  if (!b) return MX_EINVAL;
  mx_context *c = b->ctx;
  mx_photons all = batch_view(b);
  for (size_t s = 0; s < b->src.size(); s++) {
    uint32_t n0 = b->start[s], ns = b->start[s + 1] - n0;
    if (ns == 0) continue;
    // a view of the source's slice: offset pointers, stride of the batch
    mx_photons q = all;
    q.n = ns;
    q.stride = all.n;
    q.energy += n0; q.x += n0; q.p += n0; q.arrival_time += n0; q.flags += n0; q.tag += n0;
    q.mirror_shell += n0; q.order += n0; q.ccd_num += n0; q.y_pixel += n0; q.z_pixel += n0; q.dither_state += n0;
    int r = mx_generate_source(c, &b->src[s], n0, seed, &q, stream);
    if (r) return r;
    MxTables T = c->T;
    T.grating = b->dsrc[s].grating;
    T.chip_off = b->dsrc[s].chip_off;
    T.nchips = b->dsrc[s].nchips;
    r = mx_trace_tables(c, T, &q, MX_STAGE_ALL, nullptr, nullptr, seed, (cudaStream_t) stream, true);
    if (r) return r;
  }
  return MX_OK;
}

int mx_batch_photons(mx_batch *b, mx_photons *dev_view, const uint32_t **source_start) {
  if (!b) return MX_EINVAL;
  if (dev_view) *dev_view = batch_view(b);
  if (source_start) *source_start = b->start.data();
  return MX_OK;
}

uint64_t mx_batch_total_photons(const mx_batch *b) { return b ? b->total : 0; }

// The autotuner: block sizes of 64 to 256 threads, resident block counts
// per SM from the largest down to half of it, and five work-tile sizes,
// each timed with CUDA events over `trials` graph launches after one
// warm-up launch (which also captures that candidate's graph).  The
// fastest mean wins and is remembered under the batch's hash.
int mx_batch_tune(mx_batch *b, int trials, mx_batch_params *best) {
  if (!b) return MX_EINVAL;
  mx_context *c = b->ctx;
  if (trials < 1) trials = 1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(b->key);
    if (it != g_tune_cache.end()) {
      b->params = it->second;
      b->have_params = true;
      drop_graph(b);
      if (best) *best = b->params;
      return MX_OK;
    }
  }
  // block sizes up to the kernel's bound, warp tiles from one warp's worth
  // of photons to 1024, and resident blocks per SM from the register limit
  // down to half of it
  std::vector<mx_batch_params> cand;
  const int blocks[4] = {64, 128, 192, 256};
  const int tiles[5] = {32, 64, 128, 256, 1024};
  for (int bl : blocks) {
    int maxb = 0;
    int r = batch_max_blocks(b, bl, &maxb);
    if (r) return r;
    if (maxb < 1) continue;
    std::vector<int> per = {maxb};
    for (int v : {(3 * maxb + 3) / 4, maxb / 2})
      if (v >= 1 && v != per.back()) per.push_back(v);
    for (int pb : per)
      for (int t : tiles) {
        mx_batch_params q;
        q.block = bl; q.tile = t; q.blocks_per_sm = pb; q.reserved = 0;
        cand.push_back(q);
      }
  }
  if (cand.empty()) return mx_fail(c, MX_ERANGE, "mx_batch_tune: no launch shape fits");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = 1e30f;
  mx_batch_params win = cand[0];
  int r = MX_OK;
  for (const mx_batch_params &q : cand) {
    if ((r = mx_batch_set_params(b, &q)) != MX_OK) break;
    if ((r = mx_batch_run(b, 0x7A11u, c->stream)) != MX_OK) break;
    cudaEventRecord(e0, c->stream);
    for (int t = 0; t < trials && r == MX_OK; t++) r = mx_batch_run(b, 0x7A11u + t, c->stream);
    cudaEventRecord(e1, c->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (r != MX_OK) break;
    if (e != cudaSuccess) { r = mx_cuda_fail(c, e, "mx_batch_tune"); break; }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= trials;
    if (ms < best_ms) { best_ms = ms; win = q; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r != MX_OK) return r;
  if ((r = mx_batch_set_params(b, &win)) != MX_OK) return r;
  b->have_params = true;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[b->key] = win;
  }
  if (best) *best = win;
  return MX_OK;
}

}  // extern "C"
