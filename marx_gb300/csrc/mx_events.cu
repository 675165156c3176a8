// marx2fits's per-event coordinates (marx/src/marx2fits.c) as a device pass
// over an event list: CHIPX/CHIPY, EXPNO, FLTGRADE/GRADE, DETX/DETY, sky
// X/Y and TDETX/TDETY.  Each event is independent except for ACIS frames:
// marx2fits keeps the dither state of a frame's first event for the whole
// frame (read_dither_value, marx2fits.c:3567-3581), so the pass finds each
// event's frame start with a max-scan over the event order.
//
// This file is compiled without fused multiply-add contraction: DETX/DETY
// are pure arithmetic in the reference (pixlib.c:135-222, detpix.c:182-208)
// and round bit for bit like it; the sky columns also call sin, cos, acos,
// asin and atan, which agree with the host's to an ulp or so.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mx_context.h"
#include "mx_device.cuh"

using namespace mx;

namespace mx_ev {

constexpr int EV_BLOCK = 256;
constexpr int EV_MAX_FACETS = 6;

struct EvFacet {
  double x_ll[3], xhat[3], yhat[3];
  double xps, yps, xoff, yoff, tdx, tdy;   // pixel sizes, pixel of the LL corner, tiled offsets
  int32_t tiled, pad;                      // 0: ACIS-I chips 0, 2; 1: ACIS-I chips 1, 3; 2: x + tdx, y + tdy
};

struct EvGeom {
  EvFacet f[EV_MAX_FACETS];
  int32_t nf, first_id, acis, pad;
  double fp_delta, fp_x0, fp_y0;       // focal-plane system (detpix.c:42-63)
  const float *sp;                     // sub-pixel rows: energies, dx, dy (npoints each)
  const int32_t *sp_row;               // [2][256]: FI/BI x fltgrade -> offset of the row in sp, -1: none
  const int32_t *sp_n;                 // [2][256]: npoints
};

struct EvArgs {
  mx_events e;
  mx_event_params p;
  uint64_t seed;
  double roll_c, roll_s;               // cos, sin of Roll_Nom (host libm, as the reference)
  int frames;                          // frame runs decide the dither
  unsigned long long *bad;
};

// FLTGRADE of each of the 3 x 3 sub-pixels, four equally likely values
// (Flight_Grade_Table, marx2fits.c:3838-3849): rows -- 0- +- -0 00 +0 -+ 0+ ++.
__constant__ int16_t kFlightGrades[9][4] = {
    {10, 11, 138, 139}, {2, 34, 130, 162}, {18, 22, 50, 54},
    {8, 12, 136, 140},  {0, 0, 0, 0},      {16, 17, 48, 49},
    {72, 76, 104, 108}, {64, 65, 68, 69},  {80, 81, 208, 209}};
// ASCA grade of each flight grade (the CALDB grade map the reference
// tabulates as Grade_Map, marx2fits.c:3792-3810), one digit per fltgrade.
__constant__ char kGradeMap[257] =
    "0125115735663577446755677777777711251157577757774467556777777777"
    "2277227767776777667777777777777755775577677767777777777777777777"
    "1125115735663577557777777777777711251157577757775577777777777777"
    "5577557777777777667777777777777777777777777777777777777777777777";

__device__ __forceinline__ double event_uniform(uint64_t seed, uint32_t k, uint32_t slot) {
  uint32_t c[4] = {k, slot, 0x5A5A0004u, 0u};
  philox(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  uint64_t b = ((uint64_t) c[0] << 32) | c[1];
  return (double) (b >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ uint32_t row_of(const mx_events &e, uint32_t k) { return e.index ? e.index[k] : k; }

// time.dat as marx2fits reads it: a float widened to double.
__device__ __forceinline__ double event_time(const EvArgs &a, uint32_t row) {
  if (a.e.time) return (double) a.e.time[row];
  return (double) (float) (a.e.time64[row] + a.p.time_offset);
}

// compute_expno (marx2fits.c:3741-3761) for event k
__device__ __forceinline__ int64_t frame_of(const EvArgs &a, uint32_t k) {
  return (int64_t) (event_time(a, row_of(a.e, k)) / a.p.frame_time);
}

// JDMv_length (vector.c:77-97)
__device__ __forceinline__ double jdm_length(double ax, double ay, double az) {
  double x = fabs(ax), y = fabs(ay), z = fabs(az), t;
  if (z < x) { t = z; z = x; x = t; }
  if (z < y) { t = z; z = y; y = t; }
  if (z == 0.0) return 0.0;
  x = x / z; y = y / z;
  return z * sqrt(1.0 + x * x + y * y);
}
// JDMv_normalize (vector.c:99-109)
__device__ __forceinline__ D3 jdm_normalize(D3 a) {
  double len = jdm_length(a.x, a.y, a.z);
  if (len != 0.0) { a.x = a.x / len; a.y = a.y / len; a.z = a.z / len; }
  return a;
}
// JDMv_rotate_unit_vector1 (vector.c:187-206)
__device__ __forceinline__ D3 jdm_rotate_unit(D3 p, D3 n, double c, double s) {
  double pn = p.x * n.x + p.y * n.y + p.z * n.z;
  double b = pn * (1.0 - c);
  D3 x3;   // JDMv_pcross_prod (n, p)
  x3.z = n.x * p.y - n.y * p.x;
  x3.x = n.y * p.z - n.z * p.y;
  x3.y = n.z * p.x - n.x * p.z;
  D3 d = mk(c * p.x + b * n.x + s * x3.x, c * p.y + b * n.y + s * x3.y, c * p.z + b * n.z + s * x3.z);
  return jdm_normalize(d);
}

// marx_compute_acis_subpix (acis_subpix.c:284-320)
static __device__ void subpix(const EvGeom &G, int ccd, float energy, int fltgrade, float &dx, float &dy) {
  int kind = (ccd == 5 || ccd == 7) ? 1 : 0;   // BI chips (read_subpixel_file, acis_subpix.c:246-252)
  int off = __ldg(G.sp_row + kind * 256 + fltgrade);
  if (off < 0) { dx = dy = 0.0f; return; }
  unsigned n = (unsigned) __ldg(G.sp_n + kind * 256 + fltgrade);
  const float *e = G.sp + off, *xs = e + n, *ys = xs + n;
  unsigned j = bsearch_f(energy, e, n);
  if (j == 0) j++;
  if (j == n) j--;
  float e0 = __ldg(e + j - 1), e1 = __ldg(e + j);
  double w1 = ((double) energy - e0) / (double) (e1 - e0);
  double w0 = 1.0 - w1;
  dx = (float) (w0 * __ldg(xs + j - 1) + w1 * __ldg(xs + j));
  dy = (float) (w0 * __ldg(ys + j - 1) + w1 * __ldg(ys + j));
}

// Inclusive max-scan of v over the block (EV_BLOCK threads).
__device__ __forceinline__ uint32_t block_max_scan(uint32_t v, uint32_t *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v = max(v, o);
  }
  if (lane == 31) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < EV_BLOCK / 32 ? sh[lane] : 0u;
#pragma unroll
    for (int d = 1; d < EV_BLOCK / 32; d <<= 1) {
      uint32_t o = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w = max(w, o);
    }
    if (lane < EV_BLOCK / 32) sh[lane] = w;
  }
  __syncthreads();
  uint32_t r = warp ? max(v, sh[warp - 1]) : v;
  __syncthreads();
  return r;
}

// A frame starts at event k when k is the first event or its frame number
// differs from the previous event's.
__device__ __forceinline__ uint32_t frame_start(const EvArgs &a, uint32_t k) {
  if (k >= a.e.n) return 0u;
  if (k == 0) return 0u;
  return frame_of(a, k) != frame_of(a, k - 1) ? k : 0u;
}

// Last frame start of each tile of EV_BLOCK events.
__global__ void __launch_bounds__(EV_BLOCK) mx_event_frame_tiles(EvArgs a, uint32_t ntiles, uint32_t *tile_max) {
  __shared__ uint32_t sh[32];
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    uint32_t k = t * EV_BLOCK + threadIdx.x;
    uint32_t m = block_max_scan(frame_start(a, k), sh);
    if (threadIdx.x == EV_BLOCK - 1) tile_max[t] = m;
  }
}

// Exclusive max-scan over the tiles, in place (one block of 1024 threads).
__global__ void __launch_bounds__(1024) mx_event_frame_prefix(uint32_t ntiles, uint32_t *tile_max) {
  __shared__ uint32_t carry;
  __shared__ uint32_t sh[32];
  if (threadIdx.x == 0) carry = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t base = 0; base < ntiles; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    uint32_t incl = i < ntiles ? tile_max[i] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl = max(incl, o);
    }
    if (lane == 31) sh[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = sh[lane];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t o = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w = max(w, o);
      }
      sh[lane] = w;
    }
    __syncthreads();
    const uint32_t before = max(warp ? sh[warp - 1] : 0u, carry);   // everything ahead of this warp
    incl = max(incl, before);
    uint32_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = before;
    __syncthreads();
    if (i < ntiles) tile_max[i] = excl;
    if (threadIdx.x == 1023) carry = incl;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(EV_BLOCK) mx_event_kernel(EvArgs a, EvGeom G, uint32_t ntiles, const uint32_t *tile_pre) {
  __shared__ uint32_t sh[32];
  const mx_events &e = a.e;
  const mx_event_params &p = a.p;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  double last_roll = nan, roll_s = 0.0, roll_c = 1.0;   // NaN never equals a roll: the first event computes
  for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const uint32_t k = t * EV_BLOCK + threadIdx.x;
    uint32_t first = k;   // the event whose dither state this event uses
    if (a.frames) first = max(block_max_scan(frame_start(a, k), sh), tile_pre[t]);
    if (k >= e.n) continue;
    const uint32_t row = row_of(e, k), drow = row_of(e, first);
    const int ccd = e.ccd_id[row];
    const int fi = ccd - G.first_id;
    // read_float32_add_1 (marx2fits.c:3460-3470): CHIPX is xpixel + 1 in float
    const float chipx = e.xpixel[row] + 1.0f, chipy = e.ypixel[row] + 1.0f;
    if (e.chipx) e.chipx[k] = chipx;
    if (e.chipy) e.chipy[k] = chipy;
    // EXPNO (compute_expno): the frame number, or the event number less one
    // when there are no frames
    if (e.expno) e.expno[k] = G.acis ? (p.frame_time > 0.0 ? (int32_t) frame_of(a, k) : (int32_t) k - 1) : 0;
    if (fi < 0 || fi >= G.nf) {
      atomicAdd(a.bad, 1ull);
      if (e.detx) e.detx[k] = nan;
      if (e.dety) e.dety[k] = nan;
      if (e.x) e.x[k] = nan;
      if (e.y) e.y[k] = nan;
      if (e.tdetx) e.tdetx[k] = -1;
      if (e.tdety) e.tdety[k] = -1;
      if (e.fltgrade) e.fltgrade[k] = 0;
      if (e.grade) e.grade[k] = 0;
      continue;
    }
    const EvFacet &g = G.f[fi];
    const double ux = e.uniforms ? e.uniforms[k] : event_uniform(a.seed, k, 0);
    // FLTGRADE (compute_fltgrade, marx2fits.c:3854-3866) and GRADE (compute_grade)
    int fltgrade = 0;
    if (G.acis) {
      const double cx = (double) chipx, cy = (double) chipy;
      int sx = (int) (3.0 * (cx - floor(cx))), sy = (int) (3.0 * (cy - floor(cy)));
      fltgrade = kFlightGrades[3 * sy + sx][min((int) (4 * ux), 3)];   // u = 1 stays in the row
    }
    if (e.fltgrade) e.fltgrade[k] = (int16_t) fltgrade;
    if (e.grade) e.grade[k] = (int16_t) (G.acis ? kGradeMap[fltgrade & 0xff] - '0' : 0);
    // TDETX, TDETY (compute_tdetxy; acis_i_to_tiled, acis_s_to_tiled,
    // acis_geom.c:106-135, 183-203; hrc_i_to_tiled, hrc_i_geom.c:215-233;
    // hrc_s_to_tiled, hrc_s_geom.c:476-514)
    if (e.tdetx || e.tdety) {
      const unsigned ix = (unsigned) chipx, iy = (unsigned) chipy;
      float xf, yf;
      if (g.tiled == 0) { xf = (float) (g.tdx + iy); yf = (float) (g.tdy - ix); }
      else if (g.tiled == 1) { xf = (float) (g.tdx - iy); yf = (float) (g.tdy + ix); }
      else { xf = (float) (ix + g.tdx); yf = (float) (iy + g.tdy); }
      if (xf < 0.0f) xf = 0.0f;
      if (yf < 0.0f) yf = 0.0f;
      if (e.tdetx) e.tdetx[k] = (int32_t) ((unsigned) xf + 1u);
      if (e.tdety) e.tdety[k] = (int32_t) ((unsigned) yf + 1u);
    }
    // the dither state (read_dither_value): zero for an undithered run
    double d_ra = 0, d_dec = 0, d_roll = 0, d_dy = 0, d_dz = 0, d_th = 0;
    if (p.dithered) {
      if (e.sky_ra) d_ra = (double) e.sky_ra[drow];
      if (e.sky_dec) d_dec = (double) e.sky_dec[drow];
      if (e.sky_roll) d_roll = (double) e.sky_roll[drow];
      if (e.det_dy) d_dy = (double) e.det_dy[drow];
      if (e.det_dz) d_dz = (double) e.det_dz[drow];
      if (e.det_theta) d_th = (double) e.det_theta[drow];
    }
    // compute_detxy (marx2fits.c:3676-3736): chip pixel from 1-based CHIPX
    double x = (double) chipx - 1.0, y = (double) chipy - 1.0;
    switch (p.pixel_adjust) {
      case MX_PIXADJ_EXACT: break;
      case MX_PIXADJ_NONE: x = floor(x) + 0.5; y = floor(y) + 0.5; break;
      case MX_PIXADJ_RANDOMIZE: {
        const double u1 = e.uniforms ? e.uniforms[(size_t) e.n + k] : event_uniform(a.seed, k, 1);
        const double u2 = e.uniforms ? e.uniforms[2 * (size_t) e.n + k] : event_uniform(a.seed, k, 2);
        x = floor(x) + u1;
        y = floor(y) + u2;
        break;
      }
      default: {   // EDSER
        float dx, dy;
        subpix(G, ccd, e.b_energy ? e.b_energy[row] : 0.0f, fltgrade, dx, dy);
        x = floor(x) + 0.5 + dx;
        y = floor(y) + 0.5 + dy;
        break;
      }
    }
    // marx_init_chip_to_mnc (pixlib.c:135-198) with the detector offsets and
    // motion, then marx_chip_to_mnc (pixlib.c:201-222)
    double ct = 1.0, st = 0.0;
    if (d_th != 0.0) { ct = cos(d_th); st = sin(d_th); }
    const double yoff = p.det_offset[1] + d_dy, zoff = p.det_offset[2] + d_dz;
    D3 ofs = mk(p.det_offset[0] - p.focal_length, yoff + ct * g.x_ll[1] - st * g.x_ll[2],
                zoff + st * g.x_ll[1] + ct * g.x_ll[2]);
    D3 e1 = mk(g.xhat[0], ct * g.xhat[1] - st * g.xhat[2], st * g.xhat[1] + ct * g.xhat[2]);
    D3 e2 = mk(g.yhat[0], ct * g.yhat[1] - st * g.yhat[2], st * g.yhat[1] + ct * g.yhat[2]);
    e1 = mk(g.xps * e1.x, g.xps * e1.y, g.xps * e1.z);
    e2 = mk(g.yps * e2.x, g.yps * e2.y, g.yps * e2.z);
    x -= g.xoff;
    y -= g.yoff;
    D3 mnc = jdm_normalize(mk(ofs.x + e1.x * x + e2.x * y, ofs.y + e1.y * x + e2.y * y, ofs.z + e1.z * x + e2.z * y));
    // marx_mnc_to_fpc (detpix.c:182-208)
    double detx = nan, dety = nan;
    if (mnc.x != 0.0) {
      const double factor = 1.0 / (G.fp_delta * mnc.x);
      detx = G.fp_x0 - factor * mnc.y;
      dety = G.fp_y0 + factor * mnc.z;
    } else {
      atomicAdd(a.bad, 1ull);
    }
    if (e.detx) e.detx[k] = detx;
    if (e.dety) e.dety[k] = dety;
    if (!e.x && !e.y) continue;
    // compute_xy_sky (marx2fits.c:3869-3910)
    double sx, sy;
    if (!p.dithered) {
      const double dx = detx - G.fp_x0, dy = dety - G.fp_y0;
      sx = G.fp_x0 + a.roll_c * dx + a.roll_s * dy;
      sy = G.fp_y0 - a.roll_s * dx + a.roll_c * dy;
    } else {
      // marx_undither_mnc -> unapply_dither (dither.c:583-607)
      // dither offsets are arcseconds: the short series rounds like the host's sin and cos
      double sra, cra, sdec, cdec;
      sincos_small(d_ra, &sra, &cra);
      sincos_small(d_dec, &sdec, &cdec);
      const double cos_t = cdec * cra;
      D3 n = mk(0.0, -sdec, cdec * sra);
      const double sin_t = jdm_length(n.x, n.y, n.z);
      if (sin_t >= 1e-20) {
        n = mk(n.x / sin_t, n.y / sin_t, n.z / sin_t);
        mnc = jdm_rotate_unit(mnc, n, cos_t, sin_t);
      }
      if (d_roll != last_roll) {   // one roll for a whole run under INTERNAL dither
        sincos(d_roll, &roll_s, &roll_c);
        last_roll = d_roll;
      }
      mnc = jdm_rotate_unit(mnc, mk(1.0, 0.0, 0.0), roll_c, roll_s);
      // marx_mnc_to_ra_dec (pixlib.c:499-523)
      double perp = sqrt(mnc.x * mnc.x + mnc.y * mnc.y);
      if (perp > 1.0) perp = 1.0;
      const double dec = mnc.z <= 0 ? acos(perp) : -acos(perp);
      const double q = -mnc.x / perp;
      const double ra = mnc.y <= 0.0 ? acos(q) : -acos(q);
      // marx_compute_ra_dec_offsets (pixlib.c:531-570) about (0, 0): cos(dec)
      // and cos(d_dec) are the same value there
      double sdec_s, c, sra_s, cra_s;
      sincos(dec, &sdec_s, &c);
      sincos(ra, &sra_s, &cra_s);
      const double factor = c * (1 - cra_s);
      double sin_dd = sdec_s + factor * 0.0;
      if (fabs(sin_dd) > 1.0) sin_dd = sin_dd < 0 ? -1.0 : 1.0;
      const double ddec = asin(sin_dd);
      const double num = c * sra_s, den = c - factor * 1.0;
      double dra;
      if (den >= 0) dra = atan(num / den);
      else dra = num >= 0 ? atan(num / den) + PI : atan(num / den) - PI;
      sx = -dra / G.fp_delta + G.fp_x0;
      sy = ddec / G.fp_delta + G.fp_y0;
    }
    if (e.x) e.x[k] = sx;
    if (e.y) e.y[k] = sy;
  }
}

// The facets, focal-plane system and sub-pixel tables of the context's
// detector.
struct EvTables {
  EvGeom G;
  std::vector<char> blob;
  size_t o_sp = 0, o_row = 0, o_n = 0;
};

static bool event_tables(const mx_context *c, EvTables &out, std::string &err) {
  const mx_config &cfg = c->cfg;
  const HostModel &M = c->hm;
  EvGeom &G = out.G;
  memset(&G, 0, sizeof(G));
  const double arcsec = PI / (3600.0 * 180.0);
  // AXAF-FP-1.1 (ACIS), AXAF-FP-2.1 (HRC-I), AXAF-FP-2.3 (HRC-S)
  // (Focal_Plane_Coord_Info, detpix.c:42-63)
  switch (cfg.detector) {
    case MX_DETECTOR_ACIS_I:
    case MX_DETECTOR_ACIS_S: G.fp_delta = 0.492 * arcsec; G.fp_x0 = G.fp_y0 = 4096.5; G.acis = 1; break;
    case MX_DETECTOR_HRC_I: G.fp_delta = 0.13175 * arcsec; G.fp_x0 = G.fp_y0 = 16384.5; break;
    case MX_DETECTOR_HRC_S: G.fp_delta = 0.1318 * arcsec; G.fp_x0 = G.fp_y0 = 32768.5; break;
    default: err = "event coordinates need an ACIS or HRC detector"; return false;
  }
  const MxTables &T = M.T;
  G.nf = T.nchips;
  if (G.nf < 1 || G.nf > EV_MAX_FACETS) { err = "detector without facets"; return false; }
  G.first_id = M.chips[T.chip_off].id;
  // tiled offsets (acis_geom.c:37-47, hrc_i_geom.c:136-137, hrc_s_geom.c:321-328)
  static const double acis_i_tx[4] = {3061, 5131, 3061, 5131}, acis_i_ty[4] = {5131, 4107, 4085, 3061};
  static const double acis_s_tx[6] = {791, 1833, 2875, 3917, 4959, 6001};
  static const double hrc_s_ty[3] = {-12.0, 16444.0, 32900.0};
  for (int i = 0; i < G.nf; i++) {
    const MxChipDev &ch = M.chips[T.chip_off + i];
    if (ch.id != G.first_id + i) { err = "facet ids are not consecutive"; return false; }
    EvFacet &f = G.f[i];
    memcpy(f.x_ll, ch.x_ll, sizeof(f.x_ll));
    memcpy(f.xhat, ch.xhat, sizeof(f.xhat));
    memcpy(f.yhat, ch.yhat, sizeof(f.yhat));
    f.tiled = 2;
    if (G.acis) {
      // tweak_acis_pixel_size (acis_geom.c:54-66); the LL corner is pixel 0
      f.xps = ch.xlen / 1024.0; f.yps = ch.ylen / 1024.0;
      if (cfg.detector == MX_DETECTOR_ACIS_I) {
        f.tdx = acis_i_tx[ch.id]; f.tdy = acis_i_ty[ch.id];
        f.tiled = (ch.id == 0 || ch.id == 2) ? 0 : 1;
      } else {
        f.tdx = acis_s_tx[ch.id - 4]; f.tdy = 1702;
      }
    } else {
      // 6.429 micron pixels (hrc_i_geom.c:277-278, hrc_s_geom.c:559-560)
      f.xps = f.yps = 6.429e-3;
      const MxHrcDev &h = T.hrc;
      if (cfg.detector == MX_DETECTOR_HRC_I) {
        f.xoff = h.ll_cxcy[0]; f.yoff = h.ll_cxcy[1];   // LL_CXCY (hrc_i_geom.c:139-140)
        f.tdx = -1.0; f.tdy = 0.0;
      } else {
        // _marx_hrc_s_compute_pixel (hrc_s_geom.c:343-392) at the LL corner
        const double u = h.u_active0 + 0.0 / h.pix[0], v = h.v_active0[i] + 0.0 / h.pix[1];
        f.xoff = h.cxcy0[i][0] + (u - h.uv0[i][0]);
        f.yoff = h.cxcy0[i][1] + (v - h.uv0[i][1]);
        f.tdx = 0.0; f.tdy = hrc_s_ty[i];
      }
    }
  }
  // ACIS sub-pixel offsets (read_subpix_ext, acis_subpix.c:96-186)
  std::vector<float> sp;
  std::vector<int32_t> row(512, -1), npts(512, 0);
  if (G.acis) {
    const char *kinds[2] = {"acis/subpix_fi", "acis/subpix_bi"};
    for (int kd = 0; kd < 2; kd++) {
      size_t ni, nt;
      const int32_t *idx = c->pack.get<int32_t>(std::string(kinds[kd]) + "/rows", &ni, err);
      const float *tab = c->pack.get<float>(std::string(kinds[kd]) + "/table", &nt, err);
      if (!idx || !tab) return false;
      // rows: (fltgrade, npoints) pairs; table: per row energies, dx, dy of `rep` floats
      const size_t nrows = ni / 2;
      if (nrows == 0 || nt % (3 * nrows)) { err = kinds[kd] + std::string(": malformed"); return false; }
      const size_t rep = nt / (3 * nrows);
      for (size_t r = 0; r < nrows; r++) {
        const int fg = idx[2 * r], np = idx[2 * r + 1];
        if (fg < 0 || fg >= 256) { err = "Illegal flight grade in subpix column"; return false; }
        if (np <= 0) { row[kd * 256 + fg] = -1; continue; }
        if (np == 1) { err = "Expecting Number of points (NPOINTS) to be greater than 1"; return false; }
        if ((size_t) np > rep) { err = "NPOINTS is greater than repeat count"; return false; }
        row[kd * 256 + fg] = (int32_t) sp.size();
        npts[kd * 256 + fg] = np;
        for (int w = 0; w < 3; w++) {
          const float *src = tab + (w * nrows + r) * rep;
          sp.insert(sp.end(), src, src + np);
        }
      }
    }
  }
  if (sp.empty()) sp.push_back(0.0f);
  auto put = [&](const void *d, size_t bytes) {
    size_t off = (out.blob.size() + 255) & ~(size_t) 255;
    out.blob.resize(off + bytes);
    memcpy(out.blob.data() + off, d, bytes);
    return off;
  };
  out.o_sp = put(sp.data(), sp.size() * sizeof(float));
  out.o_row = put(row.data(), row.size() * sizeof(int32_t));
  out.o_n = put(npts.data(), npts.size() * sizeof(int32_t));
  return true;
}

static int ensure_event_tables(mx_context *c) {
  if (c->events_ready) return MX_OK;
  EvTables t;
  std::string err;
  if (!event_tables(c, t, err)) return mx_fail(c, MX_EINVAL, err);
  cudaError_t e = c->ev_tab.ensure(t.blob.size());
  if (e == cudaSuccess) e = cudaMemcpy(c->ev_tab.ptr, t.blob.data(), t.blob.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "uploading the event tables");
  char *b = (char *) c->ev_tab.ptr;
  t.G.sp = (const float *) (b + t.o_sp);
  t.G.sp_row = (const int32_t *) (b + t.o_row);
  t.G.sp_n = (const int32_t *) (b + t.o_n);
  static_assert(sizeof(EvGeom) <= sizeof(c->ev_geom), "event geometry larger than its slot");
  memcpy(c->ev_geom, &t.G, sizeof(EvGeom));
  c->events_ready = true;
  return MX_OK;
}

static int check_params(mx_context *c, const mx_event_params *p, const mx_events *ev) {
  if (!p || !ev) return mx_fail(c, MX_EINVAL, "mx_event_coords: null argument");
  if (ev->n == 0) return MX_OK;
  if (!ev->ccd_id || !ev->xpixel || !ev->ypixel) return mx_fail(c, MX_EINVAL, "mx_event_coords: ccd_id, xpixel and ypixel are required");
  if (!ev->time && !ev->time64) return mx_fail(c, MX_EINVAL, "mx_event_coords: no time column");
  if (p->pixel_adjust < MX_PIXADJ_EDSER || p->pixel_adjust > MX_PIXADJ_EXACT)
    return mx_fail(c, MX_EINVAL, "mx_event_coords: unknown pixel adjustment");
  if (!(p->focal_length > 0)) return mx_fail(c, MX_EINVAL, "mx_event_coords: focal length must be positive");
  return MX_OK;
}

static int launch_events(mx_context *c, const mx_event_params *params, const mx_events *ev, uint64_t seed, cudaStream_t st) {
  int rc = ensure_event_tables(c);
  if (rc != MX_OK) return rc;
  EvGeom G;
  memcpy(&G, c->ev_geom, sizeof(EvGeom));
  EvArgs a;
  a.e = *ev;
  a.p = *params;
  // marx2fits turns EDSER into RANDOMIZE for an HRC (marx2fits.c:3307-3308)
  if (!G.acis && a.p.pixel_adjust == MX_PIXADJ_EDSER) a.p.pixel_adjust = MX_PIXADJ_RANDOMIZE;
  a.seed = seed;
  const double theta = params->roll_nom * PI / 180.0;
  a.roll_c = cos(theta);
  a.roll_s = sin(theta);
  a.frames = G.acis && a.p.dithered && a.p.frame_time > 0.0 && a.p.pixel_adjust != MX_PIXADJ_EXACT;
  a.bad = c->d_event_bad;
  const uint32_t ntiles = (ev->n + EV_BLOCK - 1) / EV_BLOCK;
  const uint32_t grid = (uint32_t) std::min<uint64_t>(ntiles, (uint64_t) c->num_sms * 8);
  uint32_t *tiles = nullptr;
  if (a.frames) {
    cudaError_t e = c->ev_scan.ensure((size_t) ntiles * sizeof(uint32_t));
    if (e != cudaSuccess) return mx_cuda_fail(c, e, "allocating the frame scan");
    tiles = (uint32_t *) c->ev_scan.ptr;
    mx_event_frame_tiles<<<grid, EV_BLOCK, 0, st>>>(a, ntiles, tiles);
    mx_event_frame_prefix<<<1, 1024, 0, st>>>(ntiles, tiles);
    c->launches += 2;
  }
  mx_event_kernel<<<grid, EV_BLOCK, 0, st>>>(a, G, ntiles, tiles);
  c->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "launching the event pass");
  return MX_OK;
}

}  // namespace mx_ev

using namespace mx_ev;

extern "C" {

int mx_event_coords(mx_context *c, const mx_event_params *params, const mx_events *ev, uint64_t seed, void *stream) {
  if (!c) return MX_EINVAL;
  int rc = check_params(c, params, ev);
  if (rc != MX_OK || ev->n == 0) return rc;
  return launch_events(c, params, ev, seed, (cudaStream_t) stream);
}

int mx_event_coords_host(mx_context *c, const mx_event_params *params, const mx_events *h, uint64_t seed) {
  if (!c) return MX_EINVAL;
  int rc = check_params(c, params, h);
  if (rc != MX_OK || h->n == 0) return rc;
  const size_t n = h->n;
  size_t rows = n;   // input rows: the largest index + 1
  if (h->index) {
    uint32_t m = 0;
    for (size_t k = 0; k < n; k++) m = std::max(m, h->index[k]);
    rows = (size_t) m + 1;
  }
  struct In { const void *src; size_t bytes; const void **dst; };
  mx_events d = *h;
  std::vector<In> ins = {
      {h->index, n * 4, (const void **) &d.index},       {h->ccd_id, rows, (const void **) &d.ccd_id},
      {h->xpixel, rows * 4, (const void **) &d.xpixel},  {h->ypixel, rows * 4, (const void **) &d.ypixel},
      {h->time, rows * 4, (const void **) &d.time},      {h->time64, rows * 8, (const void **) &d.time64},
      {h->sky_ra, rows * 4, (const void **) &d.sky_ra},  {h->sky_dec, rows * 4, (const void **) &d.sky_dec},
      {h->sky_roll, rows * 4, (const void **) &d.sky_roll}, {h->det_dy, rows * 4, (const void **) &d.det_dy},
      {h->det_dz, rows * 4, (const void **) &d.det_dz},  {h->det_theta, rows * 4, (const void **) &d.det_theta},
      {h->b_energy, rows * 4, (const void **) &d.b_energy}, {h->uniforms, 3 * n * 8, (const void **) &d.uniforms}};
  struct Out { void *dst; size_t bytes; void **dev; };
  std::vector<Out> outs = {
      {h->chipx, n * 4, (void **) &d.chipx}, {h->chipy, n * 4, (void **) &d.chipy},
      {h->detx, n * 8, (void **) &d.detx},   {h->dety, n * 8, (void **) &d.dety},
      {h->x, n * 8, (void **) &d.x},         {h->y, n * 8, (void **) &d.y},
      {h->tdetx, n * 4, (void **) &d.tdetx}, {h->tdety, n * 4, (void **) &d.tdety},
      {h->expno, n * 4, (void **) &d.expno}, {h->fltgrade, n * 2, (void **) &d.fltgrade},
      {h->grade, n * 2, (void **) &d.grade}};
  size_t total = 0;
  auto align = [](size_t b) { return (b + 255) & ~(size_t) 255; };
  for (auto &i : ins) if (i.src) total += align(i.bytes);
  for (auto &o : outs) if (o.dst) total += align(o.bytes);
  cudaError_t e = c->ev_io.ensure(total);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "allocating event staging");
  cudaStream_t st = c->stream;
  char *b = (char *) c->ev_io.ptr;
  size_t off = 0;
  unsigned long long bad0 = 0;
  e = cudaMemcpyAsync(&bad0, c->d_event_bad, sizeof(bad0), cudaMemcpyDeviceToHost, st);
  for (auto &i : ins) {
    if (!i.src || e != cudaSuccess) continue;
    *i.dst = b + off;
    e = cudaMemcpyAsync(b + off, i.src, i.bytes, cudaMemcpyHostToDevice, st);
    off += align(i.bytes);
  }
  for (auto &o : outs) {
    if (!o.dst) continue;
    *o.dev = b + off;
    off += align(o.bytes);
  }
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "copying events to the device");
  rc = launch_events(c, params, &d, seed, st);
  if (rc != MX_OK) return rc;
  for (auto &o : outs) {
    if (!o.dst || e != cudaSuccess) continue;
    e = cudaMemcpyAsync(o.dst, *o.dev, o.bytes, cudaMemcpyDeviceToHost, st);
  }
  unsigned long long bad1 = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad1, c->d_event_bad, sizeof(bad1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "event pass");
  if (bad1 != bad0) return mx_fail(c, MX_EINVAL, "event with a chip id outside the detector or without a focal-plane position");
  return MX_OK;
}

int mx_event_bad_count(mx_context *c, unsigned long long *count, int reset) {
  if (!c || !count) return MX_EINVAL;
  cudaError_t e = cudaMemcpy(count, c->d_event_bad, sizeof(*count), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && reset) e = cudaMemset(c->d_event_bad, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "reading the bad-event counter");
  return MX_OK;
}

}  // extern "C"
