// Differentiable form: weighted-ray focal-plane image, the MSE between two
// images, and the adjoint of the image with respect to the 18 geometry and
// pointing parameters.
//
// Forward: one persistent kernel traces each ray in FP64 (mxd::weighted_ray
// over double) and splats it with an 11 x 11 Gaussian.  The splat is
// accumulated in 64-bit fixed point -- exact integer sums, so the image does
// not depend on the order of the atomics and repeats bit for bit -- first in
// a 64 x 64 shared-memory window about the image centre, which takes nearly
// every ray of a point source, and then in the global accumulator.  A warp
// splats its 32 rays together, one ray at a time, each lane adding four of
// the 121 taps, so the lanes of one atomic instruction never collide.
//
// Adjoint: the ray is traced again with Dual6 scalars (FP64 value, FP32
// derivatives with respect to the six parameters that move it), following
// the decisions recorded by the forward pass; dL/dimage over the ray's
// 11 x 11 window gives dL/d(u, v, w), and the ray's derivative of
// (u, v, w) turns that into six parameter contributions.  Nothing per ray
// is stored between the passes except the decision byte.  A block takes
// the rays of a tile whose decision byte says they reached the focal plane
// (a ballot and prefix sum into shared memory, in ascending order) and
// traces only those, so that its lanes do not idle through the rays that
// were lost.  Sums are deterministic: fixed tiles per block, fixed warp
// order, fixed block order, one final reduction.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "mx_context.h"
#include "mx_diff.cuh"

using mxd::Dual6;

namespace {

constexpr int DBLOCK = 256;
constexpr int DWARPS = DBLOCK / 32;
constexpr int WIN = 64;                             // shared window side, pixels
constexpr int STAGE_W = 2 + 2 * mxd::TAPS;          // ic, jc, 11 y taps x w, 11 z taps
constexpr int STAGE_STRIDE = STAGE_W + 1;           // odd stride: conflict-free per-lane rows
constexpr int ADJ_STAGE = 9;                        // 6 contributions, shell, 2 pad
constexpr int ADJ_TILE = 8 * DBLOCK;                // rays a block sorts its hits out of at a time
constexpr int NP = MX_DIFF_NPARAM;

struct ImageGeom {
  int nx, ny;
  int wx0, wy0, wnx, wny;        // shared window: origin and extent in pixels
  int shift;                     // fixed-point right shift of each tap product
  int pad;
  double cy, cz, inv_pitch, cx_pix, cz_pix;
  float half_inv_s2;             // 1 / (2 sigma^2)
  float inv_s2;                  // 1 / sigma^2
  float knorm;                   // 1 / (sqrt(2 pi) sigma)
  float pad2;
};

// What the aperture sampling needs of each shell (project_photon_to_hrma).
struct Aperture {
  double area[4], rmin[4], rmax[4];
  uint32_t shutter[4];
  int32_t ideal, area_uniform;
};

struct FwdArgs {
  mxd::Optic<double> opt[4][2];
  mxd::Between<double> mid[4];
  mxd::RayConst rc[4];
  Aperture ap;
  double p0[3];
  double vig;
  ImageGeom g;
};

struct AdjArgs {
  mxd::Optic<Dual6> opt[4][2];
  mxd::Between<Dual6> mid[4];
  mxd::RayConst rc[4];
  Aperture ap;
  Dual6 p0[3];
  double vig;
  ImageGeom g;
};

__host__ __device__ constexpr size_t align_up(size_t b) { return (b + 15) & ~(size_t) 15; }

// Strut shadows (intersects_struts, hrma.c:928-968) at the three planes,
// evaluated on the ray's values.
struct StrutTest {
  const MxTables *T;
  template <class S>
  __device__ bool operator()(int set, const mxd::V3<S> &x, const mxd::V3<S> &p) const {
    if (!T->use_struts) return false;
    return mx::struts_block(*T, set, mx::mk(mxd::val(x.x), mxd::val(x.y), mxd::val(x.z)),
                            mx::mk(mxd::val(p.x), mxd::val(p.y), mxd::val(p.z)));
  }
  // The cap struts for a ray in the paraboloid's frame: screened on its
  // MARX-frame coordinates formed in single precision (as the trace's
  // cap_struts_block does), decided in double near a bar edge.
  template <class S>
  __device__ bool cap(const mxd::Optic<S> &P, const mxd::Between<S> &B, const mxd::V3<S> &x, const mxd::V3<S> &p) const {
    if (!T->use_struts) return false;
    const float xx = mx::d2f_trunc(mxd::val(x.x)), xy = mx::d2f_trunc(mxd::val(x.y)), xz = mx::d2f_trunc(mxd::val(x.z));
    const float px = mx::d2f_trunc(mxd::val(p.x)), py = mx::d2f_trunc(mxd::val(p.y)), pz = mx::d2f_trunc(mxd::val(p.z));
    const float *m = B.bwdf;
    const int s = mx::struts_screen(*T, 1, fmaf(m[0], xx, fmaf(m[1], xy, m[2] * xz)) - B.tof[0],
                                    fmaf(m[3], xx, fmaf(m[4], xy, m[5] * xz)) - B.tof[1],
                                    fmaf(m[6], xx, fmaf(m[7], xy, m[8] * xz)) - B.tof[2],
                                    fmaf(m[0], px, fmaf(m[1], py, m[2] * pz)), fmaf(m[3], px, fmaf(m[4], py, m[5] * pz)),
                                    fmaf(m[6], px, fmaf(m[7], py, m[8] * pz)));
    if (s >= 0) return s == 1;
    mxd::V3<S> pm = mxd::matv(P.bwd, p), xm = mxd::matv(P.bwd, x) - mxd::v3<S>(P.to[0], P.to[1], P.to[2]);
    return mx::struts_block_exact(*T, 1, mx::mk(mxd::val(xm.x), mxd::val(xm.y), mxd::val(xm.z)),
                                  mx::mk(mxd::val(pm.x), mxd::val(pm.y), mxd::val(pm.z)));
  }
};

// The aperture point of ray `tag`: the shell pick, radius and azimuth the
// mirror stage draws for the photon of that tag (mirror_front), with the
// vignetting draw consumed but turned into a weight.
__device__ __forceinline__ bool aperture(const Aperture &ap, uint64_t seed, uint32_t tag, int &si, double &ry,
                                         double &rz) {
  mx::Rng rng;
  rng.U = nullptr; rng.N = nullptr; rng.seed = seed; rng.n = 0; rng.i = 0; rng.tag = tag; rng.overrun = false;
  rng.window(MX_U_MIRROR, 12, MX_N_MIRROR, 2);
  if (!ap.ideal) (void) rng.uniform();
  si = -1;
  for (int guard = 0; guard < 64 && si < 0; guard++) {
    const double r = rng.uniform();
    if (rng.overrun) return false;
    for (int i = 0; i < 4; i++)
      if (mx::lt_pos(r, ap.area[i])) { si = i; break; }
  }
  if (si < 0) return false;
  double radius;
  const double r0 = ap.rmin[si], r1 = ap.rmax[si];
  if (ap.area_uniform) radius = mx::sqrt_fast(r0 * r0 + (r1 * r1 - r0 * r0) * rng.uniform());
  else radius = r0 + (r1 - r0) * rng.uniform();
  double theta;
  for (int guard = 0;; guard++) {
    theta = rng.uniform();
    const unsigned quad = mx::quarter_of(theta);
    if (rng.overrun || guard >= 64) return false;
    if (ap.shutter[si] & (1u << quad)) break;
  }
  double st, ct;
  mx::sincospi_fast(fma(theta, 2.0, -0.25), &st, &ct);   // angle 2 pi (u - 1/8)
  ry = radius * st;
  rz = radius * ct;
  return true;
}

// Nearest pixel and the ray's offset from it on both axes; false when the
// ray's 11 x 11 window misses the image.
__device__ __forceinline__ bool splat_origin(const ImageGeom &g, double y, double z, int &ic, int &jc, float &fu,
                                             float &fv) {
  const double u = mxd::pixel_coord(y, g.cy, g.inv_pitch, g.cx_pix);
  const double v = mxd::pixel_coord(z, g.cz, g.inv_pitch, g.cz_pix);
  if (!(u > -(mxd::HALF + 1.0) && u < g.nx + (double) mxd::HALF && v > -(mxd::HALF + 1.0) &&
        v < g.ny + (double) mxd::HALF))
    return false;
  const double uc = floor(u + 0.5), vc = floor(v + 0.5);
  ic = (int) uc; jc = (int) vc;
  fu = (float) (u - uc); fv = (float) (v - vc);
  return true;
}

__device__ __forceinline__ float tap(const ImageGeom &g, int k, float f) {
  const float d = FSUB((float) (k - mxd::HALF), f);
  return FMUL(g.knorm, mxd::exp_neg(FMUL(FMUL(d, d), g.half_inv_s2)));
}

}  // namespace

// ------------------------------------------------------------ forward --
namespace {

// Splat the warp's rays: lane L's ray is valid when valid is set, with its
// window origin and taps computed by that lane into its stage row; then
// the warp adds the 121 taps of each valid ray together.
__device__ __forceinline__ void splat_warp(const ImageGeom &g, bool valid, double y, double z, double w,
                                           uint32_t *stage, unsigned long long *win, unsigned long long *acc,
                                           int lane) {
  int ic = 0, jc = 0;
  float fu = 0.f, fv = 0.f;
  if (valid) valid = w > 0.0 && splat_origin(g, y, z, ic, jc, fu, fv);
  if (valid) {
    uint32_t *row = stage + lane * STAGE_STRIDE;
    const uint32_t wq = __double2uint_rn(fmin(MX_DMUL(w, 2147483648.0), 4294967295.0));   // w 2^31
    row[0] = (uint32_t) ic;
    row[1] = (uint32_t) jc;
#pragma unroll
    for (int k = 0; k < mxd::TAPS; k++) {
      const uint32_t gy = __float2uint_rn(FMUL(tap(g, k, fu), 2147483648.0f));   // K 2^31
      row[2 + k] = (uint32_t) (((unsigned long long) wq * gy) >> 32);             // w K 2^30
      row[2 + mxd::TAPS + k] = __float2uint_rn(FMUL(tap(g, k, fv), 2147483648.0f));
    }
  }
  __syncwarp();
  unsigned vm = __ballot_sync(0xffffffffu, valid);
  while (vm) {
    const int r = __ffs(vm) - 1;
    vm &= vm - 1;
    const uint32_t *row = stage + r * STAGE_STRIDE;
    const int ric = (int) row[0], rjc = (int) row[1];
    for (int t = lane; t < mxd::TAPS * mxd::TAPS; t += 32) {
      const int kz = t / mxd::TAPS, ky = t - mxd::TAPS * kz;
      const int col = ric - mxd::HALF + ky, rr = rjc - mxd::HALF + kz;
      if ((unsigned) col < (unsigned) g.nx && (unsigned) rr < (unsigned) g.ny) {
        const unsigned long long c = ((unsigned long long) row[2 + ky] * row[2 + mxd::TAPS + kz]) >> g.shift;
        if (c) {
          const unsigned wc = (unsigned) (col - g.wx0), wr = (unsigned) (rr - g.wy0);
          if (wc < (unsigned) g.wnx && wr < (unsigned) g.wny) atomicAdd(win + wr * g.wnx + wc, c);
          else atomicAdd(acc + (size_t) rr * g.nx + col, c);
        }
      }
    }
  }
  __syncwarp();
}

// SPLAT: accumulate the image; otherwise write each ray's y, z, w.
// part[block][4]: the block's sum w, sum w y, sum w z and hits.
template <bool SPLAT>
__global__ void __launch_bounds__(DBLOCK) diff_forward_kernel(const __grid_constant__ FwdArgs args, const __grid_constant__ MxTables T,
                                                               uint64_t n, uint64_t seed, uint8_t *codes, int mode,
                                                               unsigned long long *acc, double *part, double *yzw) {
  extern __shared__ __align__(16) unsigned char smem[];
  FwdArgs &A = *reinterpret_cast<FwdArgs *>(smem);
  unsigned long long *win = reinterpret_cast<unsigned long long *>(smem + align_up(sizeof(FwdArgs)));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t *stage = reinterpret_cast<uint32_t *>(win + (SPLAT ? WIN * WIN : 0)) + warp * 32 * STAGE_STRIDE;
  {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&args);
    uint32_t *dst = reinterpret_cast<uint32_t *>(smem);
    for (int k = threadIdx.x; k < (int) (sizeof(FwdArgs) / 4); k += DBLOCK) dst[k] = src[k];
    if (SPLAT)
      for (int k = threadIdx.x; k < WIN * WIN; k += DBLOCK) win[k] = 0ull;
  }
  __syncthreads();
  const bool replay = mode == MX_DIFF_REPLAY;
  const StrutTest struts{&T};
  mxd::V3<double> p0 = mxd::v3<double>(A.p0[0], A.p0[1], A.p0[2]);
  double sw = 0.0, swy = 0.0, swz = 0.0, hits = 0.0;
  const uint64_t step = (uint64_t) gridDim.x * DWARPS * 32;
  for (uint64_t base = ((uint64_t) blockIdx.x * DWARPS + warp) * 32; base < n; base += step) {
    const uint64_t i = base + lane;
    bool hit = false;
    double y = 0.0, z = 0.0, w = 0.0;
    if (i < n) {
      uint8_t code = replay ? codes[i] : 0;
      int si;
      double ry, rz;
      if (aperture(A.ap, seed, (uint32_t) i, si, ry, rz))
        hit = mxd::weighted_ray<double>(A.opt[si][0], A.opt[si][1], A.mid[si], A.rc[si], ry, rz, p0, replay, code, struts,
                                        y, z, w);
      else
        code = 0;
      if (mode == MX_DIFF_RECORD) codes[i] = code;
      if (hit) {
        w = w * A.vig;
        sw += w; swy += w * y; swz += w * z; hits += 1.0;
      }
      if (!SPLAT) {
        yzw[i] = hit ? y : __longlong_as_double(0x7ff8000000000000ll);
        yzw[n + i] = hit ? z : __longlong_as_double(0x7ff8000000000000ll);
        yzw[2 * n + i] = hit ? w : 0.0;
      }
    }
    if (SPLAT) splat_warp(A.g, hit, y, z, w, stage, win, acc, lane);
  }
  // block partial moments, fixed order
  for (int o = 16; o > 0; o >>= 1) {
    sw += __shfl_down_sync(0xffffffffu, sw, o);
    swy += __shfl_down_sync(0xffffffffu, swy, o);
    swz += __shfl_down_sync(0xffffffffu, swz, o);
    hits += __shfl_down_sync(0xffffffffu, hits, o);
  }
  __syncthreads();
  double *red = reinterpret_cast<double *>(win + (SPLAT ? WIN * WIN : 0));   // reuses the stage
  if (lane == 0) { red[4 * warp] = sw; red[4 * warp + 1] = swy; red[4 * warp + 2] = swz; red[4 * warp + 3] = hits; }
  if (SPLAT) {
    for (int k = threadIdx.x; k < A.g.wnx * A.g.wny; k += DBLOCK) {
      const unsigned long long v = win[k];
      if (v) atomicAdd(acc + (size_t) (A.g.wy0 + k / A.g.wnx) * A.g.nx + A.g.wx0 + k % A.g.wnx, v);
    }
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int k = 0; k < DWARPS; k++) s += red[4 * k + threadIdx.x];
    part[4 * blockIdx.x + threadIdx.x] = s;
  }
}

// image = acc 2^(shift - 61) / n_rays
__global__ void diff_image_kernel(const unsigned long long *acc, size_t npix, double scale, double *image) {
  for (size_t k = (size_t) blockIdx.x * blockDim.x + threadIdx.x; k < npix; k += (size_t) gridDim.x * blockDim.x)
    image[k] = (double) acc[k] * scale;
}

// out[v] = scale * sum over b of part[b * nv + v], in block order.
__global__ void diff_sum_kernel(const double *part, int nblocks, int nv, double scale, double *out) {
  const int v = threadIdx.x;
  if (v >= nv) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; b++) s += part[(size_t) b * nv + v];
  out[v] = s * scale;
}

// loss = mean (image - target)^2 and, optionally, its gradient; one block,
// fixed reduction order.
__global__ void __launch_bounds__(1024) diff_mse_kernel(const double *image, const double *target, size_t npix,
                                                        double *dl, double *loss) {
  __shared__ double red[32];
  double s = 0.0;
  const double inv = 1.0 / (double) npix;
  for (size_t k = threadIdx.x; k < npix; k += blockDim.x) {
    const double r = image[k] - target[k];
    s += r * r;
    if (dl) dl[k] = 2.0 * r * inv;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int) (blockDim.x >> 5); k++) t += red[k];
    *loss = t * inv;
  }
}

}  // namespace

// ------------------------------------------------------------ adjoint --
namespace {

// dl/dimage at pixel (row, col): from the shared window, else from global
// memory, 0 outside the image.
__device__ __forceinline__ float resid_at(const ImageGeom &g, const float *rw, const double *dl, int row, int col) {
  const unsigned wc = (unsigned) (col - g.wx0), wr = (unsigned) (row - g.wy0);
  if (wc < (unsigned) g.wnx && wr < (unsigned) g.wny) return rw[wr * (WIN + 1) + wc];
  if ((unsigned) col < (unsigned) g.nx && (unsigned) row < (unsigned) g.ny)
    return (float) __ldg(dl + (size_t) row * g.nx + col);
  return 0.f;
}

// part[block][NP] = sum over the block's rays of dl/dimage . d(image)/dtheta
// (before the 1/n_rays factor).  Compiled for two resident blocks per SM
// (128 registers): the tangents then spill about 600 bytes per thread to
// local memory, but twice the warps hide the FP64 and load latencies that
// left one block of 248 registers 43 % FP64-busy (2.45 -> 1.83 ms per 4e6
// rays).
__global__ void __launch_bounds__(DBLOCK, 2) diff_adjoint_kernel(const __grid_constant__ AdjArgs args, uint64_t n,
                                                               uint64_t seed, const uint8_t *codes,
                                                               const double *dl, double *part) {
  extern __shared__ __align__(16) unsigned char smem[];
  AdjArgs &A = *reinterpret_cast<AdjArgs *>(smem);
  float *rw = reinterpret_cast<float *>(smem + align_up(sizeof(AdjArgs)));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *stage = rw + WIN * (WIN + 1) + warp * 32 * ADJ_STAGE;
  {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&args);
    uint32_t *dst = reinterpret_cast<uint32_t *>(smem);
    for (int k = threadIdx.x; k < (int) (sizeof(AdjArgs) / 4); k += DBLOCK) dst[k] = src[k];
    for (int k = threadIdx.x; k < args.g.wnx * args.g.wny; k += DBLOCK) {
      const int r = k / args.g.wnx, c = k - r * args.g.wnx;
      rw[r * (WIN + 1) + c] = (float) dl[(size_t) (args.g.wy0 + r) * args.g.nx + args.g.wx0 + c];
    }
  }
  __syncthreads();
  const ImageGeom &g = A.g;
  const mxd::V3<Dual6> p0 = mxd::v3<Dual6>(A.p0[0], A.p0[1], A.p0[2]);
  const StrutTest none{nullptr};   // decisions are replayed: the strut test is never called
  uint32_t *list = reinterpret_cast<uint32_t *>(rw + WIN * (WIN + 1) + DWARPS * 32 * ADJ_STAGE);   // ADJ_TILE entries
  uint32_t *wcnt = list + ADJ_TILE;                                                 // DWARPS entries
  double pacc = 0.0;               // lane p < NP: this warp's sum for parameter p
  for (uint64_t tile = (uint64_t) blockIdx.x * ADJ_TILE; tile < n; tile += (uint64_t) gridDim.x * ADJ_TILE) {
    // The rays of the tile that reached the focal plane, in ascending order:
    // only they contribute, and lanes given the others would idle through
    // the whole ray.
    uint32_t nh = 0;
    for (int j = 0; j < ADJ_TILE / DBLOCK; j++) {
      const uint64_t i = tile + (uint64_t) j * DBLOCK + threadIdx.x;
      const bool hit = i < n && (codes[i] & mxd::RAY_HIT);
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (lane == 0) wcnt[warp] = (uint32_t) __popc(m);
      __syncthreads();
      uint32_t off = nh, tot = nh;
      for (int k = 0; k < DWARPS; k++) {
        const uint32_t c = wcnt[k];
        off += k < warp ? c : 0u;
        tot += c;
      }
      if (hit) list[off + __popc(m & ((1u << lane) - 1u))] = (uint32_t) (i - tile);
      __syncthreads();
      nh = tot;
    }
    for (uint32_t b0 = 0; b0 < nh; b0 += DBLOCK) {
      const uint32_t kk = b0 + threadIdx.x;
      const bool valid = kk < nh;
      if (!__any_sync(0xffffffffu, valid)) continue;   // the warp has no ray in this round
      const uint64_t i = valid ? tile + list[kk] : 0;
      float c6[mxd::ND];
#pragma unroll
      for (int k = 0; k < mxd::ND; k++) c6[k] = 0.f;
      int si = -1;
      uint8_t code = valid ? codes[i] : 0;
      double ry, rz;
      if (valid && aperture(A.ap, seed, (uint32_t) i, si, ry, rz)) {
        Dual6 y, z, w;
        int ic, jc;
        float fu, fv;
        if (mxd::weighted_ray<Dual6>(A.opt[si][0], A.opt[si][1], A.mid[si], A.rc[si], ry, rz, p0, true, code, none, y,
                                     z, w) &&
            w.v > 0.0 && splat_origin(g, y.v, z.v, ic, jc, fu, fv)) {
          float ky[mxd::TAPS], kyd[mxd::TAPS], kz[mxd::TAPS], kzd[mxd::TAPS];
#pragma unroll
          for (int k = 0; k < mxd::TAPS; k++) {
            ky[k] = tap(g, k, fu);
            kyd[k] = ((float) (k - mxd::HALF) - fu) * g.inv_s2 * ky[k];
            kz[k] = tap(g, k, fv);
            kzd[k] = ((float) (k - mxd::HALF) - fv) * g.inv_s2 * kz[k];
          }
          float sw = 0.f, su = 0.f, sv = 0.f;
          const bool inside = ic - mxd::HALF >= g.wx0 && ic + mxd::HALF < g.wx0 + g.wnx &&
                              jc - mxd::HALF >= g.wy0 && jc + mxd::HALF < g.wy0 + g.wny;
          if (inside) {
            const float *base_row = rw + (jc - mxd::HALF - g.wy0) * (WIN + 1) + (ic - mxd::HALF - g.wx0);
#pragma unroll
            for (int a = 0; a < mxd::TAPS; a++) {
              const float *q = base_row + a * (WIN + 1);
              float t = 0.f, td = 0.f;
#pragma unroll
              for (int b = 0; b < mxd::TAPS; b++) { t += q[b] * ky[b]; td += q[b] * kyd[b]; }
              sw += kz[a] * t; su += kz[a] * td; sv += kzd[a] * t;
            }
          } else {
#pragma unroll
            for (int a = 0; a < mxd::TAPS; a++) {
              float t = 0.f, td = 0.f;
#pragma unroll
              for (int b = 0; b < mxd::TAPS; b++) {
                const float r = resid_at(g, rw, dl, jc - mxd::HALF + a, ic - mxd::HALF + b);
                t += r * ky[b]; td += r * kyd[b];
              }
              sw += kz[a] * t; su += kz[a] * td; sv += kzd[a] * t;
            }
          }
          const float vig = (float) A.vig, wv = (float) w.v * vig, ip = (float) g.inv_pitch;
#pragma unroll
          for (int k = 0; k < mxd::ND; k++) c6[k] = vig * sw * w.d[k] + wv * ip * (su * y.d[k] + sv * z.d[k]);
        } else
          si = -1;
      }
      float *row = stage + lane * ADJ_STAGE;
#pragma unroll
      for (int k = 0; k < mxd::ND; k++) row[k] = c6[k];
      row[mxd::ND] = __int_as_float(si);
      __syncwarp();
      if (lane < NP) {
        // lanes 0..15: shell lane/4, slot lane%4; lanes 16, 17: source slots 4, 5
        const int want = lane < 16 ? (lane >> 2) : -2, slot = lane < 16 ? (lane & 3) : lane - 12;
        float s = 0.f;
        for (int r = 0; r < 32; r++) {
          const float *q = stage + r * ADJ_STAGE;
          const int sr = __float_as_int(q[mxd::ND]);
          if (sr == want || (want == -2 && sr >= 0)) s += q[slot];
        }
        pacc += (double) s;
      }
      __syncwarp();
    }
    __syncthreads();   // the list is refilled for the next tile
  }
  __syncthreads();
  double *red = reinterpret_cast<double *>(rw);   // the window is no longer read
  if (lane < NP) red[warp * NP + lane] = pacc;
  __syncthreads();
  if (threadIdx.x < NP) {
    double s = 0.0;
    for (int k = 0; k < DWARPS; k++) s += red[k * NP + threadIdx.x];
    part[(size_t) blockIdx.x * NP + threadIdx.x] = s;
  }
}

}  // namespace

// --------------------------------------------------------------- host --
struct mx_diff {
  mx_context *ctx = nullptr;
  mx_diff_config cfg;
  ImageGeom g;
  Aperture ap;
  mxd::RayConst rc[4];
  double vig = 1.0;
  DevBuf codes, acc, part, out;   // out: 4 moments, then NP gradient values
  double *h_out = nullptr;        // pinned: moments and gradient read back
  bool recorded = false;
  int fwd_blocks = 0, rays_blocks = 0, adj_blocks = 0;
  size_t fwd_smem = 0, rays_smem = 0, adj_smem = 0;
};

namespace {

constexpr double PI_D = 3.14159265358979323846264338327950288;
constexpr double ARCSEC = PI_D / (180.0 * 3600.0);

int diff_fail(mx_diff *d, int code, const std::string &msg) { return mx_fail(d ? d->ctx : nullptr, code, msg); }

// Both optics of every shell at theta, with derivatives: tilts enter az_mis
// and el_mis (degrees in the geometry file) and decenters x0 and y0 (mm),
// as read_hrma_geometry_file (hrma.c:319-391) and init_hrma_shells take
// them; the rotations are rebuilt as init_yaw_pitch does.
int build_optics(mx_diff *d, const double *theta, mxd::Optic<Dual6> opt[4][2], mxd::Between<Dual6> mid[4],
                 Dual6 p0[3]) {
  mx_context *c = d->ctx;
  std::string err;
  size_t cnt = 0;
  const double *rdb = c->pack.get<double>("hrma/rdb", &cnt, err);
  if (!rdb || cnt != 72) return diff_fail(d, MX_EPACK, "mx_diff: hrma/rdb missing from the table pack");
  for (int s = 0; s < 4; s++) {
    const MxShellDev &h = c->hm.shells[s];
    const double cap_pos = c->cfg.hrma_cap_x + c->cfg.shell_xoffset[s];
    for (int o = 0; o < 2; o++) {
      const double *q = rdb + (4 * o + s) * 9;   // x0 y0 z0 p k rho0 az el l
      mxd::Optic<Dual6> &op = opt[s][o];
      op.a = h.a[o]; op.b = h.b[o]; op.c = h.c[o]; op.xmin = h.xmin[o]; op.xmax = h.xmax[o];
      Dual6 x0 = mxd::mkd(q[0] + theta[4 * s + 2] * 1e-3);
      x0.d[2] = 1e-3f;
      Dual6 y0 = mxd::mkd(q[1] + theta[4 * s + 3] * 1e-3);
      y0.d[3] = 1e-3f;
      op.to[0] = mxd::mkd(-(-q[2]) - cap_pos);
      op.to[1] = 0.0 - x0;
      op.to[2] = y0;
      Dual6 az = mxd::mkd(-(q[6] + theta[4 * s] / 3600.0) * (PI_D / 180.0));
      az.d[0] = (float) -ARCSEC;
      Dual6 el = mxd::mkd(-(q[7] + theta[4 * s + 1] / 3600.0) * (PI_D / 180.0));
      el.d[1] = (float) -ARCSEC;
      mxd::yaw_pitch<Dual6>(op.fwd, op.bwd, az, el);
      for (int r = 0; r < 3; r++) op.ff[r] = op.fwd[3 * r] * (h.front_position + op.to[0]);
    }
    const mxd::Optic<Dual6> &P = opt[s][0], &H = opt[s][1];
    mxd::Between<Dual6> &B = mid[s];
    mxd::mat3_mul<Dual6>(B.m, H.fwd, P.bwd);
    const Dual6 dt[3] = {H.to[0] - P.to[0], H.to[1] - P.to[1], H.to[2] - P.to[2]};
    for (int r = 0; r < 3; r++) B.c[r] = H.fwd[3 * r] * dt[0] + H.fwd[3 * r + 1] * dt[1] + H.fwd[3 * r + 2] * dt[2];
    for (int k = 0; k < 9; k++) B.bwdf[k] = (float) P.bwd[k].v;
    for (int r = 0; r < 3; r++) B.tof[r] = (float) P.to[r].v;
  }
  Dual6 ay = mxd::mkd((d->cfg.src_y + theta[16]) * ARCSEC);
  ay.d[4] = (float) ARCSEC;
  Dual6 az = mxd::mkd((d->cfg.src_z + theta[17]) * ARCSEC);
  az.d[5] = (float) ARCSEC;
  mxd::V3<Dual6> p = mxd::unit(mxd::v3<Dual6>(mxd::mkd(-1.0), 0.0 - mxd::dtan(ay), 0.0 - mxd::dtan(az)));
  p0[0] = p.x; p0[1] = p.y; p0[2] = p.z;
  return MX_OK;
}

int check_theta(mx_diff *d, const double *theta) {
  if (!theta) return diff_fail(d, MX_EINVAL, "mx_diff: theta is null");
  for (int k = 0; k < NP; k++)
    if (!std::isfinite(theta[k]) || fabs(theta[k]) > 3600.0)
      return diff_fail(d, MX_EINVAL, "mx_diff: theta[" + std::to_string(k) + "] must be finite and within +-3600");
  return MX_OK;
}

int fill_fwd(mx_diff *d, const double *theta, FwdArgs &F) {
  mxd::Optic<Dual6> opt[4][2];
  mxd::Between<Dual6> mid[4];
  Dual6 p0[3];
  int r = build_optics(d, theta, opt, mid, p0);
  if (r) return r;
  memset(&F, 0, sizeof(F));
  for (int s = 0; s < 4; s++) {
    for (int k = 0; k < 9; k++) F.mid[s].m[k] = mid[s].m[k].v;
    for (int k = 0; k < 3; k++) F.mid[s].c[k] = mid[s].c[k].v;
    for (int k = 0; k < 9; k++) F.mid[s].bwdf[k] = mid[s].bwdf[k];
    for (int k = 0; k < 3; k++) F.mid[s].tof[k] = mid[s].tof[k];
  }
  for (int s = 0; s < 4; s++)
    for (int o = 0; o < 2; o++) {
      const mxd::Optic<Dual6> &a = opt[s][o];
      mxd::Optic<double> &b = F.opt[s][o];
      b.a = a.a; b.b = a.b; b.c = a.c; b.xmin = a.xmin; b.xmax = a.xmax;
      for (int k = 0; k < 3; k++) b.to[k] = a.to[k].v;
      for (int k = 0; k < 9; k++) { b.fwd[k] = a.fwd[k].v; b.bwd[k] = a.bwd[k].v; }
      for (int k = 0; k < 3; k++) b.ff[k] = a.ff[k].v;
    }
  for (int s = 0; s < 4; s++) F.rc[s] = d->rc[s];
  F.ap = d->ap;
  for (int k = 0; k < 3; k++) F.p0[k] = p0[k].v;
  F.vig = d->vig;
  F.g = d->g;
  return MX_OK;
}

int fill_adj(mx_diff *d, const double *theta, AdjArgs &A) {
  memset(&A, 0, sizeof(A));
  int r = build_optics(d, theta, A.opt, A.mid, A.p0);
  if (r) return r;
  for (int s = 0; s < 4; s++) A.rc[s] = d->rc[s];
  A.ap = d->ap;
  A.vig = d->vig;
  A.g = d->g;
  return MX_OK;
}

template <class K>
cudaError_t occupancy(K kernel, size_t smem, int num_sms, int *blocks) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  if (e != cudaSuccess) return e;
  int per = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, DBLOCK, smem);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  *blocks = per * num_sms;
  return cudaSuccess;
}

}  // namespace

extern "C" {

mx_diff *mx_diff_create(mx_context *c, const mx_diff_config *cfg) {
  if (!c || !cfg) { mx_fail(c, MX_EINVAL, "mx_diff_create: null argument"); return nullptr; }
  const mx_diff_config &k = *cfg;
  std::string bad;
  if (k.n_rays < 1 || k.n_rays > MX_DIFF_MAX_RAYS) bad = "n_rays must be in 1 .. 2^32-1";
  else if (!(k.energy > 0.0) || !std::isfinite(k.energy)) bad = "energy must be positive";
  else if (!(k.pitch > 0.0) || !std::isfinite(k.pitch)) bad = "pitch must be positive";
  else if (!(k.sigma >= 0.5 && k.sigma <= 1.0)) bad = "sigma must be within 0.5 .. 1 pixel";
  else if (k.nx < 16 || k.nx > 4096 || k.ny < 16 || k.ny > 4096) bad = "nx and ny must be within 16 .. 4096";
  else if (!std::isfinite(k.src_y) || !std::isfinite(k.src_z) || fabs(k.src_y) > 3600.0 || fabs(k.src_z) > 3600.0)
    bad = "source angles must be finite and within +-3600 arcsec";
  else if (!std::isfinite(k.center_y) || !std::isfinite(k.center_z)) bad = "image centre must be finite";
  else if (c->T.source_distance > 0.0) bad = "weighted rays need a source at infinity (SourceDistance 0)";
  if (!bad.empty()) { mx_fail(c, MX_EINVAL, "mx_diff_create: " + bad); return nullptr; }

  mx_diff *d = new mx_diff();
  d->ctx = c;
  d->cfg = k;
  ImageGeom &g = d->g;
  memset(&g, 0, sizeof(g));
  g.nx = (int) k.nx; g.ny = (int) k.ny;
  g.wnx = g.nx < WIN ? g.nx : WIN; g.wny = g.ny < WIN ? g.ny : WIN;
  g.wx0 = g.nx / 2 - g.wnx / 2; g.wy0 = g.ny / 2 - g.wny / 2;
  g.cy = k.center_y; g.cz = k.center_z;
  g.inv_pitch = 1.0 / k.pitch;
  g.cx_pix = 0.5 * g.nx - 0.5; g.cz_pix = 0.5 * g.ny - 0.5;
  g.half_inv_s2 = (float) (0.5 / (k.sigma * k.sigma));
  g.inv_s2 = (float) (1.0 / (k.sigma * k.sigma));
  g.knorm = (float) (1.0 / (std::sqrt(2.0 * PI_D) * k.sigma));
  // Each tap product is below w K^2 2^61 with w < 2; a pixel sums at most
  // n_rays of them, so shifting by log2(n K^2 / 4) + 1 keeps it in 64 bits.
  const double kmax = g.knorm;
  int shift = (int) std::ceil(std::log2((double) k.n_rays * kmax * kmax / 4.0)) + 1;
  g.shift = shift < 0 ? 0 : shift;

  const MxTables &T = c->T;
  for (int s = 0; s < 4; s++) {
    const MxShellDev &h = c->hm.shells[s];
    d->ap.area[s] = h.area_fraction;
    d->ap.rmin[s] = h.min_radius;
    d->ap.rmax[s] = h.max_radius;
    d->ap.shutter[s] = h.shutter;
    mxd::RayConst &rc = d->rc[s];
    rc.front = h.front_position;
    rc.weighted = T.opt_n > 0;
    rc.beta = 0.0; rc.delta = 1.0; rc.corr = 1.0;
    if (rc.weighted) {
      // the optical constants and correction at the ray energy, as the
      // mirror stage interpolates them (float tables, float energy)
      const float fe = (float) k.energy;
      const float *optc = c->hm.optc.data();
      const double *slope = c->hm.optc_slope.data();
      const unsigned on = (unsigned) T.opt_n;
      rc.beta = mx::interp_f(fe, optc, optc + on, slope, on);
      rc.delta = mx::interp_f(fe, optc, optc + 2 * on, slope + (on - 1), on);
      if (T.use_scale) {
        const float *ce = optc + 3 * on + h.corr_off;
        rc.corr = std::sqrt((double) mx::interp_f(fe, ce, ce + h.corr_n, slope + h.corr_slope_off, (unsigned) h.corr_n));
      }
    }
  }
  d->ap.ideal = T.ideal;
  d->ap.area_uniform = T.area_uniform;
  d->vig = T.ideal ? 1.0 : T.hrma_vig;

  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) {
    d->fwd_smem = align_up(sizeof(FwdArgs)) + sizeof(unsigned long long) * WIN * WIN + 4 * DWARPS * 32 * STAGE_STRIDE;
    d->rays_smem = align_up(sizeof(FwdArgs)) + 4 * DWARPS * 32 * STAGE_STRIDE;
    d->adj_smem = align_up(sizeof(AdjArgs)) + 4 * WIN * (WIN + 1) + 4 * DWARPS * 32 * ADJ_STAGE + 4 * ADJ_TILE +
                  4 * DWARPS;
    e = occupancy(diff_forward_kernel<true>, d->fwd_smem, c->num_sms, &d->fwd_blocks);
  }
  if (e == cudaSuccess) e = occupancy(diff_forward_kernel<false>, d->rays_smem, c->num_sms, &d->rays_blocks);
  if (e == cudaSuccess) e = occupancy(diff_adjoint_kernel, d->adj_smem, c->num_sms, &d->adj_blocks);
  const int maxb = std::max(d->fwd_blocks, std::max(d->rays_blocks, d->adj_blocks));
  if (e == cudaSuccess) e = d->codes.ensure(k.n_rays);
  if (e == cudaSuccess) e = d->acc.ensure(sizeof(unsigned long long) * k.nx * k.ny);
  if (e == cudaSuccess) e = d->part.ensure(sizeof(double) * (size_t) maxb * NP);
  if (e == cudaSuccess) e = d->out.ensure(sizeof(double) * (4 + NP));
  if (e == cudaSuccess) e = cudaMallocHost(&d->h_out, sizeof(double) * (4 + NP));
  if (e == cudaSuccess) e = cudaMemset(d->codes.ptr, 0, k.n_rays);
  if (e != cudaSuccess) {
    mx_cuda_fail(c, e, "mx_diff_create");
    mx_diff_destroy(d);
    return nullptr;
  }
  return d;
}

void mx_diff_destroy(mx_diff *d) {
  if (!d) return;
  d->codes.release(); d->acc.release(); d->part.release(); d->out.release();
  if (d->h_out) cudaFreeHost(d->h_out);
  delete d;
}

int mx_diff_forward(mx_diff *d, const double *theta, int mode, double *image, double *moments, void *stream) {
  if (!d) return mx_fail(nullptr, MX_EINVAL, "mx_diff_forward: null handle");
  if (!image) return diff_fail(d, MX_EINVAL, "mx_diff_forward: image is null");
  if (mode != MX_DIFF_RECORD && mode != MX_DIFF_REPLAY && mode != MX_DIFF_FRESH)
    return diff_fail(d, MX_EINVAL, "mx_diff_forward: unknown mode");
  if (mode == MX_DIFF_REPLAY && !d->recorded)
    return diff_fail(d, MX_EINVAL, "mx_diff_forward: MX_DIFF_REPLAY before any MX_DIFF_RECORD call");
  int r = check_theta(d, theta);
  if (r) return r;
  FwdArgs F;
  if ((r = fill_fwd(d, theta, F))) return r;
  mx_context *c = d->ctx;
  cudaStream_t st = (cudaStream_t) stream;
  const size_t npix = (size_t) d->cfg.nx * d->cfg.ny;
  cudaError_t e = cudaMemsetAsync(d->acc.ptr, 0, npix * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_diff_forward");
  diff_forward_kernel<true><<<d->fwd_blocks, DBLOCK, d->fwd_smem, st>>>(
      F, c->T, d->cfg.n_rays, d->cfg.seed, (uint8_t *) d->codes.ptr, mode, (unsigned long long *) d->acc.ptr,
      (double *) d->part.ptr, nullptr);
  const double scale = std::ldexp(1.0, d->g.shift - 61) / (double) d->cfg.n_rays;
  diff_image_kernel<<<2 * c->num_sms, 256, 0, st>>>((const unsigned long long *) d->acc.ptr, npix, scale, image);
  diff_sum_kernel<<<1, 32, 0, st>>>((const double *) d->part.ptr, d->fwd_blocks, 4, 1.0, (double *) d->out.ptr);
  c->launches += 3;
  if ((e = cudaGetLastError()) != cudaSuccess) return mx_cuda_fail(c, e, "mx_diff_forward: launch");
  if (mode == MX_DIFF_RECORD) d->recorded = true;
  if (moments) {
    e = cudaMemcpyAsync(d->h_out, d->out.ptr, 4 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_diff_forward: moments");
    memcpy(moments, d->h_out, 4 * sizeof(double));
  }
  return MX_OK;
}

int mx_diff_rays(mx_diff *d, const double *theta, int mode, double *yzw, void *stream) {
  if (!d) return mx_fail(nullptr, MX_EINVAL, "mx_diff_rays: null handle");
  if (!yzw) return diff_fail(d, MX_EINVAL, "mx_diff_rays: yzw is null");
  if (mode != MX_DIFF_RECORD && mode != MX_DIFF_REPLAY && mode != MX_DIFF_FRESH)
    return diff_fail(d, MX_EINVAL, "mx_diff_rays: unknown mode");
  if (mode == MX_DIFF_REPLAY && !d->recorded)
    return diff_fail(d, MX_EINVAL, "mx_diff_rays: MX_DIFF_REPLAY before any MX_DIFF_RECORD call");
  int r = check_theta(d, theta);
  if (r) return r;
  FwdArgs F;
  if ((r = fill_fwd(d, theta, F))) return r;
  mx_context *c = d->ctx;
  cudaStream_t st = (cudaStream_t) stream;
  diff_forward_kernel<false><<<d->rays_blocks, DBLOCK, d->rays_smem, st>>>(
      F, c->T, d->cfg.n_rays, d->cfg.seed, (uint8_t *) d->codes.ptr, mode, nullptr, (double *) d->part.ptr, yzw);
  c->launches += 1;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mx_cuda_fail(c, e, "mx_diff_rays: launch");
  if (mode == MX_DIFF_RECORD) d->recorded = true;
  return MX_OK;
}

int mx_diff_mse(mx_diff *d, const double *image, const double *target, double *dl_dimage, double *loss,
                void *stream) {
  if (!d) return mx_fail(nullptr, MX_EINVAL, "mx_diff_mse: null handle");
  if (!image || !target || !loss) return diff_fail(d, MX_EINVAL, "mx_diff_mse: image, target and loss are required");
  diff_mse_kernel<<<1, 1024, 0, (cudaStream_t) stream>>>(image, target, (size_t) d->cfg.nx * d->cfg.ny, dl_dimage, loss);
  d->ctx->launches += 1;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MX_OK : mx_cuda_fail(d->ctx, e, "mx_diff_mse: launch");
}

int mx_diff_adjoint_async(mx_diff *d, const double *theta, const double *dl_dimage, double *grad_dev, void *stream) {
  if (!d) return mx_fail(nullptr, MX_EINVAL, "mx_diff_adjoint: null handle");
  if (!dl_dimage || !grad_dev) return diff_fail(d, MX_EINVAL, "mx_diff_adjoint: dl_dimage and grad are required");
  if (!d->recorded) return diff_fail(d, MX_EINVAL, "mx_diff_adjoint: no MX_DIFF_RECORD call yet");
  int r = check_theta(d, theta);
  if (r) return r;
  AdjArgs A;
  if ((r = fill_adj(d, theta, A))) return r;
  mx_context *c = d->ctx;
  cudaStream_t st = (cudaStream_t) stream;
  diff_adjoint_kernel<<<d->adj_blocks, DBLOCK, d->adj_smem, st>>>(A, d->cfg.n_rays, d->cfg.seed,
                                                                   (const uint8_t *) d->codes.ptr, dl_dimage,
                                                                   (double *) d->part.ptr);
  diff_sum_kernel<<<1, 32, 0, st>>>((const double *) d->part.ptr, d->adj_blocks, NP, 1.0 / (double) d->cfg.n_rays,
                                    grad_dev);
  c->launches += 2;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MX_OK : mx_cuda_fail(c, e, "mx_diff_adjoint: launch");
}

int mx_diff_adjoint(mx_diff *d, const double *theta, const double *dl_dimage, double *grad, void *stream) {
  if (!d) return mx_fail(nullptr, MX_EINVAL, "mx_diff_adjoint: null handle");
  if (!grad) return diff_fail(d, MX_EINVAL, "mx_diff_adjoint: grad is null");
  double *gdev = (double *) d->out.ptr + 4;
  int r = mx_diff_adjoint_async(d, theta, dl_dimage, gdev, stream);
  if (r) return r;
  cudaStream_t st = (cudaStream_t) stream;
  cudaError_t e = cudaMemcpyAsync(d->h_out + 4, gdev, NP * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return mx_cuda_fail(d->ctx, e, "mx_diff_adjoint: reading the gradient");
  memcpy(grad, d->h_out + 4, NP * sizeof(double));
  return MX_OK;
}

}  // extern "C"
