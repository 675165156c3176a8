// Weighted-ray trace for the differentiable form.
//
// A weighted ray takes the aperture point a photon of the same tag would
// take in the plain trace (project_photon_to_hrma, hrma.c:984-1050), then
// follows the HRMA geometry (compute_conic_intersection hrma.c:411-478,
// reflect_from_conic hrma.c:488-545, _marx_hrma_mirror_reflect
// hrma.c:1183-1339) without normal blur or scattering, and is projected
// onto the focal plane x = 0.  Instead of being absorbed at random it
// carries a weight: vignetting times, at each reflection, the Fresnel
// reflectivity (reflect.c:39-77) times the effective-area correction.
//
// The trace is written once over a scalar type S.  S = double gives the
// forward ray; S = Dual6 carries with each FP64 value its FP32 derivatives
// with respect to the six parameters that can move this ray: its shell's
// two tilts and two decenters and the source's two angular offsets.
#pragma once
#include <stdint.h>

#include <cmath>
#include <type_traits>

#include "mx_device.cuh"

#ifdef __CUDACC__
#define MXG __host__ __device__ __forceinline__
#else
#define MXG inline
#endif

namespace mxd {

constexpr int ND = 6;   // tangent slots: tilt az, tilt el, decenter x, decenter y, source y, source z

struct Dual6 {
  double v;
  float d[ND];
};

// A value rounded to single precision for the tangents, which are single
// precision anyway: on the device by truncation on the integer pipe (a
// conversion instruction would take an FP64-pipe slot).
MXG float tof(double x) {
#ifdef __CUDA_ARCH__
  return mx::d2f_trunc(x);
#else
  return (float) x;
#endif
}

MXG double val(double a) { return a; }
MXG double val(const Dual6 &a) { return a.v; }

MXG Dual6 mkd(double v) {
  Dual6 r; r.v = v;
  for (int k = 0; k < ND; k++) r.d[k] = 0.f;
  return r;
}
MXG Dual6 operator+(const Dual6 &a, const Dual6 &b) {
  Dual6 r; r.v = a.v + b.v;
  for (int k = 0; k < ND; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
MXG Dual6 operator-(const Dual6 &a, const Dual6 &b) {
  Dual6 r; r.v = a.v - b.v;
  for (int k = 0; k < ND; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
MXG Dual6 operator-(const Dual6 &a) {
  Dual6 r; r.v = -a.v;
  for (int k = 0; k < ND; k++) r.d[k] = -a.d[k];
  return r;
}
MXG Dual6 operator*(const Dual6 &a, const Dual6 &b) {
  Dual6 r; r.v = a.v * b.v;
  const float av = tof(a.v), bv = tof(b.v);
  for (int k = 0; k < ND; k++) r.d[k] = av * b.d[k] + bv * a.d[k];
  return r;
}
MXG Dual6 operator*(double s, const Dual6 &a) {
  Dual6 r; r.v = s * a.v;
  const float f = tof(s);
  for (int k = 0; k < ND; k++) r.d[k] = f * a.d[k];
  return r;
}
MXG Dual6 operator*(const Dual6 &a, double s) { return s * a; }
MXG Dual6 operator+(const Dual6 &a, double s) { Dual6 r = a; r.v = a.v + s; return r; }
MXG Dual6 operator+(double s, const Dual6 &a) { Dual6 r = a; r.v = s + a.v; return r; }
MXG Dual6 operator-(const Dual6 &a, double s) { Dual6 r = a; r.v = a.v - s; return r; }
MXG Dual6 operator-(double s, const Dual6 &a) {
  Dual6 r; r.v = s - a.v;
  for (int k = 0; k < ND; k++) r.d[k] = -a.d[k];
  return r;
}
MXG Dual6 operator/(const Dual6 &a, const Dual6 &b) {
  Dual6 r; r.v = a.v / b.v;
  const float ib = 1.0f / tof(b.v), q = tof(r.v);
  for (int k = 0; k < ND; k++) r.d[k] = (a.d[k] - q * b.d[k]) * ib;
  return r;
}
MXG Dual6 operator/(double s, const Dual6 &b) {
  Dual6 r; r.v = s / b.v;
  const float g = -tof(r.v) / tof(b.v);
  for (int k = 0; k < ND; k++) r.d[k] = g * b.d[k];
  return r;
}
MXG Dual6 operator/(const Dual6 &a, double s) {
  Dual6 r; r.v = a.v / s;
  const float f = 1.0f / tof(s);
  for (int k = 0; k < ND; k++) r.d[k] = a.d[k] * f;
  return r;
}
// 1 / a: for the double rays the Newton-Raphson reciprocal (within one ulp)
MXG double drcp(double a) { return mx::rcp_fast(a); }
MXG Dual6 drcp(const Dual6 &a) { return 1.0 / a; }
// a < b and a == 0 on the values, on the integer pipe
MXG bool vlt(double a, double b) { return mx::dkey(a) < mx::dkey(b); }
MXG bool vzero(double a) { return mx::is_zero(a); }
MXG double dsqrt(double a) { return sqrt(a); }
MXG Dual6 dsqrt(const Dual6 &a) {
  Dual6 r; r.v = sqrt(a.v);
  const float h = 0.5f / tof(r.v);
  for (int k = 0; k < ND; k++) r.d[k] = h * a.d[k];
  return r;
}
// 1 / sqrt(a): one reciprocal square root instead of a square root and a
// division (normalisations, the Fresnel root).
MXG double drsqrt(double a) { return mx::mx_rsqrt(a); }
MXG Dual6 drsqrt(const Dual6 &a) {
  Dual6 r; r.v = mx::mx_rsqrt(a.v);
  const float t = tof(r.v), h = -0.5f * t * t * t;
  for (int k = 0; k < ND; k++) r.d[k] = h * a.d[k];
  return r;
}
MXG double dcopysign(double a, double b) { return copysign(a, b); }
MXG Dual6 dcopysign(const Dual6 &a, const Dual6 &b) { return (a.v < 0.0) != (b.v < 0.0) ? -a : a; }
MXG double dabs(double a) { return fabs(a); }
MXG Dual6 dabs(const Dual6 &a) { return a.v < 0.0 ? -a : a; }
MXG double dsin(double a) { return sin(a); }
MXG double dcos(double a) { return cos(a); }
MXG Dual6 dsin(const Dual6 &a) {
  Dual6 r; r.v = sin(a.v);
  const float c = cosf(tof(a.v));
  for (int k = 0; k < ND; k++) r.d[k] = c * a.d[k];
  return r;
}
MXG Dual6 dcos(const Dual6 &a) {
  Dual6 r; r.v = cos(a.v);
  const float s = -sinf(tof(a.v));
  for (int k = 0; k < ND; k++) r.d[k] = s * a.d[k];
  return r;
}
MXG double dtan(double a) { return tan(a); }
MXG Dual6 dtan(const Dual6 &a) {
  Dual6 r; r.v = tan(a.v);
  const float t = tof(r.v), s = 1.0f + t * t;
  for (int k = 0; k < ND; k++) r.d[k] = s * a.d[k];
  return r;
}

// A constant of type S (no derivatives).
template <class S> MXG S cst(double v);
template <> MXG double cst<double>(double v) { return v; }
template <> MXG Dual6 cst<Dual6>(double v) { return mkd(v); }

template <class S> struct V3 { S x, y, z; };
template <class S> MXG V3<S> v3(S x, S y, S z) { V3<S> r; r.x = x; r.y = y; r.z = z; return r; }
template <class S> MXG V3<S> operator+(const V3<S> &a, const V3<S> &b) { return v3<S>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class S> MXG V3<S> operator-(const V3<S> &a, const V3<S> &b) { return v3<S>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class S> MXG V3<S> scale(const S &s, const V3<S> &a) { return v3<S>(s * a.x, s * a.y, s * a.z); }
template <class S> MXG S dotp(const V3<S> &a, const V3<S> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class S> MXG V3<S> unit(const V3<S> &a) {
  S inv = drsqrt(dotp(a, a));
  return scale(inv, a);
}
template <class S> MXG V3<S> matv(const S *m, const V3<S> &v) {
  return v3<S>(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
               m[6] * v.x + m[7] * v.y + m[8] * v.z);
}

// ------------------------------------------------ HRMA optic geometry --
// One optic of one shell: conic x^2 + y^2 + z^2 = a x^2 + b x + c between
// xmin and xmax in its own frame, the MARX -> optic translation `to` and the
// pitch/yaw rotations fwd (into the optic's frame) and bwd (back).
template <class S> struct Optic {
  double a, b, c, xmin, xmax;
  S to[3];
  S fwd[9], bwd[9];
  S ff[3];   // fwd (front + to[0], 0, 0): the aperture plane's part of fwd (x + to)
};

// A shell's way from the paraboloid's frame to the hyperboloid's: back to
// the MARX frame (P.bwd, less P.to), then in (plus H.to, H.fwd) as one
// matrix and offset, x' = m x + c, p' = m p, with m = H.fwd P.bwd and
// c = H.fwd (H.to - P.to); and P.bwd, P.to in float for the cap struts'
// screen in that frame.
template <class S> struct Between {
  S m[9], c[3];
  float bwdf[9], tof[3];
};

// The rotation builders of init_yaw_pitch (hrma.c:842-880), over S.
template <class S> MXG void rot_z(S m[9], const S &theta) {
  S c = dcos(theta), s = 0.0 - dsin(theta);
  m[0] = c; m[1] = s; m[2] = cst<S>(0.0);
  m[3] = 0.0 - s; m[4] = c; m[5] = m[2];
  m[6] = m[2]; m[7] = m[2]; m[8] = cst<S>(1.0);
}
template <class S> MXG void rot_axis(S m[9], const S n[3], const S &theta) {
  S c = dcos(theta), s = dsin(theta), c1 = 1.0 - c;
  S n0 = n[0], n1 = n[1], n2 = n[2];
  S n01 = n0 * n1 * c1, n02 = n0 * n2 * c1, n12 = n1 * n2 * c1;
  m[0] = n0 * n0 * c1 + c; m[1] = n01 - s * n2; m[2] = n02 + s * n1;
  m[3] = n01 + s * n2; m[4] = n1 * n1 * c1 + c; m[5] = n12 - s * n0;
  m[6] = n02 - s * n1; m[7] = n12 + s * n0; m[8] = n2 * n2 * c1 + c;
}
template <class S> MXG void mat3_mul(S c[9], const S a[9], const S b[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
// fwd = R(ny, -el) Rz(-az) and bwd = Rz(az) R(ny, el), ny = Rz(-az) e_y, as
// the reference builds them from the geometry file's az_mis and el_mis.
template <class S> MXG void yaw_pitch(S fwd[9], S bwd[9], const S &az, const S &el) {
  S rz[9], ry[9], ny[3];
  rot_z(rz, 0.0 - az);
  ny[0] = rz[1]; ny[1] = rz[4]; ny[2] = rz[7];
  rot_axis(ry, ny, 0.0 - el);
  mat3_mul(fwd, ry, rz);
  rot_axis(ry, ny, el);
  rot_z(rz, az);
  mat3_mul(bwd, rz, ry);
}

// Fresnel reflectivity averaged over polarisations (reflect.c:39-77) for a
// grazing cosine cos_t and refractive index 1 - delta + i beta.
template <class S> MXG S fresnel(const S &cos_t, double beta, double delta) {
#ifdef __CUDA_ARCH__
  if constexpr (std::is_same<S, double>::value) {
    // the value alone: in double-float on the FP32 pipe (mx::reflectivity_df,
    // beta and delta are floats), within about 2^-40 of the expression below
    mx::F2 num, den;
    mx::reflectivity_df(cos_t, mx::d2f_trunc(beta), mx::d2f_trunc(delta), num, den);
    return mx::df_to(mx::df_div(num, den));
  }
#endif
  const double nr = 1.0 - delta, ni = beta;
  const double sr = nr * nr - ni * ni, si = 2.0 * nr * ni;
  S sin2 = 1.0 - cos_t * cos_t;
  S wr = sr - sin2;
  const double wi = si;
  // the principal square root of wr + i wi: with q^2 = h = (r + |wr|) / 2,
  // q = h / sqrt(h) and wi / (2 q) = (wi / 2) / sqrt(h), one reciprocal
  // square root for both
  S r = dsqrt(wr * wr + wi * wi);
  S rr, ri;
  if (val(wr) >= 0.0) {
    S h = 0.5 * (r + wr), inv = drsqrt(h);
    rr = h * inv; ri = (0.5 * wi) * inv;
  } else {
    S h = 0.5 * (r - wr), inv = drsqrt(h);
    rr = (0.5 * wi) * inv; ri = h * inv;
    if (val(rr) < 0.0) { rr = 0.0 - rr; ri = 0.0 - ri; }
  }
  S a1 = (cos_t - rr) * (cos_t - rr) + ri * ri, b1 = (cos_t + rr) * (cos_t + rr) + ri * ri;
  S pr = cos_t * sr, pi_ = cos_t * si;
  S a2 = (pr - rr) * (pr - rr) + (pi_ - ri) * (pi_ - ri);
  S b2 = (pr + rr) * (pr + rr) + (pi_ + ri) * (pi_ + ri);
  return 0.5 * (a1 * b2 + a2 * b1) / (b1 * b2);
}

// compute_conic_intersection (hrma.c:411-478) with the roots of
// JDMquadratic_root (qroot.c:36-70).  root < 0: choose as the reference does
// (a root inside [xmin, xmax), the larger x when both are) and report the
// choice in *chosen (0 = the -2c/(b f) root, 1 = the -b f/(2a) root).
// root 0 or 1: take that root without the x-limit test, so that the ray
// stays on the same branch while the optic moves.  Returns false on a miss.
template <class S>
MXG bool conic_hit(const Optic<S> &o, V3<S> &x0, const V3<S> &p, V3<S> &n, int root, int *chosen) {
  S t_plus = (0.0 - x0.x) * drcp(p.x);
  S x_y = x0.y + t_plus * p.y, x_z = x0.z + t_plus * p.z;
  S alpha = o.a * (p.x * p.x) - 1.0;
  S beta = o.b * p.x - 2.0 * (p.y * x_y + p.z * x_z);
  S gamma = o.c - x_z * x_z - x_y * x_y;
  if (vzero(val(alpha))) return false;
  S bsqr = beta * beta, ac4 = alpha * gamma * 4.0;
  if (!vlt(val(ac4), val(bsqr))) return false;
  // the roots -2 gamma / (beta f) and -beta f / (2 alpha) of the reference,
  // f = 1 + sqrt(1 - 4 alpha gamma / beta^2), from b f = beta + sign(beta)
  // sqrt(beta^2 - 4 alpha gamma) and one reciprocal of alpha b f
  S bf = beta + dcopysign(dsqrt(bsqr - ac4), beta), inv = drcp(alpha * bf);
  S tp = (-2.0 * gamma) * alpha * inv, tm = (-0.5 * bf) * bf * inv;
  int pick = root;
  if (root < 0) {
    const double xp = val(p.x) * val(tp), xm = val(p.x) * val(tm);
    const bool okp = !vlt(xp, o.xmin) && vlt(xp, o.xmax), okm = !vlt(xm, o.xmin) && vlt(xm, o.xmax);
    if (okp) pick = (okm && vlt(xp, xm)) ? 1 : 0;
    else if (okm) pick = 1;
    else return false;
    *chosen = pick;
  }
  S t = pick ? tm : tp;
  x0 = v3<S>(p.x * t, x_y + p.y * t, x_z + p.z * t);
  n = unit(v3<S>((o.a - 1.0) * x0.x + 0.5 * o.b, 0.0 - x0.y, 0.0 - x0.z));
  return true;
}

// Per-ray decision byte: what the ray did the last time it was traced
// afresh.  Replaying it keeps the traced function smooth in the parameters.
enum : uint8_t { RAY_HIT = 1, RAY_ROOT_P = 2, RAY_ROOT_H = 4 };

// Everything a weighted ray needs besides the two optics of its shell.
struct RayConst {
  double front;        // front_position of the shell (aperture plane)
  double beta, delta;  // optical constants at the ray energy
  double corr;         // effective-area correction per reflection
  bool weighted;       // false: unit weights (ideal mirrors)
};

// One weighted ray from the aperture point (front, ry, rz) -- ry, rz as
// r sin(phi), r cos(phi) -- along the source direction p0, through the
// paraboloid P and hyperboloid H of its shell, to the focal plane.
// replay: code holds the decisions to follow; otherwise they are made here
// and written to code (0 when the ray is lost).  blocked(set, x, p) is the
// strut test at the pre-collimator (0) and post-collimator (2), and
// blocked.cap(P, B, x, p) at the cap for a ray given in the paraboloid's
// frame.  B takes the ray from the paraboloid's frame to the hyperboloid's.
template <class S, class Struts>
MXG bool weighted_ray(const Optic<S> &P, const Optic<S> &H, const Between<S> &B, const RayConst &rc, double ry,
                      double rz, const V3<S> &p0, bool replay, uint8_t &code, const Struts &blocked, S &y, S &z,
                      S &w) {
  int rootP = replay ? ((code & RAY_ROOT_P) ? 1 : 0) : -1;
  int rootH = replay ? ((code & RAY_ROOT_H) ? 1 : 0) : -1;
  if (replay && !(code & RAY_HIT)) return false;
  if (!replay) code = 0;
  V3<S> p = p0;
  if (!replay && blocked(0, v3<S>(cst<S>(rc.front), ry - P.to[1], rz - P.to[2]), p)) return false;
  // fwd (x + to) with x + to = (front + to[0], ry, rz): (ry - to[1]) + to[1]
  // is ry to within an ulp of to[1]
  V3<S> x = v3<S>(P.ff[0] + P.fwd[1] * ry + P.fwd[2] * rz, P.ff[1] + P.fwd[4] * ry + P.fwd[5] * rz,
                  P.ff[2] + P.fwd[7] * ry + P.fwd[8] * rz);
  p = matv(P.fwd, p);
  V3<S> n;
  int ch = 0;
  if (!conic_hit(P, x, p, n, rootP, &ch)) return false;
  if (!replay) rootP = ch;
  S pdn = dotp(p, n);
  S wt = rc.weighted ? fresnel(dabs(pdn), rc.beta, rc.delta) * rc.corr : cst<S>(1.0);
  p = p - scale(2.0 * pdn, n);
  if (!replay && blocked.cap(P, B, x, p)) return false;
  p = matv(B.m, p);
  x = matv(B.m, x) + v3<S>(B.c[0], B.c[1], B.c[2]);
  if (!conic_hit(H, x, p, n, rootH, &ch)) return false;
  if (!replay) rootH = ch;
  pdn = dotp(p, n);
  if (rc.weighted) wt = wt * (fresnel(dabs(pdn), rc.beta, rc.delta) * rc.corr);
  p = p - scale(2.0 * pdn, n);
  p = matv(H.bwd, p);
  x = matv(H.bwd, x);
  x = x - v3<S>(H.to[0], H.to[1], H.to[2]);
  if (!replay && blocked(2, x, p)) return false;
  S t = (0.0 - x.x) * drcp(p.x);
  y = x.y + t * p.y;
  z = x.z + t * p.z;
  w = wt;
  if (!replay) code = (uint8_t) (RAY_HIT | (rootP ? RAY_ROOT_P : 0) | (rootH ? RAY_ROOT_H : 0));
  return true;
}

}  // namespace mxd

namespace mxd {

// exp(-x) for x >= 0 in single precision with every operation explicitly
// rounded (Cody-Waite reduction x = n ln2 + r with ln2 in two parts, then
// the Taylor series of exp(-r) to r^7, |r| <= ln2 / 2: truncation error
// below 6e-9), so host and device give the same bits.  Used for the splat
// taps, whose image must be reproducible by the CPU restatement.
MXG float exp_neg(float x) {
  if (!(x < 80.0f)) return 0.0f;
  const int n = (int) FADD(FMUL(x, 1.44269502f), 0.5f);
  const float fn = (float) n;
  const float r = FSUB(FSUB(x, FMUL(fn, 0.693145752f)), FMUL(fn, 1.42860677e-06f));
  const float s = -r;
  float p = FADD(1.0f, FMUL(s, 1.0f / 7.0f));
  p = FADD(1.0f, FMUL(FMUL(s, 1.0f / 6.0f), p));
  p = FADD(1.0f, FMUL(FMUL(s, 0.2f), p));
  p = FADD(1.0f, FMUL(FMUL(s, 0.25f), p));
  p = FADD(1.0f, FMUL(FMUL(s, 1.0f / 3.0f), p));
  p = FADD(1.0f, FMUL(FMUL(s, 0.5f), p));
  p = FADD(1.0f, FMUL(s, p));
  return FMUL(p, mx::u2f((uint32_t) (127 - n) << 23));   // 2^-n, n <= 115
}

// Splat geometry shared by the forward image, the adjoint and the CPU
// restatement.  Pixel (row j, column i) is centred at focal-plane
// y = cy + (i - (nx/2 - 1/2)) pitch, z = cz + (j - (ny/2 - 1/2)) pitch.
constexpr int TAPS = 11, HALF = 5;

// Continuous pixel coordinate of a focal-plane position, its nearest
// pixel and the offset from it, in the explicitly rounded order the CPU
// restatement follows.
MXG double pixel_coord(double y, double c, double inv_pitch, double centre_pix) {
  return MX_DADD(MX_DMUL(y - c, inv_pitch), centre_pix);
}

}  // namespace mxd
