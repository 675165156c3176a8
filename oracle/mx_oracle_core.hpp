// CPU restatement of the MARX photon-trace stages (the oracle).  Test
// infrastructure only.  Each function names the reference function it
// restates (paths inside MARX 5.5.3) and keeps its order of operations, so
// that compiled without fused multiply-add it rounds like the reference.
//
// Templated on the real type R: R = double for tracing, R = Counted for the
// FP64 operation count used as the roofline's algorithmic unit.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace mxo {

constexpr double PI = 3.14159265358979323846264338327950288;   // jdmath.h:539
constexpr double HBAR_C = 1.973269631e-4;                      // marx.h:477 (keV um)

// ------------------------------------------------------- counting double --
struct Counted {
  double v;
  static thread_local double ops;
  Counted() : v(0) {}
  Counted(double x) : v(x) {}
  explicit operator double() const { return v; }
};
inline Counted operator+(Counted a, Counted b) { Counted::ops += 1; return a.v + b.v; }
inline Counted operator-(Counted a, Counted b) { Counted::ops += 1; return a.v - b.v; }
inline Counted operator*(Counted a, Counted b) { Counted::ops += 1; return a.v * b.v; }
inline Counted operator/(Counted a, Counted b) { Counted::ops += 1; return a.v / b.v; }
inline Counted operator-(Counted a) { return -a.v; }
inline Counted &operator+=(Counted &a, Counted b) { a = a + b; return a; }
inline Counted &operator-=(Counted &a, Counted b) { a = a - b; return a; }
inline Counted &operator*=(Counted &a, Counted b) { a = a * b; return a; }
inline Counted &operator/=(Counted &a, Counted b) { a = a / b; return a; }
inline bool operator<(Counted a, Counted b) { return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { return a.v != b.v; }
inline Counted sqrt(Counted a) { Counted::ops += 1; return std::sqrt(a.v); }
inline Counted sin(Counted a) { Counted::ops += 1; return std::sin(a.v); }
inline Counted cos(Counted a) { Counted::ops += 1; return std::cos(a.v); }
inline Counted tan(Counted a) { Counted::ops += 1; return std::tan(a.v); }
inline Counted pow(Counted a, Counted b) { Counted::ops += 1; return std::pow(a.v, b.v); }
inline Counted atan2(Counted a, Counted b) { Counted::ops += 1; return std::atan2(a.v, b.v); }
inline Counted fmod(Counted a, Counted b) { Counted::ops += 1; return std::fmod(a.v, b.v); }
inline Counted fabs(Counted a) { return std::fabs(a.v); }
using std::sqrt; using std::sin; using std::cos; using std::tan; using std::pow;
using std::atan2; using std::fmod; using std::fabs;
inline double dv(Counted a) { return a.v; }
inline double dv(double a) { return a; }

// ------------------------------------------------------------- variates --
// Philox4x32-10 (Salmon et al., SC'11 "Parallel random numbers: as easy as
// 1, 2, 3"), the engine's counter-based generator.
inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t) 0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t) 0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t) (p0 >> 32), lo0 = (uint32_t) p0;
    uint32_t hi1 = (uint32_t) (p1 >> 32), lo1 = (uint32_t) p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
  }
}
// Uniform slot k of photon `tag`: 53 random bits in [0, 1).
inline double philox_uniform(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0001u, 0u};
  philox4x32_10(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  uint64_t b = ((uint64_t) c[0] << 32) | c[1];
  return (double) (b >> 11) * (1.0 / 9007199254740992.0);
}
// Normal slot k: Box-Muller in single precision on 24-bit uniforms, with
// ln u = e ln 2 + 2 atanh((m-1)/(m+1)) and cos(2 pi u) from Taylor series on
// [0, pi/2), every operation rounded separately (no fused multiply-add).
inline float series_logf(float u) {
  uint32_t b; std::memcpy(&b, &u, 4);
  int e = (int) ((b >> 23) & 0xffu) - 127;
  uint32_t mb = (b & 0x7fffffu) | 0x3f800000u;
  float m; std::memcpy(&m, &mb, 4);
  if (m > 1.41421356f) { m = m * 0.5f; e += 1; }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float poly = s2 * (0.333333333f + s2 * (0.2f + s2 * (0.142857143f + s2 * (0.111111111f + s2 * 0.0909090909f))));
  float lnm = (2.0f * s) * (1.0f + poly);
  float fe = (float) e;
  return fe * 0.693145752f + (fe * 1.42860677e-06f + lnm);
}
inline float series_cos2pi(float u) {
  float x4 = u * 4.0f;
  int q = (int) x4;
  float f = x4 - (float) q;
  float t = f * 1.57079632679f, t2 = t * t;
  float c = 1.0f + t2 * (-0.5f + t2 * (4.16666667e-02f + t2 * (-1.38888889e-03f + t2 * (2.48015873e-05f +
            t2 * (-2.75573192e-07f + t2 * 2.08767570e-09f)))));
  float s = t * (1.0f + t2 * (-1.66666667e-01f + t2 * (8.33333333e-03f + t2 * (-1.98412698e-04f +
            t2 * (2.75573192e-06f + t2 * (-2.50521084e-08f + t2 * 1.60590438e-10f))))));
  return q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
}
inline double philox_normal(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0002u, 0u};
  philox4x32_10(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  float u1 = (float) ((c[0] >> 8) + 1u) * (1.0f / 16777216.0f);
  float u2 = (float) (c[1] >> 8) * (1.0f / 16777216.0f);
  float r = std::sqrt(-2.0f * series_logf(u1));
  return (double) (r * series_cos2pi(u2));
}

// Source-level draw k of photon `tag` (photon generation), its own domain.
inline double source_uniform(uint64_t seed, uint32_t tag, uint32_t k) {
  uint32_t c[4] = {tag, k, 0x5A5A0003u, 0u};
  philox4x32_10(c, (uint32_t) seed, (uint32_t) (seed >> 32));
  uint64_t b = ((uint64_t) c[0] << 32) | c[1];
  return (double) (b >> 11) * (1.0 / 9007199254740992.0);
}

struct Variates {
  // pre-drawn slot arrays (slot-major) or Philox
  const double *U = nullptr, *N = nullptr;
  uint32_t n = 0, i = 0;
  uint64_t seed = 0;
  uint32_t tag = 0;
  int upos = 0, uend = 0, npos = 0, nend = 0;
  bool overrun = false;
  void window(int ub, int uc, int nb, int nc) { upos = ub; uend = ub + uc; npos = nb; nend = nb + nc; }
  double uniform() {
    if (upos >= uend) { overrun = true; return 0.5; }
    int k = upos++;
    return U ? U[(size_t) k * n + i] : philox_uniform(seed, tag, (uint32_t) k);
  }
  double normal() {
    if (npos >= nend) { overrun = true; return 0.0; }
    int k = npos++;
    return N ? N[(size_t) k * n + i] : philox_normal(seed, tag, (uint32_t) k);
  }
};

// -------------------------------------------------------------- vectors --
template <class R> struct V3 { R x, y, z; };

template <class R> inline R dot(const V3<R> &a, const V3<R> &b) {  // vector.c:72
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class R> inline V3<R> cross(const V3<R> &a, const V3<R> &b) {  // vector.c:39
  V3<R> c;
  c.z = a.x * b.y - a.y * b.x;
  c.x = a.y * b.z - a.z * b.y;
  c.y = a.z * b.x - a.x * b.z;
  return c;
}
template <class R> inline R v_length(V3<R> a) {  // JDMv_length, vector.c:77-97
  R x = fabs(a.x), y = fabs(a.y), z = fabs(a.z), t;
  if (z < x) { t = z; z = x; x = t; }
  if (z < y) { t = z; z = y; y = t; }
  if (z == R(0.0)) return R(0.0);
  x = x / z; y = y / z;
  return z * sqrt(R(1.0) + x * x + y * y);
}
template <class R> inline void normalize(V3<R> &a) {  // JDMv_normalize, vector.c:99
  R len = v_length(a);
  if (len != R(0.0)) { a.x = a.x / len; a.y = a.y / len; a.z = a.z / len; }
}
template <class R> inline V3<R> ax1_bx2(R a, const V3<R> &x1, R b, const V3<R> &x2) {  // vector.c:118
  V3<R> c;
  c.x = a * x1.x + b * x2.x; c.y = a * x1.y + b * x2.y; c.z = a * x1.z + b * x2.z;
  return c;
}
template <class R>
inline V3<R> ax1_bx2_cx3(R a, const V3<R> &x1, R b, const V3<R> &x2, R c, const V3<R> &x3) {
  V3<R> d;  // vector.c:130
  d.x = a * x1.x + b * x2.x + c * x3.x;
  d.y = a * x1.y + b * x2.y + c * x3.y;
  d.z = a * x1.z + b * x2.z + c * x3.z;
  return d;
}
template <class R> inline V3<R> vsum(const V3<R> &a, const V3<R> &b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> vdiff(const V3<R> &a, const V3<R> &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

template <class R> inline V3<R> rotate_vector1(const V3<R> &p, const V3<R> &n, R c, R s) {
  R pn = dot(p, n);  // JDMv_rotate_vector1, vector.c:188-196
  return ax1_bx2_cx3(c, p, pn * (R(1.0) - c), n, s, cross(n, p));
}
template <class R> inline V3<R> rotate_unit_vector1(const V3<R> &p, const V3<R> &n, R c, R s) {
  V3<R> u = rotate_vector1(p, n, c, s);  // vector.c:198-205
  normalize(u);
  return u;
}
template <class R> inline V3<R> rotate_unit_vector(const V3<R> &p, const V3<R> &n, R theta) {
  return rotate_unit_vector1(p, n, cos(theta), sin(theta));  // vector.c:208
}

template <class R> struct M3 { R m[3][3]; };
template <class R> inline V3<R> mvmul(const M3<R> &a, const V3<R> &v) {  // JDM3m_vector_mul, rotate.c:121
  V3<R> b;
  b.x = a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z;
  b.y = a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z;
  b.z = a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z;
  return b;
}

// -------------------------------------------------- searches, interpolation --
inline unsigned binary_search_f(float x, const float *xp, unsigned n) {  // finterpo.c:37
  unsigned n0 = 0, n1 = n, n2;
  while (n1 > n0 + 1) {
    n2 = (n0 + n1) / 2;
    if (xp[n2] >= x) { if (xp[n2] == x) return n2; n1 = n2; }
    else n0 = n2;
  }
  if (x >= xp[n0]) return n1;
  return n0;
}
inline unsigned binary_search_d(double x, const double *xp, unsigned n) {  // dinterpo.c:30
  unsigned n0 = 0, n1 = n, n2;
  while (n1 > n0 + 1) {
    n2 = (n0 + n1) / 2;
    if (xp[n2] >= x) { if (xp[n2] == x) return n2; n1 = n2; }
    else n0 = n2;
  }
  if (x >= xp[n0]) return n1;
  return n0;
}
// JDMinterpolate_f, finterpo.c:59-86: float abscissa, double slope.
template <class R> inline float interpolate_f(float x, const float *xp, const float *yp, unsigned n) {
  if (n == 1) return yp[0];
  unsigned n1 = binary_search_f(x, xp, n), n0 = n1 - 1;
  if (n1 < n && x == xp[n1]) return yp[n1];
  if (n1 == n) { n1--; n0--; }
  if (n1 == 0) n0 = 1;
  R x0 = (double) xp[n0], x1 = (double) xp[n1];
  if (x1 == x0) return yp[n1];
  R dy = (double) (float) (yp[n1] - yp[n0]);  // float subtraction, as in C
  return (float) dv(R((double) yp[n0]) + dy / (x1 - x0) * (R((double) x) - x0));
}

// --------------------------------------------------------- complex math --
template <class R> struct Cx { R r, i; };
template <class R> inline Cx<R> c_mul(Cx<R> a, Cx<R> b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
template <class R> inline Cx<R> c_div(Cx<R> z1, Cx<R> z2) {  // complex.c:54
  R r1 = z1.r, i1 = z1.i, r2 = z2.r, i2 = z2.i, ratio, denom;
  Cx<R> z;
  if (fabs(r2) > fabs(i2)) {
    ratio = i2 / r2; denom = r2 + i2 * ratio;
    z.r = (r1 + ratio * i1) / denom; z.i = (i1 - r1 * ratio) / denom;
  } else {
    ratio = r2 / i2; denom = r2 * ratio + i2;
    z.r = (r1 * ratio + i1) / denom; z.i = (i1 * ratio - r1) / denom;
  }
  return z;
}
template <class R> inline Cx<R> c_a_bz(R a, R b, Cx<R> z1) { return {a + b * z1.r, b * z1.i}; }  // complex.c:140
template <class R> inline Cx<R> c_az1_bz2(R a, Cx<R> z1, R b, Cx<R> z2) {  // complex.c:148
  return {a * z1.r + b * z2.r, a * z1.i + b * z2.i};
}
template <class R> inline R c_abs(Cx<R> z) {  // complex.c:157
  R fr = fabs(z.r), fi = fabs(z.i), ratio;
  if (fr > fi) { ratio = z.i / z.r; return fr * sqrt(R(1.0) + ratio * ratio); }
  if (fi == R(0.0)) return R(0.0);
  ratio = z.r / z.i;
  return fi * sqrt(R(1.0) + ratio * ratio);
}
template <class R> inline Cx<R> c_sqrt(Cx<R> a) {  // complex.c:201
  R r = c_abs(a);
  if (r == R(0.0)) return a;
  if (a.r >= R(0.0)) { a.r = sqrt(R(0.5) * (r + a.r)); a.i = R(0.5) * a.i / a.r; }
  else {
    r = sqrt(R(0.5) * (r - a.r));
    a.r = R(0.5) * a.i / r; a.i = r;
    if (a.r < R(0.0)) { a.r = -a.r; a.i = -a.i; }
  }
  return a;
}
// marx_reflectivity, reflect.c:39-77
template <class R> inline R reflectivity(R cos_theta, R beta, R delta) {
  Cx<R> n{R(1.0) - delta, beta};
  R sin_theta = sqrt(R(1.0) - cos_theta * cos_theta);
  Cx<R> nsqr = c_mul(n, n);
  Cx<R> root = c_sqrt(c_a_bz(-sin_theta * sin_theta, R(1.0), nsqr));
  Cx<R> num = c_a_bz(cos_theta, R(-1.0), root), den = c_a_bz(cos_theta, R(1.0), root);
  Cx<R> e_perp = c_div(num, den);
  num = c_az1_bz2(cos_theta, nsqr, R(-1.0), root);
  den = c_az1_bz2(cos_theta, nsqr, R(1.0), root);
  Cx<R> e_par = c_div(num, den);
  return R(0.5) * (e_par.r * e_par.r + e_par.i * e_par.i + e_perp.r * e_perp.r + e_perp.i * e_perp.i);
}

// ----------------------------------------------------------------- model --
struct FoldArray { double e_alpha, p_min, delta_p, p_max, norm, expon; unsigned num; const float *theta; };
struct FoldTable { std::vector<FoldArray> arr; std::vector<double> e_alphas; };

struct Shell {
  double length_p, length_h, xoffset, p_blur, h_blur, p_scat, h_scat;
  double osac[2][9];  // rdb x0 y0 z0 p k rho0 az el l, [0]=P [1]=H
  double a[2], b[2], c[2], xmin[2], xmax[2];
  V3<double> to_osac[2];
  double front_position, area_fraction, min_radius, max_radius;
  unsigned shutter_bitmap, num_open;
  M3<double> fwd[2], bwd[2];
  const float *corr_e = nullptr, *corr_f = nullptr; unsigned corr_n = 0;
  FoldTable fold[2];
};

struct Grating {
  double dispersion_angle, theta_blur, period, dp_over_p, vig, rowland;
  unsigned num_orders, num_energies;
  std::vector<int> order_list;
  std::vector<float> energies;
  std::vector<float> cum;  // [order][energy]
  bool have_sectors = false;
  std::vector<double> s_min, s_max, s_dtheta, s_dtheta_blur, s_dpp, s_dpp_blur;
};

struct Chip {
  int id;
  V3<double> x_ll, x_lr, x_ul, x_ur, xhat, yhat, normal;
  double xlen, ylen, xpix, ypix, xoff, yoff;
};

struct Model {
  mx_config cfg;
  Shell sh[4];
  double cap;
  bool ideal, use_blur, use_wfold, use_struts, use_scale;
  const float *opt_e = nullptr, *opt_beta = nullptr, *opt_delta = nullptr; unsigned opt_n = 0;
  Grating gr[4];
  std::vector<Chip> chips;
  // dither
  double ra_amp, dec_amp, roll_amp, nominal_roll, aspect_blur;
  double frame_time;
};

// --------------------------------------------------------------- mirror --
// blur_normal, hrma.c:1054-1093
template <class R> inline void blur_normal(V3<R> &n, R blur, Variates &v) {
  R n_y = n.y, n_z = n.z;
  R len = sqrt(n_y * n_y + n_z * n_z);
  V3<R> perp{R(0.0), n_z / len, -n_y / len};
  R phi = R(2.0 * PI) * R(v.uniform());
  perp = rotate_unit_vector(perp, n, phi);
  phi = blur * R(1.0 / 3600.0 * PI / 180.0);
  phi = phi * R(v.normal());
  n = rotate_unit_vector(n, perp, phi);
}

// JDMquadratic_root, qroot.c:36-70
template <class R> inline int quadratic_root(R a, R b, R c, R &rplus, R &rminus) {
  if (a == R(0.0)) return -1;
  R bsqr = b * b, ac4 = a * c * R(4), nb2a = -b / (R(2.0) * a);
  if (bsqr > ac4) {
    R factor = R(1.0) + sqrt(R(1.0) - ac4 / bsqr);
    rplus = R(-2.0) * c / (b * factor);
    rminus = nb2a * factor;
    return 1;
  }
  if (bsqr == ac4) { rplus = rminus = nb2a; return 1; }
  return 0;
}

// compute_conic_intersection, hrma.c:411-478
template <class R>
inline int conic_intersection(R a, R b, R c, V3<R> &x0, const V3<R> &p, V3<R> &normal, R xmin, R xmax) {
  R t_plus = -x0.x / p.x, t_minus;
  R x_y = x0.y + t_plus * p.y, x_z = x0.z + t_plus * p.z;
  R alpha = a * p.x * p.x - R(1.0);
  R beta = b * p.x - R(2.0) * (p.y * x_y + p.z * x_z);
  R gamma = c - x_z * x_z - x_y * x_y;
  if (alpha == R(0.0)) {
    if (beta == R(0.0)) return -1;
    t_plus = t_minus = -gamma / beta;
  } else if (0 >= quadratic_root(alpha, beta, gamma, t_plus, t_minus)) return -1;
  R x_plus = p.x * t_plus, x_minus = p.x * t_minus;
  if ((x_plus >= xmin) && (x_plus < xmax)) {
    if ((x_minus >= xmin) && (x_minus < xmax) && (x_minus > x_plus)) {
      x0.x = x_minus; x0.y = x_y + p.y * t_minus; x0.z = x_z + p.z * t_minus;
    } else {
      x0.x = x_plus; x0.y = x_y + p.y * t_plus; x0.z = x_z + p.z * t_plus;
    }
  } else if ((x_minus >= xmin) && (x_minus < xmax)) {
    x0.x = x_minus; x0.y = x_y + p.y * t_minus; x0.z = x_z + p.z * t_minus;
  } else return -1;
  normal.x = (a - R(1)) * x0.x + R(0.5) * b;
  normal.y = -x0.y;
  normal.z = -x0.z;
  normalize(normal);
  return 0;
}

// interpolate_theta, wfold.c:304-332
template <class R> inline R interpolate_theta(const FoldArray &f, R p) {
  if (p < R(f.p_min)) return R(0.0);
  if (p > R(f.p_max)) return pow(R(f.norm) * (R(1.0) - p), R(f.expon));
  R delta_i = (p - R(f.p_min)) / R(f.delta_p);
  unsigned i = (unsigned) dv(delta_i);
  if (i + 1 >= f.num) return R((double) f.theta[f.num - 1]);
  delta_i -= R((double) i);
  return (R(1.0) - delta_i) * R((double) f.theta[i]) + delta_i * R((double) f.theta[i + 1]);
}
// marx_wfold_table_interp, wfold.c:334-363
template <class R> inline R wfold_interp(const FoldTable &t, R energy, R sin_alpha, R r) {
  unsigned num = (unsigned) t.arr.size();
  if (num == 1) return interpolate_theta(t.arr[0], r);
  R e_alpha = energy * sin_alpha;
  unsigned i = binary_search_d(dv(e_alpha), t.e_alphas.data(), num);
  if (i == num) i--;
  if (i == 0) i++;
  R th0 = interpolate_theta(t.arr[i - 1], r), th1 = interpolate_theta(t.arr[i], r);
  R e0 = t.e_alphas[i - 1], e1 = t.e_alphas[i];
  return th0 + (th1 - th0) * (e_alpha - e0) / (e1 - e0);
}

// reflect_from_conic, hrma.c:488-545.  Returns -2 missed, -1 absorbed, 0 ok.
template <class R>
inline int reflect_from_conic(const Model &M, const Shell &h, int o, V3<R> &x, V3<R> &p, R energy,
                              R beta, R delta, R corr, Variates &v) {
  V3<R> normal;
  if (-1 == conic_intersection(R(h.a[o]), R(h.b[o]), R(h.c[o]), x, p, normal, R(h.xmin[o]), R(h.xmax[o])))
    return -2;
  if (M.use_blur) blur_normal(normal, R(o == 0 ? h.p_blur : h.h_blur), v);
  R p_dot_n = dot(p, normal);
  if (!M.ideal) {
    R r = v.uniform();
    R rfl = reflectivity(fabs(p_dot_n), beta, delta);
    if (r >= rfl * corr) return -1;
  }
  p = ax1_bx2(R(1.0), p, R(-2.0) * p_dot_n, normal);
  if (!M.use_wfold) return 0;
  R sin_grazing = -p_dot_n;
  R r = v.uniform();
  R dg = wfold_interp(h.fold[o], energy, sin_grazing, r);
  dg *= R(o == 0 ? h.p_scat : h.h_scat);
  if (dg > R(PI / 4)) return -1;
  if (R(v.uniform()) < R(0.5)) dg = -dg;
  p = rotate_unit_vector(p, cross(p, normal), dg);
  return 0;
}

struct Strut { double xpos, half_width; };
static const Strut PRE_STRUTS[2] = {{1492.060, 0.5 * 0.5 * 25.4}, {942.266, 0.5 * 0.5 * 25.4}};
static const Strut CAP_STRUTS[2] = {{0.5 * 1.965 * 25.4, 0.5 * 0.75 * 25.4}, {-0.5 * 1.965 * 25.4, 0.5 * 0.75 * 25.4}};
static const Strut POST_STRUTS[2] = {{-1050.353, 0.5 * 0.5 * 25.4}, {-1271.333, 0.5 * 0.5 * 25.4}};

// intersects_struts, hrma.c:928-968
template <class R>
inline int intersects_struts(const Model &M, const V3<R> &X, const V3<R> &P, uint32_t &flags, const Strut *s) {
  R theta = R(30.0 * (PI / 180.0));
  R ct = cos(theta), st = sin(theta);
  for (int k = 0; k < 2; k++) {
    R hw = s[k].half_width;
    R x = X.x, y = X.y, z = X.z, px = P.x, py = P.y, pz = P.z;
    R t = (R(s[k].xpos) + R(M.cap) - x) / px;
    y += py * t; z += pz * t;
    for (int i = 0; i < 3; i++) {
      if (i != 0) { R tmp = ct * y - st * z; z = st * y + ct * z; y = tmp; }
      if (((-hw < y) && (y < hw)) || ((-hw < z) && (z < hw))) { flags |= MX_PHOTON_MIRROR_VBLOCKED; return 1; }
    }
  }
  return 0;
}

struct Photon {
  double energy, t;
  V3<double> x, p;
  uint32_t flags;
  int shell, order, ccd;
  float ypix, zpix;
  float dith[3];
};

// project_photon_to_hrma, hrma.c:984-1050
template <class R>
inline void project_photon_to_hrma(const Model &M, Photon &ph, V3<R> &x, V3<R> &p, Variates &v) {
  for (;;) {
    R r = v.uniform();
    if (v.overrun) return;
    for (int i = 0; i < 4; i++) {
      const Shell &h = M.sh[i];
      if (r < R(h.area_fraction)) {
        ph.shell = i;
        R radius;
        if (M.cfg.aperture_area_uniform) {  // engine option: uniform in area
          R r0 = R(h.min_radius), r1 = R(h.max_radius);
          radius = sqrt(r0 * r0 + (r1 * r1 - r0 * r0) * R(v.uniform()));
        } else
          radius = R(h.min_radius) + (R(h.max_radius) - R(h.min_radius)) * R(v.uniform());
        R theta;
        unsigned quad;
        do {
          theta = v.uniform();
          quad = (unsigned) dv(R(4.0) * theta);
          if (v.overrun) return;
        } while (0 == (h.shutter_bitmap & (1u << quad)));
        theta = R(2.0 * PI) * (theta - R(1.0 / 8.0));
        x.z = radius * cos(theta);
        x.y = radius * sin(theta);
        x.x = h.front_position;
        x.z -= R(h.to_osac[0].z);
        x.y -= R(h.to_osac[0].y);
        if (M.cfg.source_distance > 0.0) {
          p = ax1_bx2(R(1.0), x, R(M.cfg.source_distance), p);
          normalize(p);
        }
        if (M.use_struts) intersects_struts(M, x, p, ph.flags, PRE_STRUTS);
        return;
      }
    }
  }
}

// _marx_hrma_mirror_reflect per-photon body, hrma.c:1183-1339
template <class R> inline void mirror_photon(const Model &M, Photon &ph, Variates &v) {
  v.window(MX_U_MIRROR, 12, MX_N_MIRROR, 2);
  if (!M.ideal) {
    if (v.uniform() > M.cfg.hrma_vig) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;
    if (ph.flags & MX_BAD_PHOTON_MASK) return;
  }
  V3<R> x{ph.x.x, ph.x.y, ph.x.z}, p{ph.p.x, ph.p.y, ph.p.z};
  project_photon_to_hrma(M, ph, x, p, v);
  if (v.overrun) return;
  const Shell &h = M.sh[ph.shell];
  auto store = [&]() { ph.x = {dv(x.x), dv(x.y), dv(x.z)}; ph.p = {dv(p.x), dv(p.y), dv(p.z)}; };
  V3<R> to_p{h.to_osac[0].x, h.to_osac[0].y, h.to_osac[0].z}, to_h{h.to_osac[1].x, h.to_osac[1].y, h.to_osac[1].z};
  M3<R> fp, bp, fh, bh;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      fp.m[i][j] = h.fwd[0].m[i][j]; bp.m[i][j] = h.bwd[0].m[i][j];
      fh.m[i][j] = h.fwd[1].m[i][j]; bh.m[i][j] = h.bwd[1].m[i][j];
    }
  x = vsum(x, to_p);
  x = mvmul(fp, x);
  p = mvmul(fp, p);
  R energy = ph.energy, beta, delta, corr = R(1.0);
  if (M.opt_n == 0) { beta = R(0.0); delta = R(1.0); corr = R(1.0); }
  else {
    beta = (double) interpolate_f<R>((float) ph.energy, M.opt_e, M.opt_beta, M.opt_n);
    delta = (double) interpolate_f<R>((float) ph.energy, M.opt_e, M.opt_delta, M.opt_n);
    if (M.use_scale) corr = sqrt(R((double) interpolate_f<R>((float) ph.energy, h.corr_e, h.corr_f, h.corr_n)));
  }
  int st = reflect_from_conic(M, h, 0, x, p, energy, beta, delta, corr, v);
  if (st != 0) { ph.flags |= MX_PHOTON_UNREFLECTED; store(); return; }
  p = mvmul(bp, p);
  x = mvmul(bp, x);
  x = vdiff(x, to_p);
  if (M.use_struts && 1 == intersects_struts(M, x, p, ph.flags, CAP_STRUTS)) { store(); return; }
  x = vsum(x, to_h);
  p = mvmul(fh, p);
  x = mvmul(fh, x);
  if (0 != reflect_from_conic(M, h, 1, x, p, energy, beta, delta, corr, v)) {
    ph.flags |= MX_PHOTON_UNREFLECTED; store(); return;
  }
  p = mvmul(bh, p);
  x = mvmul(bh, x);
  x = vdiff(x, to_h);
  if (M.use_struts) intersects_struts(M, x, p, ph.flags, POST_STRUTS);
  store();
}

// --------------------------------------------------------------- dither --
// apply_dither, dither.c:551-581
template <class R> inline V3<R> apply_dither(R ra, R dec, R roll, V3<R> p) {
  p = rotate_unit_vector(p, V3<R>{R(1), R(0), R(0)}, -roll);
  R cos_ra = cos(ra), sin_ra = sin(ra), cos_dec = cos(dec), sin_dec = sin(dec);
  R cos_theta = cos_dec * cos_ra;
  V3<R> n{R(0), sin_dec, -cos_dec * sin_ra};
  R sin_theta = v_length(n);
  if (sin_theta <= R(1e-20)) return p;
  n.x /= sin_theta; n.y /= sin_theta; n.z /= sin_theta;
  return rotate_unit_vector1(p, n, cos_theta, sin_theta);
}
// dither_ray + get_internal_dither, dither.c:167-182, 609-628
template <class R> inline void dither_photon(const Model &M, Photon &ph, Variates &v) {
  v.window(0, 0, MX_N_DITHER, 2);
  R t = R(M.cfg.start_time) + R(ph.t);
  t = R(2.0 * PI) * t;
  float fra = (float) dv(R(M.ra_amp) * sin(t / R(M.cfg.dither_period[0]) + R(M.cfg.dither_phase[0])));
  float fdec = (float) dv(R(M.dec_amp) * sin(t / R(M.cfg.dither_period[1]) + R(M.cfg.dither_phase[1])));
  float froll = (float) dv(R(M.nominal_roll) + R(M.roll_amp) * sin(t / R(M.cfg.dither_period[2]) + R(M.cfg.dither_phase[2])));
  ph.dith[0] = fra; ph.dith[1] = fdec; ph.dith[2] = froll;
  R dra = R(M.aspect_blur) * R(v.normal());
  R ddec = R(M.aspect_blur) * R(v.normal());
  V3<R> p{ph.p.x, ph.p.y, ph.p.z};
  p = apply_dither(R((double) fra) + dra, R((double) fdec) + ddec, R((double) froll), p);
  ph.p = {dv(p.x), dv(p.y), dv(p.z)};
}

// -------------------------------------------------------------- grating --
template <class R> inline V3<R> rotate_x(V3<R> a, R theta) {  // rotate, diffract.c:690-701
  R c = cos(theta), s = sin(theta), ay = a.y, az = a.z;
  a.y = c * ay - s * az;
  a.z = s * ay + c * az;
  return a;
}
// newtons_quartic + intersect, diffract.c:622-687
template <class R> inline int rowland_intersect(V3<R> &x0, const V3<R> &p, R rowland) {
  R t = -x0.x / p.x;
  x0.x = R(0.0);
  x0.y = x0.y + p.y * t;
  x0.z = x0.z + p.z * t;
  R pxpz_len = p.x * p.x + p.z * p.z;
  R x2 = x0.z * x0.z + x0.y * x0.y;
  R r2 = rowland * rowland;
  R pdotx = dot(p, x0);
  R a = R(4.0) * pdotx;
  R b = R(2.0) * x2 + a * pdotx - r2 * pxpz_len;
  R c = a * x2 - R(2.0) * r2 * p.z * x0.z;
  R d = x2 * x2 - r2 * x0.z * x0.z;
  R t0 = -rowland * sqrt(pxpz_len);
  R a2 = R(2.0) * a, a3 = R(3.0) * a, b2 = R(2.0) * b;
  unsigned max_it = 10;
  for (;;) {
    R tt2 = t0 * t0;
    R num = tt2 * (R(3.0) * tt2 + a2 * t0 + b) - d;
    R den = tt2 * (R(4.0) * t0 + a3) + b2 * t0 + c;
    t = num / den;
    if (fabs(t - t0) < R(1.0e-4)) break;
    max_it--;
    if (max_it == 0) return -1;
    t0 = t;
  }
  x0 = ax1_bx2(R(1.0), x0, t, p);
  return 0;
}

// diffract_photon, diffract.c:706-823 (theta = 0 for the HETG)
template <class R> inline int diffract_photon(const Grating &g, Photon &ph, V3<R> &X, V3<R> &P, int order, Variates &v) {
  R nlod = R((double) order * (2.0 * PI * HBAR_C)) / R(g.period) / R(ph.energy);
  V3<R> x = X, p = P;
  V3<R> n = x;
  normalize(n);
  n.x = -n.x; n.y = -n.y; n.z = -n.z;
  V3<R> l{n.z, R(0.0), -n.x};
  normalize(l);
  V3<R> d = cross(n, l);
  R dtheta, dpp;
  if (g.have_sectors) {
    R sector = atan2(x.y, x.z);
    if (sector < R(0)) sector = R(2 * PI) + sector;
    unsigned ns = (unsigned) g.s_min.size();
    unsigned sn = binary_search_d(dv(sector), g.s_min.data(), ns);
    if (sn == 0) return -1;  // below the first sector: the reference reads out of bounds here
    sn = sn - 1;
    if ((R(g.s_max[sn]) <= sector) || (R(g.s_min[sn]) > sector)) return -1;
    dtheta = R(g.s_dtheta[sn]) + R(g.s_dtheta_blur[sn]) * R(v.normal());
    dpp = R(g.s_dpp[sn]) + R(g.s_dpp_blur[sn]) * R(v.normal());
  } else {
    dtheta = R(g.theta_blur) * R(v.normal());
    dpp = R(g.dp_over_p) * R(v.normal());
  }
  R theta = R(0.0);
  theta -= dtheta;
  if (theta != R(0.0)) {
    R c = cos(theta), s = sin(theta);
    V3<R> lt = l, dt = d;
    l = ax1_bx2(c, lt, s, dt);
    d = ax1_bx2(-s, lt, c, dt);
  }
  R p_d = nlod + dot(p, d);
  R p_l = dot(p, l);
  R p_n = R(1.0) - p_l * p_l - p_d * p_d;
  if (p_n < R(0.0)) return -1;
  p_n = sqrt(p_n);
  p = ax1_bx2(p_d, d, p_n, n);
  P = ax1_bx2(R(1.0), p, p_l, l);
  if (dpp == R(0)) return 0;
  R factor = nlod * dpp;
  V3<R> dp = ax1_bx2(-factor, d, factor * (p_d / p_n), n);
  P.x += dp.x; P.y += dp.y; P.z += dp.z;
  normalize(P);
  return 0;
}

// diffract, diffract.c:974-1130, for one photon: vignetting, rotation into
// the grating frame, Rowland torus, per-photon cumulative efficiencies
// (JDMinterpolate_n_fvector, finterpo.c:134-190), order choice
// (diffract_photon_from_grating, diffract.c:828-849), rotation back.
template <class R> inline void grating_photon(const Model &M, Photon &ph, Variates &v) {
  v.window(MX_U_GRATING, 2, MX_N_GRATING, 2);
  const Grating &g = M.gr[ph.shell];
  if (v.uniform() > g.vig) ph.flags |= MX_PHOTON_MIRROR_VBLOCKED;
  if (ph.flags & MX_BAD_PHOTON_MASK) return;
  V3<R> x{ph.x.x, ph.x.y, ph.x.z}, p{ph.p.x, ph.p.y, ph.p.z};
  R th = R(-1 * g.dispersion_angle);
  x = rotate_x(x, th);
  p = rotate_x(p, th);
  if (-1 == rowland_intersect(x, p, R(g.rowland))) ph.flags |= MX_PHOTON_UNDIFFRACTED;
  // cumulative efficiencies at this photon's energy
  float xe = (float) ph.energy;
  unsigned n = g.num_energies, idx = 1;
  while (idx < n - 1 && (double) xe > (double) g.energies[idx]) idx++;
  R x_0 = (double) g.energies[idx - 1], x_1 = (double) g.energies[idx], dx = x_1 - x_0;
  R r = v.uniform();
  int chosen = -1;
  for (unsigned k = 0; k < g.num_orders; k++) {
    const float *row = g.cum.data() + (size_t) k * n;
    float ck;
    if (dx == R(0.0)) ck = row[idx - 1];
    else {
      R y0 = (double) row[idx - 1], y1 = (double) row[idx];
      ck = (float) dv(y0 + (y1 - y0) * (R((double) xe) - x_0) / dx);
    }
    if (r <= R((double) ck)) { chosen = (int) k; break; }
  }
  if (chosen < 0) ph.flags |= MX_PHOTON_UNDIFFRACTED;
  else {
    ph.order = g.order_list[chosen];
    if (-1 == diffract_photon(g, ph, x, p, ph.order, v)) ph.flags |= MX_PHOTON_UNDIFFRACTED;
  }
  th = R(1 * g.dispersion_angle);
  x = rotate_x(x, th);
  p = rotate_x(p, th);
  ph.x = {dv(x.x), dv(x.y), dv(x.z)};
  ph.p = {dv(p.x), dv(p.y), dv(p.z)};
}

// ------------------------------------------------------------- detector --
// intersect_with_detector_plane, detector.c:56-109
template <class R>
inline int detector_plane(const Chip &g, const V3<R> &x0, const V3<R> &p, V3<R> &x, R &dx, R &dy, int must_hit) {
  V3<R> normal{g.normal.x, g.normal.y, g.normal.z}, xll{g.x_ll.x, g.x_ll.y, g.x_ll.z};
  R pdotn = dot(p, normal);
  if (pdotn == R(0)) return -1;
  V3<R> r = vdiff(x0, xll);
  r = ax1_bx2(R(1.0), r, R(-1.0) * dot(r, normal) / pdotn, p);
  int hit = 1;
  R rx = dot(r, V3<R>{g.xhat.x, g.xhat.y, g.xhat.z});
  if ((rx < R(0.0)) || (rx >= R(g.xlen))) { if (must_hit) return 0; hit = 0; }
  R ry = dot(r, V3<R>{g.yhat.x, g.yhat.y, g.yhat.z});
  if ((ry < R(0.0)) || (ry >= R(g.ylen))) { if (must_hit) return 0; hit = 0; }
  x = vsum(r, xll);
  dx = rx; dy = ry;
  return hit;
}

// _marx_acis_i_detect / _marx_acis_s_detect per-photon body (acis-i.c:124-157,
// acis-s.c:203-239) with _marx_intersect_with_detector (detector.c:112-168),
// _marx_transform_ray[_reverse] (trans.c:66-90) and _marx_acis_apply_streak
// (acis-i.c:60-93).  QE and pulse height are not modelled (DetIdeal).
template <class R> inline void detect_photon(const Model &M, Photon &ph, Variates &v) {
  v.window(MX_U_DETECT, 2, MX_N_DETECT, 2);
  V3<R> x{ph.x.x, ph.x.y, ph.x.z}, p{ph.p.x, ph.p.y, ph.p.z};
  V3<R> off{M.cfg.det_offset[0], M.cfg.det_offset[1], M.cfg.det_offset[2]};
  // identity rotation (no detector dither for INTERNAL): x -= offset
  x.x -= off.x; x.y -= off.y; x.z -= off.z;
  x = V3<R>{R(1) * x.x + R(0) * x.y + R(0) * x.z, R(0) * x.x + R(1) * x.y + R(0) * x.z, R(0) * x.x + R(0) * x.y + R(1) * x.z};
  p = V3<R>{R(1) * p.x + R(0) * p.y + R(0) * p.z, R(0) * p.x + R(1) * p.y + R(0) * p.z, R(0) * p.x + R(0) * p.y + R(1) * p.z};
  const Chip *hitg = nullptr;
  V3<R> xh;
  R dx = 0, dy = 0;
  for (const Chip &g : M.chips)
    if (1 == detector_plane(g, x, p, xh, dx, dy, 1)) { hitg = &g; break; }
  if (hitg == nullptr && M.cfg.det_extend) {
    R best_r2 = -1, bdx = 0, bdy = 0;
    V3<R> bx{0, 0, 0};
    for (const Chip &g : M.chips) {
      V3<R> xx; R ddx, ddy;
      if (-1 == detector_plane(g, x, p, xx, ddx, ddy, 0)) continue;
      R ex = ddx - R(0.5) * R(g.xlen), ey = ddy - R(0.5) * R(g.ylen);
      R r2 = ex * ex + ey * ey;
      if ((r2 < best_r2) || (hitg == nullptr)) { hitg = &g; bx = xx; bdx = ddx; bdy = ddy; best_r2 = r2; }
    }
    if (hitg) { xh = bx; dx = bdx; dy = bdy; }
  }
  if (hitg == nullptr) {
    ph.flags |= MX_PHOTON_MISSED_DETECTOR;
    ph.ccd = -1;
  } else {
    const Chip &d = *hitg;
    x = xh;
    ph.ccd = d.id;
    ph.ypix = (float) dv(dx / R(d.xpix));
    ph.zpix = (float) dv(dy / R(d.ypix));
    if (M.cfg.acis_frame_transfer_time > 0.0) {
      R t = R(M.cfg.start_time) + R(ph.t);
      t = fmod(t, R(M.frame_time));
      if (t > R(M.cfg.acis_exposure_time)) {
        ph.zpix = (float) dv(R(1.0) + R(1022.0) * R(v.uniform()));
        R xp = (R((double) ph.ypix) - R(d.xoff)) * R(d.xpix);
        R yp = (R((double) ph.zpix) - R(d.yoff)) * R(d.ypix);
        V3<R> dd = ax1_bx2(xp, V3<R>{d.xhat.x, d.xhat.y, d.xhat.z}, yp, V3<R>{d.yhat.x, d.yhat.y, d.yhat.z});
        x = vsum(V3<R>{d.x_ll.x, d.x_ll.y, d.x_ll.z}, dd);
        p = vdiff(x, V3<R>{R(M.cfg.focal_length), R(0), R(0)});
        normalize(p);
        ph.flags |= MX_PHOTON_ACIS_STREAKED;
      }
    }
  }
  p = V3<R>{R(1) * p.x + R(0) * p.y + R(0) * p.z, R(0) * p.x + R(1) * p.y + R(0) * p.z, R(0) * p.x + R(0) * p.y + R(1) * p.z};
  x = V3<R>{R(1) * x.x + R(0) * x.y + R(0) * x.z, R(0) * x.x + R(1) * x.y + R(0) * x.z, R(0) * x.x + R(0) * x.y + R(1) * x.z};
  x.x += off.x; x.y += off.y; x.z += off.z;
  ph.x = {dv(x.x), dv(x.y), dv(x.z)};
  ph.p = {dv(p.x), dv(p.y), dv(p.z)};
}

// The whole trace for one photon; stages as in marx.c process_photons
// (marx.c:240-273) preceded by the dither applied at photon creation
// (source.c:357).  Photons with a bad flag skip later stages, as
// marx_prune_photons drops them from sorted_index.
// A photon whose stage ran out of pre-drawn variates is not traced further
// (an engine rule; the reference draws from an unbounded stream).
template <class R> inline bool trace_photon(const Model &M, Photon &ph, uint32_t stages, Variates &v) {
  if ((stages & MX_STAGE_DITHER) && M.cfg.dither == MX_DITHER_INTERNAL) dither_photon<R>(M, ph, v);
  if ((stages & MX_STAGE_MIRROR) && !(ph.flags & MX_BAD_PHOTON_MASK)) mirror_photon<R>(M, ph, v);
  if (v.overrun) return true;
  if ((stages & MX_STAGE_GRATING) && M.cfg.grating == MX_GRATING_HETG && !(ph.flags & MX_BAD_PHOTON_MASK))
    grating_photon<R>(M, ph, v);
  if (v.overrun) return true;
  if ((stages & MX_STAGE_DETECT) && M.cfg.detector != MX_DETECTOR_NONE && !(ph.flags & MX_BAD_PHOTON_MASK))
    detect_photon<R>(M, ph, v);
  return v.overrun;
}

}  // namespace mxo
