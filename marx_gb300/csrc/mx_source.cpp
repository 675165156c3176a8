// Source direction from sky coordinates: the pointing set-up of the dither
// module (setup_pointing_ra_dec, dither.c:125-155), marx_compute_elaz
// (source.c:108-134, with marx_compute_ra_dec_offsets, pixlib.c:525-572)
// and the rotations of select_source (source.c:148-180).  Host code run
// once per source; the vector helpers restate jdmath's (vector.c) in its
// order of operations.
#include <cmath>

#include "../../include/marx_gb300.h"

namespace {

const double PI_ = 3.14159265358979323846264338327950288;
struct V { double x, y, z; };

double vlen(V a) {   // JDMv_length (vector.c:77)
  double x = fabs(a.x), y = fabs(a.y), z = fabs(a.z), t;
  if (z < x) { t = z; z = x; x = t; }
  if (z < y) { t = z; z = y; y = t; }
  if (z == 0.0) return 0.0;
  x = x / z; y = y / z;
  return z * sqrt(1.0 + x * x + y * y);
}
V normalize(V a) {   // JDMv_normalize (vector.c:92)
  double l = vlen(a);
  if (l != 0.0) { a.x = a.x / l; a.y = a.y / l; a.z = a.z / l; }
  return a;
}
double dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V cross(V a, V b) {   // JDMv_cross_prod (vector.c:29)
  V c;
  c.z = a.x * b.y - a.y * b.x;
  c.x = a.y * b.z - a.z * b.y;
  c.y = a.z * b.x - a.x * b.z;
  return c;
}
V rotate_unit(V p, V n, double theta) {   // JDMv_rotate_unit_vector (vector.c:188-212)
  double c = cos(theta), s = sin(theta), pn = dot(p, n);
  V x = cross(n, p), d;
  d.x = c * p.x + pn * (1.0 - c) * n.x + s * x.x;
  d.y = c * p.y + pn * (1.0 - c) * n.y + s * x.y;
  d.z = c * p.z + pn * (1.0 - c) * n.z + s * x.z;
  return normalize(d);
}
V spherical(double theta, double phi) {   // JDMv_spherical_to_vector (vector.c:273) with r = 1
  double s = sin(theta);
  V p;
  p.x = 1.0 * s * cos(phi);
  p.y = 1.0 * s * sin(phi);
  p.z = 1.0 * cos(theta);
  return p;
}
void to_spherical(V p, double *thetap, double *phip) {   // JDMv_unit_vector_to_spherical (vector.c:214)
  if (fabs(p.z) >= 1.0) { *thetap = p.z >= 1.0 ? 0 : PI_; *phip = 0; return; }
  double theta = acos(p.z), st = sin(theta), phi;
  if (fabs(p.x) <= fabs(p.y)) {
    phi = acos(p.x / st);
    if (p.y < 0.0) phi = -phi;
  } else {
    phi = asin(p.y / st);
    if (p.x < 0) phi = phi >= 0 ? PI_ - phi : -PI_ - phi;
  }
  *thetap = theta; *phip = phi;
}
double normalize_angle(double x) {   // dither.c:113-122
  x = fmod(x, 2 * PI_);
  if (x >= PI_) x -= (2 * PI_);
  if (x < -PI_) x += (2 * PI_);
  return x;
}
// marx_compute_ra_dec_offsets (pixlib.c:525-572): (ra, dec) as offsets
// from (ra0, dec0).
void ra_dec_offsets(double ra0, double dec0, double ra, double dec, double *dra, double *ddec) {
  double d_ra = ra - ra0, d_dec = dec - dec0, c = cos(dec), factor = c * (1 - cos(d_ra));
  double sdd = sin(d_dec) + factor * sin(dec0);
  if (fabs(sdd) > 1.0) sdd = sdd < 0 ? -1 : 1;
  double new_dec = asin(sdd), num = c * sin(d_ra), den = cos(d_dec) - factor * cos(dec0), new_ra;
  if (den >= 0) new_ra = atan(num / den);
  else new_ra = num >= 0 ? atan(num / den) + PI_ : atan(num / den) - PI_;
  *dra = new_ra; *ddec = new_dec;
}
// The nominal pointing of init_aspsol_dither (dither.c:455-464): the file's
// keywords in radians, moved below pi (no fmod, unlike the parameter file's
// roll).
double aspsol_nominal(double deg) {
  double a = deg * (PI_ / 180.0);
  if (a >= PI_) a -= (2.0 * PI_);
  return a;
}

}  // namespace

extern "C" int mx_source_direction(const mx_config *cfg, double ra, double dec, double out[3]) {
  if (!cfg || !out) return MX_EINVAL;
  // DitherModel FILE: init_aspsol_dither replaces the nominal pointing by
  // the aspect solution's keywords (carried in cfg) with its own reduction
  const bool file = cfg->dither == MX_DITHER_FILE;
  const double nom_ra = file ? aspsol_nominal(cfg->ra_nom) : cfg->ra_nom * (PI_ / 180.0);
  const double nom_dec = file ? aspsol_nominal(cfg->dec_nom) : cfg->dec_nom * (PI_ / 180.0);
  const double nom_roll = file ? aspsol_nominal(cfg->roll_nom) : normalize_angle(cfg->roll_nom * (PI_ / 180.0));
  const double yoff = cfg->pointing_offset[0] * (PI_ / (180.0 * 3600.0));
  const double zoff = cfg->pointing_offset[1] * (PI_ / (180.0 * 3600.0));
  // setup_pointing_ra_dec: the pointing from the nominal direction and the offsets
  double ct = cos(PI_ / 2.0 - nom_dec), st = sin(PI_ / 2.0 - nom_dec), cp = cos(nom_ra), sp = sin(nom_ra);
  V nom = {st * cp, st * sp, ct}, a = {-sp, cp, 0.0}, d = {ct * cp, ct * sp, -st};
  d.x = -d.x; d.y = -d.y; d.z = -d.z;
  double cd = cos(zoff), ca = cd * cos(yoff), sa = cd * sin(yoff), sd = sin(zoff);
  V p = {ca * nom.x + sa * a.x + sd * d.x, ca * nom.y + sa * a.y + sd * d.y, ca * nom.z + sa * a.z + sd * d.z};
  p = rotate_unit(p, nom, nom_roll);
  double pdec, pra;
  to_spherical(p, &pdec, &pra);
  pdec = PI_ * 0.5 - pdec;
  const double proll = nom_roll;
  // marx_compute_elaz
  const double sra = ra * (PI_ / 180.0), sdec = dec * (PI_ / 180.0);
  V src = spherical(PI_ / 2.0 - sdec, sra), pnt = spherical(PI_ / 2.0 - pdec, pra);
  src = rotate_unit(src, pnt, -proll);
  double el, az;
  to_spherical(src, &el, &az);
  el = PI_ / 2.0 - el;
  ra_dec_offsets(pra, pdec, az, el, &az, &el);
  // select_source
  V q = spherical(0.5 * PI_ - zoff, yoff);
  q = rotate_unit(q, V{0, -1, 0}, el);
  q = rotate_unit(q, V{0, 0, 1}, az);
  q = rotate_unit(q, V{1, 0, 0}, nom_roll);
  if (q.x <= 0.0) return MX_EINVAL;   // "Rays will not hit the telescope"
  out[0] = -q.x; out[1] = -q.y; out[2] = -q.z;
  return MX_OK;
}

// init_aspsol_dither and get_single_aspsol_point (dither.c:282-340,
// 438-500): each row's pointing (ra, dec) is unrolled about the nominal
// pointing by the row's roll and taken as offsets from it; angles reduced
// to [-pi, pi); times relative to TSTART, which init_aspsol_dither takes off
// the first row a second time.  Row 0 of the output is the reader's static
// start state (all zero), the left end of the first interval.
int mx_aspsol_convert(const double *rows, uint32_t n, double ra_nom, double dec_nom, double roll_nom, double tstart,
                      double *out_t, double *out_v) {
  if (!rows || !out_t || !out_v) return MX_EINVAL;
  const double nra = aspsol_nominal(ra_nom), ndec = aspsol_nominal(dec_nom);
  (void) roll_nom;   // the unrolled rows keep their own roll (Aspsol.roll1 -= Nominal_Roll is left out there)
  const V nominal = spherical(PI_ / 2.0 - ndec, nra);
  for (int k = 0; k < 8; k++) out_v[k] = 0.0;
  out_t[0] = 0.0;
  for (uint32_t i = 0; i < n; i++) {
    const double *b = rows + 7 * (size_t) i;
    double t = b[0], ra = b[1] * (PI_ / 180.0), dec = b[2] * (PI_ / 180.0), roll = b[3] * (PI_ / 180.0);
    double dth = b[6] * (PI_ / 180.0);
    V p = spherical(PI_ / 2.0 - dec, ra);
    p = rotate_unit(p, nominal, -roll);
    to_spherical(p, &dec, &ra);
    dec = PI_ / 2.0 - dec;
    ra = normalize_angle(ra);
    dec = normalize_angle(dec);
    roll = normalize_angle(roll);
    dth = normalize_angle(dth);
    ra_dec_offsets(nra, ndec, ra, dec, &ra, &dec);
    t -= tstart;
    if (i == 0) t -= tstart;
    double *v = out_v + 8 * (size_t) (i + 1);
    out_t[i + 1] = t;
    v[0] = ra; v[1] = dec; v[2] = roll; v[3] = b[4]; v[4] = b[5]; v[5] = dth; v[6] = 0.0; v[7] = 0.0;
  }
  return MX_OK;
}
