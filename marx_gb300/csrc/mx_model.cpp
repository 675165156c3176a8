// Host-side model derivation: table pack + mx_config -> the flat device
// tables of mx_model.h.  Pure C++ (no CUDA), so it is also exercised by the
// CPU test suite.
//
// The derived quantities follow the reference's init code: get_shell_geometry
// (hrma.c:551-602), init_hrma_shells (hrma.c:671-745), init_yaw_pitch
// (hrma.c:842-897) with JDM3m_rot_z_matrix / JDM3m_rot_matrix / JDM3m_mul
// (rotate.c:60-119), the WFold reader's delta_p adjustment (wfold.c:191-197),
// sum_file_efficiencies (diffract.c:1254-1300), read_sector_info
// (diffract.c:1897-1948), the CALDB chip patching and basis
// (caldb.c:256-491, detector.c:383-402, acis_geom.c:54-67) and the dither
// parameter scaling (dither.c:508-547).  Host libm evaluates the init-time
// sines and cosines, as it does in the reference.
#include "mx_host.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace mx {

static const double PI_ = 3.14159265358979323846264338327950288;
static const double HBAR_C = 1.973269631e-4;   // marx.h:477, keV um

bool Pack::load(const char *path, std::string &err) {
  FILE *f = fopen(path, "rb");
  if (!f) { err = std::string("cannot open table pack ") + (path ? path : "(null)"); return false; }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<char> b((size_t) (sz > 0 ? sz : 0));
  size_t got = sz > 0 ? fread(b.data(), 1, (size_t) sz, f) : 0;
  fclose(f);
  if ((long) got != sz || sz < 16 || memcmp(b.data(), "MXPACK01", 8) != 0) { err = "not a table pack"; return false; }
  uint32_t n;
  memcpy(&n, b.data() + 8, 4);
  if (16 + 104ull * n > (unsigned long long) sz) { err = "table pack header truncated"; return false; }
  for (uint32_t i = 0; i < n; i++) {
    const char *e = b.data() + 16 + 104 * i;
    char name[49] = {0};
    memcpy(name, e, 48);
    Section s;
    uint32_t dt, nd;
    uint64_t dims[4], off, nb;
    memcpy(&dt, e + 48, 4); memcpy(&nd, e + 52, 4); memcpy(dims, e + 56, 32);
    memcpy(&off, e + 88, 8); memcpy(&nb, e + 96, 8);
    if (off + nb > (uint64_t) sz || dt > 2) { err = std::string("bad pack section ") + name; return false; }
    s.dtype = (int) dt;
    s.count = nb / (dt == 1 ? 8 : 4);
    s.data.assign(b.data() + off, b.data() + off + nb);
    sections[name] = std::move(s);
  }
  return true;
}

template <class T> const T *Pack::get(const std::string &name, size_t *count, std::string &err) const {
  auto it = sections.find(name);
  if (it == sections.end()) { err = "table pack lacks " + name; return nullptr; }
  int want = sizeof(T) == 8 ? 1 : (std::is_same<T, float>::value ? 0 : 2);
  if (it->second.dtype != want) { err = "table pack section " + name + " has the wrong type"; return nullptr; }
  if (count) *count = it->second.count;
  return reinterpret_cast<const T *>(it->second.data.data());
}
template const double *Pack::get<double>(const std::string &, size_t *, std::string &) const;
template const float *Pack::get<float>(const std::string &, size_t *, std::string &) const;
template const int32_t *Pack::get<int32_t>(const std::string &, size_t *, std::string &) const;

// ---------------------------------------------------------------- matrices --
static void rot_z(double m[9], double theta) {
  double c = cos(theta), s = sin(theta);
  s = -s;
  double r[9] = {c, s, 0.0, -s, c, 0.0, 0.0, 0.0, 1.0};
  memcpy(m, r, sizeof(r));
}
static void rot_axis(double m[9], const double n[3], double theta) {
  double c = cos(theta), s = sin(theta), c1 = 1 - c;
  double n0 = n[0], n1 = n[1], n2 = n[2];
  double n01 = n0 * n1 * c1, n02 = n0 * n2 * c1, n12 = n1 * n2 * c1;
  m[0] = n0 * n0 * c1 + c; m[1] = n01 - s * n2; m[2] = n02 + s * n1;
  m[3] = n01 + s * n2; m[4] = n1 * n1 * c1 + c; m[5] = n12 - s * n0;
  m[6] = n02 - s * n1; m[7] = n12 + s * n0; m[8] = n2 * n2 * c1 + c;
}
static void mat3_mul(double c[9], const double a[9], const double b[9]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
static double vlen(const double a[3]) {  // JDMv_length (vector.c:77)
  double x = fabs(a[0]), y = fabs(a[1]), z = fabs(a[2]), t;
  if (z < x) { t = z; z = x; x = t; }
  if (z < y) { t = z; z = y; y = t; }
  if (z == 0.0) return 0.0;
  x = x / z; y = y / z;
  return z * sqrt(1.0 + x * x + y * y);
}
static void vnorm(double a[3]) {
  double l = vlen(a);
  if (l != 0.0) { a[0] = a[0] / l; a[1] = a[1] / l; a[2] = a[2] / l; }
}

// Slope of each interval of a float table exactly as JDMinterpolate_f
// (finterpo.c:83) forms it: float difference of the ordinates over the
// double difference of the abscissae.  The kernels then only multiply.
static void append_slopes(std::vector<double> &out, const float *x, const float *y, unsigned n) {
  for (unsigned k = 0; k + 1 < n; k++) {
    double x0 = x[k], x1 = x[k + 1];
    float dy = y[k + 1] - y[k];
    out.push_back(x1 == x0 ? 0.0 : (double) dy / (x1 - x0));
  }
}

// True if every energy row of a cumulative table [energy][order] is
// non-decreasing in the order index (the trace may then bisect it).
static bool rows_monotone(const float *cum, size_t nenergy, int norders) {
  for (size_t j = 0; j < nenergy; j++)
    for (int k = 0; k + 1 < norders; k++)
      if (!(cum[j * norders + k] <= cum[j * norders + k + 1])) return false;
  return true;
}

// JDMbinary_search_f (finterpo.c:37-57): the first index with xp >= x (an
// equal element returns its index), n if every element is smaller.
static unsigned jdm_bsearch_f(float x, const float *xp, unsigned n) {
  unsigned n0 = 0, n1 = n;
  while (n1 > n0 + 1) {
    unsigned n2 = (n0 + n1) / 2;
    if (xp[n2] >= x) {
      if (xp[n2] == x) return n2;
      n1 = n2;
    } else
      n0 = n2;
  }
  if (x >= xp[n0]) return n1;
  return n0;
}

// JDMinterpolate_f (finterpo.c:59-86); the ordinate difference is a float
// difference, the rest is double, as the reference writes it.
static float jdm_interp_f(float x, const float *xp, const float *yp, unsigned n) {
  if (n == 1) return yp[0];
  unsigned n1 = jdm_bsearch_f(x, xp, n), n0 = n1 - 1;
  if (n1 < n && x == xp[n1]) return yp[n1];
  if (n1 == n) { n1--; n0--; }
  if (n1 == 0) n0 = 1;
  double x0 = xp[n0], x1 = xp[n1];
  if (x1 == x0) return yp[n1];
  return (float) (yp[n0] + (yp[n1] - yp[n0]) / (x1 - x0) * (x - x0));
}

// JDMinterpolate_n_fvector (finterpo.c:134-190) of ny columns at sorted x.
static void jdm_interp_n(const float *x, unsigned n, const float *oldx, const float *const *oldy, unsigned oldn,
                         unsigned ny, float *const *out) {
  unsigned pos = 1;
  for (unsigned j = 0; j < n; j++) {
    double xv = x[j];
    while (pos < oldn - 1 && xv > oldx[pos]) pos++;
    double x0 = oldx[pos - 1], x1 = oldx[pos], dx = x1 - x0;
    for (unsigned i = 0; i < ny; i++) {
      if (dx == 0.0) out[i][j] = oldy[i][pos - 1];
      else {
        double y0 = oldy[i][pos - 1], y1 = oldy[i][pos];
        out[i][j] = (float) (y0 + (y1 - y0) * (xv - x0) / dx);
      }
    }
  }
}

// grating_efficiency (diffract.c:269-305) of a bar grating without material
// layers (the LETG support gratings): the transmission factor is exp(0) = 1.
static double bar_efficiency(int order, double energy, double beta, double delta, double period, double bar_height,
                             double bar_width) {
  double a = 1.0 - bar_width / period;
  double k = energy / HBAR_C;
  double kh = bar_height * k;
  double khb = kh * beta;
  double ekhb = exp(-khb);
  double eff;
  if (order != 0) {
    double mpi = order * PI_;
    a = sin(mpi * a) / mpi;
    eff = a * a * (1 + ekhb * (ekhb - 2.0 * cos(kh * delta)));
  } else {
    double b = 1 - a;
    eff = a * a + b * ekhb * (b * ekhb + 2 * a * cos(kh * delta));
  }
  return eff * 1.0;
}

// The LETG (_marx_letg_init, diffract.c:1727-1860): per-shell primary
// efficiencies from the CALDB table (init_file_efficiencies with scale 1,
// sum_file_efficiencies), the fine and coarse support gratings computed on
// the grating energy grid (marx_create_grating_opt_const_tables,
// diffract.c:1167-1188, read_grating_optical_consts :195-258,
// init_one_grating :350-440), and the primary efficiencies divided by the
// supports' total efficiencies (diffract.c:1790-1857).
static bool build_letg(const Pack &pk, const mx_config &cfg, HostModel &M, std::string &err) {
  MxTables &T = M.T;
  const int nf = cfg.leg_fine_orders, nc = cfg.leg_coarse_orders;
  if (nf < 0 || nc < 0 || nf > 127 || nc > 127 || (nf && nf % 2 == 0) || (nc && nc % 2 == 0)) {
    err = "legFineNumOrders and legCoarseNumOrders must be odd and at most 127"; return false;
  }
  if (nf == 0 || nc == 0) { err = "the LETG needs both support gratings (legFineNumOrders, legCoarseNumOrders > 0)"; return false; }
  // grating energy grid: 1024 points from 0.03 keV in steps of (10 - 0.03) / 1024
  const unsigned NE = 1024;
  std::vector<float> E(NE);
  {
    double d = (10.0 - 0.03) / NE, e = 0.03;
    for (unsigned i = 0; i < NE; i++) { E[i] = (float) e; e += d; }
  }
  size_t cnt;
  const float *oc = pk.get<float>("grating/optconst", &cnt, err);   // [7][rows]: E beta delta gold poly cr ni
  if (!oc) return false;
  unsigned rows = (unsigned) (cnt / 7);
  if (rows < 2) { err = "grating optical constants malformed"; return false; }
  std::vector<float> beta(NE), delta(NE);
  {
    const float *oy[2] = {oc + rows, oc + 2 * rows};
    float *out[2] = {beta.data(), delta.data()};
    jdm_interp_n(E.data(), NE, oc, oy, rows, 2, out);
  }
  // support gratings: cumulative efficiencies [order][energy] over the
  // order list 0, +1, -1, +2, -2, ...
  auto support = [&](int norders, double period, double bh, double bw, std::vector<float> &cum) {
    cum.assign((size_t) norders * NE, 0.0f);
    for (unsigned i = 0; i < NE; i++) {
      double sum = 0.0;
      for (int k = 0; k < norders; k++) {
        int order = (k & 1) ? (k + 1) / 2 : -(k / 2);
        sum += bar_efficiency(order, E[i], beta[i], delta[i], period, bh, bw);
        cum[(size_t) k * NE + i] = (float) sum;
      }
    }
  };
  std::vector<float> fine, coarse;
  support(nf, cfg.leg_fine_period, cfg.leg_fine_bar_height, cfg.leg_fine_bar_width, fine);
  support(nc, cfg.leg_coarse_period, cfg.leg_coarse_bar_height, cfg.leg_coarse_bar_width, coarse);
  const float *fine_tot = fine.data() + (size_t) (nf - 1) * NE, *coarse_tot = coarse.data() + (size_t) (nc - 1) * NE;

  const bool acis = cfg.detector == MX_DETECTOR_ACIS_I || cfg.detector == MX_DETECTOR_ACIS_S;
  for (int i = 0; i < 4; i++) {
    MxGratingDev &g = M.gratings[4 + i];
    memset(&g, 0, sizeof(g));
    if (!(cfg.letg_period[i] > 0)) { err = "LETG period must be > 0"; return false; }
    size_t ne, neff;
    const float *e = pk.get<float>("letg/geff" + std::to_string(i) + "/energy", &ne, err);
    const float *eff = pk.get<float>("letg/geff" + std::to_string(i) + "/eff", &neff, err);
    if (!e || !eff) return false;
    unsigned no = (unsigned) (neff / ne);
    if (ne < 2 || no < 3 || (no % 2) != 1) { err = "grating efficiency table malformed"; return false; }
    int max_order = (int) (no / 2);
    std::vector<float> cum(eff, eff + neff);   // [order][energy]
    for (unsigned j = 0; j < ne; j++) {         // sum_file_efficiencies with scale 1
      double sum = 0.0;
      for (unsigned k = 0; k < no; k++) { sum += 1.0 * (double) cum[k * ne + j]; cum[k * ne + j] = (float) sum; }
      if (sum > 1.0)
        for (unsigned k = 0; k < no; k++) cum[k * ne + j] = (float) (cum[k * ne + j] / sum);
    }
    for (unsigned j = 0; j < ne; j++) {         // divide out the fine support grating
      float f = jdm_interp_f(e[j], E.data(), fine_tot, NE);
      f = (float) (1.0 / f);
      if (f <= 0) continue;
      for (unsigned k = 0; k < no; k++) cum[k * ne + j] *= f;
    }
    for (unsigned j = 0; j < ne; j++) {         // and the coarse one, met three times
      float f = jdm_interp_f(e[j], E.data(), coarse_tot, NE);
      f = f * f * f;
      if (f <= 0) continue;
      f = (float) (1.0 / f);
      for (unsigned k = 0; k < no; k++) cum[k * ne + j] *= f;
    }
    g.geff_off = (int32_t) M.geff_energy.size();
    M.geff_energy.insert(M.geff_energy.end(), e, e + ne);
    g.cum_off = (int32_t) M.geff_cum.size();
    for (unsigned j = 0; j < ne; j++)
      for (unsigned k = 0; k < no; k++) M.geff_cum.push_back(cum[k * ne + j]);   // [energy][order]
    g.nenergy = (int32_t) ne; g.norders = (int32_t) no; g.max_order = max_order;
    g.monotone = rows_monotone(M.geff_cum.data() + g.cum_off, ne, (int) no);
    g.order_off = (int32_t) M.order_k.size();
    for (unsigned k = 0; k < no; k++) {
      int order = (int) k - max_order;
      M.order_k.push_back(order * (2.0 * PI_ * HBAR_C) / cfg.letg_period[i]);
    }
    double disp = (cfg.letg_theta[i] * (PI_ / 180.0));
    if (acis) disp += cfg.letg_acis_dtheta * (PI_ / 180.0);
    double th = -1 * disp;
    g.cos_m = cos(th); g.sin_m = sin(th);
    th = 1 * disp;
    g.cos_p = cos(th); g.sin_p = sin(th);
    g.theta_blur = (cfg.letg_dtheta[i] * (PI_ / 180.0) / 60.0);
    g.dp_over_p = cfg.letg_dpp[i];
    g.vig = cfg.letg_vig[i];
    g.rowland = cfg.leg_rowland;
    g.nsec = 0;
  }
  // support tables on the device: the energy grid, [energy][order] per grating
  M.support_energy = E;
  M.support_cum.clear();
  M.support_k.clear();
  auto put = [&](const std::vector<float> &cum, int norders, double period) {
    int32_t off = (int32_t) M.support_cum.size();
    for (unsigned i = 0; i < NE; i++)
      for (int k = 0; k < norders; k++) M.support_cum.push_back(cum[(size_t) k * NE + i]);
    int32_t koff = (int32_t) M.support_k.size();
    for (int k = 0; k < norders; k++) {
      int order = (k & 1) ? (k + 1) / 2 : -(k / 2);
      M.support_k.push_back(order * (2.0 * PI_ * HBAR_C) / period);
    }
    return std::make_pair(off, koff);
  };
  auto pf = put(fine, nf, cfg.leg_fine_period), pc = put(coarse, nc, cfg.leg_coarse_period);
  const double angle[4] = {PI_ / 2.0, PI_ / 3.0, 2.0 * PI_ / 3.0, 0.0};
  for (int s = 0; s < 4; s++) {
    MxSupportDev &d = T.supports[s];
    const bool isf = s == 0;
    d.cum_off = isf ? pf.first : pc.first;
    d.order_off = isf ? pf.second : pc.second;
    d.norders = isf ? nf : nc;
    d.monotone = rows_monotone(M.support_cum.data() + d.cum_off, NE, d.norders);
    d.rotate = angle[s] != 0.0;
    d.cos_t = cos(angle[s]); d.sin_t = sin(angle[s]);
  }
  T.support_nenergy = (int32_t) NE;
  return true;
}

// ------------------------------------------------------------------ HRC --
static void v3_sum(double r[3], const double a[3], const double b[3]) { for (int k = 0; k < 3; k++) r[k] = a[k] + b[k]; }
static void v3_diff(double r[3], const double a[3], const double b[3]) { for (int k = 0; k < 3; k++) r[k] = a[k] - b[k]; }
static double v3_dot(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void v3_ax_by(double r[3], double a, const double x[3], double b, const double y[3]) {  // JDMv_ax1_bx2
  for (int k = 0; k < 3; k++) r[k] = a * x[k] + b * y[k];
}
static void v3_cross(double c[3], const double a[3], const double b[3]) {  // JDMv_cross_prod (vector.c:29)
  double t[3];
  t[2] = a[0] * b[1] - a[1] * b[0];
  t[0] = a[1] * b[2] - a[2] * b[1];
  t[1] = a[2] * b[0] - a[0] * b[2];
  memcpy(c, t, sizeof(t));
}

// A facet from its four corners: the CALDB aimpoint and origin offset
// (_marx_caldb_patch_aimpoint, caldb.c:468-491), then the basis
// (_marx_compute_detector_basis, detector.c:383-401).
static MxChipDev facet(int id, const double ll0[3], const double lr0[3], const double ul0[3], const double aim[3],
                       const double orig[3]) {
  MxChipDev c;
  memset(&c, 0, sizeof(c));
  c.id = id;
  double ofs[3], ll[3], lr[3], ul[3], xh[3], yh[3];
  v3_sum(ofs, aim, orig);
  v3_sum(ll, ll0, ofs); v3_sum(lr, lr0, ofs); v3_sum(ul, ul0, ofs);
  v3_diff(xh, lr, ll); v3_diff(yh, ul, ll);
  c.xlen = vlen(xh); c.ylen = vlen(yh);
  vnorm(xh); vnorm(yh);
  double nrm[3];
  v3_cross(nrm, xh, yh);
  for (int k = 0; k < 3; k++) { c.x_ll[k] = ll[k]; c.xhat[k] = xh[k]; c.yhat[k] = yh[k]; c.normal[k] = nrm[k]; }
  c.xpix = c.ypix = 1.0; c.inv_xpix = c.inv_ypix = 1.0;
  for (int k = 0; k < 3; k++) {
    c.f_ll[k] = (float) c.x_ll[k]; c.f_xhat[k] = (float) c.xhat[k];
    c.f_yhat[k] = (float) c.yhat[k]; c.f_normal[k] = (float) c.normal[k];
  }
  c.f_xlen = (float) c.xlen; c.f_ylen = (float) c.ylen;
  return c;
}

// Append a bdat table (energies, values) to the HRC float tables with the
// interval slopes JDMinterpolate_f forms (float dy over double dx).
static bool hrc_table(const Pack &pk, const std::string &name, int col, HostModel &M, MxTabDev &t, std::string &err) {
  size_t cnt;
  const float *a = pk.get<float>(name, &cnt, err);
  if (!a) return false;
  int ncol = name.find("optconst") != std::string::npos ? 3 : 2;
  unsigned n = (unsigned) (cnt / ncol);
  if (n < 1) { err = name + ": empty table"; return false; }
  t.x_off = (int32_t) M.hrc_tab.size();
  M.hrc_tab.insert(M.hrc_tab.end(), a, a + n);
  t.y_off = (int32_t) M.hrc_tab.size();
  M.hrc_tab.insert(M.hrc_tab.end(), a + (size_t) col * n, a + (size_t) (col + 1) * n);
  t.s_off = (int32_t) M.hrc_slope.size();
  append_slopes(M.hrc_slope, a, a + (size_t) col * n, n);
  M.hrc_slope.push_back(0.0);
  t.n = (int32_t) n;
  return true;
}

// fixup_blur_parms (hrcblur.c:105-188): amplitudes to weights, pixels to mm.
static bool hrc_blur(const double *b, double pixelsize, MxHrcDev &h, std::string &err) {
  double g1s = b[0], g1x = b[1], g1y = b[2], g1w = b[3], g2s = b[4], g2x = b[5], g2y = b[6], g2w = b[7];
  double l1h = b[8], l1x = b[9], l1y = b[10], l1w = b[11], l1r = b[12];
  if (g1w < 0 || g2w < 0 || l1w < 0 || g1s <= 0 || g2s <= 0 || l1h <= 0 || l1r <= 0) {
    err = "One or more of the HRC blur parameters has an invalid/unsupported value"; return false;
  }
  const double fwhm_to_sigma = 0.42466090014400953;
  g1s *= pixelsize; g1x *= pixelsize; g1y *= pixelsize;
  g2s *= pixelsize; g2x *= pixelsize; g2y *= pixelsize;
  l1h *= pixelsize; l1x *= pixelsize; l1y *= pixelsize; l1r *= pixelsize;
  g2x -= g1x; g2y -= g1y; l1x -= g1x; l1y -= g1y;
  g1s *= fwhm_to_sigma; g2s *= fwhm_to_sigma; l1h *= 0.5;
  double norm = 1.0 / (2 * PI_ * g1s * g1s);
  g1w /= norm;
  norm = 1.0 / (2 * PI_ * g2s * g2s);
  g2w /= norm;
  double g2 = l1h; g2 = g2 * g2;
  norm = 1.0 / (g2 * PI_ * log(1 + l1r * l1r / g2));
  l1w /= norm;
  norm = g1w + g2w + l1w;
  if (norm > 0) { g1w /= norm; g2w /= norm; l1w /= norm; }
  h.g1_sigma = g1s; h.g1_w = g1w; h.g2_sigma = g2s; h.g2_x = g2x; h.g2_y = g2y; h.g2_w = g2w;
  h.l1_hwhm = l1h; h.l1_x = l1x; h.l1_y = l1y; h.l1_rmax = l1r; h.l1_w = l1w;
  return true;
}

// The HRC-I (hrc_i_geom.c:48-130, hrc-i.c:183-228) or HRC-S (hrc_s_geom.c,
// hrc-s.c:352-441, drake.c:148-246).  Facets go to chips[10] (HRC-I) and
// chips[11..13] (HRC-S MCPs 1, 2, 3).
// The ACIS FEF regions of the detector's chips (read_fef_file,
// process_rows, process_region_rows and map_fef_to_region,
// acis_fef.c:194-295, 619-874).  The pack holds the FUNCTION table's rows
// as acis/fef/rows (CCD_ID, CHIPX_LO, CHIPX_HI, CHIPY_LO, CHIPY_HI,
// REGNUM) and acis/fef/vals (ENERGY, CHANNEL, then G<k>_FWHM, G<k>_POS,
// G<k>_AMPL per gaussian).  Consecutive rows of one REGNUM are one region,
// its energies ascending.
static bool build_fef(const Pack &pk, int min_ccd, int max_ccd, HostModel &M, std::string &err) {
  const int REG = 32, NREG = 1024 / REG;
  const double FWHM_TO_SIGMA = 0.4246609001440095;
  size_t nr, nv;
  const int32_t *rows = pk.get<int32_t>("acis/fef/rows", &nr, err);
  const float *vals = pk.get<float>("acis/fef/vals", &nv, err);
  if (!rows || !vals) return false;
  nr /= 6;
  if (nr == 0 || nv % nr) { err = "acis/fef tables malformed"; return false; }
  const size_t ncol = nv / nr;
  if (ncol < 5 || (ncol - 2) % 3) { err = "acis/fef tables malformed"; return false; }
  const int ng = (int) ((ncol - 2) / 3);
  if (ng > MX_FEF_GAUSSIANS) { err = "FEF with more gaussians per row than the engine's " + std::to_string(MX_FEF_GAUSSIANS); return false; }
  M.fef_map.assign((size_t) 10 * NREG * NREG, -1);
  M.fef.clear(); M.fef_f.clear(); M.fef_slope.clear();
  auto finish = [&](const std::vector<size_t> &run) -> bool {   // the rows of one region
    const int32_t *q = rows + 6 * run[0];
    const int ccd = q[0], xmin = q[1], xmax = q[2], ymin = q[3], ymax = q[4];
    MxFefDev f;
    memset(&f, 0, sizeof(f));
    f.n_e = (int32_t) run.size();
    f.n_g = ng;
    f.e_off = (int32_t) M.fef_f.size();
    for (size_t r : run) M.fef_f.push_back(vals[r * ncol]);
    for (size_t r : run) M.fef_f.push_back(vals[r * ncol + 1]);
    f.g_off = (int32_t) M.fef_f.size();
    for (size_t r : run)
      for (int k = 0; k < ng; k++) {
        const float *g = vals + r * ncol + 2 + 3 * k;
        M.fef_f.push_back(g[2]);                                   // amp
        M.fef_f.push_back(g[1]);                                   // center
        M.fef_f.push_back((float) (FWHM_TO_SIGMA * g[0]));         // sigma
      }
    // check_fef_validity: energies and channels increasing
    const float *e = M.fef_f.data() + f.e_off, *ch = e + f.n_e;
    for (int k = 0; k + 1 < f.n_e; k++)
      if (!(e[k] < e[k + 1]) || !(ch[k] < ch[k + 1])) {
        err = "Fef Map does not have monotonically increasing energies and PHAs"; return false;
      }
    f.s_off = (int32_t) M.fef_slope.size();
    append_slopes(M.fef_slope, ch, e, (unsigned) f.n_e);
    // check_region_values, map_fef_to_region
    if (ccd < 0 || ccd >= 10) { err = "Invalid CCD_ID value in gain file"; return false; }
    if (xmin < 1 || ymin < 1 || xmax > 1024 || ymax > 1024) { err = "CHIPX/Y_LO/HI value out of range"; return false; }
    if ((xmax % REG) || (ymax % REG) || ((xmin - 1) % REG) || ((ymin - 1) % REG)) {
      err = "Expecting ACIS gain region size to be a multiple of 32"; return false;
    }
    const int idx = (int) M.fef.size();
    M.fef.push_back(f);
    for (int i = (xmin - 1) / REG; i < xmax / REG; i++)
      for (int j = (ymin - 1) / REG; j < ymax / REG; j++) M.fef_map[((size_t) ccd * NREG + i) * NREG + j] = idx;
    return true;
  };
  // rows of other chips are skipped; a region is a run of rows with one REGNUM
  std::vector<size_t> run;
  int last_reg = -1;
  for (size_t r = 0; r < nr; r++) {
    const int ccd = rows[6 * r];
    if (ccd < min_ccd || ccd > max_ccd) continue;
    const int reg = rows[6 * r + 5];
    if (!run.empty() && reg == last_reg) { run.push_back(r); continue; }
    if (!run.empty() && !finish(run)) return false;
    run.assign(1, r);
    last_reg = reg;
  }
  if (!run.empty() && !finish(run)) return false;
  return true;
}

// JDMbinary_search_d (dinterpo.c:30): the same bisection over doubles.
static unsigned jdm_bsearch_d(double x, const double *xp, unsigned n) {
  unsigned n0 = 0, n1 = n;
  while (n1 > n0 + 1) {
    unsigned n2 = (n0 + n1) / 2;
    if (xp[n2] >= x) {
      if (xp[n2] == x) return n2;
      n1 = n2;
    } else
      n0 = n2;
  }
  if (x >= xp[n0]) return n1;
  return n0;
}

// An energy -> value table of the ACIS response in fef_f / fef_slope.
static MxTabDev response_table(HostModel &M, const float *x, const float *y, unsigned n) {
  MxTabDev t;
  t.n = (int32_t) n;
  t.x_off = (int32_t) M.fef_f.size();
  M.fef_f.insert(M.fef_f.end(), x, x + n);
  t.y_off = (int32_t) M.fef_f.size();
  M.fef_f.insert(M.fef_f.end(), y, y + n);
  t.s_off = (int32_t) M.fef_slope.size();
  append_slopes(M.fef_slope, x, y, n);
  return t;
}

// The chips' CALDB QE (_marx_read_acis_qe, caldb.c:504-575) and
// contamination (read_contam_file_for_ccd and compute_tau_values,
// aciscontam.c:236-487) for the ACIS response with DetIdeal = no.  The
// contamination's epoch is cfg.tstart_mjdsecs.
static bool build_contam(const Pack &pk, const mx_config &cfg, int min_ccd, int max_ccd, HostModel &M,
                         std::string &err) {
  MxContamDev z;
  memset(&z, 0, sizeof(z));
  M.contam.assign(10, z);
  for (int ccd = min_ccd; ccd <= max_ccd; ccd++) {
    MxContamDev &c = M.contam[ccd];
    const std::string k = "acis/contam" + std::to_string(ccd) + "/";
    size_t nq;
    const float *qe = pk.get<float>("acis/qe" + std::to_string(ccd), &nq, err);
    if (!qe) return false;
    if (nq / 2 < 2) { err = "Expecting more than 2 rows in the ACIS QE file"; return false; }
    c.qe = response_table(M, qe, qe + nq / 2, (unsigned) (nq / 2));
    size_t nr, ne, nm, nt, n0, n1;
    const int32_t *rows = pk.get<int32_t>(k + "rows", &nr, err);
    if (!rows) { err = "Unable to open acis contam file for CCD " + std::to_string(ccd); return false; }
    const unsigned L = (unsigned) (nr / 3);
    if (L > MX_CONTAM_LAYERS) { err = "The number of layers in the contamination file is larger than supported"; return false; }
    const float *en = pk.get<float>(k + "energy", &ne, err), *mu = pk.get<float>(k + "mu", &nm, err);
    const double *tm = pk.get<double>(k + "time", &nt, err);
    const float *t0s = pk.get<float>(k + "tau0", &n0, err), *t1s = pk.get<float>(k + "tau1", &n1, err);
    if (!en || !mu || !tm || !t0s || !t1s || L == 0) { if (err.empty()) err = "contamination table malformed"; return false; }
    const size_t re = ne / L, rt = nt / L;
    if (nm / L != re || n0 / L != rt || n1 / L != rt) { err = "contamination table malformed"; return false; }
    const bool has_fxy = pk.sections.count(k + "fxy") > 0;
    const float *fxy = nullptr;
    size_t nf = 0;
    if (has_fxy) {
      fxy = pk.get<float>(k + "fxy", &nf, err);
      const int32_t *blk = pk.get<int32_t>(k + "fxyblk", nullptr, err);
      if (!fxy || !blk) return false;
      c.blk = blk[0];
      if (c.blk <= 0 || c.blk * (1024 / c.blk) != 1024) { err = "Invalid fxyblk value"; return false; }
      if (nf / L != (size_t) (1024 / c.blk) * (1024 / c.blk)) { err = "The FXY column has the wrong size"; return false; }
      c.mode = 2;
    } else if (ccd <= 3) {
      // fxy_acis0..3 (aciscontam.c:138-156)
      static const double cx[4] = {1024.5, 0.5, 0.5, 1024.5};
      c.mode = 0; c.x0 = cx[ccd]; c.y0 = 1024.5;
    } else
      c.mode = 1;   // fxy_acis456789
    c.nl = (int32_t) L;
    for (unsigned l = 0; l < L; l++) {
      if (rows[3 * l] != 0) { err = "Expecting COMPONENT=0 in the contamination file"; return false; }
      const unsigned n_e = (unsigned) rows[3 * l + 1], n_t = (unsigned) rows[3 * l + 2];
      if (n_t <= 1 || n_e <= 1) { err = "Expecting n_energy or n_time to be greater than 1"; return false; }
      if (n_t > rt) { err = "n_time value is larger than data arrays"; return false; }
      if (n_e > re) { err = "n_energy value is larger than data arrays"; return false; }
      const double *times = tm + l * rt;
      const float *e = en + l * re, *m = mu + l * re, *tau0s = t0s + l * rt, *tau1s = t1s + l * rt;
      for (unsigned i = 0; i + 1 < n_t; i++)
        if (!(times[i] < times[i + 1])) { err = "Expecting the time grid to be monotonically increasing"; return false; }
      for (unsigned i = 0; i + 1 < n_e; i++)
        if (!(e[i] < e[i + 1])) { err = "Expecting the ENERGY grid to be monotonically increasing"; return false; }
      // compute_tau_values
      unsigned b1 = jdm_bsearch_d(cfg.tstart_mjdsecs, times, n_t), b0 = b1 - 1;
      if (b1 == n_t) { b1--; b0--; }
      if (b1 == 0) { b1 = 1; b0 = 0; }
      const double t = (cfg.tstart_mjdsecs - times[b0]) / (times[b1] - times[b0]);
      c.tau0[l] = tau0s[b0] + (double) (tau0s[b1] - tau0s[b0]) * t;
      c.tau1[l] = tau1s[b0] + (double) (tau1s[b1] - tau1s[b0]) * t;
      c.mu[l] = response_table(M, e, m, n_e);
      if (has_fxy) {
        const size_t per = nf / L;
        c.fxy_off[l] = (int32_t) M.fef_f.size();
        M.fef_f.insert(M.fef_f.end(), fxy + l * per, fxy + (l + 1) * per);
      }
    }
  }
  return true;
}

static bool build_hrc(const Pack &pk, const mx_config &cfg, HostModel &M, std::string &err) {
  MxTables &T = M.T;
  MxHrcDev &h = T.hrc;
  memset(&h, 0, sizeof(h));
  h.kind = cfg.detector;
  h.blur = !cfg.det_ideal;
  M.hrc_tab.clear(); M.hrc_slope.clear();
  auto table = [&](const char *name, int col, MxTabDev &t) {
    if (cfg.det_ideal) { memset(&t, 0, sizeof(t)); return true; }   // _marx_hrc_read_efficiencies: perfect
    return hrc_table(pk, name, col, M, t, err);
  };
  double pixelsize;
  if (cfg.detector == MX_DETECTOR_HRC_I) {
    size_t n;
    const double *g = pk.get<double>("hrc/i_geom", &n, err);
    const double *aim = pk.get<double>("hrc/aimpt_i", nullptr, err), *org = pk.get<double>("hrc/origin_i", nullptr, err);
    if (!g || !aim || !org) return false;
    if (n != 15) { err = "hrc/i_geom malformed"; return false; }
    const double xps = g[0], yps = g[1];
    const double *LL_XYZ = g + 2, *Center_XYZ = g + 5, *LLtoLR = g + 8, *Center_CXCY = g + 11, *Aim_CXCY = g + 13;
    // setup_coordinate_xforms (hrc_i_geom.c:48-101)
    double a[3] = {LLtoLR[0], LLtoLR[1], LLtoLR[2]};
    double len = vlen(a);
    if (len == 0.0) { err = "Length of vector from LL to LR must be non-zero"; return false; }
    double il = 1.0 / len;
    for (int k = 0; k < 3; k++) a[k] = il * a[k];
    double center[3] = {Center_XYZ[0], Center_XYZ[1], Center_XYZ[2]}, LL[3] = {LL_XYZ[0], LL_XYZ[1], LL_XYZ[2]};
    double ll[3], lr[3], LR[3], UR[3], UL[3], t3[3];
    v3_diff(ll, LL, center);
    if (vlen(ll) == 0.0) { err = "The LL corner must not be the center"; return false; }
    v3_ax_by(lr, 1.0, ll, -2.0 * v3_dot(a, ll), a);
    v3_sum(LR, center, lr);
    for (int k = 0; k < 3; k++) t3[k] = -1.0 * ll[k];
    v3_sum(UR, center, t3);
    for (int k = 0; k < 3; k++) t3[k] = -1.0 * lr[k];
    v3_sum(UL, center, t3);
    if (xps <= 0.0 || yps <= 0.0) { err = "X and Y Pixel sizes must be larger than 0"; return false; }
    double b[3];
    v3_diff(b, UL, LL);
    vnorm(b);
    double llc0 = Center_CXCY[0] + v3_dot(ll, a) / xps, llc1 = Center_CXCY[1] + v3_dot(ll, b) / yps;
    double dx[3];
    v3_ax_by(t3, (llc0 - Aim_CXCY[0]) * xps, a, (llc1 - Aim_CXCY[1]) * yps, b);
    v3_diff(dx, t3, LL);
    double LL2[3], LR2[3], UL2[3];
    v3_sum(LL2, LL, dx); v3_sum(LR2, LR, dx); v3_sum(UL2, UL, dx);
    M.chips[10] = facet(0, LL2, LR2, UL2, aim, org);
    h.ll_cxcy[0] = llc0; h.ll_cxcy[1] = llc1;
    h.pix[0] = xps; h.pix[1] = yps; h.inv_pix[0] = 1.0 / xps; h.inv_pix[1] = 1.0 / yps;
    pixelsize = 0.5 * (xps * 0.25 + yps * 0.25);
    if (!table("hrc/qe_i", 1, h.mcp[0]) || !table("hrc/uvis_i", 1, h.filt[0])) return false;
    if (!hrc_blur(cfg.hrc_i_blur, pixelsize, h, err)) return false;
    T.chip_off = 10; T.nchips = 1;
  } else {
    size_t n;
    const double *g = pk.get<double>("hrc/s_geom", &n, err);
    const double *aim = pk.get<double>("hrc/aimpt_s", nullptr, err), *org = pk.get<double>("hrc/origin_s", nullptr, err);
    if (!g || !aim || !org) return false;
    if (n != 45) { err = "hrc/s_geom malformed"; return false; }
    const double vps = g[0], *V_Active = g + 1, ups = g[7], *U_Active = g + 8, *Aim_Off = g + 10;
    const double *UV[3] = {g + 13, g + 17, g + 15};      // left, middle, right
    const double *XYZ0[3] = {g + 19, g + 25, g + 22};
    const double *CXCY[3] = {g + 28, g + 32, g + 30};
    const double deg = PI_ / 180.0;
    const double left_t = g[34] * deg, right_t = g[35] * deg, det_t = g[36] * deg;
    const double *ion = g + 37;   // T L R X SL SR GapL GapR
    // _marx_hrc_s_geom_init and setup_alphas_and_betas (hrc_s_geom.c:134-180, 446-478)
    double xyz[3][3];
    for (int m = 0; m < 3; m++)
      for (int k = 0; k < 3; k++) xyz[m][k] = XYZ0[m][k] + Aim_Off[k];
    const double alpha[3] = {0.0, 0.0, ups};
    const double beta[3][3] = {{-1.0 * sin(left_t) * vps, -1.0 * cos(left_t) * vps, 0.0},
                               {0.0, -1.0 * vps, 0.0},
                               {1.0 * sin(right_t) * vps, -1.0 * cos(right_t) * vps, 0.0}};
    auto uv_xyz = [&](int m, double u, double v, double out[3]) {   // map_uv_to_xyz (hrc_s_geom.c:98-109)
      double du = u - UV[m][0], dv = v - UV[m][1];
      for (int k = 0; k < 3; k++) out[k] = xyz[m][k] + du * alpha[k] + dv * beta[m][k];
    };
    // rotate_mcp (hrc_s_geom.c:211-224): JDMv_rotate_vector1 about (-1, 0, 0), no normalisation
    const double st = sin(det_t), ct = cos(det_t), axis[3] = {-1, 0, 0};
    auto rot = [&](double p[3]) {
      double pn = v3_dot(p, axis), nxp[3];
      v3_cross(nxp, axis, p);
      double q[3];
      for (int k = 0; k < 3; k++) q[k] = ct * p[k] + pn * (1.0 - ct) * axis[k] + st * nxp[k];
      memcpy(p, q, sizeof(q));
    };
    for (int m = 0; m < 3; m++) {
      double ll[3], lr[3], ul[3];
      uv_xyz(m, U_Active[0], V_Active[2 * m + 1], ul);
      uv_xyz(m, U_Active[0], V_Active[2 * m], ll);
      uv_xyz(m, U_Active[1], V_Active[2 * m], lr);
      rot(ll); rot(lr); rot(ul);
      M.chips[11 + m] = facet(m + 1, ll, lr, ul, aim, org);
      h.v_active0[m] = V_Active[2 * m];
      h.uv0[m][0] = UV[m][0]; h.uv0[m][1] = UV[m][1];
      h.cxcy0[m][0] = CXCY[m][0]; h.cxcy0[m][1] = CXCY[m][1];
    }
    h.u_active0 = U_Active[0];
    h.pix[0] = ups; h.pix[1] = vps; h.inv_pix[0] = 1.0 / ups; h.inv_pix[1] = 1.0 / vps;
    pixelsize = 0.5 * (ups * 0.25 + vps * 0.25);
    // MCP regions: facet ids 1, 2, 3 -> QE files 2, 1, 0 (all mcp_qe_s); filters 0..3
    for (int k = 0; k < 3; k++)
      if (!table("hrc/qe_s", 1, h.mcp[k])) return false;
    const char *uv[4] = {"hrc/uvis_s0", "hrc/uvis_s1", "hrc/uvis_s2", "hrc/uvis_s3"};
    for (int k = 0; k < 4; k++)
      if (!table(uv[k], 1, h.filt[k])) return false;
    if (!hrc_blur(cfg.hrc_s_blur, pixelsize, h, err)) return false;
    // geometric centre of the middle MCP (hrc-s.c:424-431), ion shield
    const MxChipDev &mid = M.chips[12];
    double ur[3], half[3], ur0[3], ofs[3];
    uv_xyz(1, U_Active[1], V_Active[3], ur0);   // the middle MCP's x_ur corner, rotated and offset
    rot(ur0);
    v3_sum(ofs, aim, org);
    v3_sum(ur, ur0, ofs);
    v3_ax_by(half, 0.5, mid.x_ll, 0.5, ur);
    double off[3] = {cfg.det_offset[0], cfg.det_offset[1], cfg.det_offset[2]}, gc[3];
    v3_sum(gc, off, half);
    h.shield_yc = gc[1]; h.shield_zc = gc[2];
    h.shield_t = ion[0]; h.shield_l = ion[1]; h.shield_r = ion[2]; h.shield_x = ion[3];
    h.shield_sl = ion[4]; h.shield_sr = ion[5];
    h.shield_sr_gap = ion[5] + ion[7];
    h.shield_sl_gap = ion[4] + ion[6];
    // Drake flat (_marx_drake_flat_init, drake.c:148-246)
    h.drake_n = 0;
    if (cfg.hrc_hesf) {
      int np = cfg.hesf_n;
      if (np <= 0 || np > 4) { err = "HESFN must lie in 1..4"; return false; }
      double cx = cfg.hesf_offset_x, cz = cfg.hesf_offset_z;
      for (int i = 0; i < np; i++) {
        double ang = cfg.hesf_theta[i] * (PI_ / 180.0);
        double hh = cfg.hesf_height[i], htt = hh * tan(ang);
        for (int side = 0; side < 2; side++) {
          MxPlateDev &r = h.plates[i + side * np];
          double e1[3] = {0.0, side ? -1.0 : 1.0, 0.0}, e2[3] = {hh, 0.0, -htt}, nrm[3], a[3];
          double l2 = vlen(e2);
          vnorm(e2);
          if (side == 0) v3_cross(nrm, e1, e2); else v3_cross(nrm, e2, e1);
          double corner[3] = {cx, side ? -cfg.hesf_gap_y2 : cfg.hesf_gap_y1, cz};
          v3_sum(a, gc, corner);
          for (int k = 0; k < 3; k++) { r.a[k] = a[k]; r.e1[k] = e1[k]; r.e2[k] = e2[k]; r.normal[k] = nrm[k]; }
          r.len1 = cfg.hesf_length; r.len2 = l2;
        }
        cz -= htt;
        cx += hh;
      }
      h.drake_n = 2 * np;
      h.drake_cr_width = cfg.hesf_cr_width;
      if (!hrc_table(pk, "hrc/optconst_c", 1, M, h.c_beta, err) || !hrc_table(pk, "hrc/optconst_c", 2, M, h.c_delta, err) ||
          !hrc_table(pk, "hrc/optconst_cr", 1, M, h.cr_beta, err) || !hrc_table(pk, "hrc/optconst_cr", 2, M, h.cr_delta, err))
        return false;
    }
    T.chip_off = 11; T.nchips = 3;
  }
  if (M.hrc_tab.empty()) { M.hrc_tab.push_back(0.f); M.hrc_slope.push_back(0.0); }
  return true;
}

bool build_model(const Pack &pk, const mx_config &cfg, HostModel &M, std::string &err) {
  M = HostModel();
  MxTables &T = M.T;
  memset(&T, 0, sizeof(T));
  static const int ids[4] = {1, 3, 4, 6};
  T.ideal = cfg.hrma_ideal != 0;
  T.use_blur = !T.ideal && cfg.use_blur;
  T.use_wfold = !T.ideal && cfg.use_wfold;
  T.use_struts = cfg.use_struts != 0;
  T.use_scale = cfg.use_scale_factors != 0;
  T.area_uniform = cfg.aperture_area_uniform != 0;
  T.hrma_vig = cfg.hrma_vig;
  T.source_distance = cfg.source_distance;
  T.cap = cfg.hrma_cap_x;
  double th30 = 30.0 * (PI_ / 180.0);
  T.cos30 = cos(th30); T.sin30 = sin(th30);
  const double sx[3][2] = {{1492.060, 942.266}, {0.5 * 1.965 * 25.4, -0.5 * 1.965 * 25.4}, {-1050.353, -1271.333}};
  const double sw[3][2] = {{0.5 * 0.5 * 25.4, 0.5 * 0.5 * 25.4}, {0.5 * 0.75 * 25.4, 0.5 * 0.75 * 25.4},
                           {0.5 * 0.5 * 25.4, 0.5 * 0.5 * 25.4}};
  memcpy(T.strut_xpos, sx, sizeof(sx));
  memcpy(T.strut_half_width, sw, sizeof(sw));
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 2; k++) {
      T.strut_xf[a][k] = (float) (sx[a][k] + T.cap);
      T.strut_hwf[a][k] = (float) sw[a][k];
    }
  T.cos30f = (float) T.cos30; T.sin30f = (float) T.sin30;

  if (cfg.hrma_vig < 0 || cfg.hrma_vig > 1) { err = "HRMAVig must lie in [0,1]"; return false; }
  for (int i = 0; i < 4; i++)
    if (!(cfg.hetg_period[i] > 0) && cfg.grating == MX_GRATING_HETG) { err = "HETG period must be > 0"; return false; }

  // ---- HRMA shells
  size_t cnt;
  const double *rdb = pk.get<double>("hrma/rdb", &cnt, err);
  if (!rdb) return false;
  if (cnt != 72) { err = "hrma/rdb must hold 8 x 9 values"; return false; }
  const float *opt = pk.get<float>("hrma/optconst", &cnt, err);
  if (!opt) return false;
  unsigned optn = (unsigned) (cnt / 3);
  T.opt_n = T.ideal ? 0 : (int32_t) optn;
  M.optc.assign(opt, opt + 3 * optn);
  append_slopes(M.optc_slope, opt, opt + optn, optn);          // beta
  append_slopes(M.optc_slope, opt, opt + 2 * optn, optn);      // delta
  double total_area = 0.0;
  M.shells.resize(4);
  for (int i = 0; i < 4; i++) {
    MxShellDev &h = M.shells[i];
    memset(&h, 0, sizeof(h));
    double cap_pos = cfg.hrma_cap_x + cfg.shell_xoffset[i];
    double len[2];
    for (int o = 0; o < 2; o++) {
      const double *q = rdb + (4 * o + i) * 9;   // x0 y0 z0 p k rho0 az el l
      len[o] = q[8];
      h.c[o] = q[5] * q[5]; h.b[o] = -2.0 * q[4]; h.a[o] = 1.0 - q[3];
      h.am1[o] = h.a[o] - 1.0; h.hb[o] = 0.5 * h.b[o];
      h.xmin[o] = -0.5 * q[8]; h.xmax[o] = 0.5 * q[8];
      h.to_osac[o][0] = -(-q[2]) - cap_pos;
      h.to_osac[o][1] = (-q[0]);
      h.to_osac[o][2] = -(-q[1]);
      double el = -q[7] * (PI_ / 180.0), az = -q[6] * (PI_ / 180);
      double rz[9], ry[9], ny[3];
      rot_z(rz, -az);
      ny[0] = rz[1]; ny[1] = rz[4]; ny[2] = rz[7];   // rz * (0,1,0)
      ny[0] = rz[0] * 0 + rz[1] * 1 + rz[2] * 0;
      ny[1] = rz[3] * 0 + rz[4] * 1 + rz[5] * 0;
      ny[2] = rz[6] * 0 + rz[7] * 1 + rz[8] * 0;
      rot_axis(ry, ny, -el);
      mat3_mul(h.fwd[o], ry, rz);
      rot_axis(ry, ny, el);
      rot_z(rz, az);
      mat3_mul(h.bwd[o], rz, ry);
    }
    mat3_mul(h.mid, h.fwd[1], h.bwd[0]);
    {
      const double dt[3] = {h.to_osac[1][0] - h.to_osac[0][0], h.to_osac[1][1] - h.to_osac[0][1],
                            h.to_osac[1][2] - h.to_osac[0][2]};
      for (int r = 0; r < 3; r++)
        h.mid_off[r] = h.fwd[1][3 * r] * dt[0] + h.fwd[1][3 * r + 1] * dt[1] + h.fwd[1][3 * r + 2] * dt[2];
      for (int k = 0; k < 9; k++) h.bwd0f[k] = (float) h.bwd[0][k];
      for (int r = 0; r < 3; r++) h.osac0f[r] = (float) h.to_osac[0][r];
    }
    const double *qp = rdb + i * 9;
    h.front_position = cap_pos - qp[2] + h.xmax[0];
    for (int r = 0; r < 3; r++) h.front_fwd[r] = h.fwd[0][3 * r] * (h.front_position + h.to_osac[0][0]);
    auto radius = [](double a, double b, double c, double x) { return sqrt(c + x * (b + x * (a - 1))); };
    h.min_radius = radius(h.a[0], h.b[0], h.c[0], h.xmin[0]);
    h.max_radius = radius(h.a[0], h.b[0], h.c[0], h.xmax[0]);
    h.min_radius -= len[0] * tan(0.67 * PI_ / 180);
    h.dr = h.max_radius - h.min_radius;
    h.shutter = cfg.shutters[i] & 0xF;
    unsigned nopen = (unsigned) __builtin_popcount(h.shutter);
    if (nopen) total_area += (nopen / 4.0) * (h.max_radius - h.min_radius) * (h.max_radius + h.min_radius);
    h.area_fraction = total_area;
    h.blur[0] = cfg.blur_p[i] * (1.0 / 3600.0 * PI_ / 180.0);
    h.blur[1] = cfg.blur_h[i] * (1.0 / 3600.0 * PI_ / 180.0);
    h.scat[0] = cfg.scat_p[i]; h.scat[1] = cfg.scat_h[i];
    const float *corr = pk.get<float>("hrma/corr" + std::to_string(ids[i]), &cnt, err);
    if (!corr) return false;
    h.corr_off = (int32_t) (M.optc.size() - 3 * optn);
    h.corr_n = (int32_t) (cnt / 2);
    M.optc.insert(M.optc.end(), corr, corr + cnt);
    h.corr_slope_off = (int32_t) M.optc_slope.size();
    append_slopes(M.optc_slope, corr, corr + h.corr_n, (unsigned) h.corr_n);
  }
  if (total_area <= 0.0) { err = "The mirror geometric area is 0.  Check shutters."; return false; }
  M.geom_area_cm2 = (total_area * PI_) / 100.0;
  for (auto &h : M.shells) h.area_fraction = h.area_fraction / total_area;
  T.optc_len = (int32_t) M.optc.size();
  if (M.optc_slope.empty()) M.optc_slope.push_back(0.0);
  T.slope_len = (int32_t) M.optc_slope.size();

  // ---- WFold tables: index 2*shell + optic
  M.fold_hdr.assign((size_t) 8 * MX_FOLD_MAX * 8, 0.0);
  M.fold_ealpha.assign((size_t) 8 * MX_FOLD_MAX, 0.0);
  M.fold_inv_de.assign((size_t) 8 * MX_FOLD_MAX, 0.0);
  M.fold_theta.assign((size_t) 8 * MX_FOLD_MAX * MX_FOLD_THETA, 0.0f);
  for (int i = 0; i < 4; i++)
    for (int o = 0; o < 2; o++) {
      std::string base = std::string("wfold/") + (o ? "h" : "p") + std::to_string(ids[i]);
      size_t nh, nt;
      const double *hd = pk.get<double>(base + "/hdr", &nh, err);
      const float *th = pk.get<float>(base + "/theta", &nt, err);
      if (!hd || !th) return false;
      size_t narr = nh / 7, nmax = narr ? nt / narr : 0;
      if (narr == 0 || narr > MX_FOLD_MAX || nmax > MX_FOLD_THETA) { err = base + ": table too large"; return false; }
      int t = 2 * i + o;
      T.fold_num[t] = (uint32_t) narr;
      for (size_t a = 0; a < narr; a++) {
        double *dst = &M.fold_hdr[((size_t) t * MX_FOLD_MAX + a) * 8];
        memcpy(dst, hd + 7 * a, 7 * sizeof(double));
        if (hd[7 * a + 6] > (double) nmax || hd[7 * a + 6] < 1) { err = base + ": bad angle count"; return false; }
        M.fold_ealpha[(size_t) t * MX_FOLD_MAX + a] = hd[7 * a];
        dst[7] = 1.0 / hd[7 * a + 2];
        if (a + 1 < narr) M.fold_inv_de[(size_t) t * MX_FOLD_MAX + a] = 1.0 / (hd[7 * (a + 1)] - hd[7 * a]);
        memcpy(&M.fold_theta[((size_t) t * MX_FOLD_MAX + a) * MX_FOLD_THETA], th + a * nmax, nmax * sizeof(float));
      }
    }

  // ---- HETG
  // The HETG tables are built whatever the configured grating, so that a
  // batch of sources can choose per source.
  T.grating = cfg.grating;
  if (cfg.grating != MX_GRATING_NONE && cfg.grating != MX_GRATING_HETG && cfg.grating != MX_GRATING_LETG) {
    err = "unsupported grating"; return false;
  }
  M.gratings.assign(MX_MAX_GRATINGS, MxGratingDev());
  {
    for (int i = 0; i < 4; i++) {
      MxGratingDev &g = M.gratings[i];
      memset(&g, 0, sizeof(g));
      size_t ne, neff;
      const float *e = pk.get<float>("hetg/geff" + std::to_string(i) + "/energy", &ne, err);
      const float *eff = pk.get<float>("hetg/geff" + std::to_string(i) + "/eff", &neff, err);
      if (!e || !eff) return false;
      unsigned no = (unsigned) (neff / ne);
      if (ne < 2 || no < 3 || (no % 2) != 1) { err = "grating efficiency table malformed"; return false; }
      int max_order = (int) (no / 2);
      std::vector<float> cum(eff, eff + neff);   // [order][energy]
      if (cfg.max_order > 0) {
        for (unsigned j = 0; j < ne; j++) {
          double tot = 0.0, kept = 0.0;
          for (unsigned k = 0; k < no; k++) {
            tot += (double) cum[k * ne + j];
            if (abs((int) k - max_order) <= cfg.max_order) kept += (double) cum[k * ne + j];
          }
          for (unsigned k = 0; k < no; k++)
            cum[k * ne + j] = (abs((int) k - max_order) <= cfg.max_order && kept > 0.0)
                                  ? (float) ((double) cum[k * ne + j] * (tot / kept)) : 0.0f;
        }
      }
      for (unsigned j = 0; j < ne; j++) {   // sum_file_efficiencies with scale 1
        double sum = 0.0;
        for (unsigned k = 0; k < no; k++) { sum += 1.0 * (double) cum[k * ne + j]; cum[k * ne + j] = (float) sum; }
        if (sum > 1.0)
          for (unsigned k = 0; k < no; k++) cum[k * ne + j] = (float) (cum[k * ne + j] / sum);
      }
      g.geff_off = (int32_t) M.geff_energy.size();
      M.geff_energy.insert(M.geff_energy.end(), e, e + ne);
      g.cum_off = (int32_t) M.geff_cum.size();
      for (unsigned j = 0; j < ne; j++)
        for (unsigned k = 0; k < no; k++) M.geff_cum.push_back(cum[k * ne + j]);   // [energy][order]
      g.nenergy = (int32_t) ne; g.norders = (int32_t) no; g.max_order = max_order;
      g.monotone = rows_monotone(M.geff_cum.data() + g.cum_off, ne, (int) no);
      g.order_off = (int32_t) M.order_k.size();
      for (unsigned k = 0; k < no; k++) {
        int order = (int) k - max_order;
        M.order_k.push_back(order * (2.0 * PI_ * HBAR_C) / cfg.hetg_period[i]);
      }
      double disp = (cfg.hetg_theta[i] * (PI_ / 180.0));
      double th = -1 * disp;
      g.cos_m = cos(th); g.sin_m = sin(th);
      th = 1 * disp;
      g.cos_p = cos(th); g.sin_p = sin(th);
      g.theta_blur = (cfg.hetg_dtheta[i] * (PI_ / 180.0) / 60.0);
      g.dp_over_p = cfg.hetg_dpp[i];
      g.vig = cfg.hetg_vig[i];
      g.rowland = i < 2 ? cfg.meg_rowland : cfg.heg_rowland;
      g.nsec = 0;
      if (cfg.use_sector_files) {
        size_t ns;
        const double *s = pk.get<double>("hetg/sector" + std::to_string(ids[i]), &ns, err);
        if (!s) return false;
        ns /= 6;
        if (ns == 0 || ns > MX_MAX_SECTORS) { err = "sector table size"; return false; }
        g.sec_off = (int32_t) M.sectors.size();
        g.nsec = (int32_t) ns;
        std::vector<double> cols(6 * ns);
        for (size_t k = 0; k < ns; k++) {
          cols[0 * ns + k] = s[6 * k] * (PI_ / 180.0);
          cols[1 * ns + k] = s[6 * k + 1] * (PI_ / 180.0);
          cols[2 * ns + k] = s[6 * k + 2] * (PI_ / (180.0 * 60.0));
          cols[3 * ns + k] = s[6 * k + 3] * (PI_ / (180.0 * 60.0));
          cols[4 * ns + k] = s[6 * k + 4];
          cols[5 * ns + k] = s[6 * k + 5];
        }
        M.sectors.insert(M.sectors.end(), cols.begin(), cols.end());
      }
    }
  }
  if (cfg.grating == MX_GRATING_LETG && !build_letg(pk, cfg, M, err)) return false;
  if (M.geff_energy.empty()) M.geff_energy.push_back(0.f);
  if (M.geff_cum.empty()) M.geff_cum.push_back(0.f);
  if (M.order_k.empty()) M.order_k.push_back(0.0);
  if (M.sectors.empty()) M.sectors.push_back(0.0);

  // ---- detector chips: ACIS-I (ids 0-3, aimpoint AI2) then ACIS-S (ids
  // 4-9, aimpoint AS1), each set as the reference builds it for that
  // detector; a chip's index in the table is its id.
  if (cfg.detector < MX_DETECTOR_NONE || cfg.detector > MX_DETECTOR_HRC_S) { err = "unsupported detector"; return false; }
  const bool acis = cfg.detector == MX_DETECTOR_ACIS_I || cfg.detector == MX_DETECTOR_ACIS_S;
  {
    size_t ng = 0;
    const double *geom = pk.get<double>("acis/geom", &ng, err);
    const double *orig = pk.get<double>("acis/origin", nullptr, err);
    const double *aim_i = pk.get<double>("acis/aimpt_i", nullptr, err);
    const double *aim_s = pk.get<double>("acis/aimpt_s", nullptr, err);
    if (!geom || !orig || !aim_i || !aim_s) return false;
    ng /= 13;
    for (int id = 0; id <= 9; id++) {
      const double *aim = id < 4 ? aim_i : aim_s;
      double ofs[3] = {aim[0] + orig[0], aim[1] + orig[1], aim[2] + orig[2]};
      double ll[3] = {0, 0, 0}, lr[3] = {0, 0, 0}, ul[3] = {0, 0, 0};
      bool found = false;
      for (size_t r = 0; r < ng; r++)
        if ((int) geom[13 * r] == id) {
          const double *q = geom + 13 * r;
          for (int k = 0; k < 3; k++) { ll[k] = q[1 + k]; lr[k] = q[4 + k]; ul[k] = q[7 + k]; }
          found = true;
        }
      if (!found) { err = "chip missing from the geometry table"; return false; }
      MxChipDev c;
      memset(&c, 0, sizeof(c));
      c.id = id;
      double xh[3], yh[3];
      for (int k = 0; k < 3; k++) {
        lr[k] = lr[k] + ofs[k]; ll[k] = ll[k] + ofs[k]; ul[k] = ul[k] + ofs[k];
        xh[k] = lr[k] - ll[k]; yh[k] = ul[k] - ll[k];
      }
      c.xlen = vlen(xh); c.ylen = vlen(yh);
      vnorm(xh); vnorm(yh);
      for (int k = 0; k < 3; k++) { c.x_ll[k] = ll[k]; c.xhat[k] = xh[k]; c.yhat[k] = yh[k]; }
      c.normal[2] = xh[0] * yh[1] - xh[1] * yh[0];
      c.normal[0] = xh[1] * yh[2] - xh[2] * yh[1];
      c.normal[1] = xh[2] * yh[0] - xh[0] * yh[2];
      c.xpix = c.xlen / 1024.0; c.ypix = c.ylen / 1024.0;
      c.inv_xpix = 1.0 / c.xpix; c.inv_ypix = 1.0 / c.ypix;
      for (int k = 0; k < 3; k++) {
        c.f_ll[k] = (float) c.x_ll[k]; c.f_xhat[k] = (float) c.xhat[k];
        c.f_yhat[k] = (float) c.yhat[k]; c.f_normal[k] = (float) c.normal[k];
      }
      c.f_xlen = (float) c.xlen; c.f_ylen = (float) c.ylen;
      M.chips.push_back(c);
    }
    if (acis && cfg.acis_exposure_time <= 0) {
      err = "ACIS_Exposure_Time must be greater than 0"; return false;
    }
    M.chips.resize(MX_MAX_CHIPS);
    T.chip_off = cfg.detector == MX_DETECTOR_ACIS_S ? 4 : 0;
    T.nchips = cfg.detector == MX_DETECTOR_NONE ? 0 : (cfg.detector == MX_DETECTOR_ACIS_I ? 4 : 6);
    T.det_kind = cfg.detector;
    T.det_ideal = cfg.det_ideal != 0;
    M.hrc_tab.clear(); M.hrc_slope.clear();
    memset(&T.hrc, 0, sizeof(T.hrc));
    if (!acis && cfg.detector != MX_DETECTOR_NONE && !build_hrc(pk, cfg, M, err)) return false;
    if (M.hrc_tab.empty()) { M.hrc_tab.push_back(0.f); M.hrc_slope.push_back(0.0); }
    // the FEF when the pack carries one (the reference's ACIS detector needs
    // the file; without it the detection stays geometric)
    M.fef_map.clear(); M.fef.clear(); M.fef_f.clear(); M.fef_slope.clear();
    T.acis_fef = 0;
    if (acis && pk.sections.count("acis/fef/rows")) {
      if (!build_fef(pk, cfg.detector == MX_DETECTOR_ACIS_I ? 0 : 4, cfg.detector == MX_DETECTOR_ACIS_I ? 3 : 9, M, err))
        return false;
      T.acis_fef = M.fef.empty() ? 0 : 1;
    }
    T.fef_nregions = (int32_t) M.fef.size();
    // the QE and contamination acceptance of DetIdeal = no, when the pack
    // carries contamination tables (without them ACIS detection is ideal)
    M.contam.clear();
    T.acis_qe = 0;
    if (acis && !cfg.det_ideal && pk.sections.count(std::string("acis/contam") +
                                                    (cfg.detector == MX_DETECTOR_ACIS_I ? "0" : "4") + "/rows")) {
      if (!build_contam(pk, cfg, cfg.detector == MX_DETECTOR_ACIS_I ? 0 : 4, cfg.detector == MX_DETECTOR_ACIS_I ? 3 : 9,
                        M, err))
        return false;
      T.acis_qe = 1;
    }
    if (M.contam.empty()) { MxContamDev z; memset(&z, 0, sizeof(z)); M.contam.assign(10, z); }
    if (M.fef_map.empty()) M.fef_map.push_back(-1);
    if (M.fef.empty()) { MxFefDev z; memset(&z, 0, sizeof(z)); M.fef.push_back(z); }
    if (M.fef_f.empty()) M.fef_f.push_back(0.f);
    if (M.fef_slope.empty()) M.fef_slope.push_back(0.0);
    T.det_extend = cfg.det_extend != 0;
    for (int k = 0; k < 3; k++) T.det_offset[k] = cfg.det_offset[k];
    T.frame_transfer = cfg.acis_frame_transfer_time < 0.0 ? 0.0 : cfg.acis_frame_transfer_time;
    T.exposure = cfg.acis_exposure_time;
    T.frame_time = T.frame_transfer + T.exposure;
    T.inv_frame_time = 1.0 / T.frame_time;
    T.focal_length = cfg.focal_length;
  }

  // ---- dither
  if (cfg.dither < MX_DITHER_NONE || cfg.dither > MX_DITHER_FILE) { err = "unknown dither model"; return false; }
  T.dither = cfg.dither != MX_DITHER_NONE;
  T.dither_file = cfg.dither == MX_DITHER_FILE;
  T.aspect_blur = cfg.aspect_blur * (PI_ / (180.0 * 3600.0));
  if (T.aspect_blur < 0) T.aspect_blur = 0.0;
  for (int k = 0; k < 3; k++) {
    T.dith_amp[k] = cfg.dither_amp[k] * (PI_ / (180.0 * 3600));
    T.dith_period[k] = cfg.dither_period[k];
    T.dith_phase[k] = cfg.dither_phase[k];
    if (cfg.dither == MX_DITHER_INTERNAL && !(cfg.dither_period[k] > 0)) { err = "dither periods must be > 0"; return false; }
    T.dith_inv_period[k] = cfg.dither_period[k] > 0 ? 1.0 / cfg.dither_period[k] : 0.0;
    int e = 0;
    frexp(T.dith_amp[k], &e);   // |amp| = m 2^e, 1/2 <= m < 1
    T.dith_amp_exp[k] = e;
  }
  double roll = cfg.roll_nom * (PI_ / 180.0);
  double xr = fmod(roll, 2 * PI_);
  if (xr >= PI_) xr -= (2 * PI_);
  if (xr < -PI_) xr += (2 * PI_);
  T.nominal_roll = xr;
  T.roll_f = (float) (T.nominal_roll + 0.0);
  // With no roll amplitude every photon is rolled by the same float angle
  // (get_internal_dither, dither.c:175): its sine and cosine are taken once
  // here as the per-photon code would take them (series below 1e-3 rad).
  T.roll_fixed = !T.dither_file && T.dith_amp[2] == 0.0;
  {
    double a = -(double) (float) (T.nominal_roll + 0.0);
    T.roll_zero = T.roll_fixed && a == 0.0;
    if (fabs(a) < 1e-3) {
      double a2 = a * a;
      T.roll_sin = a + a * a2 * (-1.0 / 6.0 + a2 * (1.0 / 120.0 + a2 * (-1.0 / 5040.0)));
      T.roll_cos = 1.0 + a2 * (-0.5 + a2 * (1.0 / 24.0 + a2 * (-1.0 / 720.0)));
    } else {
      T.roll_sin = sin(a); T.roll_cos = cos(a);
    }
  }
  T.start_time = cfg.start_time;
  return true;
}

}  // namespace mx
