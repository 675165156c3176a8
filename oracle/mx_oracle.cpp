// Model set-up and C entry points of the CPU oracle (test infrastructure).
// Set-up restates the reference's init functions: get_shell_geometry
// (hrma.c:551-602), init_hrma_shells (hrma.c:671-745), init_yaw_pitch
// (hrma.c:842-897), the grating init (diffract.c:1254-1300, 1551-1624,
// 1897-1948), chip geometry (caldb.c:256-491, detector.c:383-402,
// acis_geom.c:54-67) and the dither parameter scaling (dither.c:508-547).
#include "mx_oracle.h"
#include "mx_oracle_core.hpp"

#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <thread>
#include <algorithm>

namespace mxo {
thread_local double Counted::ops = 0;
}
using namespace mxo;

static thread_local std::string g_err;

struct PackSection { int dtype; int ndim; uint64_t dims[4]; std::vector<char> data; };

static bool read_pack(const char *path, std::map<std::string, PackSection> &out) {
  FILE *f = fopen(path, "rb");
  if (!f) { g_err = std::string("cannot open pack ") + path; return false; }
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<char> b(sz);
  if ((long) fread(b.data(), 1, sz, f) != sz) { fclose(f); g_err = "short read"; return false; }
  fclose(f);
  if (sz < 16 || memcmp(b.data(), "MXPACK01", 8) != 0) { g_err = "bad pack magic"; return false; }
  uint32_t n;
  memcpy(&n, b.data() + 8, 4);
  for (uint32_t i = 0; i < n; i++) {
    const char *e = b.data() + 16 + 104 * i;
    char name[49] = {0};
    memcpy(name, e, 48);
    PackSection s;
    uint32_t dt, nd;
    uint64_t off, nb;
    memcpy(&dt, e + 48, 4); memcpy(&nd, e + 52, 4);
    memcpy(s.dims, e + 56, 32); memcpy(&off, e + 88, 8); memcpy(&nb, e + 96, 8);
    if (off + nb > (uint64_t) sz) { g_err = "pack section out of range"; return false; }
    s.dtype = (int) dt; s.ndim = (int) nd;
    s.data.assign(b.data() + off, b.data() + off + nb);
    out[name] = std::move(s);
  }
  return true;
}

struct mxo_model {
  Model M;
  std::map<std::string, PackSection> pack;
};

template <class T> static const T *sec(mxo_model *m, const std::string &name, size_t *count = nullptr) {
  auto it = m->pack.find(name);
  if (it == m->pack.end()) { g_err = "pack lacks " + name; return nullptr; }
  if (count) *count = it->second.data.size() / sizeof(T);
  return reinterpret_cast<const T *>(it->second.data.data());
}

static void rot_z_matrix(M3<double> &m, double theta) {  // rotate.c:60
  double c = cos(theta), s = sin(theta);
  s = -s;
  m.m[0][0] = c; m.m[0][1] = s; m.m[0][2] = 0.0;
  m.m[1][0] = -s; m.m[1][1] = c; m.m[1][2] = 0.0;
  m.m[2][0] = 0.0; m.m[2][1] = 0.0; m.m[2][2] = 1.0;
}
static void rot_matrix(M3<double> &m, V3<double> n, double theta) {  // rotate.c:81
  double c = cos(theta), s = sin(theta), c1 = 1 - c;
  double n0 = n.x, n1 = n.y, n2 = n.z;
  double n01 = n0 * n1 * c1, n02 = n0 * n2 * c1, n12 = n1 * n2 * c1;
  m.m[0][0] = n0 * n0 * c1 + c; m.m[0][1] = n01 - s * n2; m.m[0][2] = n02 + s * n1;
  m.m[1][0] = n01 + s * n2; m.m[1][1] = n1 * n1 * c1 + c; m.m[1][2] = n12 - s * n0;
  m.m[2][0] = n02 - s * n1; m.m[2][1] = n12 + s * n0; m.m[2][2] = n2 * n2 * c1 + c;
}
static void mmul(M3<double> &c, const M3<double> &a, const M3<double> &b) {  // rotate.c:110
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
}

// The shell's MARX -> optic translations (get_shell_geometry) and its
// pitch/yaw rotations (init_yaw_pitch) from its geometry-file rows.
static void shell_frames(Shell &h, double cap_pos) {
  for (int o2 = 0; o2 < 2; o2++) {
    double x0 = h.osac[o2][0], y0 = h.osac[o2][1], z0 = h.osac[o2][2];
    h.to_osac[o2].x = -(-z0); h.to_osac[o2].y = (-x0); h.to_osac[o2].z = -(-y0);
    h.to_osac[o2].x -= cap_pos;
  }
  for (int o2 = 0; o2 < 2; o2++) {
    double el = -h.osac[o2][7] * (PI / 180.0), az = -h.osac[o2][6] * (PI / 180);
    M3<double> rz, ry;
    rot_z_matrix(rz, -az);
    V3<double> ny = mvmul(rz, V3<double>{0, 1, 0});
    rot_matrix(ry, ny, -el);
    mmul(h.fwd[o2], ry, rz);
    rot_matrix(ry, ny, el);
    rot_z_matrix(rz, az);
    mmul(h.bwd[o2], rz, ry);
  }
}

static bool setup(mxo_model *o, const mx_config *cfg) {
  Model &M = o->M;
  if (cfg->grating == MX_GRATING_LETG || cfg->detector == MX_DETECTOR_HRC_I || cfg->detector == MX_DETECTOR_HRC_S) {
    g_err = "the restatement covers the HETG and ACIS; LETG and HRC runs are checked against the reference's outputs";
    return false;
  }
  M.cfg = *cfg;
  M.cap = cfg->hrma_cap_x;
  M.ideal = cfg->hrma_ideal != 0;
  M.use_blur = !M.ideal && cfg->use_blur;
  M.use_wfold = !M.ideal && cfg->use_wfold;
  M.use_struts = cfg->use_struts != 0;
  M.use_scale = cfg->use_scale_factors != 0;
  const double *rdb = sec<double>(o, "hrma/rdb");
  if (!rdb) return false;
  static const int ids[4] = {1, 3, 4, 6};
  double total_area = 0.0;
  for (int i = 0; i < 4; i++) {
    Shell &h = M.sh[i];
    for (int o2 = 0; o2 < 2; o2++)
      for (int k = 0; k < 9; k++) h.osac[o2][k] = rdb[(4 * o2 + i) * 9 + k];
    h.length_p = h.osac[0][8]; h.length_h = h.osac[1][8];
    h.xoffset = cfg->shell_xoffset[i];
    h.p_blur = cfg->blur_p[i]; h.h_blur = cfg->blur_h[i];
    h.p_scat = cfg->scat_p[i]; h.h_scat = cfg->scat_h[i];
    // get_shell_geometry
    double cap_pos = M.cap + h.xoffset;
    for (int o2 = 0; o2 < 2; o2++) {
      double pp = h.osac[o2][3], kk = h.osac[o2][4];
      double r = h.osac[o2][5], len = h.osac[o2][8];
      h.c[o2] = r * r; h.b[o2] = -2.0 * kk; h.a[o2] = 1.0 - pp;
      h.xmin[o2] = -0.5 * len; h.xmax[o2] = 0.5 * len;
    }
    shell_frames(h, cap_pos);
    h.front_position = cap_pos - h.osac[0][2] + h.xmax[0];
    // init_hrma_shells
    auto radius = [](double a, double b, double c, double x) { return sqrt(c + x * (b + x * (a - 1))); };
    h.min_radius = radius(h.a[0], h.b[0], h.c[0], h.xmin[0]);
    h.max_radius = radius(h.a[0], h.b[0], h.c[0], h.xmax[0]);
    h.min_radius -= h.length_p * tan(0.67 * PI / 180);
    h.shutter_bitmap = cfg->shutters[i] & 0xF;
    h.num_open = (unsigned) __builtin_popcount(h.shutter_bitmap);
    if (h.num_open)
      total_area += (h.num_open / 4.0) * (h.max_radius - h.min_radius) * (h.max_radius + h.min_radius);
    h.area_fraction = total_area;
    // correction factors and WFold tables
    size_t cnt = 0;
    const float *corr = sec<float>(o, "hrma/corr" + std::to_string(ids[i]), &cnt);
    if (!corr) return false;
    h.corr_n = (unsigned) (cnt / 2); h.corr_e = corr; h.corr_f = corr + h.corr_n;
    for (int o2 = 0; o2 < 2; o2++) {
      std::string base = std::string("wfold/") + (o2 ? "h" : "p") + std::to_string(ids[i]);
      size_t nh = 0, nt = 0;
      const double *hdr = sec<double>(o, base + "/hdr", &nh);
      const float *th = sec<float>(o, base + "/theta", &nt);
      if (!hdr || !th) return false;
      unsigned narr = (unsigned) (nh / 7), nmax = (unsigned) (nt / narr);
      FoldTable &t = h.fold[o2];
      t.arr.clear(); t.e_alphas.clear();
      for (unsigned a = 0; a < narr; a++) {
        const double *q = hdr + 7 * a;
        t.arr.push_back(FoldArray{q[0], q[1], q[2], q[3], q[4], q[5], (unsigned) q[6], th + (size_t) a * nmax});
        t.e_alphas.push_back(q[0]);
      }
    }
  }
  if (total_area <= 0.0) { g_err = "mirror geometric area is 0"; return false; }
  for (int i = 0; i < 4; i++) M.sh[i].area_fraction = M.sh[i].area_fraction / total_area;
  size_t cnt = 0;
  const float *opt = sec<float>(o, "hrma/optconst", &cnt);
  if (!opt) return false;
  if (M.ideal) M.opt_n = 0;
  else { M.opt_n = (unsigned) (cnt / 3); M.opt_e = opt; M.opt_beta = opt + M.opt_n; M.opt_delta = opt + 2 * M.opt_n; }

  // grating
  if (cfg->grating == MX_GRATING_HETG) {
    for (int i = 0; i < 4; i++) {
      Grating &g = M.gr[i];
      size_t ne = 0, neff = 0;
      const float *e = sec<float>(o, "hetg/geff" + std::to_string(i) + "/energy", &ne);
      const float *eff = sec<float>(o, "hetg/geff" + std::to_string(i) + "/eff", &neff);
      if (!e || !eff) return false;
      g.num_energies = (unsigned) ne;
      g.num_orders = (unsigned) (neff / ne);
      g.energies.assign(e, e + ne);
      int max_order = (int) (g.num_orders / 2);
      g.order_list.resize(g.num_orders);
      for (int k = -max_order; k <= max_order; k++) g.order_list[k + max_order] = k;
      g.cum.assign(eff, eff + neff);
      if (cfg->max_order > 0) {  // optional order cut, renormalised to the full efficiency
        for (unsigned j = 0; j < ne; j++) {
          double tot = 0.0, kept = 0.0;
          for (unsigned k = 0; k < g.num_orders; k++) {
            tot += (double) g.cum[k * ne + j];
            if (abs(g.order_list[k]) <= cfg->max_order) kept += (double) g.cum[k * ne + j];
          }
          for (unsigned k = 0; k < g.num_orders; k++)
            g.cum[k * ne + j] = (abs(g.order_list[k]) <= cfg->max_order && kept > 0.0)
                                    ? (float) ((double) g.cum[k * ne + j] * (tot / kept)) : 0.0f;
        }
      }
      // sum_file_efficiencies, diffract.c:1254-1300 (scale 1)
      for (unsigned j = 0; j < ne; j++) {
        double sum = 0.0;
        for (unsigned k = 0; k < g.num_orders; k++) {
          sum += 1.0 * (double) g.cum[k * ne + j];
          g.cum[k * ne + j] = (float) sum;
        }
        if (sum > 1.0)
          for (unsigned k = 0; k < g.num_orders; k++) g.cum[k * ne + j] = (float) (g.cum[k * ne + j] / sum);
      }
      g.dispersion_angle = (cfg->hetg_theta[i] * (PI / 180.0));
      g.theta_blur = (cfg->hetg_dtheta[i] * (PI / 180.0) / 60.0);
      g.period = cfg->hetg_period[i];
      g.dp_over_p = cfg->hetg_dpp[i];
      g.vig = cfg->hetg_vig[i];
      g.rowland = (i < 2) ? cfg->meg_rowland : cfg->heg_rowland;
      g.have_sectors = cfg->use_sector_files != 0;
      if (g.have_sectors) {
        size_t ns = 0;
        const double *s = sec<double>(o, "hetg/sector" + std::to_string(ids[i]), &ns);
        if (!s) return false;
        ns /= 6;
        g.s_min.resize(ns); g.s_max.resize(ns); g.s_dtheta.resize(ns);
        g.s_dtheta_blur.resize(ns); g.s_dpp.resize(ns); g.s_dpp_blur.resize(ns);
        for (size_t k = 0; k < ns; k++) {
          g.s_min[k] = s[6 * k] * (PI / 180.0);
          g.s_max[k] = s[6 * k + 1] * (PI / 180.0);
          g.s_dtheta[k] = s[6 * k + 2] * (PI / (180.0 * 60.0));
          g.s_dtheta_blur[k] = s[6 * k + 3] * (PI / (180.0 * 60.0));
          g.s_dpp[k] = s[6 * k + 4];
          g.s_dpp_blur[k] = s[6 * k + 5];
        }
      }
    }
  }

  // detector chips
  M.chips.clear();
  if (cfg->detector != MX_DETECTOR_NONE) {
    size_t ng = 0;
    const double *geom = sec<double>(o, "acis/geom", &ng);
    const double *orig = sec<double>(o, "acis/origin");
    const double *aim = sec<double>(o, cfg->detector == MX_DETECTOR_ACIS_I ? "acis/aimpt_i" : "acis/aimpt_s");
    if (!geom || !orig || !aim) return false;
    ng /= 13;
    int lo = cfg->detector == MX_DETECTOR_ACIS_I ? 0 : 4, hi = cfg->detector == MX_DETECTOR_ACIS_I ? 3 : 9;
    V3<double> stf{aim[0], aim[1], aim[2]}, stt{orig[0], orig[1], orig[2]};
    V3<double> ofs = vsum(stf, stt);
    for (int id = lo; id <= hi; id++) {
      Chip c{};
      c.id = id;
      for (size_t r = 0; r < ng; r++)
        if ((int) geom[13 * r] == id) {
          const double *q = geom + 13 * r;
          c.x_ll = {q[1], q[2], q[3]}; c.x_lr = {q[4], q[5], q[6]};
          c.x_ul = {q[7], q[8], q[9]}; c.x_ur = {q[10], q[11], q[12]};
        }
      c.x_lr = vsum(c.x_lr, ofs); c.x_ll = vsum(c.x_ll, ofs);
      c.x_ur = vsum(c.x_ur, ofs); c.x_ul = vsum(c.x_ul, ofs);
      c.xhat = vdiff(c.x_lr, c.x_ll); c.yhat = vdiff(c.x_ul, c.x_ll);
      c.xlen = v_length(c.xhat); c.ylen = v_length(c.yhat);
      normalize(c.xhat); normalize(c.yhat);
      c.normal = cross(c.xhat, c.yhat);
      c.xpix = c.xlen / 1024.0; c.ypix = c.ylen / 1024.0;
      c.xoff = 0; c.yoff = 0;
      M.chips.push_back(c);
    }
    if (cfg->acis_exposure_time <= 0) { g_err = "ACIS_Exposure_Time must be greater than 0"; return false; }
    double ftt = cfg->acis_frame_transfer_time < 0.0 ? 0.0 : cfg->acis_frame_transfer_time;
    M.cfg.acis_frame_transfer_time = ftt;
    M.frame_time = ftt + cfg->acis_exposure_time;
  }

  // dither (dither.c:508-547, 170-182)
  M.aspect_blur = cfg->aspect_blur * (PI / (180.0 * 3600.0));
  if (M.aspect_blur < 0) M.aspect_blur = 0.0;
  M.ra_amp = cfg->dither_amp[0] * (PI / (180.0 * 3600));
  M.dec_amp = cfg->dither_amp[1] * (PI / (180.0 * 3600));
  M.roll_amp = cfg->dither_amp[2] * (PI / (180.0 * 3600));
  double roll = cfg->roll_nom * (PI / 180.0);
  double xr = fmod(roll, 2 * PI);
  if (xr >= PI) xr -= (2 * PI);
  if (xr < -PI) xr += (2 * PI);
  M.nominal_roll = xr;
  return true;
}

extern "C" {

mxo_model *mxo_create(const char *pack_path, const mx_config *cfg) {
  auto *o = new mxo_model();
  if (!read_pack(pack_path, o->pack) || !setup(o, cfg)) { delete o; return nullptr; }
  return o;
}
void mxo_destroy(mxo_model *m) { delete m; }
const char *mxo_last_error(void) { return g_err.c_str(); }

static void load_photon(const mx_photons *ph, uint32_t i, Photon &q) {
  uint32_t n = ph->stride ? ph->stride : ph->n;
  q.energy = ph->energy[i];
  q.t = ph->arrival_time ? ph->arrival_time[i] : 0.0;
  q.x = ph->x ? V3<double>{ph->x[i], ph->x[n + i], ph->x[2 * n + i]} : V3<double>{0, 0, 0};
  q.p = {ph->p[i], ph->p[n + i], ph->p[2 * n + i]};
  q.flags = ph->flags ? ph->flags[i] : 0;
  q.shell = ph->mirror_shell ? ph->mirror_shell[i] : 0;
  q.order = ph->order ? ph->order[i] : 0;
  q.ccd = ph->ccd_num ? ph->ccd_num[i] : -1;
  q.ypix = ph->y_pixel ? ph->y_pixel[i] : 0.f;
  q.zpix = ph->z_pixel ? ph->z_pixel[i] : 0.f;
  for (int k = 0; k < 3; k++) q.dith[k] = ph->dither_state ? ph->dither_state[k * n + i] : 0.f;
}
static void store_photon(const mx_photons *ph, uint32_t i, const Photon &q) {
  uint32_t n = ph->stride ? ph->stride : ph->n;
  if (ph->x) { ph->x[i] = q.x.x; ph->x[n + i] = q.x.y; ph->x[2 * n + i] = q.x.z; }
  ph->p[i] = q.p.x; ph->p[n + i] = q.p.y; ph->p[2 * n + i] = q.p.z;
  if (ph->flags) ph->flags[i] = q.flags;
  if (ph->mirror_shell) ph->mirror_shell[i] = (int8_t) q.shell;
  if (ph->order) ph->order[i] = (int8_t) q.order;
  if (ph->ccd_num) ph->ccd_num[i] = (int8_t) q.ccd;
  if (ph->y_pixel) ph->y_pixel[i] = q.ypix;
  if (ph->z_pixel) ph->z_pixel[i] = q.zpix;
  if (ph->dither_state) for (int k = 0; k < 3; k++) ph->dither_state[k * n + i] = q.dith[k];
}

int mxo_trace(const mxo_model *m, const mx_photons *ph, uint32_t stages, const double *U, const double *N,
              uint64_t seed, int nthreads) {
  if (!m || !ph || !ph->energy || !ph->p) return MX_EINVAL;
  if ((U == nullptr) != (N == nullptr)) return MX_EINVAL;
  unsigned nt = nthreads > 0 ? (unsigned) nthreads : std::max(1u, std::thread::hardware_concurrency());
  uint32_t n = ph->n;
  nt = std::min<unsigned>(nt, std::max<uint32_t>(1, n / 256 + 1));
  std::vector<int> bad(nt, 0);
  auto work = [&](unsigned w) {
    for (uint32_t i = w; i < n; i += nt) {
      Photon q;
      load_photon(ph, i, q);
      Variates v;
      v.U = U; v.N = N; v.n = n; v.i = i; v.seed = seed;
      v.tag = ph->tag ? ph->tag[i] : i;
      if (trace_photon<double>(m->M, q, stages, v)) { q.flags |= MX_PHOTON_VARIATE_OVERRUN; bad[w]++; }
      store_photon(ph, i, q);
    }
  };
  if (nt == 1) work(0);
  else {
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nt; w++) th.emplace_back(work, w);
    for (auto &t : th) t.join();
  }
  int tot = 0;
  for (int b : bad) tot += b;
  return tot;
}

int mxo_count_flops(const mxo_model *m, const mx_photons *ph, uint32_t stages, uint64_t seed, double *counts) {
  if (!m || !ph) return MX_EINVAL;
  Counted::ops = 0;
  for (uint32_t i = 0; i < ph->n; i++) {
    Photon q;
    load_photon(ph, i, q);
    Variates v;
    v.n = ph->n; v.i = i; v.seed = seed; v.tag = ph->tag ? ph->tag[i] : i;
    trace_photon<Counted>(m->M, q, stages, v);
    store_photon(ph, i, q);
  }
  counts[0] = Counted::ops;
  counts[1] = ph->n;
  return 0;
}

int mxo_detector_geometry(const mxo_model *m, double *out, int max_chips) {
  int n = 0;
  for (const Chip &c : m->M.chips) {
    if (n >= max_chips) break;
    double *o = out + 20 * n++;
    o[0] = c.id;
    o[1] = c.x_ll.x; o[2] = c.x_ll.y; o[3] = c.x_ll.z;
    o[4] = c.xhat.x; o[5] = c.xhat.y; o[6] = c.xhat.z;
    o[7] = c.yhat.x; o[8] = c.yhat.y; o[9] = c.yhat.z;
    o[10] = c.normal.x; o[11] = c.normal.y; o[12] = c.normal.z;
    o[13] = c.xlen; o[14] = c.ylen; o[15] = c.xpix; o[16] = c.ypix;
    o[17] = c.xoff; o[18] = c.yoff; o[19] = 0;
  }
  return n;
}

double mxo_philox_uniform(uint64_t seed, uint32_t tag, uint32_t slot) { return philox_uniform(seed, tag, slot); }
double mxo_philox_normal(uint64_t seed, uint32_t tag, uint32_t slot) { return philox_normal(seed, tag, slot); }
double mxo_source_uniform(uint64_t seed, uint32_t tag, uint32_t k) { return source_uniform(seed, tag, k); }

}  // extern "C"

// ------------------------------------------------- weighted rays (oracle) --
// CPU restatement of the differentiable form's forward pass: the mirror
// stage of mirror_photon above on the aperture point of each ray's tag,
// with the shell geometry perturbed as the geometry file would carry it,
// no normal blur or scattering, reflectivity times correction as a weight
// instead of the random absorption test, then the focal plane x = 0 and
// the engine's fixed-point Gaussian splat.

// exp(-x), x >= 0: Cody-Waite reduction and the Taylor series of exp(-r)
// to r^7, each operation rounded to single precision in the engine's order.
static float exp_neg_f(float x) {
  if (!(x < 80.0f)) return 0.0f;
  const int n = (int) (x * 1.44269502f + 0.5f);
  const float fn = (float) n;
  const float r = (x - fn * 0.693145752f) - fn * 1.42860677e-06f;
  const float s = -r;
  float p = 1.0f + s * (1.0f / 7.0f);
  p = 1.0f + (s * (1.0f / 6.0f)) * p;
  p = 1.0f + (s * 0.2f) * p;
  p = 1.0f + (s * 0.25f) * p;
  p = 1.0f + (s * (1.0f / 3.0f)) * p;
  p = 1.0f + (s * 0.5f) * p;
  p = 1.0f + s * p;
  uint32_t b = (uint32_t) (127 - n) << 23;
  float scale;
  memcpy(&scale, &b, 4);
  return p * scale;
}

template <class R>
static bool weighted_ray(const Model &M, uint64_t seed, uint32_t tag, const V3<double> &p0d, double energy,
                         double &y, double &z, double &w) {
  Variates v;
  v.seed = seed; v.tag = tag;
  v.window(MX_U_MIRROR, 12, MX_N_MIRROR, 2);
  R wt = R(1.0);
  if (!M.ideal) { v.uniform(); wt = R(M.cfg.hrma_vig); }
  Photon ph{};
  V3<R> x{R(0.0), R(0.0), R(0.0)}, p{R(p0d.x), R(p0d.y), R(p0d.z)};
  project_photon_to_hrma<R>(M, ph, x, p, v);
  if (v.overrun || (ph.flags & MX_PHOTON_MIRROR_VBLOCKED)) return false;
  const Shell &h = M.sh[ph.shell];
  R beta = R(0.0), delta = R(1.0), corr = R(1.0);
  if (M.opt_n) {
    beta = (double) interpolate_f<R>((float) energy, M.opt_e, M.opt_beta, M.opt_n);
    delta = (double) interpolate_f<R>((float) energy, M.opt_e, M.opt_delta, M.opt_n);
    if (M.use_scale) corr = sqrt(R((double) interpolate_f<R>((float) energy, h.corr_e, h.corr_f, h.corr_n)));
  }
  uint32_t flags = 0;
  for (int o = 0; o < 2; o++) {
    V3<R> to{R(h.to_osac[o].x), R(h.to_osac[o].y), R(h.to_osac[o].z)};
    M3<R> fw, bw;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) { fw.m[i][j] = h.fwd[o].m[i][j]; bw.m[i][j] = h.bwd[o].m[i][j]; }
    x = vsum(x, to);
    x = mvmul(fw, x);
    p = mvmul(fw, p);
    V3<R> n;
    if (-1 == conic_intersection(R(h.a[o]), R(h.b[o]), R(h.c[o]), x, p, n, R(h.xmin[o]), R(h.xmax[o]))) return false;
    R pdn = dot(p, n);
    if (!M.ideal) wt *= reflectivity(fabs(pdn), beta, delta) * corr;
    p = ax1_bx2(R(1.0), p, R(-2.0) * pdn, n);
    p = mvmul(bw, p);
    x = mvmul(bw, x);
    x = vdiff(x, to);
    if (M.use_struts && intersects_struts(M, x, p, flags, o == 0 ? CAP_STRUTS : POST_STRUTS)) return false;
  }
  R t = -x.x / p.x;
  y = dv(x.y + t * p.y);
  z = dv(x.z + t * p.z);
  w = dv(wt);
  return true;
}

extern "C" float mxo_splat_exp(float x) { return exp_neg_f(x); }

// The model with theta added to the geometry-file rows of every shell, as
// the reference would read it from a perturbed HRMA_Geometry_File, and the
// source direction at theta.
static void perturbed(const mxo_model *m, const mx_diff_config *cfg, const double *theta, Model &M, V3<double> &p0) {
  M = m->M;
  for (int s = 0; s < 4; s++) {
    Shell &h = M.sh[s];
    for (int o = 0; o < 2; o++) {
      h.osac[o][0] += theta[4 * s + 2] * 1e-3;
      h.osac[o][1] += theta[4 * s + 3] * 1e-3;
      h.osac[o][6] += theta[4 * s] / 3600.0;
      h.osac[o][7] += theta[4 * s + 1] / 3600.0;
    }
    shell_frames(h, M.cap + h.xoffset);
  }
  const double arcsec = PI / (180.0 * 3600.0);
  p0 = V3<double>{-1.0, -tan((cfg->src_y + theta[16]) * arcsec), -tan((cfg->src_z + theta[17]) * arcsec)};
  normalize(p0);
}

extern "C" int mxo_weighted_flops(const mxo_model *m, const mx_diff_config *cfg, const double *theta, double *counts) {
  if (!m || !cfg || !theta || !counts) return MX_EINVAL;
  Model M;
  V3<double> p0;
  perturbed(m, cfg, theta, M, p0);
  Counted::ops = 0;
  double hits = 0.0;
  for (uint64_t i = 0; i < cfg->n_rays; i++) {
    double y, z, w;
    if (weighted_ray<Counted>(M, cfg->seed, (uint32_t) i, p0, cfg->energy, y, z, w)) hits += 1.0;
  }
  counts[0] = Counted::ops;
  counts[1] = (double) cfg->n_rays;
  counts[2] = hits;
  return 0;
}

// The engine's fixed-point splat of one ray of weight w at (y, z) into the
// 64-bit accumulators A (w 2^31 x K 2^31 x K 2^31 >> shift per tap).
struct SplatGeom {
  int nx, ny, shift;
  float knorm, half_inv_s2;
  double inv_pitch, cxp, czp, cy, cz;
  SplatGeom(const mx_diff_config *cfg, uint64_t n) {
    nx = (int) cfg->nx; ny = (int) cfg->ny;
    knorm = (float) (1.0 / (std::sqrt(2.0 * PI) * cfg->sigma));
    half_inv_s2 = (float) (0.5 / (cfg->sigma * cfg->sigma));
    const double kmax = knorm;
    shift = (int) std::ceil(std::log2((double) n * kmax * kmax / 4.0)) + 1;
    if (shift < 0) shift = 0;
    inv_pitch = 1.0 / cfg->pitch; cxp = 0.5 * nx - 0.5; czp = 0.5 * ny - 0.5;
    cy = cfg->center_y; cz = cfg->center_z;
  }
  void add(std::vector<uint64_t> &A, double y, double z, double w) const {
    const double u = (y - cy) * inv_pitch + cxp, vv = (z - cz) * inv_pitch + czp;
    if (!(u > -6.0 && u < nx + 5.0 && vv > -6.0 && vv < ny + 5.0)) return;
    const double uc = std::floor(u + 0.5), vc = std::floor(vv + 0.5);
    const int ic = (int) uc, jc = (int) vc;
    const float fu = (float) (u - uc), fv = (float) (vv - vc);
    const uint32_t wq = (uint32_t) std::nearbyint(std::fmin(w * 2147483648.0, 4294967295.0));
    uint32_t a[11], b[11];
    for (int k = 0; k < 11; k++) {
      float d = (float) (k - 5) - fu;
      uint32_t gy = (uint32_t) std::nearbyint((double) (knorm * exp_neg_f((d * d) * half_inv_s2) * 2147483648.0f));
      a[k] = (uint32_t) (((uint64_t) wq * gy) >> 32);
      float e = (float) (k - 5) - fv;
      b[k] = (uint32_t) std::nearbyint((double) (knorm * exp_neg_f((e * e) * half_inv_s2) * 2147483648.0f));
    }
    for (int kz = 0; kz < 11; kz++) {
      int row = jc - 5 + kz;
      if (row < 0 || row >= ny) continue;
      for (int ky = 0; ky < 11; ky++) {
        int col = ic - 5 + ky;
        if (col < 0 || col >= nx) continue;
        A[(size_t) row * nx + col] += ((uint64_t) a[ky] * b[kz]) >> shift;
      }
    }
  }
  void finish(const std::vector<std::vector<uint64_t>> &acc, uint64_t n, double *image) const {
    const double scale = std::ldexp(1.0, shift - 61) / (double) n;
    for (size_t k = 0; k < (size_t) nx * ny; k++) {
      uint64_t s = 0;
      for (const auto &A : acc) s += A[k];
      image[k] = (double) s * scale;
    }
  }
};

extern "C" int mxo_weighted(const mxo_model *m, const mx_diff_config *cfg, const double *theta, double *yzw,
                            double *image, int nthreads) {
  if (!m || !cfg || !theta || cfg->n_rays < 1 || cfg->n_rays > 0xffffffffull) return MX_EINVAL;
  Model M;
  V3<double> p0;
  perturbed(m, cfg, theta, M, p0);
  const uint64_t n = cfg->n_rays;
  const SplatGeom g(cfg, n);
  unsigned nt = nthreads > 0 ? (unsigned) nthreads : std::max(1u, std::thread::hardware_concurrency());
  nt = (unsigned) std::min<uint64_t>(nt, n / 1024 + 1);
  std::vector<std::vector<uint64_t>> acc(image ? nt : 0);
  auto work = [&](unsigned wk) {
    std::vector<uint64_t> *A = image ? &acc[wk] : nullptr;
    if (A) A->assign((size_t) g.nx * g.ny, 0);
    for (uint64_t i = wk; i < n; i += nt) {
      double y = 0, z = 0, w = 0;
      bool hit = weighted_ray<double>(M, cfg->seed, (uint32_t) i, p0, cfg->energy, y, z, w);
      if (yzw) {
        yzw[i] = hit ? y : NAN;
        yzw[n + i] = hit ? z : NAN;
        yzw[2 * n + i] = hit ? w : 0.0;
      }
      if (A && hit && w > 0.0) g.add(*A, y, z, w);
    }
  };
  if (nt == 1) work(0);
  else {
    std::vector<std::thread> th;
    for (unsigned w = 0; w < nt; w++) th.emplace_back(work, w);
    for (auto &t : th) t.join();
  }
  if (image) g.finish(acc, n, image);
  return 0;
}

// The image of given rays (yzw: 3 x n, y and z in mm, weight; rays of
// weight 0 or non-finite position are skipped) with the engine's splat, as
// mxo_weighted images its own rays: for rays traced elsewhere (the
// reference's mirror stage).
extern "C" int mxo_splat(const mx_diff_config *cfg, const double *yzw, uint64_t n, double *image) {
  if (!cfg || !yzw || !image || n < 1) return MX_EINVAL;
  const SplatGeom g(cfg, n);
  std::vector<std::vector<uint64_t>> acc(1);
  acc[0].assign((size_t) g.nx * g.ny, 0);
  for (uint64_t i = 0; i < n; i++) {
    const double y = yzw[i], z = yzw[n + i], w = yzw[2 * n + i];
    if (w > 0.0 && std::isfinite(y) && std::isfinite(z)) g.add(acc[0], y, z, w);
  }
  g.finish(acc, n, image);
  return 0;
}

// Pre-drawn slot arrays holding the Philox variates of tags first_tag ..
// first_tag + n - 1 (U: MX_NUM_U x n, N: MX_NUM_N x n, slot-major): the
// draws the engine's Philox mode gives those photons.
extern "C" void mxo_philox_slots(uint64_t seed, uint32_t first_tag, uint64_t n, double *U, double *N) {
  for (uint64_t i = 0; i < n; i++) {
    const uint32_t tag = first_tag + (uint32_t) i;
    if (U)
      for (uint32_t k = 0; k < MX_NUM_U; k++) U[k * n + i] = philox_uniform(seed, tag, k);
    if (N)
      for (uint32_t k = 0; k < MX_NUM_N; k++) N[k * n + i] = philox_normal(seed, tag, k);
  }
}
