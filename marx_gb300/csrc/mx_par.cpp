// The marx.par parameters behind mx_config: one table of (name, parameter
// type, module, field), read either through a caller's reader callback (the
// compatibility shim passes the reference's parameter-file library there) or
// from a .par file with command-line style overrides.
//
// The names, types ('r' real, 'i' integer, 'b' boolean, 's' string) and the
// module that reads each parameter are those of marx/par/marx.par and of the
// parameter tables of hrma.c:244-286, diffract.c:550-614 and :1727-1860,
// detector.c:45-52, acis-i.c:170-176, hrc-i.c, hrc-s.c, drake.c:148-246 and
// dither.c:85-110.
#include <cerrno>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/marx_gb300.h"
#include "mx_host.h"

extern int mx_fail(struct mx_context *c, int code, const std::string &msg);

namespace {

enum Kind { K_DOUBLE, K_INT, K_BOOL, K_SHUTTER, K_GRATING, K_DETECTOR, K_DITHER, K_MIRROR };

struct ParamDef {
  std::string name;
  char type;          // marx.par type letter
  uint32_t group;     // MX_PARAMS_*
  Kind kind;
  size_t offset;      // into mx_config (K_MIRROR: unused)
};

#define OFF(f) offsetof(mx_config, f)

const std::vector<ParamDef> &table() {
  static std::vector<ParamDef> t;
  if (!t.empty()) return t;
  const int shells[4] = {1, 3, 4, 6};
  auto add = [](const std::string &n, char ty, uint32_t g, Kind k, size_t off) { t.push_back({n, ty, g, k, off}); };
  auto real = [&](const std::string &n, uint32_t g, size_t off) { add(n, 'r', g, K_DOUBLE, off); };
  const uint32_t M = MX_PARAMS_MIRROR, G = MX_PARAMS_GRATING, D = MX_PARAMS_DETECTOR, A = MX_PARAMS_DITHER;
  char b[64];
  // HRMA (hrma.c:244-286, mirror.c:48-60)
  add("MirrorType", 's', M, K_MIRROR, 0);
  real("HRMA_Cap_X", M, OFF(hrma_cap_x));
  real("HRMAVig", M, OFF(hrma_vig));
  add("HRMA_Ideal", 'b', M, K_BOOL, OFF(hrma_ideal));
  add("HRMA_Use_Blur", 'b', M, K_BOOL, OFF(use_blur));
  add("HRMA_Use_WFold", 'b', M, K_BOOL, OFF(use_wfold));
  add("HRMA_Use_Struts", 'b', M, K_BOOL, OFF(use_struts));
  add("HRMA_Use_Scale_Factors", 'b', M, K_BOOL, OFF(use_scale_factors));
  for (int i = 0; i < 4; i++) {
    const int s = shells[i];
    snprintf(b, sizeof b, "HRMA_P%dH%d_XOffset", s, s); real(b, M, OFF(shell_xoffset) + 8 * i);
    snprintf(b, sizeof b, "P%dBlur", s); real(b, M, OFF(blur_p) + 8 * i);
    snprintf(b, sizeof b, "H%dBlur", s); real(b, M, OFF(blur_h) + 8 * i);
    snprintf(b, sizeof b, "P%dScatFactor", s); real(b, M, OFF(scat_p) + 8 * i);
    snprintf(b, sizeof b, "H%dScatFactor", s); real(b, M, OFF(scat_h) + 8 * i);
    snprintf(b, sizeof b, "Shutters%d", s); add(b, 's', M, K_SHUTTER, OFF(shutters) + 4 * i);
  }
  // gratings (grating.c:44-60, diffract.c:550-614, :1727-1860)
  add("GratingType", 's', G, K_GRATING, OFF(grating));
  add("Use_HETG_Sector_Files", 'b', G, K_BOOL, OFF(use_sector_files));
  real("MEGRowlandDiameter", G, OFF(meg_rowland));
  real("HEGRowlandDiameter", G, OFF(heg_rowland));
  real("LEGRowlandDiameter", G, OFF(leg_rowland));
  real("LETG_ACIS_dTheta", G, OFF(letg_acis_dtheta));
  const char *gq[5] = {"Theta", "dTheta", "Period", "dPoverP", "Vig"};
  const size_t hoff[5] = {OFF(hetg_theta), OFF(hetg_dtheta), OFF(hetg_period), OFF(hetg_dpp), OFF(hetg_vig)};
  const size_t loff[5] = {OFF(letg_theta), OFF(letg_dtheta), OFF(letg_period), OFF(letg_dpp), OFF(letg_vig)};
  for (int i = 0; i < 4; i++)
    for (int q = 0; q < 5; q++) {
      snprintf(b, sizeof b, "HETG_Shell%d_%s", shells[i], gq[q]); real(b, G, hoff[q] + 8 * i);
      snprintf(b, sizeof b, "LETG_Shell%d_%s", shells[i], gq[q]); real(b, G, loff[q] + 8 * i);
    }
  add("legFineNumOrders", 'i', G, K_INT, OFF(leg_fine_orders));
  add("legCoarseNumOrders", 'i', G, K_INT, OFF(leg_coarse_orders));
  real("legFinePeriod", G, OFF(leg_fine_period));
  real("legFineBarHeight", G, OFF(leg_fine_bar_height));
  real("legFineBarWidth", G, OFF(leg_fine_bar_width));
  real("legCoarsePeriod", G, OFF(leg_coarse_period));
  real("legCoarseBarHeight", G, OFF(leg_coarse_bar_height));
  real("legCoarseBarWidth", G, OFF(leg_coarse_bar_width));
  // detectors (detector.c:45-52, acis-i.c:170-176, hrcblur.c, drake.c:148-246)
  add("DetectorType", 's', D, K_DETECTOR, OFF(detector));
  add("DetIdeal", 'b', D, K_BOOL, OFF(det_ideal));
  add("DetExtendFlag", 'b', D, K_BOOL, OFF(det_extend));
  real("DetOffsetX", D, OFF(det_offset));
  real("DetOffsetY", D, OFF(det_offset) + 8);
  real("DetOffsetZ", D, OFF(det_offset) + 16);
  real("ACIS_Exposure_Time", D, OFF(acis_exposure_time));
  real("ACIS_Frame_Transfer_Time", D, OFF(acis_frame_transfer_time));
  const char *blur[13] = {"G1FWHM", "G1Xctr", "G1Yctr", "G1Amp", "G2FWHM", "G2Xctr", "G2Yctr",
                          "G2Amp",  "L1FWHM", "L1Xctr", "L1Yctr", "L1Amp", "L1Rmax"};
  for (int k = 0; k < 13; k++) {
    snprintf(b, sizeof b, "HRC-I-Blur%s", blur[k]); real(b, D, OFF(hrc_i_blur) + 8 * k);
    snprintf(b, sizeof b, "HRC-S-Blur%s", blur[k]); real(b, D, OFF(hrc_s_blur) + 8 * k);
  }
  add("HRC-HESF", 'b', D, K_BOOL, OFF(hrc_hesf));
  add("HESFN", 'i', D, K_INT, OFF(hesf_n));
  real("HESFOffsetX", D, OFF(hesf_offset_x));
  real("HESFOffsetZ", D, OFF(hesf_offset_z));
  real("HESFGapY1", D, OFF(hesf_gap_y1));
  real("HESFGapY2", D, OFF(hesf_gap_y2));
  real("HESFLength", D, OFF(hesf_length));
  real("HESFCrWidth", D, OFF(hesf_cr_width));
  for (int k = 0; k < 4; k++) {
    snprintf(b, sizeof b, "HESFHeight%d", k + 1); real(b, D, OFF(hesf_height) + 8 * k);
    snprintf(b, sizeof b, "HESFTheta%d", k + 1); real(b, D, OFF(hesf_theta) + 8 * k);
  }
  // aspect dither and pointing (dither.c:85-160)
  add("DitherModel", 's', A, K_DITHER, OFF(dither));
  real("AspectBlur", A, OFF(aspect_blur));
  real("RA_Nom", A, OFF(ra_nom));
  real("Dec_Nom", A, OFF(dec_nom));
  real("Roll_Nom", A, OFF(roll_nom));
  real("PointingOffsetY", A, OFF(pointing_offset));
  real("PointingOffsetZ", A, OFF(pointing_offset) + 8);
  const char *ax[3] = {"RA", "Dec", "Roll"};
  for (int k = 0; k < 3; k++) {
    snprintf(b, sizeof b, "DitherAmp_%s", ax[k]); real(b, A, OFF(dither_amp) + 8 * k);
    snprintf(b, sizeof b, "DitherPeriod_%s", ax[k]); real(b, A, OFF(dither_period) + 8 * k);
    snprintf(b, sizeof b, "DitherPhase_%s", ax[k]); real(b, A, OFF(dither_phase) + 8 * k);
  }
  return t;
}

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n"), z = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, z - a + 1);
}

bool parse_bool(const std::string &v, int &out) {
  std::string l;
  for (char ch : v) l += (char) tolower((unsigned char) ch);
  if (l == "yes" || l == "y" || l == "true" || l == "1") { out = 1; return true; }
  if (l == "no" || l == "n" || l == "false" || l == "0") { out = 0; return true; }
  return false;
}

// One parameter's text into the configuration.
int apply(mx_config *cfg, const ParamDef &d, const std::string &raw) {
  const std::string v = trim(raw);
  char *base = (char *) cfg;
  auto bad = [&](const char *what) {
    return mx_fail(nullptr, MX_EINVAL, "parameter " + d.name + ": " + what + " '" + v + "'");
  };
  switch (d.kind) {
    case K_DOUBLE: {
      char *end = nullptr;
      errno = 0;
      double x = strtod(v.c_str(), &end);
      if (v.empty() || *end || errno) return bad("not a number");
      memcpy(base + d.offset, &x, sizeof x);
      return MX_OK;
    }
    case K_INT: {
      char *end = nullptr;
      errno = 0;
      long x = strtol(v.c_str(), &end, 10);
      if (v.empty() || *end || errno || x < INT32_MIN || x > INT32_MAX) return bad("not an integer");
      int32_t y = (int32_t) x;
      memcpy(base + d.offset, &y, sizeof y);
      return MX_OK;
    }
    case K_BOOL: {
      int x;
      if (!parse_bool(v, x)) return bad("not a boolean");
      int32_t y = x;
      memcpy(base + d.offset, &y, sizeof y);
      return MX_OK;
    }
    case K_SHUTTER: {
      // _marx_parse_shutter_string (mirror.c:112): four characters, '0' an
      // open quadrant, '1' a closed one
      if (v.size() != 4) return bad("not four shutter characters");
      uint32_t m = 0;
      for (int q = 0; q < 4; q++) {
        if (v[q] == '0') m |= 1u << q;
        else if (v[q] != '1') return bad("not a shutter string");
      }
      memcpy(base + d.offset, &m, sizeof m);
      return MX_OK;
    }
    case K_GRATING: {
      int32_t g = v == "NONE" ? MX_GRATING_NONE : v == "HETG" ? MX_GRATING_HETG : v == "LETG" ? MX_GRATING_LETG : -1;
      if (g < 0) return bad("GratingType not supported");
      cfg->grating = g;
      return MX_OK;
    }
    case K_DETECTOR: {
      int32_t k = v == "NONE" ? MX_DETECTOR_NONE : v == "ACIS-I" ? MX_DETECTOR_ACIS_I : v == "ACIS-S" ? MX_DETECTOR_ACIS_S
                : v == "HRC-I" ? MX_DETECTOR_HRC_I : v == "HRC-S" ? MX_DETECTOR_HRC_S : -1;
      if (k < 0) return bad("DetectorType not supported");
      cfg->detector = k;
      return MX_OK;
    }
    case K_DITHER: {
      int32_t k = v == "NONE" ? MX_DITHER_NONE : v == "INTERNAL" ? MX_DITHER_INTERNAL : v == "FILE" ? MX_DITHER_FILE : -1;
      if (k < 0) return bad("DitherModel not supported");
      cfg->dither = k;
      return MX_OK;
    }
    case K_MIRROR:
      if (v != "HRMA") return bad("MirrorType not supported (HRMA only)");
      return MX_OK;
  }
  return bad("unknown parameter kind");
}

// Fields of a parameter-file line, split at commas outside double quotes,
// quotes removed.
std::vector<std::string> csv_fields(const std::string &line) {
  std::vector<std::string> f(1);
  bool q = false;
  for (char ch : line) {
    if (ch == '"') q = !q;
    else if (ch == ',' && !q) f.emplace_back();
    else f.back() += ch;
  }
  return f;
}

}  // namespace

namespace mx {

const std::string *ParSet::find(const std::string &name) const {
  for (size_t k = kv.size(); k-- > 0;)   // a later line or override wins
    if (kv[k].first == name) return &kv[k].second;
  return nullptr;
}

bool load_par(const char *path, const char *const *overrides, int n_overrides, ParSet &out, std::string &err) {
  FILE *f = fopen(path, "r");
  if (!f) { err = std::string("cannot open ") + path; return false; }
  out.kv.clear();
  char line[4096];
  while (fgets(line, sizeof line, f)) {
    std::string s = trim(line);
    if (s.empty() || s[0] == '#') continue;
    std::vector<std::string> fl = csv_fields(s);
    if (fl.size() >= 4) out.kv.emplace_back(trim(fl[0]), trim(fl[3]));
  }
  fclose(f);
  for (int k = 0; k < n_overrides; k++) {
    const char *o = overrides ? overrides[k] : nullptr;
    const char *eq = o ? strchr(o, '=') : nullptr;
    if (!eq) { err = std::string("override without '=': ") + (o ? o : ""); return false; }
    out.kv.emplace_back(trim(std::string(o, eq - o)), trim(std::string(eq + 1)));
  }
  return true;
}

int par_reader(void *user, const char *name, char type, char *value, size_t len) {
  (void) type;
  const std::string *v = ((const ParSet *) user)->find(name);
  if (!v || len == 0) return -1;
  snprintf(value, len, "%s", v->c_str());
  return 0;
}

}  // namespace mx

extern "C" {

int mx_config_read_params(mx_config *cfg, uint32_t groups, mx_param_reader read, void *user, int required) {
  if (!cfg || !read) return mx_fail(nullptr, MX_EINVAL, "mx_config_read_params: null argument");
  char buf[1024];
  for (const ParamDef &d : table()) {
    if (!(d.group & groups)) continue;
    buf[0] = 0;
    if (read(user, d.name.c_str(), d.type, buf, sizeof buf) != 0) {
      if (required) return mx_fail(nullptr, MX_EINVAL, "parameter " + d.name + " is missing");
      continue;
    }
    int r = apply(cfg, d, buf);
    if (r) return r;
  }
  return MX_OK;
}

int mx_param_type(const char *name, char *type, uint32_t *group) {
  if (!name) return MX_EINVAL;
  for (const ParamDef &d : table())
    if (d.name == name) {
      if (type) *type = d.type;
      if (group) *group = d.group;
      return MX_OK;
    }
  return MX_EINVAL;
}

int mx_config_read_par(mx_config *cfg, const char *path, const char *const *overrides, int n_overrides) {
  if (!cfg || !path) return mx_fail(nullptr, MX_EINVAL, "mx_config_read_par: null argument");
  mx::ParSet pf;
  std::string err;
  if (!mx::load_par(path, overrides, n_overrides, pf, err)) return mx_fail(nullptr, MX_EINVAL, "mx_config_read_par: " + err);
  mx_config_default(cfg);
  return mx_config_read_params(cfg, MX_PARAMS_ALL, mx::par_reader, &pf, 0);
}

}  // extern "C"
