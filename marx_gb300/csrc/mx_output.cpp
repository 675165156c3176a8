// MARX's photon output: one binary column file per attribute in an output
// directory (marx_write_photons, marx/libsrc/marxio.c:395-478; file format
// marx_create_write_dump_file and marx_close_write_dump_file,
// marxio.c:70-165).  Host code: the photon list is in host memory.
//
// A column file is a 32-byte header -- the four magic bytes 83 13 89 8D,
// the column type ('E' float32, 'J' int32, 'I' int16, 'A' int8), the column
// name NUL padded from byte 5, the row count (big-endian int32) at byte 20
// and the column count (0) at byte 24 -- followed by one big-endian value
// per written photon.  Only photons without a MX_BAD_PHOTON_MASK bit are
// written.  Appending adds rows to existing files and rewrites the count.
#include <algorithm>
#include <cerrno>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/marx_gb300.h"

namespace {

struct Column {
  uint32_t mask;
  const char *file, *name;
  char type;
};

// The reference's Outfile_Info_Table (marxio.c:288-322), in its order.
const Column kColumns[] = {
    {MX_OUT_PI, "b_energy.dat", "B_ENERGY", 'E'},
    {MX_OUT_ENERGY, "energy.dat", "ENERGY", 'E'},
    {MX_OUT_TIME, "time.dat", "TIME", 'E'},
    {MX_OUT_TAG, "tag.dat", "TAG", 'J'},
    {MX_OUT_X, "xpos.dat", "XPOS", 'E'},
    {MX_OUT_X, "ypos.dat", "YPOS", 'E'},
    {MX_OUT_X, "zpos.dat", "ZPOS", 'E'},
    {MX_OUT_P, "xcos.dat", "COSX", 'E'},
    {MX_OUT_P, "ycos.dat", "COSY", 'E'},
    {MX_OUT_P, "zcos.dat", "COSZ", 'E'},
    {MX_OUT_PHA, "pha.dat", "PHA", 'I'},
    {MX_OUT_DET_NUM, "detector.dat", "CCDID", 'A'},
    {MX_OUT_DET_PIXEL, "xpixel.dat", "CHIPX", 'E'},
    {MX_OUT_DET_PIXEL, "ypixel.dat", "CHIPY", 'E'},
    {MX_OUT_DET_UV, "hrc_u.dat", "U", 'E'},
    {MX_OUT_DET_UV, "hrc_v.dat", "V", 'E'},
    {MX_OUT_SHELL, "mirror.dat", "MIRROR", 'I'},
    {MX_OUT_DET_REGION, "hrcregion.dat", "HRCREGION", 'A'},
    {MX_OUT_ORDER, "order.dat", "ORDER", 'A'},
    {MX_OUT_ORDER1, "ofine.dat", "FINE", 'A'},
    {MX_OUT_ORDER2, "ocoarse1.dat", "COARSE1", 'A'},
    {MX_OUT_ORDER3, "ocoarse2.dat", "COARSE2", 'A'},
    {MX_OUT_ORDER4, "ocoarse3.dat", "COARSE3", 'A'},
    {MX_OUT_SKY_DITHER, "sky_ra.dat", "RA", 'E'},
    {MX_OUT_SKY_DITHER, "sky_dec.dat", "DEC", 'E'},
    {MX_OUT_SKY_DITHER, "sky_roll.dat", "ROLL", 'E'},
    {MX_OUT_DET_DITHER, "det_dy.dat", "DET_DY", 'E'},
    {MX_OUT_DET_DITHER, "det_dz.dat", "DET_DZ", 'E'},
    {MX_OUT_DET_DITHER, "det_theta.dat", "DET_THETA", 'E'},
};
const int kNumColumns = sizeof(kColumns) / sizeof(kColumns[0]);

thread_local std::string g_err;

void put_be(std::vector<unsigned char> &b, uint32_t v, int bytes) {
  for (int k = bytes - 1; k >= 0; k--) b.push_back((unsigned char) (v >> (8 * k)));
}
uint32_t f2bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

// The value of column c for photon i, appended big-endian to b.
void put_value(std::vector<unsigned char> &b, int c, const mx_photons *h, size_t i, double total_time) {
  const size_t s = h->stride ? h->stride : h->n;
  auto f32 = [&](double v) { put_be(b, f2bits((float) v), 4); };
  auto col3 = [&](const double *a, int k) { return a ? a[k * s + i] : 0.0; };
  switch (c) {
    case 0: f32(h->pi ? (double) h->pi[i] : 0.0); break;             // PI (keV) from the ACIS FEF
    case 1: f32(h->energy ? h->energy[i] : 0.0); break;
    case 2: f32((h->arrival_time ? h->arrival_time[i] : 0.0) + total_time); break;
    case 3: put_be(b, h->tag ? h->tag[i] : 0u, 4); break;
    case 4: case 5: case 6: f32(col3(h->x, c - 4)); break;
    case 7: case 8: case 9: f32(col3(h->p, c - 7)); break;
    case 10: put_be(b, (uint16_t) (h->pulse_height ? h->pulse_height[i] : 0), 2); break;
    case 11: put_be(b, (uint8_t) (h->ccd_num ? h->ccd_num[i] : -1), 1); break;
    case 12: f32(h->y_pixel ? (double) h->y_pixel[i] : 0.0); break;
    case 13: f32(h->z_pixel ? (double) h->z_pixel[i] : 0.0); break;
    case 14: f32(h->u_pixel ? (double) h->u_pixel[i] : 0.0); break;
    case 15: f32(h->v_pixel ? (double) h->v_pixel[i] : 0.0); break;
    case 16: put_be(b, (uint16_t) (int16_t) (h->mirror_shell ? h->mirror_shell[i] : 0), 2); break;
    case 17: put_be(b, h->detector_region ? h->detector_region[i] : 0u, 1); break;
    case 18: put_be(b, (uint8_t) (h->order ? h->order[i] : 0), 1); break;
    case 19: case 20: case 21: case 22:
      put_be(b, (uint8_t) (h->support_orders ? h->support_orders[(c - 19) * s + i] : 0), 1); break;
    case 23: case 24: case 25: f32(h->dither_state ? (double) h->dither_state[(c - 23) * s + i] : 0.0); break;
    case 26: case 27: case 28: f32(h->det_dither ? (double) h->det_dither[(c - 26) * s + i] : 0.0); break;
    default: f32(0.0); break;
  }
}

// Marx_Photon_Attr_Type (marx.h:51-100) as an LP64 compiler lays it out:
// the record of a ray file.
struct RayRecord {
  double energy, x[3], p[3], arrival_time;
  uint32_t flags;
  float y_pixel, z_pixel, u_pixel, v_pixel;
  float dither[6];               // Marx_Dither_Type: ra, dec, roll, dy, dz, dtheta
  float pi;
  int16_t pulse_height;
  uint32_t mirror_shell;
  int8_t ccd_num, detector_region, order, support_orders[4];
  uint32_t tag;
};
static_assert(sizeof(RayRecord) == 136, "ray-file record size");
static_assert(offsetof(RayRecord, flags) == 64 && offsetof(RayRecord, dither) == 84 && offsetof(RayRecord, pi) == 108 &&
                  offsetof(RayRecord, pulse_height) == 112 && offsetof(RayRecord, mirror_shell) == 116 &&
                  offsetof(RayRecord, ccd_num) == 120 && offsetof(RayRecord, tag) == 128,
              "ray-file record layout");
const unsigned long kRayMagic = 0xF8161961UL;   // MARX_RAYFILE_MAGIC (marx.h:479)

}  // namespace

extern "C" {

int mx_write_rayfile(const mx_photons *h, uint64_t history, const char *file, int append, double total_time) {
  if (!h || !file) { g_err = "mx_write_rayfile: null argument"; return MX_EINVAL; }
  if (h->stride && h->stride < h->n) { g_err = "mx_write_rayfile: stride below n"; return MX_EINVAL; }
  FILE *f = fopen(file, append ? "ab" : "wb");
  if (!f) { g_err = std::string("Unable to open ") + file + " for writing"; return MX_EINVAL; }
  bool ok = true;
  if (!append) {
    unsigned long hdr[2] = {kRayMagic, (unsigned long) history};
    ok = fwrite(hdr, sizeof(unsigned long), 2, f) == 2;
  }
  const size_t s = h->stride ? h->stride : h->n;
  std::vector<RayRecord> buf;
  buf.reserve(h->n);
  for (size_t i = 0; i < h->n && ok; i++) {
    if (h->flags && (h->flags[i] & MX_BAD_PHOTON_MASK)) continue;
    RayRecord r;
    memset(&r, 0, sizeof(r));
    r.energy = h->energy ? h->energy[i] : 0.0;
    for (int k = 0; k < 3; k++) {
      r.x[k] = h->x ? h->x[k * s + i] : 0.0;
      r.p[k] = h->p ? h->p[k * s + i] : 0.0;
      r.dither[k] = h->dither_state ? h->dither_state[k * s + i] : 0.0f;
      r.dither[3 + k] = h->det_dither ? h->det_dither[k * s + i] : 0.0f;
    }
    r.arrival_time = (h->arrival_time ? h->arrival_time[i] : 0.0) + total_time;
    r.flags = h->flags ? h->flags[i] : 0u;
    r.y_pixel = h->y_pixel ? h->y_pixel[i] : 0.0f;
    r.z_pixel = h->z_pixel ? h->z_pixel[i] : 0.0f;
    r.u_pixel = h->u_pixel ? h->u_pixel[i] : 0.0f;
    r.v_pixel = h->v_pixel ? h->v_pixel[i] : 0.0f;
    r.pi = h->pi ? h->pi[i] : 0.0f;
    r.pulse_height = h->pulse_height ? h->pulse_height[i] : (int16_t) 0;
    r.mirror_shell = h->mirror_shell ? (uint32_t) (int32_t) h->mirror_shell[i] : 0u;
    r.ccd_num = h->ccd_num ? h->ccd_num[i] : (int8_t) 0;
    r.detector_region = h->detector_region ? (int8_t) h->detector_region[i] : (int8_t) 0;
    r.order = h->order ? h->order[i] : (int8_t) 0;
    for (int k = 0; k < 4; k++) r.support_orders[k] = h->support_orders ? h->support_orders[k * s + i] : (int8_t) 0;
    r.tag = h->tag ? h->tag[i] : 0u;
    buf.push_back(r);
  }
  if (ok && !buf.empty()) ok = fwrite(buf.data(), sizeof(RayRecord), buf.size(), f) == buf.size();
  if (fclose(f) != 0) ok = false;
  if (!ok) { g_err = std::string("write to ") + file + " failed"; return MX_EINVAL; }
  return MX_OK;
}

int mx_read_rayfile(const char *file, mx_photons *h, uint32_t max, uint64_t *offset, double *last_time,
                    uint64_t *history, uint32_t *n_read) {
  if (!file || !h || !offset || !last_time || !n_read) { g_err = "mx_read_rayfile: null argument"; return MX_EINVAL; }
  *n_read = 0;
  FILE *f = fopen(file, "rb");
  if (!f) { g_err = std::string("Unable to open rayfile ") + file; return MX_EINVAL; }
  unsigned long hdr[2];
  if (fread(hdr, sizeof(unsigned long), 2, f) != 2 || hdr[0] != kRayMagic) {
    fclose(f);
    g_err = std::string("Magic number mismatch in rayfile ") + file;
    return MX_EINVAL;
  }
  if (history) *history = hdr[1];
  if (*offset == 0) *offset = sizeof(hdr);
  if (fseek(f, (long) *offset, SEEK_SET) != 0) { fclose(f); g_err = "mx_read_rayfile: bad offset"; return MX_EINVAL; }
  const size_t cap = h->n ? std::min<size_t>(max, h->n) : max;
  std::vector<RayRecord> buf(cap);
  const size_t got = cap ? fread(buf.data(), sizeof(RayRecord), cap, f) : 0;
  fclose(f);
  const size_t s = h->stride ? h->stride : h->n;
  double t = 0.0;
  for (size_t i = 0; i < got; i++) {
    const RayRecord &r = buf[i];
    t = r.arrival_time;
    if (h->energy) h->energy[i] = r.energy;
    for (int k = 0; k < 3; k++) {
      if (h->x) h->x[k * s + i] = r.x[k];
      if (h->p) h->p[k * s + i] = r.p[k];
      if (h->dither_state) h->dither_state[k * s + i] = r.dither[k];
      if (h->det_dither) h->det_dither[k * s + i] = r.dither[3 + k];
    }
    if (h->arrival_time) h->arrival_time[i] = r.arrival_time - *last_time;
    if (h->flags) h->flags[i] = r.flags;
    if (h->tag) h->tag[i] = r.tag;
    if (h->mirror_shell) h->mirror_shell[i] = (int8_t) r.mirror_shell;
    if (h->order) h->order[i] = r.order;
    if (h->ccd_num) h->ccd_num[i] = r.ccd_num;
    if (h->y_pixel) h->y_pixel[i] = r.y_pixel;
    if (h->z_pixel) h->z_pixel[i] = r.z_pixel;
    if (h->u_pixel) h->u_pixel[i] = r.u_pixel;
    if (h->v_pixel) h->v_pixel[i] = r.v_pixel;
    if (h->pi) h->pi[i] = r.pi;
    if (h->pulse_height) h->pulse_height[i] = r.pulse_height;
    if (h->detector_region) h->detector_region[i] = (uint8_t) r.detector_region;
    if (h->support_orders)
      for (int k = 0; k < 4; k++) h->support_orders[k * s + i] = r.support_orders[k];
  }
  if (got) *last_time = t;
  *offset += got * sizeof(RayRecord);
  *n_read = (uint32_t) got;
  return MX_OK;
}

const char *mx_write_error(void) { return g_err.c_str(); }

// The history bits the reference's stages set for cfg: marx_create_photons
// (source.c:338-353), the mirror (hrma.c:1173), diffract (diffract.c:984,
// 1103, 1115) and the detectors (acis-i.c:108, acis-s.c:189, hrc-i.c:128,
// hrc-s.c:245-248).
uint32_t mx_output_history(const mx_config *cfg, uint32_t stages) {
  uint32_t h = MX_OUT_ENERGY | MX_OUT_TIME | MX_OUT_X | MX_OUT_P | MX_OUT_TAG;
  if (!cfg) return h;
  if (stages & MX_STAGE_MIRROR) h |= MX_OUT_SHELL;
  if ((stages & MX_STAGE_GRATING) && cfg->grating != MX_GRATING_NONE) {
    h |= MX_OUT_ORDER;
    if (cfg->grating == MX_GRATING_LETG)
      h |= (cfg->leg_fine_orders ? MX_OUT_ORDER1 : 0u) |
           (cfg->leg_coarse_orders ? (MX_OUT_ORDER2 | MX_OUT_ORDER3 | MX_OUT_ORDER4) : 0u);
  }
  if ((stages & MX_STAGE_DETECT) && cfg->detector != MX_DETECTOR_NONE) {
    h |= MX_OUT_DET_PIXEL | MX_OUT_DET_NUM | MX_OUT_PHA;
    if (cfg->detector == MX_DETECTOR_ACIS_I || cfg->detector == MX_DETECTOR_ACIS_S) h |= MX_OUT_PI;
    else h |= MX_OUT_DET_REGION;
    if (cfg->detector == MX_DETECTOR_HRC_S) h |= MX_OUT_DET_UV;
  }
  return h;
}

int mx_write_photons(const mx_photons *h, uint32_t history, uint32_t write_mask, int dither, const char *dir,
                     int append, double total_time) {
  if (!h || !dir) { g_err = "mx_write_photons: null argument"; return MX_EINVAL; }
  if (h->stride && h->stride < h->n) { g_err = "mx_write_photons: stride below n"; return MX_EINVAL; }
  // marx_write_photons: the columns the stages made valid; the dither state
  // whenever a dither model runs
  write_mask &= dither ? (history | MX_OUT_SKY_DITHER | MX_OUT_DET_DITHER) : history;
  std::vector<size_t> good;
  good.reserve(h->n);
  for (size_t i = 0; i < h->n; i++)
    if (!h->flags || !(h->flags[i] & MX_BAD_PHOTON_MASK)) good.push_back(i);
  for (int c = 0; c < kNumColumns; c++) {
    const Column &col = kColumns[c];
    if (!(col.mask & write_mask)) continue;
    std::string path = std::string(dir) + "/" + col.file;
    FILE *f = nullptr;
    uint32_t rows0 = 0;
    if (append && (f = fopen(path.c_str(), "r+b")) != nullptr) {
      unsigned char hdr[32];
      if (fread(hdr, 1, 32, f) != 32 || hdr[0] != 0x83 || hdr[1] != 0x13 || hdr[2] != 0x89 || hdr[3] != 0x8D) {
        fclose(f);
        g_err = path + ": not a column file";
        return MX_EINVAL;
      }
      rows0 = ((uint32_t) hdr[20] << 24) | ((uint32_t) hdr[21] << 16) | ((uint32_t) hdr[22] << 8) | hdr[23];
      fseek(f, 0, SEEK_END);
    } else {
      if (!(f = fopen(path.c_str(), "w+b"))) { g_err = "Unable to open " + path + " for writing"; return MX_EINVAL; }
      unsigned char hdr[32];
      memset(hdr, 0, sizeof(hdr));
      hdr[0] = 0x83; hdr[1] = 0x13; hdr[2] = 0x89; hdr[3] = 0x8D;
      hdr[4] = (unsigned char) col.type;
      for (int k = 0; col.name[k] && 5 + k < 32; k++) hdr[5 + k] = (unsigned char) col.name[k];
      hdr[20] = hdr[21] = hdr[22] = hdr[23] = 0;   // row and column counts
      hdr[24] = hdr[25] = hdr[26] = hdr[27] = 0;
      if (fwrite(hdr, 1, 32, f) != 32) { fclose(f); g_err = "write to " + path + " failed"; return MX_EINVAL; }
    }
    std::vector<unsigned char> buf;
    buf.reserve(good.size() * 4);
    for (size_t i : good) put_value(buf, c, h, i, total_time);
    bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    uint32_t rows = rows0 + (uint32_t) good.size();
    unsigned char cnt[4] = {(unsigned char) (rows >> 24), (unsigned char) (rows >> 16), (unsigned char) (rows >> 8),
                            (unsigned char) rows};
    ok = ok && fseek(f, 20, SEEK_SET) == 0 && fwrite(cnt, 1, 4, f) == 4;
    if (fclose(f) != 0) ok = false;
    if (!ok) { g_err = "write to " + path + " failed (errno " + std::to_string(errno) + ")"; return MX_EINVAL; }
  }
  return MX_OK;
}

}  // extern "C"
