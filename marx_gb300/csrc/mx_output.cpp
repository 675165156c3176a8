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
#include <cerrno>
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
    default: f32(0.0); break;                                        // detector dither: none with INTERNAL
  }
}

}  // namespace

extern "C" {

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
