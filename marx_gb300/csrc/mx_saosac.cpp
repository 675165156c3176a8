// The SAOSAC source (marx/libsrc/s-saosac.c:95-345): rays of an SAO
// raytrace of the mirror, read from the RAYTRACE binary table of a FITS
// file (columns RT_X, RT_Y, RT_Z, RT_COSX, RT_COSY, RT_COSZ, RT_KEV, RT_WGHT and,
// when present, RT_TIME), placed on the plane of the mirror's cap and handed
// to the grating and detector stages (the mirror stage is skipped: its
// history bit is set).  Host code: a file reader, as the reference's.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/marx_gb300.h"
#include "mx_device.cuh"

extern int mx_fail(struct mx_context *c, int code, const std::string &msg);

struct mx_saosac {
  std::vector<unsigned char> file;
  size_t data_off = 0, row_bytes = 0;
  uint64_t nrows = 0, next = 0;
  int col[9];          // byte offset of each column in a row
  char type[9];        // 'D' or 'E'
  bool has_time = false;
  double start_time = 0.0;
  double cap_x = 0.0;
};

namespace {

const char *NAMES[9] = {"RT_X", "RT_Y", "RT_Z", "RT_COSX", "RT_COSY", "RT_COSZ", "RT_KEV", "RT_WGHT", "RT_TIME"};

std::string card_value(const char *c) {
  std::string v(c + 10, 70);
  size_t a = v.find_first_not_of(' ');
  if (a == std::string::npos) return "";
  if (v[a] == '\'') {
    size_t b = v.find('\'', a + 1);
    std::string s = v.substr(a + 1, b == std::string::npos ? std::string::npos : b - a - 1);
    s.erase(s.find_last_not_of(' ') + 1);
    return s;
  }
  size_t b = v.find('/', a);
  std::string s = v.substr(a, b == std::string::npos ? std::string::npos : b - a);
  s.erase(s.find_last_not_of(' ') + 1);
  return s;
}

double be_value(const unsigned char *p, char type) {
  if (type == 'D') {
    uint64_t u = 0;
    for (int k = 0; k < 8; k++) u = (u << 8) | p[k];
    double d;
    memcpy(&d, &u, 8);
    return d;
  }
  uint32_t u = 0;
  for (int k = 0; k < 4; k++) u = (u << 8) | p[k];
  float f;
  memcpy(&f, &u, 4);
  return (double) f;
}

int fail(const std::string &m) { return mx_fail(nullptr, MX_EINVAL, m); }

}  // namespace

extern "C" {

mx_saosac *mx_saosac_open(const char *path, double hrma_cap_x) {
  if (!path) { fail("mx_saosac_open: null file name"); return nullptr; }
  FILE *f = fopen(path, "rb");
  if (!f) { fail(std::string("Unable to open proper SAOSAC rayfile called ") + path); return nullptr; }
  mx_saosac *s = new mx_saosac();
  unsigned char buf[65536];
  size_t k;
  while ((k = fread(buf, 1, sizeof buf, f)) > 0) s->file.insert(s->file.end(), buf, buf + k);
  fclose(f);
  s->cap_x = hrma_cap_x;
  // walk the HDUs to the binary table named RAYTRACE
  size_t off = 0;
  while (off + 2880 <= s->file.size()) {
    std::vector<std::pair<std::string, std::string>> hdr;
    bool end = false;
    while (!end && off + 2880 <= s->file.size()) {
      for (int i = 0; i < 36; i++) {
        const char *c = (const char *) s->file.data() + off + 80 * i;
        std::string key(c, 8);
        key.erase(key.find_last_not_of(' ') + 1);
        if (key == "END") { end = true; break; }
        if (c[8] == '=' && c[9] == ' ') hdr.emplace_back(key, card_value(c));
      }
      off += 2880;
    }
    auto get = [&](const std::string &k) -> std::string {
      for (auto &kv : hdr)
        if (kv.first == k) return kv.second;
      return "";
    };
    auto num = [&](const std::string &k) { return atoll(get(k).c_str()); };
    long long naxis = num("NAXIS"), size = 0;
    if (naxis > 0) {
      size = 1;
      for (long long i = 1; i <= naxis; i++) size *= num("NAXIS" + std::to_string(i));
      size = size * std::llabs(num("BITPIX")) / 8 + num("PCOUNT");
    }
    if (get("XTENSION") == "BINTABLE" && get("EXTNAME") == "RAYTRACE") {
      const int nf = (int) num("TFIELDS");
      int pos = 0, found = 0;
      for (int c = 0; c < 9; c++) s->col[c] = -1;
      for (int i = 1; i <= nf; i++) {
        const std::string name = get("TTYPE" + std::to_string(i)), form = get("TFORM" + std::to_string(i));
        int rep = 1;
        size_t j = 0;
        if (!form.empty() && isdigit((unsigned char) form[0])) { rep = atoi(form.c_str()); while (j < form.size() && isdigit((unsigned char) form[j])) j++; }
        const char t = j < form.size() ? form[j] : '?';
        const int width = t == 'D' || t == 'K' ? 8 : t == 'E' || t == 'J' ? 4 : t == 'I' ? 2 : 1;
        for (int c = 0; c < 9; c++)
          if (name == NAMES[c]) {
            if ((t != 'D' && t != 'E') || rep != 1) {
              fail("SAOSAC column " + name + " is not a scalar E or D column");
              delete s;
              return nullptr;
            }
            s->col[c] = pos; s->type[c] = t; found++;
          }
        pos += rep * width;
      }
      for (int c = 0; c < 8; c++)
        if (s->col[c] < 0) {
          fail(std::string("Unable to open proper SAOSAC rayfile called ") + path + ": no " + NAMES[c]);
          delete s;
          return nullptr;
        }
      s->has_time = s->col[8] >= 0;
      s->row_bytes = (size_t) num("NAXIS1");
      s->nrows = (uint64_t) num("NAXIS2");
      s->data_off = off;
      if ((long long) s->row_bytes < pos || off + s->row_bytes * s->nrows > s->file.size()) {
        fail("SAOSAC table truncated");
        delete s;
        return nullptr;
      }
      return s;
    }
    off += (size_t) ((size + 2879) / 2880 * 2880);
  }
  fail(std::string("Unable to find a RAYTRACE extension in ") + path);
  delete s;
  return nullptr;
}

// saosac_create_photons (s-saosac.c:173-300) for up to max photons.
int mx_saosac_read(mx_saosac *s, const mx_photons *h, uint32_t max, const double *u, uint64_t seed,
                   uint32_t first_tag, uint32_t *n_read) {
  if (!s || !h || !n_read || !h->energy || !h->x || !h->p) return fail("mx_saosac_read: null argument");
  const size_t st = h->stride ? h->stride : h->n;
  if (max > h->n) max = h->n;
  uint32_t n = 0, pending = 0;
  double this_time = 0.0;
  while (n < max && s->next < s->nrows) {
    const uint64_t row = s->next++;
    const unsigned char *r = s->file.data() + s->data_off + row * s->row_bytes;
    double b[9];
    for (int c = 0; c < 9; c++) b[c] = s->col[c] >= 0 ? be_value(r + s->col[c], s->type[c]) : 0.0;
    // the weight as a survival probability: one uniform per row read
    const double w = b[7];
    const double ur = u ? u[row] : mx::source_uniform(seed, (uint32_t) row, 0);
    if (ur >= w) pending |= MX_PHOTON_MIRROR_VBLOCKED;
    // the rays' origin is the fore end of the cap: project them to x = 0
    // and place them on the cap's plane (s-saosac.c:216-231)
    const double px = b[3], py = b[4], pz = b[5];
    const double t = -b[0] / px;
    const double y = b[1] + py * t, z = b[2] + pz * t;
    // shell from the radius at the intersect plane (s-saosac.c:233-259)
    const double rr = z * z + y * y;
    const int shell = rr < 138012.25 ? 3 : rr < 206116.0 ? 2 : rr < 292681.0 ? 1 : 0;
    if (s->has_time) {
      if (s->start_time == 0) s->start_time = b[8];
      this_time = b[8] - s->start_time;
    } else
      this_time += 1.0;
    if (this_time < 0) continue;   // the row is dropped; its flags stay with the next photon
    h->energy[n] = b[6];
    h->x[n] = s->cap_x - 0.016750; h->x[st + n] = y; h->x[2 * st + n] = z;
    h->p[n] = px; h->p[st + n] = py; h->p[2 * st + n] = pz;
    if (h->arrival_time) h->arrival_time[n] = this_time;
    if (h->flags) h->flags[n] = pending;
    if (h->mirror_shell) h->mirror_shell[n] = (int8_t) shell;
    if (h->tag) h->tag[n] = first_tag + n;
    pending = 0;
    n++;
  }
  if (s->has_time) s->start_time += this_time;
  *n_read = n;
  return MX_OK;
}

uint64_t mx_saosac_rows(const mx_saosac *s) { return s ? s->nrows : 0; }
int mx_saosac_has_time(const mx_saosac *s) { return s && s->has_time ? 1 : 0; }

void mx_saosac_close(mx_saosac *s) { delete s; }

}  // extern "C"
