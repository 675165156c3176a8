/* A MARX-style driver of the compatibility shim, compiled by
 * tests/test_compat_gpu.py against include/marx_gb300_compat.h and linked
 * with libmarx_gb300_compat.so.  It stands in for marx.c's process_photons
 * (marx/src/marx.c:240-273) and, for the parameters, for the reference's
 * parameter-file library: pf_get_* below read "Name=value" lines.
 *
 *   stage_fixture PARAMS INPUT OUTPUT
 *
 * INPUT:  n (u32), energy[n], p[3][n], arrival_time[n] (f64), tag[n] (u32),
 *         U[36][n], N[24][n] (f64, slot-major pre-drawn variates)
 * OUTPUT: the four *_init return values (i32), history (u64), num_sorted
 *         after the final prune (u32), sorted_index[num_sorted] (u32), 1 if
 *         a second marx_mirror_reflect left the photons as they were (i32),
 *         then the n Marx_Photon_Attr_Type records as they are in memory. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "marx_gb300_compat.h"

struct _Param_File_Type {
  int n;
  char name[512][64];
  char value[512][256];
};

static const char *lookup(Param_File_Type *pf, const char *name) {
  for (int i = pf->n - 1; i >= 0; i--)
    if (!strcmp(pf->name[i], name)) return pf->value[i];
  return NULL;
}

int pf_get_string(Param_File_Type *pf, char *name, char *buf, unsigned int len) {
  const char *v = lookup(pf, name);
  if (!v || !len) return -1;
  strncpy(buf, v, len);
  buf[len - 1] = 0;
  return 0;
}

int pf_get_double(Param_File_Type *pf, char *name, double *d) {
  const char *v = lookup(pf, name);
  char *end;
  if (!v) return -1;
  *d = strtod(v, &end);
  return *end ? -1 : 0;
}

int pf_get_integer(Param_File_Type *pf, char *name, int *i) {
  const char *v = lookup(pf, name);
  char *end;
  if (!v) return -1;
  *i = (int) strtol(v, &end, 10);
  return *end ? -1 : 0;
}

int pf_get_boolean(Param_File_Type *pf, char *name, int *b) {
  const char *v = lookup(pf, name);
  if (!v) return -1;
  if (!strcmp(v, "yes")) *b = 1;
  else if (!strcmp(v, "no")) *b = 0;
  else return -1;
  return 0;
}

static Param_File_Type *read_params(const char *path) {
  FILE *f = fopen(path, "r");
  if (!f) return NULL;
  Param_File_Type *pf = calloc(1, sizeof *pf);
  char line[512];
  while (pf->n < 512 && fgets(line, sizeof line, f)) {
    char *eq = strchr(line, '=');
    if (!eq) continue;
    *eq = 0;
    char *v = eq + 1;
    v[strcspn(v, "\r\n")] = 0;
    snprintf(pf->name[pf->n], 64, "%s", line);
    snprintf(pf->value[pf->n], 256, "%s", v);
    pf->n++;
  }
  fclose(f);
  return pf;
}

static int get(void *dst, size_t sz, size_t count, FILE *f) { return fread(dst, sz, count, f) == count ? 0 : -1; }

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  Param_File_Type *pf = read_params(argv[1]);
  FILE *in = fopen(argv[2], "rb");
  if (!pf || !in) return 3;
  unsigned int n;
  if (get(&n, 4, 1, in)) return 4;
  double *E = malloc(8 * n), *P = malloc(24 * (size_t) n), *T = malloc(8 * n);
  unsigned int *tag = malloc(4 * (size_t) n);
  double *U = malloc(8 * 36 * (size_t) n), *N = malloc(8 * 24 * (size_t) n);
  if (get(E, 8, n, in) || get(P, 8, 3 * (size_t) n, in) || get(T, 8, n, in) || get(tag, 4, n, in) ||
      get(U, 8, 36 * (size_t) n, in) || get(N, 8, 24 * (size_t) n, in))
    return 5;
  fclose(in);

  int rc[4];
  rc[0] = marx_gb300_compat_dither_init(pf);
  rc[1] = marx_mirror_init(pf);
  rc[2] = marx_grating_init(pf);
  rc[3] = marx_detector_init(pf);
  if (marx_gb300_compat_set_variates(U, N, n)) return 6;

  /* a batch as marx_create_photons leaves it (source.c:268-385) */
  Marx_Photon_Type *pt = marx_alloc_photon_type(n);
  if (!pt) return 7;
  for (unsigned int i = 0; i < n; i++) {
    Marx_Photon_Attr_Type *at = pt->attributes + i;
    at->energy = E[i];
    at->p.x = P[i]; at->p.y = P[n + i]; at->p.z = P[2 * (size_t) n + i];
    at->arrival_time = T[i];
    at->tag = tag[i];
    at->ccd_num = -1;
    pt->sorted_index[i] = i;
    pt->sorted_energies[i] = E[i];
  }
  pt->n_photons = pt->num_sorted = n;
  pt->history = MARX_ENERGY_OK | MARX_TIME_OK | MARX_X_VECTOR_OK | MARX_P_VECTOR_OK | MARX_TAG_OK;
  unsigned int nd = 0;
  if (rc[0] >= 0 && marx_gb300_compat_dither_photons(pt, &nd)) return 8;

  /* process_photons */
  if (marx_mirror_reflect(pt, 0) || marx_grating_diffract(pt, 0) || marx_detect(pt, 0)) {
    fprintf(stderr, "stage failed: %s\n", marx_gb300_compat_last_error());
    return 9;
  }
  /* a stage that already ran is skipped (its history bit) */
  Marx_Photon_Attr_Type *copy = malloc(sizeof(Marx_Photon_Attr_Type) * (size_t) n);
  memcpy(copy, pt->attributes, sizeof(Marx_Photon_Attr_Type) * (size_t) n);
  int same = marx_mirror_reflect(pt, 0) == 0 && marx_detect(pt, 0) == 0 &&
             !memcmp(copy, pt->attributes, sizeof(Marx_Photon_Attr_Type) * (size_t) n);
  marx_prune_photons(pt);

  FILE *out = fopen(argv[3], "wb");
  if (!out) return 10;
  unsigned long long hist = pt->history;
  fwrite(rc, 4, 4, out);
  fwrite(&hist, 8, 1, out);
  fwrite(&pt->num_sorted, 4, 1, out);
  fwrite(pt->sorted_index, 4, pt->num_sorted, out);
  fwrite(&same, 4, 1, out);
  fwrite(pt->attributes, sizeof(Marx_Photon_Attr_Type), n, out);
  fclose(out);
  marx_dealloc_photon_type(pt);
  marx_gb300_compat_shutdown();
  return 0;
}
