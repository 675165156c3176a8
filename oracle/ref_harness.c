/* Test harness around the reference MARX library (compiled in place from the
 * reference's own sources by oracle/Makefile).  Test infrastructure only.
 *
 * It drives the reference's stage functions over a photon list:
 *   _marx_dither_photons  (marx/libsrc/dither.c:630)
 *   marx_mirror_reflect   (marx/libsrc/mirror.c:93)
 *   marx_grating_diffract (marx/libsrc/grating.c:88)
 * and the per-photon body of _marx_acis_i_detect / _marx_acis_s_detect
 * (marx/libsrc/acis-i.c:96-160, acis-s.c:177-248) through the exported
 * pieces that body calls (_marx_transform_ray, _marx_intersect_with_detector,
 * _marx_acis_apply_streak).  For the ACIS marx_detector_init itself cannot
 * run here: it loads the ACIS FEF calibration file unconditionally and that
 * file is not shipped with the reference, so QE and pulse height are not
 * exercised (DetIdeal semantics; pulse height left at 0).  The HRC
 * detectors need no missing file: marx_detector_init and marx_detect
 * (detector.c:298-378) run as they are.
 *
 * Built twice:
 *   MXREF_INTERPOSE=1  the jdmath generator is replaced by per-photon
 *                      pre-drawn variates.  Each stage reads its uniforms
 *                      and normals from fixed slot ranges of the current
 *                      photon (MX_U_* / MX_N_* below), so the same variates
 *                      can be handed to any other implementation.
 *   MXREF_INTERPOSE=0  the reference's own generator (jdmath random.c,
 *                      gaussrnd.c), seeded with mxref_seed(); photons are
 *                      processed as one batch exactly as marx.c does.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>

#include <jdmath.h>
#include <pfile.h>
#include "acis.h"   /* the facets' tdet offsets (MARX_DET_FACET_PRIVATE_DATA) */
#include "marx.h"
#include "_marx.h"

/* Variate slot layout, shared with the engine and the port. */
#define MX_NU 36
#define MX_NN 24
#define MX_U_MIRROR 0
#define MX_U_MIRROR_N 12
#define MX_U_GRATING 12
#define MX_U_GRATING_N 2
#define MX_U_DETECT 14
#define MX_U_DETECT_N 2
#define MX_N_DITHER 0
#define MX_N_DITHER_N 2
#define MX_N_MIRROR 2
#define MX_N_MIRROR_N 2
#define MX_N_GRATING 4
#define MX_N_GRATING_N 2
#define MX_N_DETECT 6
#define MX_N_DETECT_N 2
#define MX_U_LETG 16
#define MX_U_LETG_N 6
#define MX_N_LETG 8
#define MX_N_LETG_N 10
#define MX_U_HRC 22
#define MX_U_HRC_N 6
#define MX_N_HRC 18
#define MX_N_HRC_N 2
#define MX_U_FEF 28
#define MX_U_FEF_N 8
#define MX_N_FEF 20
#define MX_N_FEF_N 4

static char Err[1024];
static void set_err(const char *s) { strncpy(Err, s, sizeof(Err) - 1); }
const char *mxref_last_error(void) { return Err; }

/* ---------------------------------------------------------------- RNG -- */
#if MXREF_INTERPOSE
static const double *Cur_U, *Cur_N;
static int U_pos, U_end, N_pos, N_end;
static int Rng_Overrun, Rng_Unexpected;

static void rng_window(const double *u, int ubase, int ucount,
                       const double *n, int nbase, int ncount)
{
   Cur_U = u; U_pos = ubase; U_end = ubase + ucount;
   Cur_N = n; N_pos = nbase; N_end = nbase + ncount;
}

double JDMrandom(void)
{
   if (Cur_U == NULL || U_pos >= U_end) { Rng_Overrun++; return 0.5; }
   return Cur_U[U_pos++];
}
double JDMgaussian_random(void)
{
   if (Cur_N == NULL || N_pos >= N_end) { Rng_Overrun++; return 0.0; }
   return Cur_N[N_pos++];
}
double JDMexpn_random(void) { Rng_Unexpected++; return 1.0; }
int JDMsrandom(unsigned long s) { (void) s; return 0; }
uint32 JDMuint32_random(void) { Rng_Unexpected++; return 0; }
int JDMseed_random(JDMRandom_Type *rt, unsigned long s) { (void) rt; (void) s; Rng_Unexpected++; return 0; }
uint32 JDMgenerate_uint32_random(JDMRandom_Type *rt) { (void) rt; Rng_Unexpected++; return 0; }
double JDMgenerate_random(JDMRandom_Type *rt) { (void) rt; Rng_Unexpected++; return 0.5; }
JDMRandom_Type *JDMcreate_random(void) { Rng_Unexpected++; return NULL; }
void JDMfree_random(JDMRandom_Type *rt) { (void) rt; }
void JDMseed_fast_random(unsigned long s) { (void) s; }
uint32 JDMfast_uint32_random(void) { Rng_Unexpected++; return 0; }
double JDMfast_random(void) { Rng_Unexpected++; return 0.5; }
#endif

/* The FEF pulse-height draws (marx_apply_acis_rmf, acis_fef.c:967-1079)
 * come from a window of their own: the library is linked with
 * --wrap=_marx_apply_acis_rmf, so the ACIS detector's call lands here. */
int __real__marx_apply_acis_rmf(_Marx_Acis_Chip_Type *c, float x, float y, double energy, float *pip,
                                short *phap);
int __wrap__marx_apply_acis_rmf(_Marx_Acis_Chip_Type *c, float x, float y, double energy, float *pip,
                                short *phap)
{
#if MXREF_INTERPOSE
   const double *su = Cur_U, *sn = Cur_N;
   int up = U_pos, ue = U_end, np = N_pos, ne = N_end, r;
   rng_window(su, MX_U_FEF, MX_U_FEF_N, sn, MX_N_FEF, MX_N_FEF_N);
   r = __real__marx_apply_acis_rmf(c, x, y, energy, pip, phap);
   Cur_U = su; Cur_N = sn; U_pos = up; U_end = ue; N_pos = np; N_end = ne;
   return r;
#else
   return __real__marx_apply_acis_rmf(c, x, y, energy, pip, phap);
#endif
}

/* ------------------------------------------------------------- set-up -- */
static Param_File_Type *Pf;
static int Have_Dither, Have_Grating, Det_Kind;   /* 0 none, 1 ACIS-I, 2 ACIS-S */
static int Acis_Fef;      /* an ACIS FEF file is present: the reference's own ACIS detector runs */
static int Grating_Is_LETG;
static Marx_Detector_Type *Det;

int mxref_setup(const char *parfile, const char *datadir, int nover,
                const char **names, const char **values)
{
   char buf[PF_MAX_LINE_LEN];
   double yoff, zoff;
   int i;

   Err[0] = 0;
   if (Pf != NULL) { pf_close_parameter_file(Pf); Pf = NULL; }
   if (NULL == (Pf = pf_open_parameter_file((char *) parfile, "rQ")))
     { set_err("cannot open parameter file"); return -1; }
   for (i = 0; i < nover; i++)
     if (-1 == pf_set_value(Pf, (char *) names[i], (char *) values[i]))
       { snprintf(Err, sizeof(Err), "cannot set %s=%s", names[i], values[i]); return -1; }

   if (-1 == marx_set_data_directory((char *) datadir))
     { set_err("bad data directory"); return -1; }

   if (-1 == _marx_init_dither(Pf, 0, &yoff, &zoff))
     { set_err("dither init failed"); return -1; }
   if (-1 == pf_get_string(Pf, "DitherModel", buf, sizeof(buf)))
     return -1;
   Have_Dither = (0 == strcmp(buf, "INTERNAL")) || (0 == strcmp(buf, "FILE"));

   if (-1 == marx_mirror_init(Pf)) { set_err("mirror init failed"); return -1; }
   if (-1 == marx_grating_init(Pf)) { set_err("grating init failed"); return -1; }
   if (-1 == pf_get_string(Pf, "GratingType", buf, sizeof(buf))) return -1;
   Have_Grating = (0 != strcmp(buf, "NONE"));
   Grating_Is_LETG = (0 == strcmp(buf, "LETG"));

   /* Detector: the part of marx_detector_init (detector.c:298-357) that does
    * not depend on the missing FEF file. */
   if (-1 == pf_get_string(Pf, "DetectorType", buf, sizeof(buf))) return -1;
   Det_Kind = 0; Det = NULL;
   if (0 == strcmp(buf, "ACIS-I")) Det_Kind = 1;
   else if (0 == strcmp(buf, "ACIS-S")) Det_Kind = 2;
   else if (0 == strcmp(buf, "HRC-I")) Det_Kind = 3;
   else if (0 == strcmp(buf, "HRC-S")) Det_Kind = 4;
   else if (0 != strcmp(buf, "NONE")) { set_err("unsupported DetectorType"); return -1; }
   if (Det_Kind >= 3)
     {
        /* The HRC needs no file that is missing here: the reference's own
         * marx_detector_init runs as it is. */
        if (-1 == marx_detector_init(Pf)) { set_err("detector init failed"); return -1; }
        if (NULL == (Det = marx_get_detector_info(buf, 0))) { set_err("detector geometry"); return -1; }
        return 0;
     }
   Acis_Fef = 0;
   if (Det_Kind)
     {
        char *fef = _marx_caldb_get_file("ACISFEF");
        if ((fef != NULL) && (1 == marx_file_exists(fef)))
          {
             /* With an FEF (DetIdeal = yes reads nothing else) marx_detector_init
              * runs as it is, and marx_detect applies the FEF pulse heights. */
             marx_free(fef);
             if (-1 == marx_detector_init(Pf)) { set_err("detector init failed"); return -1; }
             if (NULL == (Det = marx_get_detector_info(Det_Kind == 1 ? "ACIS-I" : "ACIS-S", 0)))
               { set_err("detector geometry"); return -1; }
             Acis_Fef = 1;
             return 0;
          }
        if (fef != NULL) marx_free(fef);
     }
   if (Det_Kind)
     {
        double *m = _Marx_Det_XForm_Matrix.matrix;
        m[0] = 1; m[1] = 0; m[2] = 0; m[3] = 0; m[4] = 1; m[5] = 0; m[6] = 0; m[7] = 0; m[8] = 1;
        if ((-1 == pf_get_double(Pf, "DetOffsetX", &_Marx_Det_XForm_Matrix.dx))
            || (-1 == pf_get_double(Pf, "DetOffsetY", &_Marx_Det_XForm_Matrix.dy))
            || (-1 == pf_get_double(Pf, "DetOffsetZ", &_Marx_Det_XForm_Matrix.dz))
            || (-1 == pf_get_boolean(Pf, "DetExtendFlag", &_Marx_Det_Extend_Flag)))
          { set_err("detector parameters"); return -1; }
        _Marx_Det_Ideal_Flag = 1;
        if (-1 == _marx_acis_get_generic_parms(Pf)) { set_err("ACIS parameters"); return -1; }
        if (NULL == (Det = marx_get_detector_info(Det_Kind == 1 ? "ACIS-I" : "ACIS-S", 0)))
          { set_err("detector geometry"); return -1; }
     }
   return 0;
}

/* Chip facets after the reference's CALDB patching: per chip
 * id, x_ll[3], xhat[3], yhat[3], normal[3], xlen, ylen, xpix, ypix,
 * xpixel_offset, ypixel_offset  (20 doubles). */
int mxref_detector_geometry(double *out, int max_chips)
{
   Marx_Detector_Geometry_Type *g;
   int n = 0;
   if (Det == NULL) return 0;
   for (g = Det->facet_list; g != NULL && n < max_chips; g = g->next, n++)
     {
        double *o = out + 20 * n;
        o[0] = g->id;
        o[1] = g->x_ll.x; o[2] = g->x_ll.y; o[3] = g->x_ll.z;
        o[4] = g->xhat.x; o[5] = g->xhat.y; o[6] = g->xhat.z;
        o[7] = g->yhat.x; o[8] = g->yhat.y; o[9] = g->yhat.z;
        o[10] = g->normal.x; o[11] = g->normal.y; o[12] = g->normal.z;
        o[13] = g->xlen; o[14] = g->ylen;
        o[15] = g->x_pixel_size; o[16] = g->y_pixel_size;
        o[17] = g->xpixel_offset; o[18] = g->ypixel_offset;
        o[19] = 0;
     }
   return n;
}

double mxref_focal_length(void) { return Marx_Focal_Length; }

/* The tiled-detector offsets of each facet (tdet_xoff, tdet_yoff), as
 * marx2fits's compute_tdetxy reads them. */
int mxref_facet_tdet(double *out, int max_chips)
{
   Marx_Detector_Geometry_Type *g;
   int n = 0;
   if (Det == NULL) return 0;
   for (g = Det->facet_list; g != NULL && n < max_chips; g = g->next, n++)
     {
        out[2 * n] = g->tdet_xoff;
        out[2 * n + 1] = g->tdet_yoff;
     }
   return n;
}

/* The detector's focal-plane system: fp_delta_s0 (radians), fp_x0, fp_y0
 * (detpix.c:42-63). */
int mxref_fp_system(double *out)
{
   if (Det == NULL || Det->fp_coord_info == NULL) return -1;
   out[0] = Det->fp_coord_info->fp_delta_s0;
   out[1] = Det->fp_coord_info->fp_x0;
   out[2] = Det->fp_coord_info->fp_y0;
   return 0;
}

/* ---------------------------------------------------------- detection -- */
/* Per-photon body of _marx_acis_i_detect (acis-i.c:124-157); the acis-s
 * body is the same with chip ids 4..9.  QE is skipped (DetIdeal) and the
 * pulse-height function is not available, so the streak follows every hit. */
static void detect_photons(Marx_Photon_Type *pt)
{
   unsigned int i;
   marx_prune_photons(pt);
   for (i = 0; i < pt->num_sorted; i++)
     {
        Marx_Photon_Attr_Type *at = pt->attributes + pt->sorted_index[i];
        Marx_Detector_Geometry_Type *d;
        double dx, dy;

        _marx_dither_detector(&at->dither_state);
        _marx_transform_ray(&at->x, &at->p, &_Marx_Det_XForm_Matrix);
        d = _marx_intersect_with_detector(at->x, at->p, Det->facet_list,
                                          &at->x, &dx, &dy, _Marx_Det_Extend_Flag);
        if (d == NULL)
          {
             at->flags |= PHOTON_MISSED_DETECTOR;
             at->ccd_num = -1;
          }
        else
          {
             at->ccd_num = d->id;
             at->y_pixel = dx / d->x_pixel_size;
             at->z_pixel = dy / d->y_pixel_size;
             _marx_acis_apply_streak(pt->start_time, at, d);
          }
        _marx_transform_ray_reverse(&at->x, &at->p, &_Marx_Det_XForm_Matrix);
        _marx_undither_detector(&at->dither_state);
     }
}

/* --------------------------------------------------------------- trace -- */
typedef struct
{
   double *x, *p;           /* n*3 */
   unsigned int *flags;
   int *shell, *order, *ccd;
   float *ypix, *zpix;
   float *dither;           /* n*3: ra, dec, roll */
} Out_Type;

static void fill_attr(Marx_Photon_Attr_Type *at, double e, const double *p, double t,
                      unsigned int tag)
{
   memset(at, 0, sizeof(*at));
   at->energy = e;
   at->p.x = p[0]; at->p.y = p[1]; at->p.z = p[2];
   at->arrival_time = t;
   at->tag = tag;
   at->ccd_num = -1;
}

/* Outputs beyond the core columns, NULL when not wanted: LETG support
 * orders (4 per photon), HRC pulse height, u/v pixel and detector region. */
static signed char *X_Sup;
static short *X_Pha;
static float *X_U, *X_V;
static unsigned char *X_Region;
static float *X_Pi;
/* ACIS PI (at->pi) output column, or NULL. */
void mxref_set_pi_output(float *pi) { X_Pi = pi; }
/* The detector dither (dy, dz, dtheta of at->dither_state, 3 per photon), or NULL. */
static float *X_Det;
void mxref_set_det_dither_output(float *d) { X_Det = d; }

void mxref_set_extra_outputs(signed char *sup, short *pha, float *u, float *v, unsigned char *region)
{
   X_Sup = sup; X_Pha = pha; X_U = u; X_V = v; X_Region = region;
}

static void store_attr(const Marx_Photon_Attr_Type *at, int i, double *x, double *p,
                       unsigned int *flags, int *shell, int *order, int *ccd,
                       float *ypix, float *zpix, float *dith)
{
   x[3*i] = at->x.x; x[3*i+1] = at->x.y; x[3*i+2] = at->x.z;
   p[3*i] = at->p.x; p[3*i+1] = at->p.y; p[3*i+2] = at->p.z;
   flags[i] = at->flags;
   shell[i] = (int) at->mirror_shell;
   order[i] = at->order;
   ccd[i] = at->ccd_num;
   ypix[i] = at->y_pixel; zpix[i] = at->z_pixel;
   dith[3*i] = at->dither_state.ra; dith[3*i+1] = at->dither_state.dec;
   dith[3*i+2] = at->dither_state.roll;
   if (X_Sup != NULL)
     {
        int k;
        for (k = 0; k < 4; k++) X_Sup[4*i+k] = at->support_orders[k];
     }
   if (X_Pha != NULL) X_Pha[i] = at->pulse_height;
   if (X_U != NULL) X_U[i] = at->u_pixel;
   if (X_V != NULL) X_V[i] = at->v_pixel;
   if (X_Region != NULL) X_Region[i] = at->detector_region;
   if (X_Pi != NULL) X_Pi[i] = at->pi;
   if (X_Det != NULL)
     {
        X_Det[3*i] = at->dither_state.dy; X_Det[3*i+1] = at->dither_state.dz;
        X_Det[3*i+2] = at->dither_state.dtheta;
     }
}

#define ST_DITHER 1
#define ST_MIRROR 2
#define ST_GRATING 4
#define ST_DETECT 8

#if MXREF_INTERPOSE
/* One photon at a time with its own pre-drawn variates.  U is n x MX_NU and
 * N is n x MX_NN, photon-major.  used[] receives, per photon, the number of
 * uniforms and normals each stage consumed (8 ints).  Returns the number of
 * photons whose stage ran past its slot range, or -1. */
int mxref_trace_slots(int n, const double *energy, const double *p_in, const double *t,
                      const double *U, const double *N, int stages,
                      double *x, double *p, unsigned int *flags, int *shell, int *order,
                      int *ccd, float *ypix, float *zpix, float *dith, int *used)
{
   Marx_Photon_Type pt;
   Marx_Photon_Attr_Type at;
   unsigned int sidx;
   double sen;
   int i, bad = 0;

   for (i = 0; i < n; i++)
     {
        const double *u = U + (size_t) i * MX_NU;
        const double *g = N + (size_t) i * MX_NN;
        int *us = used + 8 * i;
        unsigned int num;

        fill_attr(&at, energy[i], p_in + 3 * i, t[i], (unsigned int) i);
        memset(&pt, 0, sizeof(pt));
        pt.attributes = &at;
        pt.n_photons = 1; pt.max_n_photons = 1;
        pt.sorted_index = &sidx; pt.sorted_energies = &sen;
        pt.num_sorted = 1; sidx = 0; sen = energy[i];
        pt.history = MARX_ENERGY_OK | MARX_TIME_OK | MARX_P_VECTOR_OK | MARX_TAG_OK;
        Rng_Overrun = 0;

        memset(us, 0, 8 * sizeof(int));
        if ((stages & ST_DITHER) && Have_Dither)
          {
             rng_window(u, 0, 0, g, MX_N_DITHER, MX_N_DITHER_N);
             _marx_dither_photons(&pt, &num);
             us[1] = N_pos - MX_N_DITHER;
             if (num == 0) us[1] = -1;     /* the dither model gave no state (past the aspect solution) */
          }
        if (stages & ST_MIRROR)
          {
             rng_window(u, MX_U_MIRROR, MX_U_MIRROR_N, g, MX_N_MIRROR, MX_N_MIRROR_N);
             if (-1 == marx_mirror_reflect(&pt, 0)) { set_err("mirror"); return -1; }
             us[2] = U_pos - MX_U_MIRROR; us[3] = N_pos - MX_N_MIRROR;
          }
        if ((stages & ST_GRATING) && Have_Grating)
          {
             if (Grating_Is_LETG)
               rng_window(u, MX_U_LETG, MX_U_LETG_N, g, MX_N_LETG, MX_N_LETG_N);
             else
               rng_window(u, MX_U_GRATING, MX_U_GRATING_N, g, MX_N_GRATING, MX_N_GRATING_N);
             if (-1 == marx_grating_diffract(&pt, 0)) { set_err("grating"); return -1; }
             us[4] = U_pos - (Grating_Is_LETG ? MX_U_LETG : MX_U_GRATING);
             us[5] = N_pos - (Grating_Is_LETG ? MX_N_LETG : MX_N_GRATING);
          }
        if ((stages & ST_DETECT) && Det_Kind >= 3)
          {
             rng_window(u, MX_U_HRC, MX_U_HRC_N, g, MX_N_HRC, MX_N_HRC_N);
             pt.history &= ~MARX_DET_NUM_OK;
             if (-1 == marx_detect(&pt, 0)) { set_err("detect"); return -1; }
             us[6] = U_pos - MX_U_HRC; us[7] = N_pos - MX_N_HRC;
          }
        else if ((stages & ST_DETECT) && Det_Kind)
          {
             rng_window(u, MX_U_DETECT, MX_U_DETECT_N, g, MX_N_DETECT, MX_N_DETECT_N);
             if (Acis_Fef)
               {
                  pt.history &= ~MARX_DET_NUM_OK;
                  if (-1 == marx_detect(&pt, 0)) { set_err("detect"); return -1; }
               }
             else detect_photons(&pt);
             us[6] = U_pos - MX_U_DETECT; us[7] = N_pos - MX_N_DETECT;
          }
        rng_window(NULL, 0, 0, NULL, 0, 0);
        if (Rng_Overrun) bad++;
        store_attr(&at, i, x, p, flags, shell, order, ccd, ypix, zpix, dith);
     }
   if (Rng_Unexpected) { set_err("unexpected generator call"); return -1; }
   return bad;
}
#else
void mxref_seed(unsigned long seed) { JDMsrandom(seed); }

static const double *Sort_E;
static int cmp_energy(const void *a, const void *b)
{
   double ea = Sort_E[*(const unsigned int *) a], eb = Sort_E[*(const unsigned int *) b];
   return (ea > eb) - (ea < eb);
}

/* All photons as one batch with the reference's own generator, in energy
 * order as marx_create_photons leaves them (source.c:366).  Returns the
 * seconds spent inside the stage calls, or -1. */
double mxref_trace_batch(int n, const double *energy, const double *p_in, const double *t,
                         int stages, double *x, double *p, unsigned int *flags, int *shell,
                         int *order, int *ccd, float *ypix, float *zpix, float *dith)
{
   Marx_Photon_Type *pt;
   unsigned int i, num;
   struct timespec t0, t1;
   double secs;

   if (NULL == (pt = marx_alloc_photon_type((unsigned int) n))) return -1;
   pt->sorted_index = (unsigned int *) malloc(n * sizeof(unsigned int));
   for (i = 0; i < (unsigned int) n; i++)
     {
        fill_attr(pt->attributes + i, energy[i], p_in + 3 * i, t[i], i);
        pt->sorted_index[i] = i;
     }
   Sort_E = energy;
   qsort(pt->sorted_index, n, sizeof(unsigned int), cmp_energy);
   for (i = 0; i < (unsigned int) n; i++) pt->sorted_energies[i] = energy[pt->sorted_index[i]];
   pt->n_photons = n; pt->num_sorted = n;
   pt->history = MARX_ENERGY_OK | MARX_TIME_OK | MARX_P_VECTOR_OK | MARX_TAG_OK;

   clock_gettime(CLOCK_MONOTONIC, &t0);
   if ((stages & ST_DITHER) && Have_Dither) _marx_dither_photons(pt, &num);
   if ((stages & ST_MIRROR) && (-1 == marx_mirror_reflect(pt, 0))) goto fail;
   if ((stages & ST_GRATING) && Have_Grating && (-1 == marx_grating_diffract(pt, 0))) goto fail;
   if ((stages & ST_DETECT) && Det_Kind >= 3) { if (-1 == marx_detect(pt, 0)) goto fail; }
   else if ((stages & ST_DETECT) && Det_Kind && Acis_Fef) { if (-1 == marx_detect(pt, 0)) goto fail; }
   else if ((stages & ST_DETECT) && Det_Kind) detect_photons(pt);
   clock_gettime(CLOCK_MONOTONIC, &t1);
   secs = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);

   for (i = 0; i < (unsigned int) n; i++)
     store_attr(pt->attributes + i, i, x, p, flags, shell, order, ccd, ypix, zpix, dith);
   marx_dealloc_photon_type(pt);
   return secs;
fail:
   marx_dealloc_photon_type(pt);
   return -1;
}
#endif

/* ------------------------------------------------------------- output -- */
/* The reference's own writer (marx_write_photons, marxio.c:395-478) over a
 * photon list given as columns (component-major x, p, dither state and
 * support orders as in the engine's lists), for byte comparisons of the
 * output files.  open_mode 1 creates the files, 0 appends. */
int mxref_write_photons(const char *dir, int n, const double *energy, const double *x, const double *p,
                        const double *t, const unsigned int *flags, const unsigned int *tag,
                        const signed char *shell, const signed char *order, const signed char *ccd,
                        const float *ypix, const float *zpix, const float *dith, const signed char *sup,
                        const short *pha, const float *upix, const float *vpix, const unsigned char *region,
                        unsigned long history, unsigned long write_mask, int open_mode, double total_time)
{
   Marx_Photon_Type *pt;
   int i, k, r;

   if (NULL == (pt = marx_alloc_photon_type((unsigned int) (n > 0 ? n : 1)))) return -1;
   for (i = 0; i < n; i++)
     {
        Marx_Photon_Attr_Type *at = pt->attributes + i;
        memset(at, 0, sizeof(*at));
        at->energy = energy[i];
        at->x.x = x[i]; at->x.y = x[n + i]; at->x.z = x[2 * n + i];
        at->p.x = p[i]; at->p.y = p[n + i]; at->p.z = p[2 * n + i];
        at->arrival_time = t[i];
        at->flags = flags[i];
        at->tag = tag[i];
        at->mirror_shell = (unsigned int) shell[i];
        at->order = order[i];
        at->ccd_num = ccd[i];
        at->y_pixel = ypix[i]; at->z_pixel = zpix[i];
        at->dither_state.ra = dith[i]; at->dither_state.dec = dith[n + i]; at->dither_state.roll = dith[2 * n + i];
        for (k = 0; k < 4; k++) at->support_orders[k] = sup[k * n + i];
        at->pulse_height = pha[i];
        at->u_pixel = upix[i]; at->v_pixel = vpix[i];
        at->detector_region = region[i];
     }
   pt->n_photons = (unsigned int) n;
   pt->history = history;
   r = marx_write_photons(pt, write_mask, (char *) dir, open_mode, total_time);
   marx_dealloc_photon_type(pt);
   return r;
}

/* The reference's ray-file writer (marx_dump_to_rayfile, s-rayfile.c:109-155)
 * over the same columns, with PI. */
int mxref_dump_rayfile(const char *file, int n, const double *energy, const double *x, const double *p,
                       const double *t, const unsigned int *flags, const unsigned int *tag,
                       const signed char *shell, const signed char *order, const signed char *ccd,
                       const float *ypix, const float *zpix, const float *dith, const signed char *sup,
                       const short *pha, const float *upix, const float *vpix, const unsigned char *region,
                       const float *pi, unsigned long history, int new_file, double total_time)
{
   Marx_Photon_Type *pt;
   int i, k, r;

   if (NULL == (pt = marx_alloc_photon_type((unsigned int) (n > 0 ? n : 1)))) return -1;
   for (i = 0; i < n; i++)
     {
        Marx_Photon_Attr_Type *at = pt->attributes + i;
        memset(at, 0, sizeof(*at));
        at->energy = energy[i];
        at->x.x = x[i]; at->x.y = x[n + i]; at->x.z = x[2 * n + i];
        at->p.x = p[i]; at->p.y = p[n + i]; at->p.z = p[2 * n + i];
        at->arrival_time = t[i];
        at->flags = flags[i];
        at->tag = tag[i];
        at->mirror_shell = (unsigned int) shell[i];
        at->order = order[i];
        at->ccd_num = ccd[i];
        at->y_pixel = ypix[i]; at->z_pixel = zpix[i];
        at->dither_state.ra = dith[i]; at->dither_state.dec = dith[n + i]; at->dither_state.roll = dith[2 * n + i];
        for (k = 0; k < 4; k++) at->support_orders[k] = sup[k * n + i];
        at->pulse_height = pha[i];
        at->u_pixel = upix[i]; at->v_pixel = vpix[i];
        at->detector_region = (SIGNED_CHAR) region[i];
        at->pi = pi[i];
     }
   pt->n_photons = (unsigned int) n;
   pt->history = history;
   r = marx_dump_to_rayfile((char *) file, new_file, pt, total_time);
   marx_dealloc_photon_type(pt);
   return r;
}

/* ------------------------------------------------------------ sources -- */
/* The reference's source models (marx_create_source, source.c:388-420, and
 * the create_photons functions of s-*.c) for the parameters of the last
 * mxref_setup call.  p_out receives the source direction st->p. */
static Marx_Source_Type *Src;
int mxref_source_setup(double *p_out)
{
   if (Pf == NULL) { set_err("mxref_setup first"); return -1; }
   if (Src != NULL) { marx_close_source(Src); Src = NULL; }
   if (NULL == (Src = marx_create_source(Pf))) { set_err("source set-up failed"); return -1; }
   if (-1 == marx_open_source(Src)) { set_err("source open failed"); return -1; }
   p_out[0] = Src->p.x; p_out[1] = Src->p.y; p_out[2] = Src->p.z;
   return 0;
}

/* Replace the source's direction st->p (select_source, source.c:158-201,
 * leaves an IMAGE source's p pointing from the origin to the sky; its
 * image_create_photons expects the direction of travel). */
int mxref_source_set_direction(const double *p)
{
   if (Src == NULL) { set_err("no source"); return -1; }
   Src->p.x = p[0]; Src->p.y = p[1]; Src->p.z = p[2];
   return 0;
}

/* One photon per create_photons call.  With the slot build, photon i's
 * uniforms come from U[i*4 .. i*4+4) in the order the model draws them
 * (spectrum first); with the native build, from the reference's own
 * generator.  Energies and directions (n x 3) out. */
int mxref_source_photons(int n, const double *U, double *energy, double *p)
{
   Marx_Photon_Type pt;
   Marx_Photon_Attr_Type at;
   unsigned int num;
   int i;
   if (Src == NULL) { set_err("no source"); return -1; }
   for (i = 0; i < n; i++)
     {
        memset(&pt, 0, sizeof(pt));
        memset(&at, 0, sizeof(at));
        pt.attributes = &at; pt.max_n_photons = 1;
#if MXREF_INTERPOSE
        rng_window(U + 4 * (size_t) i, 0, 4, NULL, 0, 0);
        Rng_Overrun = 0;
#else
        (void) U;
#endif
        if (-1 == (*Src->create_photons)(Src, &pt, 1, &num)) { set_err("create_photons"); return -1; }
#if MXREF_INTERPOSE
        rng_window(NULL, 0, 0, NULL, 0, 0);
        if (Rng_Overrun) { set_err("source drew more than 4 uniforms"); return -1; }
#endif
        energy[i] = at.energy;
        p[3 * i] = at.p.x; p[3 * i + 1] = at.p.y; p[3 * i + 2] = at.p.z;
     }
   return 0;
}

/* One create_photons call for a batch of up to n photons (the SAOSAC
 * source reads its rays in batches; its times are relative to the batch
 * before, s-saosac.c:173-300).  With the slot build the uniforms come from
 * U[0 .. nu) in the order they are drawn.  Energies, positions and
 * directions (n x 3), times, flags and shells out; *num the photons made,
 * *used the uniforms drawn (slot build). */
int mxref_source_batch(int n, const double *U, int nu, double *energy, double *x, double *p, double *t,
                       unsigned int *flags, int *shell, unsigned int *num, int *used)
{
   Marx_Photon_Type pt;
   Marx_Photon_Attr_Type *at;
   unsigned int i;
   if (Src == NULL) { set_err("no source"); return -1; }
   if (NULL == (at = (Marx_Photon_Attr_Type *) calloc((size_t) n, sizeof (Marx_Photon_Attr_Type))))
     { set_err("out of memory"); return -1; }
   memset(&pt, 0, sizeof(pt));
   pt.attributes = at; pt.max_n_photons = (unsigned int) n;
#if MXREF_INTERPOSE
   rng_window(U, 0, nu, NULL, 0, 0);
   Rng_Overrun = 0;
#else
   (void) U; (void) nu;
#endif
   if (-1 == (*Src->create_photons)(Src, &pt, (unsigned int) n, num)) { free(at); set_err("create_photons"); return -1; }
#if MXREF_INTERPOSE
   *used = U_pos;
   rng_window(NULL, 0, 0, NULL, 0, 0);
   if (Rng_Overrun) { free(at); set_err("source drew more uniforms than given"); return -1; }
#endif
   for (i = 0; i < *num; i++)
     {
        energy[i] = at[i].energy; t[i] = at[i].arrival_time;
        x[3 * i] = at[i].x.x; x[3 * i + 1] = at[i].x.y; x[3 * i + 2] = at[i].x.z;
        p[3 * i] = at[i].p.x; p[3 * i + 1] = at[i].p.y; p[3 * i + 2] = at[i].p.z;
        flags[i] = at[i].flags; shell[i] = (int) at[i].mirror_shell;
     }
   free(at);
   return 0;
}
