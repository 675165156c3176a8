/* marx_gb300 compatibility shim — MARX's own stage API over the reference's
 * array-of-structures photon list, traced on the GPU.
 *
 * libmarx_gb300_compat.so exports, with the reference's names, signatures,
 * return values and per-batch semantics, the functions that MARX's
 * process_photons (marx/src/marx.c:240-273) calls back to back:
 *
 *   marx_mirror_init      marx/libsrc/mirror.c:48    marx_mirror_reflect   mirror.c:93
 *   marx_grating_init     marx/libsrc/grating.c:44   marx_grating_diffract grating.c:88
 *   marx_detector_init    marx/libsrc/detector.c:298 marx_detect           detector.c:361
 *   marx_prune_photons    marx/libsrc/photon.c:40
 *   marx_alloc_photon_type / marx_dealloc_photon_type  photon.c:67, :92
 *
 * so that a stock marx.c links against it in place of the mirror, grating,
 * detector and photon modules of libmarx (the link line is in the
 * integration notes beside this header).  Each stage:
 *   - returns 0 without work when its history bit is already set, then sets
 *     it (hrma.c:1171-1173, diffract.c:982-984, acis-i.c:105-109,
 *     hrc-i.c:125-129, hrc-s.c:242-248);
 *   - prunes first (marx_prune_photons: sorted_index keeps the photons with
 *     no BAD_PHOTON_MASK bit, in order, and sorted_energies follows it);
 *   - gathers the attributes of the photons in sorted_index into the
 *     engine's structure-of-arrays columns, traces them on the GPU through
 *     mx_trace (include/marx_gb300.h) and scatters the results back.  Photons
 *     outside sorted_index are not touched.
 * The *_init functions read their parameters by name through the
 * reference's parameter-file library (pf_get_string, pf_get_double,
 * pf_get_integer, pf_get_boolean of pfile.h), which the calling program
 * links; the shim references them weakly, so a program without them can
 * load the library but its *_init calls fail.  Errors are reported as
 * marx_error does (a message on stderr) and kept for
 * marx_gb300_compat_last_error().
 *
 * Random numbers: Philox4x32-10 keyed by (seed, photon tag), the seed the
 * RandomSeed parameter (read by marx_mirror_init when present) or
 * marx_gb300_compat_set_seed; or pre-drawn per-photon variates
 * (marx_gb300_compat_set_variates), the mode the parity tests use.
 *
 * Limits: MirrorType HRMA only (the FLATFIELD mirror is not built);
 * detector motion from an aspect solution (DitherModel FILE, the dy, dz,
 * dtheta of Marx_Dither_Type) is not applied by marx_detect: a batch that
 * carries it is refused.  The CALDB tables come from the engine's table
 * pack (MARX_GB300_PACK, else marx_gb300/caldb/marx_tables.mxpack beside
 * the library), not from DataDirectory.
 */
#ifndef MARX_GB300_COMPAT_H
#define MARX_GB300_COMPAT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The reference's types (marx.h:42-151, jdmath.h:395-399, pfile.h:37),
 * declared here with the same members in the same order so that the
 * layout is the reference's; a translation unit that includes the
 * reference's own headers first uses theirs. */
#ifndef JDMATH_H_INCLUDED
typedef struct {
  double x, y, z;
} JDMVector_Type;
#endif

#ifndef _PF_H_LOADED_
typedef struct _Param_File_Type Param_File_Type;
#endif

#ifndef _MARX_H_
typedef struct {
  float ra, dec, roll;     /* sky dither, relative to the nominal pointing (rad) */
  float dy, dz, dtheta;    /* detector motion (mm, mm, rad) */
} Marx_Dither_Type;

typedef struct {
  double energy;                 /* keV */
  JDMVector_Type x;              /* position (mm) */
  JDMVector_Type p;              /* direction */
  double arrival_time;           /* s, from Marx_Photon_Type.start_time */
  unsigned int flags;            /* PHOTON_* bits */
  float y_pixel, z_pixel;        /* chip pixel, 0-based */
  float u_pixel, v_pixel;        /* HRC-S u, v */
  Marx_Dither_Type dither_state;
  float pi;
  short pulse_height;
  unsigned int mirror_shell;     /* 0..3 */
  signed char ccd_num;
  signed char detector_region;
  signed char order;
  signed char support_orders[4];
  unsigned int tag;
} Marx_Photon_Attr_Type;

typedef struct {
  double source_distance;        /* mm, 0: source at infinity */
  Marx_Photon_Attr_Type *attributes;
  unsigned int n_photons;
  unsigned int max_n_photons;
  double total_time;
  double start_time;
  unsigned int *sorted_index;
  double *sorted_energies;
  unsigned int num_sorted;
  unsigned long history;         /* MARX_*_OK bits */
  unsigned int tag_start;
} Marx_Photon_Type;

#define PHOTON_UNDETECTED       0x01
#define PHOTON_UNREFLECTED      0x02
#define PHOTON_UNDIFFRACTED     0x04
#define PHOTON_MISSED_DETECTOR  0x08
#define PHOTON_MIRROR_VBLOCKED  0x10
#define PHOTON_DRAKE_BLOCKED    0x20
#define PHOTON_GRATING_VBLOCKED 0x40
#define BAD_PHOTON_MASK         0xFF
#define PHOTON_DRAKE_REFLECTED  0x100
#define PHOTON_ACIS_STREAKED    0x200

#define MARX_ENERGY_OK        0x00000001
#define MARX_TIME_OK          0x00000002
#define MARX_X_VECTOR_OK      0x00000004
#define MARX_P_VECTOR_OK      0x00000008
#define MARX_TAG_OK           0x00000010
#define MARX_PULSEHEIGHT_OK   0x00000020
#define MARX_PI_OK            0x00000040
#define MARX_DET_PIXEL_OK     0x00000080
#define MARX_DET_NUM_OK       0x00000100
#define MARX_DET_REGION_OK    0x00000200
#define MARX_DET_UV_PIXEL_OK  0x00000400
#define MARX_MIRROR_SHELL_OK  0x00000800
#define MARX_SKY_DITHER_OK    0x00001000
#define MARX_DET_DITHER_OK    0x00002000
#define MARX_ORDER_OK         0x00100000
#define MARX_ORDER1_OK        0x00200000
#define MARX_ORDER2_OK        0x00400000
#define MARX_ORDER3_OK        0x00800000
#define MARX_ORDER4_OK        0x01000000

int marx_mirror_init(Param_File_Type *pf);
int marx_mirror_reflect(Marx_Photon_Type *pt, int verbose);
int marx_grating_init(Param_File_Type *pf);
int marx_grating_diffract(Marx_Photon_Type *pt, int verbose);
int marx_detector_init(Param_File_Type *pf);
int marx_detect(Marx_Photon_Type *pt, int verbose);
void marx_prune_photons(Marx_Photon_Type *pt);
Marx_Photon_Type *marx_alloc_photon_type(unsigned int num);
int marx_dealloc_photon_type(Marx_Photon_Type *pt);
#endif /* _MARX_H_ */

/* Return values of the *_init functions, as the reference's (marx.h:364-376):
 * the module type (mirror: 2, HRMA; grating: 0 NONE, 1 HETG, 2 LETG;
 * detector: 0 NONE, 1 HRC-S, 2 HRC-I, 3 ACIS-S, 4 ACIS-I), or -1. */

/* ---- extensions (no counterpart in the reference) ---------------------- */

/* The aspect dither of the photons just created (_marx_dither_photons,
 * dither.c:630, which marx_create_photons runs at source.c:357), for a
 * caller whose photons come from elsewhere: every one of the n_photons
 * attributes in order, the DitherModel parameters read by
 * marx_gb300_compat_dither_init (INTERNAL or NONE).  Sets dither_state's
 * ra, dec, roll and turns p. */
int marx_gb300_compat_dither_init(Param_File_Type *pf);
int marx_gb300_compat_dither_photons(Marx_Photon_Type *pt, unsigned int *num_dithered);

/* Philox seed of the next stage calls. */
void marx_gb300_compat_set_seed(uint64_t seed);

/* Pre-drawn variates instead of Philox: U (36 x n) and N (24 x n),
 * slot-major, indexed by the photon's position in the attributes array
 * (U[k * n + i] is uniform k of attributes[i]); the slot layout is
 * MX_NUM_U / MX_NUM_N of marx_gb300.h.  The arrays stay the caller's and
 * must outlive the stage calls; NULL (both) returns to Philox.  0, or -1
 * when only one is given. */
int marx_gb300_compat_set_variates(const double *U, const double *N, unsigned int n);

/* The last error message ("" when none). */
const char *marx_gb300_compat_last_error(void);

/* Release the engine context and device buffers (the next stage call
 * builds them again). */
void marx_gb300_compat_shutdown(void);

#ifdef __cplusplus
}
#endif
#endif /* MARX_GB300_COMPAT_H */
