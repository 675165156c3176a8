/* marx_gb300 — GB300-native photon trace for the MARX stage pipeline
 * (aspect dither -> HRMA mirror -> HETG/LETG grating -> ACIS/HRC detector).
 *
 * C ABI: plain pointers, sizes and POD structs.  Every entry point returns
 * 0 on success and a negative MX_E* code on failure; mx_last_error() gives
 * the message.  Nothing aborts or traps across this boundary.
 *
 * Reference interfaces this ABI stands in for (paths inside MARX 5.5.3):
 *   marx_mirror_reflect   marx/libsrc/mirror.c:93   (marx.h:358)
 *   marx_grating_diffract marx/libsrc/grating.c:88  (marx.h:362)
 *   marx_detect           marx/libsrc/detector.c:361 (marx.h:355)
 *   _marx_dither_photons  marx/libsrc/dither.c:630  (_marx.h:142)
 *   marx_prune_photons    marx/libsrc/photon.c:40   (marx.h:155)
 * and the *_init(Param_File_Type*) functions beside them, whose parameters
 * (marx/par/marx.par) are the fields of mx_config.
 */
#ifndef MARX_GB300_H
#define MARX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status -- */
#define MX_OK            0
#define MX_EINVAL       -1   /* bad argument or configuration */
#define MX_ENOMEM       -2   /* device or host allocation failed */
#define MX_ECUDA        -3   /* a CUDA call failed */
#define MX_EPACK        -4   /* table pack missing or malformed */
#define MX_ERANGE       -5   /* size beyond a stated limit */
#define MX_EVARIATE     -6   /* a stage needed more pre-drawn variates than its slots */
#define MX_EWATCHDOG    -7   /* device-side iteration limit hit; photons flagged */

/* Per-photon flag bits: same values as marx.h:65-75 (PHOTON_*). */
#define MX_PHOTON_UNDETECTED        0x01u
#define MX_PHOTON_UNREFLECTED       0x02u
#define MX_PHOTON_UNDIFFRACTED      0x04u
#define MX_PHOTON_MISSED_DETECTOR   0x08u
#define MX_PHOTON_MIRROR_VBLOCKED   0x10u
#define MX_PHOTON_DRAKE_BLOCKED     0x20u
#define MX_PHOTON_GRATING_VBLOCKED  0x40u
#define MX_BAD_PHOTON_MASK          0xFFu
#define MX_PHOTON_DRAKE_REFLECTED   0x100u
#define MX_PHOTON_ACIS_STREAKED     0x200u
/* Engine-only bit: a stage ran out of pre-drawn variate slots. */
#define MX_PHOTON_VARIATE_OVERRUN   0x10000u
/* Engine-only bit inside the bad mask: with DitherModel FILE the photon's
 * time is at or past the aspect solution's last row.  The reference stops
 * dithering there and drops the photon and every later one from its batch
 * (get_aspsol_point, dither.c:303-306 and _marx_dither_photons, :646-656);
 * the engine flags it and later stages skip it. */
#define MX_PHOTON_ASPECT_END        0x80u

/* Stage mask for mx_trace. */
#define MX_STAGE_DITHER   0x1u   /* _marx_dither_photons (dither.c:630)   */
#define MX_STAGE_MIRROR   0x2u   /* marx_mirror_reflect  (mirror.c:93)    */
#define MX_STAGE_GRATING  0x4u   /* marx_grating_diffract (grating.c:88)  */
#define MX_STAGE_DETECT   0x8u   /* marx_detect          (detector.c:361) */
#define MX_STAGE_ALL      0xFu

/* Pre-drawn variate slots per photon.  Each stage reads its uniforms and
 * normals from a fixed slot range, in the order the reference draws them:
 *   mirror  U[0..11]: [vignetting] shell radius theta,
 *                     per optic P then H: [blur phi] [reflectivity] [wfold p, sign]
 *           N[2..3] : per optic [blur angle]
 *   HETG    U[12..13]: vignetting, order;  N[4..5]: dtheta, dP/P
 *   ACIS    U[14..15]: [QE] [streak row];  N[6..7]: reserved
 *           U[28..35], N[20..23]: the FEF pulse height (marx_apply_acis_rmf):
 *                      gaussian choice, its normal or tail draws, rejection
 *                      draws, the PI randomisation
 *   LETG    U[16..21]: vignetting, order, support orders (fine, coarse x3);
 *           N[8..17] : dtheta, dP/P of the primary, then of each support
 *   HRC     U[22..27]: MCP QE, UV/ion shield QE, blur component, radius,
 *                      azimuth (one spare);  N[18..19]: pulse height (one spare)
 *   dither  N[0..1]  : aspect blur ra, dec
 * Slot arrays are slot-major: U[k * n + i] is uniform k of photon i. */
#define MX_NUM_U 36
#define MX_NUM_N 24
#define MX_U_MIRROR   0
#define MX_U_GRATING 12
#define MX_U_DETECT  14
#define MX_U_LETG    16
#define MX_U_HRC     22
#define MX_U_FEF     28
#define MX_N_DITHER   0
#define MX_N_MIRROR   2
#define MX_N_GRATING  4
#define MX_N_DETECT   6
#define MX_N_LETG     8
#define MX_N_HRC     18
#define MX_N_FEF     20

enum { MX_GRATING_NONE = 0, MX_GRATING_HETG = 1, MX_GRATING_LETG = 2 };
enum { MX_DETECTOR_NONE = 0, MX_DETECTOR_ACIS_I = 1, MX_DETECTOR_ACIS_S = 2, MX_DETECTOR_HRC_I = 3,
       MX_DETECTOR_HRC_S = 4 };
enum { MX_DITHER_NONE = 0, MX_DITHER_INTERNAL = 1, MX_DITHER_FILE = 2 };   /* DitherModel NONE, INTERNAL, FILE */

/* Simulation parameters.  Names follow marx.par; units are marx.par's. */
typedef struct mx_config {
  /* HRMA (hrma.c:244-286) */
  double hrma_cap_x;          /* HRMA_Cap_X (mm) */
  double shell_xoffset[4];    /* HRMA_P1H1_XOffset .. P6H6 (mm), shells 1,3,4,6 */
  double blur_p[4], blur_h[4];/* P1Blur..P6Blur, H1Blur..H6Blur (arcsec) */
  double scat_p[4], scat_h[4];/* P1ScatFactor.., H1ScatFactor.. */
  double hrma_vig;            /* HRMAVig */
  int32_t hrma_ideal;         /* HRMA_Ideal */
  int32_t use_blur;           /* HRMA_Use_Blur */
  int32_t use_wfold;          /* HRMA_Use_WFold */
  int32_t use_struts;         /* HRMA_Use_Struts */
  int32_t use_scale_factors;  /* HRMA_Use_Scale_Factors */
  uint32_t shutters[4];       /* Shutters1..6 as open-quadrant bitmaps ("0000" -> 0xF) */
  double source_distance;     /* Marx_Photon_Type.source_distance (mm, 0 = infinite) */
  /* Grating (diffract.c:550-614, marx.par HETG_Shell*) */
  int32_t grating;            /* MX_GRATING_* */
  int32_t use_sector_files;   /* Use_HETG_Sector_Files */
  double hetg_theta[4];       /* HETG_Shell{1,3,4,6}_Theta (deg) */
  double hetg_dtheta[4];      /* HETG_Shell*_dTheta (arcmin, sigma) */
  double hetg_period[4];      /* HETG_Shell*_Period (um) */
  double hetg_dpp[4];         /* HETG_Shell*_dPoverP */
  double hetg_vig[4];         /* HETG_Shell*_Vig */
  double meg_rowland, heg_rowland; /* MEG/HEGRowlandDiameter (mm) */
  int32_t max_order;          /* 0: every order in the table; m>0: keep |order|<=m, renormalised */
  int32_t aperture_area_uniform; /* 0: radius uniform in [rmin,rmax] as hrma.c:1005;
                                    1: uniform in area over each shell annulus */
  /* Dither (dither.c:85-110) */
  int32_t dither;             /* MX_DITHER_* */
  int32_t reserved1;
  double dither_amp[3];       /* DitherAmp_RA, _Dec, _Roll (arcsec) */
  double dither_period[3];    /* DitherPeriod_* (s) */
  double dither_phase[3];     /* DitherPhase_* (rad) */
  double roll_nom;            /* Roll_Nom (deg) */
  double aspect_blur;         /* AspectBlur (arcsec, sigma) */
  /* Detector (detector.c:45-52, acis-i.c:170-176) */
  int32_t detector;           /* MX_DETECTOR_* */
  int32_t det_extend;         /* DetExtendFlag */
  double det_offset[3];       /* DetOffsetX/Y/Z (mm) */
  double acis_exposure_time;  /* ACIS_Exposure_Time (s) */
  double acis_frame_transfer_time; /* ACIS_Frame_Transfer_Time (s) */
  double focal_length;        /* Marx_Focal_Length (detpix.c:41) (mm) */
  double start_time;          /* Marx_Photon_Type.start_time (s) */
  /* LETG (diffract.c:1727-1860; marx.par LETG_Shell*, leg*) */
  double letg_theta[4];       /* LETG_Shell{1,3,4,6}_Theta (deg) */
  double letg_dtheta[4];      /* LETG_Shell*_dTheta (arcmin, sigma) */
  double letg_period[4];      /* LETG_Shell*_Period (um) */
  double letg_dpp[4];         /* LETG_Shell*_dPoverP */
  double letg_vig[4];         /* LETG_Shell*_Vig */
  double leg_rowland;         /* LEGRowlandDiameter (mm) */
  double letg_acis_dtheta;    /* LETG_ACIS_dTheta (deg), added with an ACIS detector */
  int32_t leg_fine_orders;    /* legFineNumOrders (2n+1; 0: no fine support grating) */
  int32_t leg_coarse_orders;  /* legCoarseNumOrders (2n+1; 0: no coarse support grating) */
  double leg_fine_period, leg_fine_bar_height, leg_fine_bar_width;       /* legFine* (um) */
  double leg_coarse_period, leg_coarse_bar_height, leg_coarse_bar_width; /* legCoarse* (um) */
  /* HRC (hrc-i.c, hrc-s.c, hrcblur.c) */
  int32_t det_ideal;          /* DetIdeal: no QE, no HRC position blur */
  int32_t reserved2;
  double hrc_i_blur[13];      /* HRC-I-Blur{G1FWHM,G1Xctr,G1Yctr,G1Amp,G2..,L1FWHM,L1Xctr,L1Yctr,L1Amp,L1Rmax} */
  double hrc_s_blur[13];      /* the same for HRC-S (1/4 pixels) */
  /* HRC-S high-energy suppression filter, the Drake flat (drake.c:148-246) */
  int32_t hrc_hesf;           /* HRC-HESF */
  int32_t hesf_n;             /* HESFN: plates per side, 1..4 */
  double hesf_offset_x, hesf_offset_z;   /* HESFOffsetX, HESFOffsetZ (mm) */
  double hesf_gap_y1, hesf_gap_y2;       /* HESFGapY1, HESFGapY2 (mm) */
  double hesf_length, hesf_cr_width;     /* HESFLength, HESFCrWidth (mm) */
  double hesf_height[4], hesf_theta[4];  /* HESFHeight1..4 (mm), HESFTheta1..4 (deg) */
  /* Pointing (dither.c:85-160) */
  double ra_nom, dec_nom;     /* RA_Nom, Dec_Nom (deg) */
  double pointing_offset[2];  /* PointingOffsetY, PointingOffsetZ (arcsec) */
  /* ACIS response with DetIdeal = no (acis-s.c:136-172): the CALDB QE and
   * the contamination of the pack's ACIS contamination tables at this epoch */
  double tstart_mjdsecs;      /* the run's start in seconds since MJDREF (marx_set_time, util.c:231) */
} mx_config;

/* Structure-of-arrays photon list.  3-vectors are component-major:
 * x[0*s + i], x[1*s + i], x[2*s + i] with s = stride (n when 0).  Which pointers must be set depends
 * on the stages run; unused outputs may be NULL. */
typedef struct mx_photons {
  uint32_t n;
  uint32_t stride;         /* distance between the components of x, p and
                              dither_state (0: n); a larger stride views a
                              slice of a longer list in place */
  double   *energy;        /* keV */
  double   *x;             /* 3n, mm (output of the mirror) */
  double   *p;             /* 3n, unit direction (input and output) */
  double   *arrival_time;  /* s, relative to start_time */
  uint32_t *flags;         /* MX_PHOTON_* */
  uint32_t *tag;           /* per-photon generator counter (Philox mode); NULL: photon i
                              draws with counter i (its index in the list) */
  int8_t   *mirror_shell;  /* 0..3 */
  int8_t   *order;         /* grating order */
  int8_t   *ccd_num;       /* chip id, -1 if missed */
  int8_t   *reserved8;
  float    *y_pixel;       /* chip x (0-based) */
  float    *z_pixel;       /* chip y (0-based) */
  float    *dither_state;  /* 3n: ra, dec, roll (rad), as Marx_Dither_Type */
  int8_t   *support_orders;/* 4n: LETG fine and three coarse support orders */
  int16_t  *pulse_height;  /* HRC pulse height; ACIS PHA from the FEF (-1: no response) */
  float    *u_pixel;       /* HRC-S u, v pixel */
  float    *v_pixel;
  uint8_t  *detector_region; /* HRC-S UV/ion shield region */
  float    *pi;            /* ACIS PI energy (keV) from the FEF (Marx_Photon_Attr_Type.pi, b_energy.dat) */
  float    *det_dither;    /* 3n: dy, dz (mm), dtheta (rad): the detector's motion of Marx_Dither_Type,
                              written by the dither stage (zero unless DitherModel is FILE) */
} mx_photons;

/* Pre-drawn variates (device pointers for mx_trace).  When both are NULL
 * the variates come from Philox4x32-10 keyed by (seed, tag). */
typedef struct mx_variates {
  const double *U;         /* MX_NUM_U * n, slot-major, uniforms in [0,1) */
  const double *N;         /* MX_NUM_N * n, slot-major, unit normals */
} mx_variates;

typedef struct mx_context mx_context;

/* Defaults = marx.par 5.5 values (HRMA, HETG, INTERNAL dither, ACIS-S). */
void mx_config_default(mx_config *cfg);

/* Load the table pack (see marx_gb300/caldb/pack.py), derive every model
 * table for cfg and upload it to the current CUDA device.  Replaces the
 * marx_mirror_init / marx_grating_init / marx_detector_init / dither init
 * sequence (mirror.c:48, grating.c:44, detector.c:298, dither.c:508). */
mx_context *mx_create(const char *pack_path, const mx_config *cfg);
int  mx_configure(mx_context *ctx, const mx_config *cfg);

/* Check a configuration against a table pack without touching the GPU:
 * MX_OK, or MX_EPACK / MX_EINVAL with the reason in mx_last_error(NULL). */
int  mx_validate_config(const char *pack_path, const mx_config *cfg);
void mx_destroy(mx_context *ctx);

/* The mirror's open aperture area in cm^2 for cfg (its shells' annuli and
 * open shutters; Marx_Mirror_Geometric_Area, hrma.c:719-736), which sets
 * the mean time between a source's photons.  Host only. */
int  mx_geometric_area(const char *pack_path, const mx_config *cfg, double *cm2);

/* Marx_Photon_Type.start_time for the photons traced next (the ACIS frame
 * streak and the aspect solution take start_time + arrival time): a launch
 * parameter, changed without rebuilding the model (MARX moves it on by each
 * batch's total time, source.c:285). */
int  mx_set_start_time(mx_context *ctx, double start_time);

/* ---------------------------------------------------- parameter files --
 * The marx.par parameters behind mx_config (marx/par/marx.par), grouped by
 * the module whose *_init reads them: the mirror (mirror.c:48, hrma.c:244-286),
 * the gratings (grating.c:44, diffract.c:550-614, :1727-1860), the detectors
 * (detector.c:298, acis-i.c:170-176, hrc-*.c, drake.c:148-246) and the aspect
 * dither (dither.c:85-160).  A reader returns one parameter's value as text
 * ("yes"/"no" for booleans), given its name and marx.par type letter
 * ('r' real, 'i' integer, 'b' boolean, 's' string); 0 when found, -1 when
 * the parameter is absent. */
#define MX_PARAMS_MIRROR   0x1u
#define MX_PARAMS_GRATING  0x2u
#define MX_PARAMS_DETECTOR 0x4u
#define MX_PARAMS_DITHER   0x8u
#define MX_PARAMS_ALL      0xFu
typedef int (*mx_param_reader)(void *user, const char *name, char type, char *value, size_t len);

/* Read the parameters of the given groups into cfg (fields of other
 * groups keep their values).  required != 0: an absent parameter is an
 * error (MX_EINVAL), as a missing parameter is to the reference's *_init;
 * otherwise it keeps cfg's value.  Unsupported values (MirrorType other than
 * HRMA, an unknown GratingType, DetectorType or DitherModel, a malformed
 * number, boolean or shutter string) are MX_EINVAL; the reason is in
 * mx_last_error(NULL). */
int  mx_config_read_params(mx_config *cfg, uint32_t groups, mx_param_reader read, void *user, int required);

/* A MARX parameter file (name,type,mode,value,... per line) plus
 * "Name=value" overrides, as the marx command line takes them (a later
 * one wins), read into cfg from mx_config_default: every parameter the
 * engine uses, absent ones at their defaults. */
int  mx_config_read_par(mx_config *cfg, const char *par_path, const char *const *overrides, int n_overrides);

/* The marx.par type letter and MX_PARAMS_* group of a parameter the engine
 * reads (MX_EINVAL for any other name). */
int  mx_param_type(const char *name, char *type, uint32_t *group);
const char *mx_last_error(const mx_context *ctx);  /* ctx may be NULL */

/* Trace photons in place on the device (pointers in ph are device
 * pointers).  Stages run back to back per photon inside one fused kernel;
 * a photon whose flags carry a MX_BAD_PHOTON_MASK bit is left untouched, as
 * marx_prune_photons leaves it out of sorted_index.  Asynchronous on
 * stream (a cudaStream_t, NULL = default stream): a list of 2^18 photons or
 * more traced with Philox draws by the wavefront kernels runs as two halves
 * at once on two streams of the context, forked from stream and joined back
 * into it, so that work queued on stream after the call starts after the
 * whole trace. */
int mx_trace(mx_context *ctx, const mx_photons *ph, uint32_t stages,
             const mx_variates *var, uint64_t seed, void *stream);

/* With an ACIS FEF or (DetIdeal = no) ACIS contamination tables in the
 * pack, every trace that runs the detector stage ends with one more launch:
 * the ACIS response of the photons on a chip (QE x contamination
 * acceptance, FEF pulse height and PI, frame-transfer streak). */

/* Kernel organisation for mx_trace / mx_trace_host.  FUSED runs every stage
 * of a photon in one kernel; WAVEFRONT splits the mirror at its two conic
 * intersections into three kernels with survivor queues between them (the
 * photons lost on the way then stop occupying SIMT lanes) and needs
 * 2 x 128 bytes of device scratch per photon; AUTO picks the wavefront from
 * MX_WAVEFRONT_MIN_PHOTONS photons up.  Both give the same per-photon
 * results. */
#define MX_MODE_AUTO 0
#define MX_MODE_FUSED 1
#define MX_MODE_WAVEFRONT 2
#define MX_WAVEFRONT_MIN_PHOTONS 65536
int mx_set_trace_mode(mx_context *ctx, int mode);

/* The wavefront trace of mx_trace with its survivor queues in a device
 * array built into the library instead of memory the context allocates, so
 * the call allocates nothing: for callers that cannot allocate device
 * memory while they trace, such as a host whose GPU memory is all reserved
 * by another allocator, or a latency-critical loop that must stay out of
 * the CUDA allocator (cudaMalloc and cudaFree may synchronise the device).
 * No counterpart in the reference (MARX allocates its photon arrays on the
 * host per batch).
 *   - at most MX_STATIC_MAX_PHOTONS photons per call (MX_ERANGE beyond);
 *     the array (2 x 128 bytes per photon, 32 MiB) is held by every GPU
 *     that loads the library until the process exits;
 *   - stages must include MX_STAGE_MIRROR: this entry point always runs
 *     the wavefront kernels, whatever mx_set_trace_mode set; pointers and
 *     argument checks as for mx_trace, except that x is always required
 *     (also without MX_STAGE_DETECT);
 *   - the current device must be the one the context was created on
 *     (MX_EINVAL otherwise);
 *   - the first call on a device looks up the array's address there, with
 *     that device current; make that first call before any stream capture;
 *   - every call shares the one array: calls that overlap on the GPU (other
 *     streams or threads) race on it, so serialise them. */
#define MX_STATIC_MAX_PHOTONS 131072
int mx_trace_static(mx_context *ctx, const mx_photons *ph, uint32_t stages, const mx_variates *var,
                    uint64_t seed, void *stream);

/* Same trace on HOST buffers: copies inputs to the device, traces and
 * copies results back; blocks until done.  A list of 2^19 photons or more
 * (tracing the mirror) is cut into chunks: copies in on one stream, copies
 * out on another and the traces on two more, ordered by events, so that the
 * copies of some chunks overlap the trace of others (pinned host memory lets
 * them run asynchronously); the results are those of one pass. */
int mx_trace_host(mx_context *ctx, const mx_photons *host, uint32_t stages,
                  const mx_variates *host_var, uint64_t seed);

/* ------------------------------------------------------------ sources --
 * A source at infinity: the input producer of the trace (the create_photons
 * functions of s-point.c:59, s-gauss.c, s-beta.c, s-disk.c, s-line.c, s-image.c, with
 * flat_energy and file_energy, spectrum.c:138-190).  Photon k gets tag
 * first_tag + k; its energy and direction come from the Philox draws of
 * that tag in the source domain (draw 0: energy, then the source's own
 * draws in the reference's order); arrival time 0 and flags 0. */
typedef struct mx_source {
  double p[3];              /* unit direction of travel (toward the mirror) */
  double energy_min, energy_max;   /* keV, FLAT spectrum */
  uint32_t num_photons;
  int32_t grating;          /* MX_GRATING_NONE or MX_GRATING_HETG */
  int32_t detector;         /* MX_DETECTOR_ACIS_I or MX_DETECTOR_ACIS_S */
  uint32_t reserved;
  /* Extended sources (s-gauss.c, s-beta.c, s-disk.c, s-line.c) about p:
   *   MX_SOURCE_GAUSS  param[0] S-GaussSigma (arcsec)
   *   MX_SOURCE_BETA   param[0] S-BetaCoreRadius (arcsec), param[1] S-BetaBeta (> 1/2)
   *   MX_SOURCE_DISK   param[0] S-DiskTheta0, param[1] S-DiskTheta1 (arcsec)
   *   MX_SOURCE_LINE   param[0] S-LinePhi (deg), param[1] S-LineTheta (arcsec)
   *   MX_SOURCE_IMAGE  param[0], param[1] degrees per pixel along NAXIS1 and NAXIS2
   *                    (|CDELT1|, |CDELT2|, or the CD matrix's row lengths; 0: 0.5 arcsec),
   *                    image: image_ny rows of image_nx pixel values (s-image.c:91-330) */
  int32_t kind;             /* MX_SOURCE_* */
  uint32_t spectrum_n;      /* > 0: FILE spectrum of spectrum_n rows (spectrum.c:182-274), else FLAT */
  double param[4];
  const double *spectrum_energy;   /* HOST arrays: energy (keV, non-decreasing) and flux density */
  const double *spectrum_flux;
  uint32_t image_nx, image_ny;     /* IMAGE: NAXIS1, NAXIS2 */
  const float *image;              /* HOST array, row-major (NAXIS2 rows of NAXIS1 pixels) */
} mx_source;
enum { MX_SOURCE_POINT = 0, MX_SOURCE_GAUSS = 1, MX_SOURCE_BETA = 2, MX_SOURCE_DISK = 3, MX_SOURCE_LINE = 4,
       MX_SOURCE_IMAGE = 5 };

/* DitherModel = FILE (init_aspsol_dither and get_single_aspsol_point,
 * dither.c:282-500): the rows of the aspect solution's ASPSOL table, n x 7
 * row-major (time (s), ra, dec, roll (deg), dy, dz (mm), dtheta (deg)) in
 * the file's order, with its RA_NOM, DEC_NOM, ROLL_NOM (deg) and TSTART (s)
 * keywords.  Each row is converted as the reference converts it (ra, dec
 * rolled into offsets from the nominal pointing; times relative to TSTART,
 * the first row's taken off twice as init_aspsol_dither does) and the table
 * kept on the device for the configuration's dither stage, which must be
 * MX_DITHER_FILE.  A photon at time t (start_time + arrival time) takes the
 * linear interpolation between the last row at or before t and the next one
 * (get_aspsol_dither, :350-371); the detector stages move the detector by
 * that row's dy, dz, dtheta (_marx_dither_detector, detector.c:275-284).
 * record_only: the rays are already dithered (_MARX_DITHER_RECORD_ONLY):
 * the state is recorded and the aspect blur applied, the pointing not moved.
 * The configuration's ra_nom, dec_nom and roll_nom should carry the file's
 * keywords, as init_aspsol_dither overrides the parameter file's.  n = 0
 * removes the table.  Times must not decrease along the photon list for the
 * result to equal the reference's forward-only reader. */
int mx_set_aspect_solution(mx_context *ctx, const double *rows, uint32_t n, double ra_nom, double dec_nom,
                           double roll_nom, double tstart, int record_only);

/* USER sources (marx/libsrc/s-user.c): a plug-in shared object exporting
 * user_open_source(argv, argc, area, px, py, pz), user_create_ray(&t,
 * &energy, &p1, &p2, &p3), user_close_source() and optionally
 * user_start_iteration().  Host-side, as in the reference.
 *
 * mx_user_source_open: marx_select_user_source + open_source (s-user.c:
 * 158-167, 250-300): dlopen `file`, split `args` (UserSourceArgs) at blanks
 * into argv and call user_open_source with the mirror's geometric area
 * (cm^2) and the source direction p.  NULL on failure (mx_user_source_error). */
typedef struct mx_user_source mx_user_source;
mx_user_source *mx_user_source_open(const char *file, const char *args, double geometric_area, const double p[3]);
/* create_photons (s-user.c:168-232) over a HOST list: host->energy holds
 * the spectrum's draws on entry; per photon user_create_ray gets the draw
 * and may replace it (a negative energy keeps the draw); p is the ray's,
 * flags 0, and while the plug-in hands back t >= 0 the arrival time is the
 * running sum of those t (times_set = 1; otherwise arrival times are left to
 * the caller, as the reference leaves them to marx_create_photons).  Stops at
 * the first ray the plug-in refuses; user_start_iteration returning -1 gives
 * no photons.  *n_created = photons made. */
int mx_user_source_create(mx_user_source *src, const mx_photons *host, uint32_t n, uint32_t *n_created,
                          int *times_set);
/* close_source: user_close_source, then the plug-in is unloaded. */
void mx_user_source_close(mx_user_source *src);
const char *mx_user_source_error(void);

/* The direction of travel p of the photons of a source at (ra, dec)
 * (degrees) for the configuration's pointing (RA_Nom, Dec_Nom, Roll_Nom,
 * PointingOffsetY/Z): setup_pointing_ra_dec (dither.c:125-155),
 * marx_compute_elaz (source.c:108-134) and select_source (source.c:136-232).
 * MX_EINVAL if the source lies behind the telescope. */
int mx_source_direction(const mx_config *cfg, double ra, double dec, double p[3]);

/* Fill energy, p, arrival_time, flags and tag of dev (device pointers,
 * dev->n = src->num_photons) with the source's photons. */
int mx_generate_source(mx_context *ctx, const mx_source *src, uint32_t first_tag, uint64_t seed,
                       const mx_photons *dev, void *stream);

/* ------------------------------------------------------------ batches --
 * Many sources of uneven size traced in ONE persistent cooperative kernel
 * launch (generation, dither, mirror, per-source grating and detector),
 * replayed from a captured CUDA graph.  Source s owns photons
 * [start[s], start[s+1]) of the batch's output list, tagged by their
 * index in it.  The kernel's block size, work-tile size and resident
 * blocks per SM are chosen by mx_batch_tune (timed trials, remembered per
 * source-table and configuration hash for the life of the process). */
typedef struct mx_batch mx_batch;
typedef struct mx_batch_params {
  int32_t block;            /* threads per block: 32 to 256 in whole warps */
  int32_t tile;             /* photons a warp claims per visit of the work counter (multiple of 32) */
  int32_t blocks_per_sm;    /* resident blocks per SM (<= the occupancy limit) */
  int32_t reserved;
} mx_batch_params;

mx_batch *mx_batch_create(mx_context *ctx, const mx_source *sources, int nsrc);
int  mx_batch_set_params(mx_batch *b, const mx_batch_params *params);
int  mx_batch_get_params(const mx_batch *b, mx_batch_params *params);
/* Time candidate parameter sets (each run `trials` times) and keep the
 * fastest; *best receives it.  A second call for an identical batch and
 * configuration returns the remembered choice without timing. */
int  mx_batch_tune(mx_batch *b, int trials, mx_batch_params *best);
/* One graph launch: the whole batch, generation to detection. */
int  mx_batch_run(mx_batch *b, uint64_t seed, void *stream);
/* The same photons traced source by source with the plain entry points
 * (mx_generate_source + mx_trace per source): the comparison baseline. */
int  mx_batch_run_sequential(mx_batch *b, uint64_t seed, void *stream);
/* Device views of the batch's photon list and the host array of nsrc + 1
 * source offsets. */
int  mx_batch_photons(mx_batch *b, mx_photons *dev_view, const uint32_t **source_start);
uint64_t mx_batch_total_photons(const mx_batch *b);
void mx_batch_destroy(mx_batch *b);

/* ----------------------------------------------- differentiable form --
 * Weighted rays: each ray takes the aperture point the mirror stage would
 * give a photon of the same tag (project_photon_to_hrma, hrma.c:984-1050)
 * and the HRMA geometry of the trace, without normal blur or scattering,
 * to the focal plane x = 0.  Instead of random absorption it carries a
 * weight: HRMAVig times, at each reflection, the Fresnel reflectivity
 * (reflect.c:39-77) times the shell's effective-area correction (1 with
 * HRMA_Ideal).  The image is the weighted rays splatted with a normalised
 * Gaussian of sigma pixels, truncated at 5 pixels, divided by n_rays.
 * No counterpart in the reference; its parameters are the ones the
 * reference reads from HRMA_Geometry_File (read_hrma_geometry_file,
 * hrma.c:319-391) and the source direction.
 *
 * theta[MX_DIFF_NPARAM] perturbs the configured model:
 *   theta[4 s + 0]  shell s az_mis   (arcsec, added to P and H rows)
 *   theta[4 s + 1]  shell s el_mis   (arcsec, added to P and H rows)
 *   theta[4 s + 2]  shell s x0       (micrometres, added to P and H rows)
 *   theta[4 s + 3]  shell s y0       (micrometres, added to P and H rows)
 *   theta[16], theta[17]  source offset in y and z (arcsec)
 * with shells s = 0..3 in the order 1, 3, 4, 6.  The source direction is
 * unit(-1, -tan(ay), -tan(az)), ay = src_y + theta[16] and
 * az = src_z + theta[17] in arcsec.
 *
 * Which root each conic gives, whether the ray hits both optics and
 * whether a strut blocks it are discrete.  MX_DIFF_RECORD decides them
 * afresh and keeps them per ray; MX_DIFF_REPLAY follows the kept decisions
 * (without the x-limit and strut tests), so the image is smooth in theta;
 * MX_DIFF_FRESH decides afresh without keeping them.  The adjoint
 * differentiates the replayed function at theta and needs a recorded set. */
#define MX_DIFF_NPARAM 18
#define MX_DIFF_RECORD 0
#define MX_DIFF_REPLAY 1
#define MX_DIFF_FRESH  2
#define MX_DIFF_MAX_RAYS 4294967295ull

typedef struct mx_diff_config {
  uint64_t n_rays;          /* rays per evaluation, tags 0 .. n_rays-1 */
  uint64_t seed;            /* Philox key of the aperture points */
  double energy;            /* keV, every ray */
  double src_y, src_z;      /* source direction before theta[16..17], arcsec */
  double center_y, center_z;/* focal-plane position of the image centre, mm */
  double pitch;             /* pixel size, mm */
  double sigma;             /* splat width in pixels, 0.5 .. 1 */
  uint32_t nx, ny;          /* image columns (focal-plane y) and rows (z), 16 .. 4096 */
} mx_diff_config;

typedef struct mx_diff mx_diff;

/* Weighted rays over the context's mirror model (its MirrorType must be
 * HRMA with a source at infinity).  NULL on error (mx_last_error(ctx)). */
mx_diff *mx_diff_create(mx_context *ctx, const mx_diff_config *cfg);
/* The image at theta into image (device, ny x nx doubles, row-major,
 * row = z).  moments (host, may be NULL) receives sum w, sum w y,
 * sum w z and the number of rays reaching the focal plane; with moments
 * the call waits for the stream. */
int mx_diff_forward(mx_diff *d, const double *theta, int mode, double *image, double *moments, void *stream);
/* Per-ray focal-plane y, z (mm) and weight w into yzw (device, 3 x n_rays,
 * column-major: y[0..n), z[0..n), w[0..n)); lost rays get w = 0. */
int mx_diff_rays(mx_diff *d, const double *theta, int mode, double *yzw, void *stream);
/* Mean squared difference of two images (device) into *loss (device) and,
 * when dl_dimage is not NULL, its gradient 2 (image - target) / (nx ny). */
int mx_diff_mse(mx_diff *d, const double *image, const double *target, double *dl_dimage, double *loss,
                void *stream);
/* The adjoint: grad (host, MX_DIFF_NPARAM) = sum over pixels of
 * dl_dimage (device) times d image / d theta at theta, through the
 * decisions of the last MX_DIFF_RECORD call.  Waits for the stream. */
int mx_diff_adjoint(mx_diff *d, const double *theta, const double *dl_dimage, double *grad, void *stream);
/* Device-side form of mx_diff_adjoint: grad_dev is a device array of
 * MX_DIFF_NPARAM doubles; does not wait. */
int mx_diff_adjoint_async(mx_diff *d, const double *theta, const double *dl_dimage, double *grad_dev,
                          void *stream);
void mx_diff_destroy(mx_diff *d);

/* Survivor compaction (marx_prune_photons, photon.c:40): writes the indices
 * of photons without MX_BAD_PHOTON_MASK bits to idx_out (device, n entries)
 * in ascending order and their count to *count_out (host). */
int mx_compact(mx_context *ctx, const uint32_t *flags, uint32_t n,
               uint32_t *idx_out, uint32_t *count_out, void *stream);

/* Device table summary, for tests: number of bytes staged per block in
 * shared memory and resident in global memory. */
int mx_table_bytes(const mx_context *ctx, size_t *shared_bytes, size_t *global_bytes);

/* Number of kernel launches issued by this context since creation. */
uint64_t mx_launch_count(const mx_context *ctx);

/* The context's own stream (a cudaStream_t), on which mx_trace_host runs. */
void *mx_stream(mx_context *ctx);

/* Photons flagged MX_PHOTON_VARIATE_OVERRUN since the last reset. */
int mx_overrun_count(mx_context *ctx, unsigned long long *count, int reset);

/* ------------------------------------------------------------- runs --
 * marx's main loop (marx/src/marx.c:545-608) on the GPU: the parameter
 * file par_path (marx.par format) with "Name=value" overrides configures
 * the engine and the run, as the marx program reads them: SourceType
 * (POINT, GAUSS, BETA, DISK, LINE) with SourceRA, SourceDEC,
 * SourceDistance and the model's S-* parameters, or SAOSAC with
 * SAOSACFile (mx_saosac_*: rays past the mirror, traced from the grating
 * on; a file without RT_TIME gives zero times and clears the rays'
 * vignetting flags, as marx_create_photons does for it); SpectrumType FLAT
 * (MinEnergy, MaxEnergy) or FILE (SpectrumFile) with SourceFlux; NumRays
 * (photons to create, or with a minus sign to detect) in batches of
 * dNumRays, or ExposureTime (s) when positive; RandomSeed (-1: from the
 * clock); OutputDir, OutputVectors, DumpToRayFile and RayFile.  Each batch
 * is created on the device (energies and directions of the source model,
 * Poisson arrival times with mean 1 / (SourceFlux x the mirror's open
 * area), tags from 0 on), traced through every stage and written to
 * OutputDir (mx_write_photons), or with DumpToRayFile = yes dithered and
 * written to RayFile (mx_write_rayfile); OutputDir then receives marx.par
 * (the parameter file with the overrides) and obs.par (the detector's
 * observation template from the table pack with the run's pointing,
 * detector, grating and times), as marx leaves them for marx2fits.
 * Results are statistically, not photon for photon, those of the
 * reference's marx: its generator differs. */
typedef struct mx_run_stats {
  uint64_t collected;      /* photons created */
  uint64_t detected;       /* photons written (no MX_BAD_PHOTON_MASK bit) */
  double total_time;       /* simulated exposure (s) */
  uint32_t iterations;     /* batches */
  uint32_t reserved;
} mx_run_stats;
int mx_run_marx(const char *pack_path, const char *par_path, const char *const *overrides, int n_overrides,
                mx_run_stats *stats);

/* ------------------------------------------------------------ output --
 * MARX's output directory format (marx_write_photons, marxio.c:395-478):
 * one big-endian column file per attribute (xpos.dat, energy.dat,
 * detector.dat, ...), rows for the photons without a MX_BAD_PHOTON_MASK
 * bit.  history holds the MX_OUT_* bits of the columns the stages made
 * valid (the reference's Marx_Photon_Type.history); write_mask the columns
 * wanted (marx.par OutputVectors); with dither != 0 the dither-state
 * columns are written whenever asked for.  append != 0 adds rows to the
 * files already in dir.  The list is in HOST memory.  Bit values as
 * marx.h:128-147. */
#define MX_OUT_ENERGY      0x00000001u
#define MX_OUT_TIME        0x00000002u
#define MX_OUT_X           0x00000004u
#define MX_OUT_P           0x00000008u
#define MX_OUT_TAG         0x00000010u
#define MX_OUT_PHA         0x00000020u
#define MX_OUT_PI          0x00000040u
#define MX_OUT_DET_PIXEL   0x00000080u
#define MX_OUT_DET_NUM     0x00000100u
#define MX_OUT_DET_REGION  0x00000200u
#define MX_OUT_DET_UV      0x00000400u
#define MX_OUT_SHELL       0x00000800u
#define MX_OUT_SKY_DITHER  0x00001000u
#define MX_OUT_DET_DITHER  0x00002000u
#define MX_OUT_ORDER       0x00100000u
#define MX_OUT_ORDER1      0x00200000u
#define MX_OUT_ORDER2      0x00400000u
#define MX_OUT_ORDER3      0x00800000u
#define MX_OUT_ORDER4      0x01000000u
int mx_write_photons(const mx_photons *host, uint32_t history, uint32_t write_mask, int dither, const char *dir,
                     int append, double total_time);
const char *mx_write_error(void);   /* message of the last mx_write_photons failure (this thread) */
/* The history bits a trace of cfg through `stages` makes valid, as the
 * reference's stages set them. */
uint32_t mx_output_history(const mx_config *cfg, uint32_t stages);

/* The SAOSAC source (s-saosac.c:95-345): rays of an SAO raytrace of the
 * mirror from the RAYTRACE binary table of a FITS file (RT_X, RT_Y, RT_Z,
 * RT_COSX, RT_COSY, RT_COSZ, RT_KEV, RT_WGHT and an optional RT_TIME;
 * scalar E or D columns).  mx_saosac_read makes up to max photons from the next rows,
 * as saosac_create_photons does: each row draws one uniform against its
 * weight (MX_PHOTON_MIRROR_VBLOCKED when u >= RT_WGHT), its ray is projected
 * to the plane x = 0 of the file's frame and placed at x = hrma_cap_x -
 * 0.01675 mm, its shell follows from the radius there, its energy is
 * RT_KEV; times are RT_TIME minus the first row's, relative to the end of
 * the batch before (without RT_TIME: 1, 2, 3, ... per batch).  A row whose
 * time falls before the start is dropped and its blocked flag passes to
 * the next photon, as in the reference.  u: one uniform per row of the
 * file, indexed by row (NULL: the Philox source draw 0 of tag = row under
 * seed).  Photons get tags first_tag, first_tag + 1, ...; written into HOST
 * columns energy, x, p (required), arrival_time, flags, mirror_shell, tag.
 * Trace them with stages MX_STAGE_DITHER | MX_STAGE_GRATING |
 * MX_STAGE_DETECT: the rays have passed the mirror.  Errors: NULL or
 * MX_EINVAL, reason in mx_last_error(NULL). */
typedef struct mx_saosac mx_saosac;
mx_saosac *mx_saosac_open(const char *file, double hrma_cap_x);
int mx_saosac_read(mx_saosac *s, const mx_photons *host, uint32_t max, const double *u, uint64_t seed,
                   uint32_t first_tag, uint32_t *n_read);
uint64_t mx_saosac_rows(const mx_saosac *s);
int mx_saosac_has_time(const mx_saosac *s);   /* 1 when the table has RT_TIME */
void mx_saosac_close(mx_saosac *s);

/* MARX ray files (DumpToRayFile and the RAYFILE source, s-rayfile.c):
 * a native-endian unsigned long magic 0xF8161961 and the history bits, then
 * one Marx_Photon_Attr_Type record (marx.h:51-100, 136 bytes on LP64
 * hosts) per photon.  mx_write_rayfile writes the photons without a
 * MX_BAD_PHOTON_MASK bit with total_time added to their arrival times
 * (marx_dump_to_rayfile, s-rayfile.c:109-155; the list itself is not
 * changed); append != 0 adds records to an existing file.  mx_read_rayfile
 * reads up to max records from byte *offset (0: from the start, after
 * checking the header) into the host columns that are not NULL, subtracts
 * *last_time from the arrival times and leaves there the last record's
 * time, as rayfile_create_photons does (s-rayfile.c:188-219); *offset
 * advances past what was read and *n_read is 0 at the end of the file.
 * Host memory. */
int mx_write_rayfile(const mx_photons *host, uint64_t history, const char *file, int append, double total_time);
int mx_read_rayfile(const char *file, mx_photons *host, uint32_t max, uint64_t *offset, double *last_time,
                    uint64_t *history, uint32_t *n_read);

/* ------------------------------------------------ event coordinates --
 * The per-event columns marx2fits derives from an output directory
 * (marx/src/marx2fits.c), for the context's detector:
 *   CHIPX, CHIPY   xpixel + 1 in single precision (read_float32_add_1, :3460)
 *   EXPNO          ACIS frame number (compute_expno, :3741)
 *   FLTGRADE,GRADE ACIS sub-pixel grade draw (compute_fltgrade, :3854;
 *                  compute_grade, :3813)
 *   DETX, DETY     focal-plane pixel (compute_detxy, :3676, through
 *                  marx_init_chip_to_mnc / marx_chip_to_mnc, pixlib.c:135-222,
 *                  and marx_mnc_to_fpc, detpix.c:182)
 *   X, Y           sky pixel (compute_xy_sky, :3869; marx_undither_mnc,
 *                  dither.c:703; marx_mnc_to_ra_dec and
 *                  marx_compute_ra_dec_offsets, pixlib.c:499-570)
 *   TDETX, TDETY   tiled detector pixel (compute_tdetxy, :3584)
 * On an ACIS run every event of one frame uses the dither state of the
 * frame's first event unless the pixel adjustment is EXACT
 * (read_dither_value, :3567).  Pixel adjustments as marx2fits --pixadj
 * (:3240-3275); EDSER takes the sub-pixel offsets of the ACIS subpix CALDB
 * file (marx_compute_acis_subpix, acis_subpix.c:284) and means RANDOMIZE
 * on an HRC, as in marx2fits. */
#define MX_PIXADJ_EDSER      0
#define MX_PIXADJ_RANDOMIZE  1
#define MX_PIXADJ_NONE       2
#define MX_PIXADJ_EXACT      3

typedef struct mx_event_params {
  double focal_length;     /* marx.par FocalLength (mm) */
  double det_offset[3];    /* marx.par DetOffsetX, DetOffsetY, DetOffsetZ (mm) */
  double roll_nom;         /* obs.par Roll_Nom (degrees): the sky rotation of an undithered run */
  double frame_time;       /* ACIS frame period: ACIS_Exposure_Time plus ACIS_Frame_Transfer_Time
                              when both are > 0; <= 0: every event is a frame of its own */
  double time_offset;      /* added to time64 before its single-precision rounding */
  int32_t dithered;        /* the run used a dither model (DitherModel != NONE) */
  int32_t pixel_adjust;    /* MX_PIXADJ_* */
} mx_event_params;

typedef struct mx_events {
  uint32_t n;              /* events */
  uint32_t reserved;
  const uint32_t *index;   /* event k reads row index[k] of the input columns; NULL: row k */
  /* inputs: the columns of an output directory (all device memory) */
  const int8_t *ccd_id;    /* detector.dat: chip / facet id */
  const float *xpixel, *ypixel;               /* xpixel.dat, ypixel.dat: 0-based chip pixels */
  const float *time;       /* time.dat; NULL: time64[row] + time_offset, rounded to single precision */
  const double *time64;
  const float *sky_ra, *sky_dec, *sky_roll;   /* dither state (radians); NULL reads 0 */
  const float *det_dy, *det_dz, *det_theta;   /* detector motion (mm, mm, radians); NULL reads 0 */
  const float *b_energy;   /* b_energy.dat (keV) for EDSER; NULL reads 0 */
  const double *uniforms;  /* [3][n] per event, slot-major: grade draw, x and y randomisation;
                              NULL: Philox4x32-10 keyed by seed */
  /* outputs, one per event (device memory); NULL columns are skipped */
  float *chipx, *chipy;
  double *detx, *dety, *x, *y;
  int32_t *tdetx, *tdety, *expno;             /* expno: ACIS only, 0 on an HRC */
  int16_t *fltgrade, *grade;                  /* ACIS only, 0 on an HRC */
} mx_events;

/* Events whose chip id is not a facet of the detector, or whose ray has no
 * focal-plane position, get NaN coordinates and count as bad
 * (mx_event_bad_count); marx2fits stops at the first such event. */
int mx_event_coords(mx_context *ctx, const mx_event_params *params, const mx_events *ev, uint64_t seed,
                    void *stream);
/* The same with every column in HOST memory; copies inside, synchronous.
 * Returns MX_EINVAL when an event was bad. */
int mx_event_coords_host(mx_context *ctx, const mx_event_params *params, const mx_events *host_ev,
                         uint64_t seed);
int mx_event_bad_count(mx_context *ctx, unsigned long long *count, int reset);

/* Measured FP64 fused-multiply-add throughput of the current device
 * (TFLOP/s), the denominator of the trace kernels' roofline. */
int mx_probe_fp64(double *tflops, double *ms);

/* The engine's own arithmetic helpers evaluated on the current device, for
 * tests that hold them to their stated error bounds (no counterpart in the
 * reference).  x and y are device pointers; n values in, n results out
 * (2n for fn 1):
 *   fn 0  y = 1/x by Newton-Raphson from a float seed (within one ulp)
 *   fn 1  y[2i], y[2i+1] = sin(pi x), cos(pi x) in double-float (within 2^-44)
 *   fn 2  y = x rounded to the nearest float (as the cast rounds it)
 *   fn 3  y = (float) sin(x), as the cast of the double sine rounds it
 *   fn 4  y = x truncated toward zero to float
 *   fn 5  x holds n triples (cos of the grazing angle, beta, delta), y gets
 *         n quadruples: the Fresnel numerator and denominator of the mirror
 *         reflectivity in double-float, then in double precision
 *   fn 6  y = (double) (unsigned) x, 0 <= x < 2^32, on the integer pipe
 *   fn 7  y = sqrt(x) from the reciprocal square root (within two ulps)
 *   fn 8  y = (unsigned) (4 x), 0 <= x < 1, from the bits of x
 * Synchronises the device.  MX_EINVAL for an unknown fn or null pointers. */
int mx_math_check(int fn, const double *x, double *y, size_t n);

#ifdef __cplusplus
}
#endif
#endif /* MARX_GB300_H */
