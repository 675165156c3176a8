// Device-side model tables, derived on the host from the table pack and an
// mx_config (see mx_host.cpp) and read by the trace kernels.
#pragma once
#include <stdint.h>
#include "../../include/marx_gb300.h"

#define MX_FOLD_MAX 256      // WFold arrays per table (the HRMA tables hold 200)
#define MX_FOLD_THETA 208    // angles per WFold array (the HRMA tables hold 201)
#define MX_MAX_CHIPS 14       // ACIS ids 0-9, then HRC-I (id 0) and HRC-S (ids 1-3)
#define MX_MAX_SECTORS 64
#define MX_MAX_GRATINGS 8     // HETG shells 1,3,4,6 then LETG shells 1,3,4,6

// One HRMA shell: both optics (index 0 = paraboloid P, 1 = hyperboloid H).
struct MxShellDev {
  double a[2], b[2], c[2], xmin[2], xmax[2];   // conic x^2+r^2 = a x^2 + b x + c, x-limits (hrma.c:555-575)
  double to_osac[2][3];                        // MARX -> OSAC translation (hrma.c:590-599)
  double fwd[2][9], bwd[2][9];                 // pitch/yaw matrices (hrma.c:842-897)
  double front_position, area_fraction, min_radius, max_radius;
  double blur[2];                              // normal blur sigma (rad)
  double scat[2];                              // WFold scattering factor
  int32_t corr_off, corr_n;                    // correction-factor table (floats after the optical constants)
  uint32_t shutter;                            // open-quadrant bitmap
  int32_t corr_slope_off;                      // its interval slopes in optc_slope
  double front_fwd[3];                         // fwd[0] (front_position + to_osac[0][0], 0, 0)
  double am1[2], hb[2];                        // a - 1 and b / 2 (the conic's normal)
  double dr;                                   // max_radius - min_radius
  // paraboloid frame -> MARX frame -> hyperboloid frame as one change:
  // x' = mid x + mid_off, p' = mid p (mid = fwd[1] bwd[0], mid_off =
  // fwd[1] (to_osac[1] - to_osac[0]))
  double mid[9], mid_off[3];
  float bwd0f[9], osac0f[3];                   // bwd[0] and to_osac[0] in float (the cap struts' screen)
  // Padding to 736 bytes (184 words): the four shells' copies in shared
  // memory start on banks 0, 24, 16 and 8, so lanes of a warp that load
  // one field of different shells do not conflict (at 704 bytes shells 0
  // and 2, and 1 and 3, shared their banks).
  double bank_pad[4];
};
static_assert(sizeof(MxShellDev) % 128 == 96, "shell records of 736 + 128 k bytes: four distinct bank offsets");

// One HETG grating (per mirror shell, diffract.c:51-77).
struct MxGratingDev {
  double vig, rowland, theta_blur, dp_over_p;
  double cos_m, sin_m, cos_p, sin_p;           // rotation by -/+ dispersion angle
  int32_t geff_off, cum_off, nenergy, norders; // cumulative efficiencies [energy][order]
  int32_t max_order, order_off, sec_off, nsec; // order_k offset; sectors [6][nsec]
  int32_t monotone, pad;                       // every energy row non-decreasing in the order index
};

// One LETG support grating as the trace meets it (diffract.c:1097-1114):
// the fine grating once at 90 degrees, the coarse grating at 60, 120 and 0.
struct MxSupportDev {
  int32_t cum_off, norders;    // cumulative efficiencies [energy][order] on the shared energy grid
  int32_t order_off, rotate;   // order constants in support_k; rotate: the angle is not zero
  double cos_t, sin_t;         // cos and sin of the angle
  int32_t monotone, pad;       // every energy row non-decreasing in the order index
};

// A float table lookup (JDMinterpolate_f) in the HRC tables: abscissae at
// hrc_tab + x_off, ordinates at hrc_tab + y_off, interval slopes at
// hrc_slope + s_off; n = 0 means a perfect efficiency (no table).
struct MxTabDev {
  int32_t x_off, y_off, s_off, n;
};

// One Drake-flat plate section (drake.c:48-58, 188-230).
struct MxPlateDev {
  double a[3], e1[3], e2[3], normal[3];
  double len1, len2;
};

// The configured HRC (hrc-i.c, hrc-s.c, hrc_i_geom.c, hrc_s_geom.c,
// hrcblur.c, drake.c), everything the detector stage reads.
struct MxHrcDev {
  int32_t kind;                 // MX_DETECTOR_HRC_I or MX_DETECTOR_HRC_S
  int32_t blur;                 // position blur on (not DetIdeal)
  // pixel mapping: HRC-I y = ll_cxcy + d / size; HRC-S per MCP (facets ids 1..3)
  double ll_cxcy[2], pix[2], inv_pix[2];       // HRC-I pixel sizes, HRC-S U and V sizes
  double u_active0, v_active0[3], uv0[3][2], cxcy0[3][2];
  // efficiencies: MCP per facet (HRC-S: facet id k uses MCP region map[k]), filter per region
  MxTabDev mcp[3], filt[4];
  // HRC-S UV/ion shield (hrc-s.c:119-185, 410-418)
  double shield_yc, shield_zc, shield_t, shield_l, shield_r, shield_sl, shield_sr, shield_sl_gap, shield_sr_gap,
      shield_x;
  // position blur (hrcblur.c:105-188), mm, centred on the first gaussian
  double g1_sigma, g1_w, g2_sigma, g2_x, g2_y, g2_w, l1_hwhm, l1_x, l1_y, l1_rmax, l1_w;
  // Drake flat (HRC-S): 2 x plates sections, carbon and chromium constants
  int32_t drake_n, pad;
  double drake_cr_width;
  MxPlateDev plates[8];
  MxTabDev c_beta, c_delta, cr_beta, cr_delta;
};

// One region of the ACIS FEF (acis_fef.c Fef_Type): n_e energies and
// channels at fef_f + e_off (energies, then channels), n_g gaussians per
// energy at fef_f + g_off as (amp, center, sigma) triples [energy][gaussian],
// the channel-to-energy interpolation slopes at fef_slope + s_off.
#define MX_FEF_GAUSSIANS 6   // gaussians per FEF row the device pass holds
#define MX_CONTAM_LAYERS 5   // MAX_LAYERS of aciscontam.c

// One chip's QE and contamination (aciscontam.c Single_Component_Contam_Type)
// for the ACIS response with DetIdeal = no.  Tables index fef_f/fef_slope.
struct MxContamDev {
  int32_t nl, mode, blk, pad;   // layers; spatial term: 0 ACIS-I radial (x0, y0), 1 ACIS-S power law, 2 fxy map
  double x0, y0;
  double tau0[MX_CONTAM_LAYERS], tau1[MX_CONTAM_LAYERS];
  MxTabDev mu[MX_CONTAM_LAYERS];    // energy -> mu per layer
  int32_t fxy_off[MX_CONTAM_LAYERS], pad2[3];
  MxTabDev qe;                      // energy -> QE (the CALDB ACIS QE)
};
struct MxFefDev {
  int32_t e_off, n_e, g_off, n_g;
  int32_t s_off, pad[3];
};

struct MxChipDev {
  double x_ll[3], xhat[3], yhat[3], normal[3];
  double xlen, ylen, xpix, ypix, xoff, yoff;
  double inv_xpix, inv_ypix;                   // correctly rounded 1/xpix, 1/ypix
  float f_ll[3], f_xhat[3], f_yhat[3], f_normal[3], f_xlen, f_ylen;   // single-precision screen copies
  int32_t id, pad;
  // Padding to 232 bytes (58 words): up to ten chips' copies in shared
  // memory start on distinct even banks, so lanes of a warp on different
  // chips do not conflict (at 224 bytes chips k and k + 4 shared banks).
  double bank_pad;
};
static_assert(sizeof(MxChipDev) == 232, "chip records of 58 words: distinct bank offsets for ten chips");

// Everything the kernels read, passed by value as a launch parameter.
struct MxTables {
  // device pointers
  const MxShellDev *shells;
  const float *optc;            // [beta-table energies | beta | delta | corr(E,f) per shell]
  int32_t optc_len;             // floats in optc
  int32_t opt_n;                // rows of the optical-constant table (0: perfect reflector)
  const double *optc_slope;     // per-interval slopes of beta, delta and each correction table
  int32_t slope_len;            // doubles in optc_slope
  int32_t pad_slope;
  const double *fold_hdr;       // [8][MX_FOLD_MAX][8]: e_alpha p_min delta_p p_max norm expon num 1/delta_p
  const double *fold_inv_de;    // [8][MX_FOLD_MAX]: 1 / (e_alpha[k+1] - e_alpha[k])
  const double *fold_ealpha;    // [8][MX_FOLD_MAX]
  const float *fold_theta;      // [8][MX_FOLD_MAX][MX_FOLD_THETA]
  uint32_t fold_num[8];         // table index = 2 * shell + optic
  const MxGratingDev *gratings;
  const float *geff_energy;
  const float *geff_cum;
  const double *order_k;        // order * (2 pi hbar c) / period, per grating and order
  const double *sectors;
  const MxChipDev *chips;
  // LETG support gratings
  MxSupportDev supports[4];
  const float *support_energy;  // the grating energy grid (marx_create_grating_opt_const_tables)
  const float *support_cum;     // [energy][order] per support grating
  const double *support_k;      // order * (2 pi hbar c) / period per support grating and order
  int32_t support_nenergy, pad_support;
  // mirror
  int32_t ideal, use_blur, use_wfold, use_struts, use_scale, area_uniform;
  double hrma_vig, source_distance, cap, cos30, sin30;
  double strut_xpos[3][2], strut_half_width[3][2];
  float strut_xf[3][2], strut_hwf[3][2], cos30f, sin30f;   // cap + strut_xpos and half widths in float
  // dither
  int32_t dither, grating;      // grating: MX_GRATING_* of the configuration
  double dith_amp[3], dith_period[3], dith_phase[3], nominal_roll, aspect_blur, start_time;
  double dith_inv_period[3];    // correctly rounded 1 / dith_period
  int32_t dith_amp_exp[3];      // dith_amp <= 2^dith_amp_exp (sine_to_float)
  float roll_f;                 // (float) nominal_roll, the roll of every photon when roll_fixed
  int32_t roll_fixed, roll_zero;// roll amplitude 0: the roll angle is the same for every photon (zero: no roll)
  double roll_cos, roll_sin;    // cos and sin of -(float) nominal_roll, when roll_fixed
  // DitherModel FILE (mx_set_aspect_solution): rows 0 .. asp_n of the
  // aspect solution, row 0 the zero state the reference's reader starts from
  int32_t dither_file, asp_record_only;
  const double *asp_t;          // [asp_n + 1] times (s, relative to TSTART)
  const double *asp_v;          // [asp_n + 1][8]: ra, dec, roll (rad), dy, dz (mm), dtheta (rad), 0, 0
  uint32_t asp_n, pad_asp;
  // detector
  int32_t nchips, det_extend;   // configured detector's chips: chips[chip_off .. chip_off + nchips)
  int32_t chip_off, pad_chip;
  double det_offset[3], frame_transfer, frame_time, exposure, focal_length;
  double inv_frame_time;
  int32_t det_kind, det_ideal;  // MX_DETECTOR_* of the configuration, DetIdeal
  // HRC tables (global memory) and parameters
  const float *hrc_tab;
  const double *hrc_slope;
  MxHrcDev hrc;
  // ACIS FEF pulse heights (acis_fef.c): 32 x 32 pixel cells of ccds 0..9 ->
  // region index (-1: none), the regions and their tables
  const int32_t *fef_map;
  const MxFefDev *fef;
  const float *fef_f;
  const double *fef_slope;
  int32_t acis_fef, fef_nregions;
  // ACIS QE x contamination acceptance (DetIdeal = no and contamination tables present)
  const MxContamDev *contam;        // [10] by chip id
  int32_t acis_qe, pad_qe;
};
