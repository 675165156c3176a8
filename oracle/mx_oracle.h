/* CPU restatement of the MARX photon trace (the oracle).  Test
 * infrastructure only: the tests, the smoke check and the bench's CPU
 * baseline call it as the checker; the product never links it.
 *
 * It follows the reference functions line by line (citations in
 * mx_oracle_core.hpp) in plain scalar double arithmetic, compiled without
 * fused multiply-add, one photon at a time.  Variates come either from
 * pre-drawn per-photon slot arrays (same layout as the engine, see
 * include/marx_gb300.h) or from the engine's Philox4x32-10 streams. */
#ifndef MX_ORACLE_H
#define MX_ORACLE_H
#include <stdint.h>
#include "../include/marx_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mxo_model mxo_model;

mxo_model *mxo_create(const char *pack_path, const mx_config *cfg);
void mxo_destroy(mxo_model *m);
const char *mxo_last_error(void);

/* Trace n photons in place (host SoA, same meaning as mx_photons).  U/N are
 * slot-major pre-drawn variates or NULL for Philox(seed, tag).  nthreads <=
 * 0 uses every hardware thread.  Returns the number of photons whose stage
 * ran out of slots, or a negative error. */
int mxo_trace(const mxo_model *m, const mx_photons *ph, uint32_t stages,
              const double *U, const double *N, uint64_t seed, int nthreads);

/* Same trace through the flop-counting arithmetic type; returns the FP64
 * operation counts summed over the photons (add/sub/mul/div/sqrt/compare
 * are 1, libm calls 1 each) in counts[0] and the number of photons that
 * ran in counts[1]. */
int mxo_count_flops(const mxo_model *m, const mx_photons *ph, uint32_t stages,
                    uint64_t seed, double *counts);

/* Chip facets as derived for the configured detector: per chip id, x_ll[3],
 * xhat[3], yhat[3], normal[3], xlen, ylen, xpix, ypix, xoff, yoff, 0. */
int mxo_detector_geometry(const mxo_model *m, double *out, int max_chips);

/* Philox variates as the engine defines them, for tests. */
double mxo_philox_uniform(uint64_t seed, uint32_t tag, uint32_t slot);
double mxo_philox_normal(uint64_t seed, uint32_t tag, uint32_t slot);
/* Photon-generation draw k of photon `tag` (energies of point sources). */
double mxo_source_uniform(uint64_t seed, uint32_t tag, uint32_t k);

/* Weighted rays of the differentiable form (mx_diff_config) at theta,
 * decisions made afresh: per-ray focal-plane y, z and weight into yzw
 * (3 x n_rays, lost rays NaN, NaN, 0; may be NULL) and the splatted image
 * into image (ny x nx; may be NULL). */
int mxo_weighted(const mxo_model *m, const mx_diff_config *cfg, const double *theta, double *yzw,
                 double *image, int nthreads);
/* FP64 operations of the weighted rays (counting arithmetic, as
 * mxo_count_flops): counts[0] operations, counts[1] rays, counts[2] rays
 * that reached the focal plane. */
int mxo_weighted_flops(const mxo_model *m, const mx_diff_config *cfg, const double *theta, double *counts);
/* The splat's single-precision exp(-x). */
float mxo_splat_exp(float x);

#ifdef __cplusplus
}
#endif
#endif
