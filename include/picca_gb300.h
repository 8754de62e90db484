/*
 * picca_gb300 C ABI: GPU (sm_103a) pair accumulation for the Lyman-alpha
 * auto-correlation (picca.cf) and delta x quasar cross-correlation
 * (picca.xcf).
 *
 * Conventions
 *  - Every pointer inside pg_forest_set / pg_xi_rows and every array argument
 *    is a DEVICE pointer allocated by the caller (e.g. PyTorch); the library
 *    only owns the small scratch buffer of a pg_plan.
 *  - Every call is stream-ordered on `stream` (a cudaStream_t passed as
 *    void*, NULL = legacy default stream) and returns a status code: 0 on
 *    success, a negative PG_ERR_* value otherwise (pg_strerror). No call
 *    aborts the process and no kernel traps: device-side problems (bin index
 *    out of range, bounded waits that expire) are written to a status word
 *    that pg_plan_stats reads back.
 *  - A plan is not thread-safe; use one plan per host thread / stream.
 *
 * Reference interfaces replaced (picca v9.21.0):
 *  - pg_cf_neighbours   <- cf.fill_neighs            py/picca/cf.py:82-135
 *  - pg_xcf_neighbours  <- xcf.fill_neighs           py/picca/xcf.py:71-123
 *  - pg_cf_xi           <- cf.compute_xi + cf.compute_xi_forest_pairs_fast
 *                          py/picca/cf.py:138-247, :250-387
 *  - pg_xcf_xi          <- xcf.compute_xi + xcf.compute_xi_forest_pairs_fast
 *                          py/picca/xcf.py:126-220, :223-322
 *  - pg_corr_params     <- the cf / xcf module globals set by
 *                          py/picca/bin/picca_cf.py:343-368 and
 *                          py/picca/bin/picca_xcf.py:351-373
 */
#ifndef PICCA_GB300_H
#define PICCA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_OK 0
#define PG_ERR_INVALID_ARGUMENT (-1)
#define PG_ERR_CUDA (-2)
#define PG_ERR_TIMEOUT (-3)
#define PG_ERR_BIN_RANGE (-4)
#define PG_ERR_NO_MEMORY (-5)
#define PG_ERR_UNSUPPORTED (-6)
#define PG_ERR_NO_DEVICE (-7)

/* pg_cf_xi / pg_xcf_xi arithmetic modes */
#define PG_MODE_FP64 0       /* all geometry and sums in FP64 (plain form)   */
#define PG_MODE_FP32_GUARD 1 /* FP32 geometry, FP64 re-decision of pairs near
                                a bin edge, FP32 block sums (xi compensated)
                                merged into FP64 rows (precision form)       */

/* Binning and cuts: the module globals of picca.cf / picca.xcf. NaN disables
 * z_min_pairs, z_max_pairs and the (zerr_cut_deg, zerr_cut_kms) cut. */
typedef struct pg_corr_params {
    double r_par_min, r_par_max, r_trans_max;
    int32_t num_bins_r_par, num_bins_r_trans;
    double z_min_pairs, z_max_pairs;
    double zerr_cut_deg, zerr_cut_kms;
    double ang_max;
    int32_t x_correlation;                      /* cf: signed r_par (two fields or --unfold-cf) */
    int32_t rmu_binning;
    int32_t ang_correlation;
    int32_t remove_same_half_plate_close_pairs;
} pg_corr_params;

/* A set of lines of sight (structure of arrays, device memory).
 * Forests: pixels of forest f are [pix_offset[f], pix_offset[f+1]) of the
 * pixel arrays (zero-weight pixels may be dropped by the caller: the
 * reference skips them). r_first / r_last are the comoving distances of the
 * first and last pixel before any dropping (xcf pre-cut, xcf.py:117-121).
 * Quasar sets: num pixels = 0 and obj_* hold the per-object values. */
typedef struct pg_forest_set {
    int64_t num;
    int64_t num_pixels;                                       /* pix_offset[num] */
    const int64_t *pix_offset;                                /* [num+1]  */
    const double *z, *r_comov, *dist_m, *weights, *delta;     /* [pixels] */
    const double *ra, *dec, *x_cart, *y_cart, *z_cart, *cos_dec, *z_qso;  /* [num] */
    const double *r_first, *r_last;                           /* [num]    */
    const double *obj_r_comov, *obj_dist_m, *obj_weight;      /* [num]    */
    const int64_t *thingid, *plate, *fiberid;                 /* [num]    */
    const int32_t *row;                                       /* [num] output row */
    int32_t num_rows;
    int32_t max_pixels;   /* upper bound of pix_offset[f+1]-pix_offset[f]; forests
                             longer than this are skipped and reported        */
} pg_forest_set;

/* Per-row (healpix) raw sums, [num_rows * num_bins] each, ACCUMULATED into
 * (the caller zeroes them): sum of w, delta-products, r_par*w, r_trans*w,
 * z*w and pair counts, before the division by the weights of
 * cf.py:242-246. */
typedef struct pg_xi_rows {
    double *weights, *xi, *r_par, *r_trans, *z;
    int64_t *num_pairs;
} pg_xi_rows;

/* Statistics of the last pg_cf_xi / pg_xcf_xi call on a plan. */
typedef struct pg_run_stats {
    int32_t status;             /* PG_OK or the first device-side error       */
    int32_t error_detail;       /* e.g. offending bin index                   */
    int64_t rechecked_pairs;    /* FP32_GUARD: pairs re-decided in FP64       */
    int64_t recheck_overflows;  /* FP32_GUARD: early recheck-queue drains     */
    int64_t work_items;         /* work items processed                        */
} pg_run_stats;

typedef struct pg_plan pg_plan;

const char *pg_strerror(int status);
int pg_version(void);

/* Create a plan on the CURRENT device (allocates a few hundred bytes of
 * device scratch) / release it. */
int pg_plan_create(pg_plan **plan);
int pg_plan_destroy(pg_plan *plan);

/* Synchronise the plan's last stream and read its statistics. */
int pg_plan_stats(pg_plan *plan, pg_run_stats *stats);

/* Neighbour lists of every forest of s1 against s2 (s2 == NULL: auto-
 * correlation of s1 with itself, keeping ra1 > ra2 as cf.py:129-135).
 * Two passes: with offsets == NULL write counts[s1->num]; then, with the
 * caller's exclusive prefix sum `offsets` ([s1->num + 1]), write the
 * neighbour indices into index[offsets[f] ..]. Neighbours are listed in
 * increasing index order of s2. */
int pg_cf_neighbours(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
                     const pg_forest_set *s2, int64_t *counts, const int64_t *offsets,
                     int32_t *index, void *stream);

/* Quasar neighbours of forests (angle, thingid, zerr and r_comov pre-cuts
 * of xcf.fill_neighs), same two-pass protocol. */
int pg_xcf_neighbours(pg_plan *plan, const pg_corr_params *params,
                      const pg_forest_set *forests, const pg_forest_set *objs,
                      int64_t *counts, const int64_t *offsets, int32_t *index, void *stream);

/* Accumulate the pair sums of forests s1[work_order[k]] (k < num_work; NULL
 * work_order: 0..num_work-1) with their neighbours in s2 (NULL: s1) into
 * rows out[s1->row[f]]. nbr_angle (optional, parallel to nbr_index) gives
 * the angular separation of each listed pair; NULL computes it from the unit
 * vectors as QSO.get_angle_between does. mode = PG_MODE_FP64 or
 * PG_MODE_FP32_GUARD. */
int pg_cf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
             const pg_forest_set *s2, const int64_t *nbr_offsets, const int32_t *nbr_index,
             const double *nbr_angle, const int32_t *work_order, int64_t num_work,
             int32_t mode, const pg_xi_rows *out, void *stream);

/* Delta x quasar version of pg_cf_xi. */
int pg_xcf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *forests,
              const pg_forest_set *objs, const int64_t *nbr_offsets, const int32_t *nbr_index,
              const double *nbr_angle, const int32_t *work_order, int64_t num_work,
              int32_t mode, const pg_xi_rows *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PICCA_GB300_H */
