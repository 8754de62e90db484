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
 *  - pg_cf_neighbours_grouped / pg_xcf_neighbours_grouped <- the same, with
 *                          the query_disc candidate healpix (cf.py:105-122,
 *                          xcf.py:92-101) as groups of the sorted sets
 *  - pg_cf_xi           <- cf.compute_xi + cf.compute_xi_forest_pairs_fast
 *                          py/picca/cf.py:138-247, :250-387
 *  - pg_xcf_xi          <- xcf.compute_xi + xcf.compute_xi_forest_pairs_fast
 *                          py/picca/xcf.py:126-220, :223-322
 *  - pg_cf_dmat         <- cf.compute_dmat + cf.compute_dmat_forest_pairs_fast
 *                          py/picca/cf.py:390-517, :519-887
 *  - pg_xcf_dmat        <- xcf.compute_dmat + xcf.compute_dmat_forest_pairs_fast
 *                          py/picca/xcf.py:325-424, :427-675
 *  - pg_cf_metal_dmat   <- cf.compute_metal_dmat  py/picca/cf.py:890-1218
 *  - pg_xcf_metal_dmat  <- xcf.compute_metal_dmat py/picca/xcf.py:677-800
 *  - pg_wick_xi_matrices, pg_cf_wick
 *                       <- cf.compute_wick_terms + cf.compute_wickT123_pairs
 *                          py/picca/cf.py:1328-1495, :1498-1626
 *  - pg_xcf_wick, pg_xcf_wick_factored
 *                       <- xcf.compute_wick_terms + xcf.compute_wickT1234_pairs
 *                          py/picca/xcf.py:838-1008, :1220-1351
 *  - pg_read_delta_file <- io.read_delta_file + Delta.from_fitsio / from_image
 *                          py/picca/io.py:333-380, py/picca/data.py:376-620
 *  - pg_project_deltas  <- Delta.project            py/picca/data.py:622-655
 *  - pg_fast_metal_dmat <- calc_fast_metal_dmat of
 *                          py/picca/bin/picca_fast_metal_dmat.py:30-251 and
 *                          py/picca/bin/picca_fast_metal_xdmat.py:28-215
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
    int64_t work_items;         /* work items processed; pg_cont_fit_select in
                                   PG_FIT_MIXED: forests finished in two-float */
    int64_t gemm_macs;          /* pg_cf_dmat: multiply-adds of the per-pair
                                   products of the eta terms               */
    int64_t visited_pairs;      /* FP32_GUARD cf: lane steps of the diagonal
                                   sweeps (pixel pairs evaluated, idle lanes
                                   included)                                   */
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

/* Launch shapes of the precision-form pair kernels on this plan (no
 * counterpart in the reference): warps per CTA and CTAs per SM (each CTA
 * keeps its own shared-memory histogram, so CTAs per SM is the number of
 * histogram replicas on an SM). 0 selects the default: the most warps the
 * shared memory allows (20 for pg_cf_xi, 16 for pg_xcf_xi) and as many CTAs
 * as fit. The results do not depend on the shape beyond the summation order
 * of the FP32-compensated sums (the pair counts are identical). The
 * no-allocation entry pg_cf_xi_static always uses the default. */
typedef struct pg_tuning {
    int32_t cf_warps, cf_blocks_per_sm;
    int32_t xcf_warps, xcf_blocks_per_sm;
} pg_tuning;
int pg_plan_set_tuning(pg_plan *plan, const pg_tuning *tuning);
int pg_plan_get_tuning(pg_plan *plan, pg_tuning *tuning);

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

/* Groups of two forest sets for the grouped neighbour search (the
 * healpix-by-healpix candidate selection of cf.fill_neighs, cf.py:105-122,
 * which asks healpy.query_disc for the healpix near each forest). The
 * query set's objects are grouped into consecutive ranges; blocks
 * [block_first[b], block_end[b]) (at most 256 queries each) all belong to
 * group block_group[b] and every query belongs to exactly one block. The
 * other set's group g holds objects [start2[g], start2[g+1]) (start2
 * non-decreasing). cand_groups[cand_offsets[G] .. cand_offsets[G+1]) lists,
 * in increasing order, every group of the other set that can hold a
 * neighbour of a query of group G (a superset is fine: each object is still
 * tested exactly). All arrays are device pointers. */
typedef struct pg_nbr_groups {
    int32_t num_groups1, num_groups2, num_blocks, reserved;
    const int64_t *start2;        /* [num_groups2 + 1] */
    const int32_t *cand_offsets;  /* [num_groups1 + 1] */
    const int32_t *cand_groups;   /* [cand_offsets[num_groups1]] */
    const int32_t *block_group;   /* [num_blocks] */
    const int64_t *block_first;   /* [num_blocks] */
    const int64_t *block_end;     /* [num_blocks] */
} pg_nbr_groups;

/* pg_cf_neighbours / pg_xcf_neighbours restricted to candidate groups (same
 * protocol, same results and order when the groups cover every neighbour). */
int pg_cf_neighbours_grouped(pg_plan *plan, const pg_corr_params *params,
                             const pg_forest_set *s1, const pg_forest_set *s2,
                             const pg_nbr_groups *groups, int64_t *counts,
                             const int64_t *offsets, int32_t *index, void *stream);
int pg_xcf_neighbours_grouped(pg_plan *plan, const pg_corr_params *params,
                              const pg_forest_set *forests, const pg_forest_set *objs,
                              const pg_nbr_groups *groups, int64_t *counts,
                              const int64_t *offsets, int32_t *index, void *stream);

/* Accumulate the pair sums of forests s1[work_order[k]] (k < num_work; NULL
 * work_order: 0..num_work-1) with their neighbours in s2 (NULL: s1) into
 * rows out[s1->row[f]]. nbr_angle (optional, parallel to nbr_index) gives
 * the angular separation of each listed pair; NULL computes it from the unit
 * vectors as QSO.get_angle_between does. mode = PG_MODE_FP64 or
 * PG_MODE_FP32_GUARD; the precision form covers the (r_par, r_trans) bins
 * with every cut and the r-mu bins without the z-pair, zerr and half-plate
 * cuts; the angular binning and r-mu with those cuts run in FP64 in either
 * mode. */
int pg_cf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
             const pg_forest_set *s2, const int64_t *nbr_offsets, const int32_t *nbr_index,
             const double *nbr_angle, const int32_t *work_order, int64_t num_work,
             int32_t mode, const pg_xi_rows *out, void *stream);

/* Delta x quasar version of pg_cf_xi. */
int pg_xcf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *forests,
              const pg_forest_set *objs, const int64_t *nbr_offsets, const int32_t *nbr_index,
              const double *nbr_angle, const int32_t *work_order, int64_t num_work,
              int32_t mode, const pg_xi_rows *out, void *stream);

/* pg_cf_xi for callers that cannot allocate device memory. No counterpart
 * in the reference. Some callers cannot call cudaMalloc (a framework owns
 * the device allocator, or every buffer is sized at start-up), and a
 * pg_plan allocates its scratch. This variant needs no plan: the scratch
 * lives in a library-owned device array of PG_STATIC_SCRATCH_BYTES bytes
 * (held by every GPU that loads the library until exit). All calls on a
 * device share that array: calls that overlap on the GPU race and give
 * wrong results. The first call with a device current looks up the
 * array's address (once per device). The call is synchronous: it
 * synchronises `stream` and copies the kernel's device-side status back
 * with a blocking cudaMemcpy, so it must not be called while `stream` (or
 * any stream) is being captured into a CUDA graph. Returns that status;
 * PG_ERR_UNSUPPORTED if the scratch would not fit in the array. */
#define PG_STATIC_SCRATCH_BYTES 4096
int pg_cf_xi_static(const pg_corr_params *params, const pg_forest_set *s1,
                    const pg_forest_set *s2, const int64_t *nbr_offsets,
                    const int32_t *nbr_index, const double *nbr_angle,
                    const int32_t *work_order, int64_t num_work, int32_t mode,
                    const pg_xi_rows *out, void *stream);

/* ------------------------------------------------------------------------ */
/* Dr16 continuum fit                                                        */
/* ------------------------------------------------------------------------ */
/* Reference interfaces replaced (picca v9.21.0):
 *  - pg_cont_fit_batch  <- expected_fluxes/utils.py:12-136 compute_continuum
 *                          with least_squares_cont_model.py:65-197 (chi2 of
 *                          the (zero_point, slope) continuum model), run for
 *                          every forest (dr16_expected_flux.py:389-425)
 *  - pg_cont_stacks     <- expected_flux.py:256-308 _compute_mean_cont,
 *                          least_squares_var_stats.py:134-198
 *                          initialize_delta_arrays, expected_flux.py:190-236
 *                          compute_delta_stack (bin sums; normalisation and
 *                          the 20 variance fits stay on the host)
 *  - pg_cont_deltas     <- dr16_expected_flux.py:706-740 populate_los_ids +
 *                          expected_flux.py:328-349 extract_deltas
 * All paths under delta_extraction/ are relative to py/picca. */

/* Raw forests (device pointers): pixels of forest f are
 * [pix_offset[f], pix_offset[f+1]). */
typedef struct pg_spectra {
    int64_t num;
    int64_t num_pixels;
    const int64_t *pix_offset;
    const double *log_lambda, *flux, *ivar, *transmission_correction;
    const double *z_qso;
} pg_spectra;

/* Current model of the Dr16 iteration (device pointers).
 * Mean continuum: linear interpolation with extrapolation on
 * (mean_cont_x, mean_cont_y), num_mean_cont points (rest-frame log lambda).
 * eta, var_lss, fudge: piecewise cubics on var_breaks[0..num_var_intervals]
 * with coefficients coef[k*num_var_intervals + i], k = 0..3 highest power
 * first (the polynomial form of scipy's not-a-knot cubic interp1d),
 * extrapolated with the end pieces. Stack of deltas: nearest-point lookup
 * on stack_x (num_stack points); NULL means 1. */
typedef struct pg_cont_model {
    int32_t num_mean_cont;
    const double *mean_cont_x, *mean_cont_y;
    int32_t num_var_intervals;
    const double *var_breaks, *eta_coef, *var_lss_coef, *fudge_coef;
    int32_t num_stack;
    const double *stack_x, *stack_y;
    double log_lambda_rest_min, log_lambda_rest_max;  /* rest-frame grid ends */
    double var_lss_mod;
    int32_t order;                /* 0: slope fixed at 0; 1: free slope */
    int32_t use_constant_weight;
} pg_cont_model;

/* Per-forest fit results (device pointers, [num]); continuum is per pixel
 * ([num_pixels], may be NULL). status: 0 ok, 1 not converged, 2 negative
 * continuum, 3 zero continuum (the bad_continuum_reason values of
 * compute_continuum). */
typedef struct pg_cont_fit {
    double *zero_point, *slope, *chi2;
    int32_t *ndata, *status, *iterations;
    double *continuum;
} pg_cont_fit;

/* Histograms of one Dr16 iteration (device pointers, ACCUMULATED into;
 * NULL skips a group): rest-frame mean continuum (mean_cont_num,
 * mean_cont_weight, [rest_bins]), variance statistics (var_mean, var_delta2,
 * var_delta4, var_npix, var_nqso, [20 * 100] = wavelength x log var_pipe
 * bins), observed-frame stack (stack_num, stack_weight, [obs_bins]). */
typedef struct pg_cont_stacks {
    int32_t rest_bins;
    double rest_grid0, rest_step;
    double *mean_cont_num, *mean_cont_weight;
    int32_t var_lambda_bins;
    double var_grid0, var_step;
    double *var_mean, *var_delta2, *var_delta4, *var_npix, *var_nqso;
    int32_t obs_bins;
    double obs_grid0, obs_step;
    double *stack_num, *stack_weight;
    /* 0: grids evenly spaced in log10(lambda), grid0 / step in log10
     * Angstrom (find_bins_log); 1: evenly spaced in lambda, grid0 = lambda of
     * the first node and step in Angstrom (find_bins_lin, bin of 10**x),
     * delta_extraction/utils.py:139-186 */
    int32_t wave_lin;
} pg_cont_stacks;

#define PG_FIT_FP64 0        /* per-pixel chi2 terms in FP64                   */
#define PG_FIT_MIXED 1       /* per-pixel terms in FP32 (FP64 inputs converted
                                on the integer pipe), exact-product FP32 2x2
                                Newton solves, a two-float finish where FP32
                                rounding could move the optimum          */

/* Fit (zero_point, slope) of every forest by damped Newton iterations on the
 * chi2 of the continuum model. start (optional, [2*num], device) gives a
 * warm start (zero_point, slope) per forest; NULL starts from the
 * ivar-weighted mean flux and slope 0 (utils.py:92-94). Iterations stop
 * when the step is below tol * max(1, |a|, |b|) or after max_iter. With a
 * start and max_iter == 0 nothing is fitted: the continuum, chi2 and status
 * are evaluated at the given (zero_point, slope). */
int pg_cont_fit_batch(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                const double *start, int32_t max_iter, double tol, int32_t mode,
                const pg_cont_fit *out, void *stream);

/* pg_cont_fit_batch restricted to the forests forest_index[0..num_index)
 * (device, int32; NULL with num_index = spectra->num: every forest). Results
 * are written at each listed forest's position; the others are untouched.
 * Used for the fallback fits of the learned warm start. In PG_FIT_MIXED the
 * per-pixel terms are FP32, the iteration stops at a step below
 * max(tol, 1e-6) * max(1, |a|, |b|), and the continuum is formed in FP32.
 * A converged mixed fit whose optimum the FP32 rounding of the gradient is
 * estimated to move by more than 2e-6 * max(1, |a|, |b|) (a forest whose
 * pixels barely separate a from b) is finished in the same call by Newton
 * steps with two-float per-pixel terms and gradient (FP64 accuracy without
 * the FP64 pipe) until the step is below 1e-11 * max(1, |a|, |b|);
 * pg_plan_stats' work_items counts those forests. */
int pg_cont_fit_select(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                       const double *start, const int32_t *forest_index, int64_t num_index,
                       int32_t max_iter, double tol, int32_t mode, const pg_cont_fit *out,
                       void *stream);

/* The learned warm start's fit (no counterpart in the reference): Newton
 * iterations with FP32 per-pixel terms from start[2*f..] (required), ended
 * by a certificate instead of a step size. Once a Newton step d = -H^-1 g of
 * chi2 is at most sqrt(ab_tol) * max(1, |a|, |b|) (the error after it is of
 * order |d|^2), the step is taken and the new point is certified with its
 * gradient g' and the last Hessian: the remaining step H^-1 g' at most
 * ab_tol * max(1, |a|, |b|) and half the Newton decrement g'.H^-1 g' / 2 (the
 * excess of chi2 over the minimum of its quadratic model) at most
 * chi2_tol * max(|chi2|, ndata). Forests not certified within max_iter get
 * status 1 (the caller re-fits them with the plain fit). No FP64 finish;
 * forests longer than 224 pixels are fitted to convergence in FP64. */
int pg_cont_fit_warm(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                     const double *start, const int32_t *forest_index, int64_t num_index,
                     int32_t max_iter, double chi2_tol, double ab_tol, const pg_cont_fit *out,
                     void *stream);

/* Accumulate the histograms of one Dr16 iteration from fitted continua
 * (forests with status != 0 are skipped, as bad_continuum_reason is). */
int pg_cont_stacks_accumulate(pg_plan *plan, const pg_spectra *spectra,
                              const pg_cont_model *model, const pg_cont_fit *fit,
                              const pg_cont_stacks *stacks, void *stream);

/* Final deltas and weights per pixel: expected flux = continuum * stack,
 * weights of compute_forest_weights, delta = flux / expected - 1 where the
 * weight is positive (0 elsewhere). Forests with status != 0 get weight 0. */
int pg_cont_deltas(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                   const pg_cont_fit *fit, double *delta, double *weights, void *stream);

/* ------------------------------------------------------------------------ */
/* Learned warm start for the continuum fit. No counterpart in the           */
/* reference: kernels of a small MLP (BF16 tensor-core GEMM with FP32        */
/* accumulation, bias-gradient column sums, MSE gradient, Adam).            */
/* All pointers are device pointers; bf16 values are passed as uint16_t.     */
/* ------------------------------------------------------------------------ */
#define PG_MLP_EPI_NONE 0
#define PG_MLP_EPI_GELU 1        /* out = gelu(acc + bias)                     */
#define PG_MLP_EPI_GELU_GRAD 2   /* out = (acc + bias) * gelu'(zin)            */

/* C[m, n] = A[m, k] B[k, n] with element strides A(i, l) = a[i*sam + l*sak],
 * B(l, j) = b[l*sbk + j*sbn]; optional bias[n], epilogue, pre-activation
 * output zout / input zin ([m, ldz] FP32), bf16 output c and/or FP32 output
 * cf ([m, ldc]; cf = result + beta * cf). */
int pg_mlp_gemm(const uint16_t *a, int64_t sam, int64_t sak, const uint16_t *b, int64_t sbk,
                int64_t sbn, int32_t m, int32_t n, int32_t k, const float *bias, int32_t epilogue,
                const float *zin, float *zout, int64_t ldz, uint16_t *c, float *cf, int64_t ldc,
                float beta, void *stream);

/* out[j] = sum_i x[i, j] for a bf16 [m, ldx] matrix. */
int pg_mlp_colsum(const uint16_t *x, int32_t m, int32_t n, int64_t ldx, float *out,
                  void *stream);

/* dy = 2 (y - t) / m as bf16 ([m, n]); loss += sum (y - t)^2 / m if loss. */
int pg_mlp_mse_grad(const float *y, const float *t, int32_t m, int32_t n, uint16_t *dy,
                    float *loss, void *stream);

/* One Adam step on n FP32 parameters (bias-corrected, optional decoupled
 * weight decay); writes the bf16 copy when params_bf16 is not NULL. */
int pg_mlp_adam(float *params, const float *grads, float *m1, float *m2, uint16_t *params_bf16,
                int64_t n, float lr, float beta1, float beta2, float eps, int32_t step,
                float weight_decay, void *stream);

/* bf16 copy of an FP32 array. */
int pg_mlp_to_bf16(const float *x, uint16_t *y, int64_t n, void *stream);

/* Inference forward pass of the warm-start network (no counterpart in the
 * reference) as one fused kernel on the 5th-generation tensor cores:
 * tcgen05.mma BF16 x BF16 -> FP32 with the accumulator in tensor memory,
 * 128 forests per tile through all four layers on one SM (bias + GELU
 * epilogues in FP32, hidden activations rounded to BF16 as in
 * pg_mlp_gemm's forward). pg_mlp_pack writes the BF16 weights of the
 * 66-256-256-256-2 network (params16: per layer W [fan_in][fan_out] then the
 * bias, as pg_mlp_to_bf16 makes them) into the operand image the kernel
 * copies to shared memory (pg_mlp_packed_elems() bf16 elements, 16-byte
 * aligned); pg_mlp_forward reads x [m, stride] bf16 (stride >= 80, a
 * multiple of 8, columns 66..79 zero), the FP32 biases from params and
 * writes y [m, 2] FP32. */
int64_t pg_mlp_packed_elems(void);
int pg_mlp_pack(const uint16_t *params16, uint16_t *packed, void *stream);
int pg_mlp_forward(pg_plan *plan, const uint16_t *packed, const float *params, const uint16_t *x,
                   int64_t m, int32_t stride, float *y, void *stream);

/* pg_mlp_features and pg_mlp_forward in one kernel (no counterpart in the
 * reference): each tile's features are formed from the spectra and the
 * current model straight into the tensor-core operand in shared memory
 * (the same values pg_mlp_features writes), then the network runs on them;
 * writes y [num, 2] FP32 and a0 [num] FP64. Measured slower than the two
 * calls (3.2 ms against 1.1 + 0.5 ms for 400k forests on a GB300): the
 * feature pass is memory-latency bound and gets only the 16 warps per SM
 * that the network's 192 KB of operand buffers leave room for. */
int pg_mlp_warm_start(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                      const uint16_t *packed, const float *params, float *y, double *a0,
                      void *stream);

/* Per-forest input features of the warm-start network: 64 bins of
 * flux / mean continuum over the rest-frame range (ivar-weighted means,
 * divided by the forest's ivar-weighted mean flux a0, minus 1; empty bins
 * 0), (z_qso - 3), and log of the mean flux*sqrt(ivar); features[f *
 * feat_stride + j] as bf16 (columns 66..feat_stride-1 zeroed); a0[f] FP64. */
int pg_mlp_features(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                    uint16_t *features, int32_t feat_stride, double *a0, void *stream);

/* ---------------------------------------------------------------------
 * Distortion matrix (py/picca/cf.py:390-887, py/picca/bin/picca_dmat.py)
 * --------------------------------------------------------------------- */

/* The model binning and redshift evolution of the distortion matrix (the cf
 * module globals num_model_bins_r_par / _r_trans,
 * redshift_evolution_in_distortion_matrix, z_ref, alpha, alpha2 set by
 * py/picca/bin/picca_dmat.py:366-400). */
#define PG_DMAT_FP64 0        /* eta products in FP64 on the CUDA cores          */
#define PG_DMAT_SPLIT_BF16 1  /* eta products on the BF16 tensor cores: rows scaled
                                 by powers of two, 48-bit fixed point split into
                                 six 8-bit digits, exact digit products and
                                 integer level sums (error below 2^-46 of the
                                 largest |row| x |column| product)            */
typedef struct pg_dmat_params {
    int32_t num_model_bins_r_par, num_model_bins_r_trans;
    int32_t redshift_evolution;
    int32_t row_capacity;  /* data + model bins of one forest pair held at once
                              (0: 512); more are processed in chunks        */
    int32_t product;       /* PG_DMAT_FP64 or PG_DMAT_SPLIT_BF16             */
    int32_t reserved;
    double z_ref, alpha, alpha2;
} pg_dmat_params;

/* Raw sums of the distortion matrix, ACCUMULATED into (the caller zeroes
 * them), before the normalisation of py/picca/bin/picca_dmat.py:487-525:
 * weights_dmat [nb], dmat [nb * nm] (dmat[data_bin * nm + model_bin]),
 * r_par_eff, r_trans_eff, z_eff, weight_eff [nm]; nb = num_bins_r_par *
 * num_bins_r_trans, nm = num_model_bins_r_par * num_model_bins_r_trans. */
typedef struct pg_dmat_sums {
    double *weights_dmat, *dmat;
    double *r_par_eff, *r_trans_eff, *z_eff, *weight_eff;
} pg_dmat_sums;

/* Device work-buffer size (bytes) pg_cf_dmat wants for forests of at most
 * max_pixels1 / max_pixels2 pixels: one slice per CTA of the persistent
 * kernel, for every resident CTA or at most max_ctas of them (max_ctas > 0;
 * pass the number of forest pairs for small runs). A smaller buffer runs
 * fewer CTAs; PG_ERR_UNSUPPORTED if the forests do not fit in shared
 * memory. */
int pg_cf_dmat_work_bytes(pg_plan *plan, const pg_corr_params *params,
                          const pg_dmat_params *dparams, int32_t max_pixels1,
                          int32_t max_pixels2, int64_t max_ctas, uint64_t *bytes);

/* Distortion matrix of the selected forest pairs (pair_first[q] of s1,
 * pair_second[q] of s2; s2 = NULL for the auto-correlation, when s1 and its
 * log_lambda / order arrays serve both sides). The pair selection (the
 * random rejection of cf.compute_dmat) is the caller's. log_lambda* are
 * pixel arrays aligned with the sets, order* per-forest polynomial orders (0
 * or 1, Delta.order). pair_angle (optional, [num_pairs]) overrides the
 * angles computed from the sets' unit vectors. Every pixel pair adds the
 * reference's eta terms; sums are FP64 and reassociated with respect to the
 * reference (agreement to a few ulp of the summed magnitudes). work is a
 * device buffer of work_bytes (pg_cf_dmat_work_bytes). rmu_binning,
 * x_correlation and the zerr / z cuts follow the reference;
 * ang_correlation is PG_ERR_UNSUPPORTED (the reference has no angular
 * distortion matrix). */
int pg_cf_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
               const pg_forest_set *s1, const pg_forest_set *s2, const double *log_lambda1,
               const double *log_lambda2, const int32_t *order1, const int32_t *order2,
               const int32_t *pair_first, const int32_t *pair_second, const double *pair_angle,
               int64_t num_pairs, void *work, uint64_t work_bytes, const pg_dmat_sums *out,
               void *stream);

/* Metal distortion matrix (py/picca/cf.py:890-1218,
 * py/picca/bin/picca_metal_dmat.py). The pixels of a set seen as absorber
 * abs: distances and redshift at z_abs = 10^log_lambda / lambda_abs - 1,
 * zfac = (1 + z_abs)^(alpha_abs - 1), and the pixel weight where z_abs is
 * below the forest's quasar redshift, 0 elsewhere; arrays aligned with the
 * set's pixel arrays. */
typedef struct pg_metal_pixels {
    const double *r_comov, *dist_m, *z, *zfac, *weights;
} pg_metal_pixels;

/* One pass of cf.compute_metal_dmat over the kept forest pairs
 * (pair_first[q] of s1, pair_second[q] of s2; s2 NULL: auto): forest 1 seen
 * as absorber abs1 (a1), forest 2 as abs2 (a2). zevol_den = (1 +
 * z_ref)^(alpha_abs1 + alpha_abs2 - 2). The reference's swapped pass for two
 * different absorbers is a second call with a1 / a2 built for abs2 / abs1.
 * Sums are ACCUMULATED into out (FP64, the reference's un-normalised
 * tuples). */
int pg_cf_metal_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                     double zevol_den, const pg_forest_set *s1, const pg_forest_set *s2,
                     const pg_metal_pixels *a1, const pg_metal_pixels *a2,
                     const int32_t *pair_first, const int32_t *pair_second,
                     const double *pair_angle, int64_t num_pairs, const pg_dmat_sums *out,
                     void *stream);

/* xcf.compute_metal_dmat (py/picca/xcf.py:677-800): the same pass with the
 * quasars as one-pixel forests (quasar_pixels: a set whose pixel k is
 * quasar k: r_comov, dist_m, weights and z the quasar's), a2 the quasars'
 * values with zfac = 1, a1 the forests' pixels seen as the absorber with
 * zfac = ((1 + z_abs) / (1 + z_ref))^(alpha_abs - 1) and zevol_den = 1.
 * r_par is signed; pairs are kept by the reference's strict distance tests
 * (r_par_min < r_par < r_par_max, r_trans < r_trans_max) for both bins. */
int pg_xcf_metal_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                      double zevol_den, const pg_forest_set *forests,
                      const pg_forest_set *quasar_pixels, const pg_metal_pixels *a1,
                      const pg_metal_pixels *a2, const int32_t *pair_first,
                      const int32_t *pair_second, const double *pair_angle, int64_t num_pairs,
                      const pg_dmat_sums *out, void *stream);

/* Wick covariance of the auto-correlation, terms T1-T3
 * (py/picca/cf.py:1328-1626, py/picca/bin/picca_wick.py). */

/* Weighted 1D correlation matrix of each listed forest of `set`,
 * X[i][k] = ((w_k w_i) xi) sqrt(v_k v_i) with xi = xi_values[m], m the
 * number of xi_bounds below |log_lambda_k - log_lambda_i| (scipy's
 * nearest-neighbour rule; xi_bounds[num_xi - 1] are the cell bounds of the
 * num_xi tabulated offsets), and v the per-pixel 1D variance. Forest
 * forests[q] is written row-major at arena + x_offsets[forests[q]]
 * (n_f^2 doubles). The diagonal is written as 0 (no Wick term uses it). */
int pg_wick_xi_matrices(pg_plan *plan, const pg_forest_set *set, const double *log_lambda,
                        const double *variance, const double *xi_bounds,
                        const double *xi_values, int32_t num_xi, const int32_t *forests,
                        int64_t num_forests, const int64_t *x_offsets, double *arena,
                        void *stream);

/* Sums of cf.compute_wick_terms / xcf.compute_wick_terms (device,
 * ACCUMULATED into): weights_wick and num_pairs_wick [nb], t1 .. t4
 * [nb * nb] (t1 only on its diagonal; t4 only for the cross, may be NULL
 * for pg_cf_wick), nb = num_bins_r_par * num_bins_r_trans. */
typedef struct pg_wick_sums {
    double *weights_wick;
    int64_t *num_pairs_wick;
    double *t1, *t2, *t3, *t4;
} pg_wick_sums;

/* Terms T1-T3 of the forest pairs (pair_first[q] of s1, pair_second[q] of
 * s2): zw1 / zw2 the per-pixel ((1 + z) / (1 + z_ref))^(alpha - 1) of each
 * side, x_offsets / arena the matrices of pg_wick_xi_matrices. Uses
 * params->r_par_min / r_par_max / r_trans_max / num_bins_* / x_correlation
 * (the Wick pixel-pair range keeps r_par_min <= r_par < r_par_max,
 * r_trans < r_trans_max). A costly pair may be listed several times as
 * slices: entry q then does slice unit_slice[q] of unit_slices[q] (both
 * optional: NULL = one slice per entry); every slice of a pair must be
 * listed exactly once. work: pg_cf_wick_work_bytes() bytes of device
 * scratch (16-byte aligned); fewer bytes run fewer CTAs. Forests must have
 * at most 32767 pixels. */
int pg_cf_wick_work_bytes(pg_plan *plan, const pg_corr_params *params, int32_t max_pixels1,
                          int32_t max_pixels2, int64_t max_ctas, uint64_t *bytes);
int pg_cf_wick(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
               const pg_forest_set *s2, const double *zw1, const double *zw2,
               const int64_t *x_offsets1, const double *arena1, const int64_t *x_offsets2,
               const double *arena2, const int32_t *pair_first, const int32_t *pair_second,
               const double *pair_angle, const int32_t *unit_slice, const int32_t *unit_slices,
               int64_t num_pairs, void *work, uint64_t work_bytes, const pg_wick_sums *out,
               void *stream);

/* Terms T1-T4 of the delta x quasar Wick covariance. A work item q is
 * forest item_forest[q] of `forests` with its neighbouring quasars
 * obj_index[item_start[q] .. item_start[q] + item_count[q]) of `objs`
 * (obj_angle, optional and aligned with obj_index, overrides the angles
 * from the unit vectors). zw1: per pixel of `forests`
 * ((1 + z) / (1 + z_ref))^(alpha - 1); zw_obj: per object
 * ((1 + z_qso) / (1 + z_ref))^(alpha_obj - 1); the objects' weights and
 * comoving distances are objs->obj_weight / obj_r_comov. r_par is signed and
 * a pair is kept when r_par_min <= r_par < r_par_max, r_trans <
 * r_trans_max. unit_slice / unit_slices cut costly items into slices as
 * for pg_cf_wick. work: pg_xcf_wick_work_bytes() bytes (16-byte aligned)
 * for forests of at most max_pixels pixels (at most 32767) and items of at
 * most max_quasars quasars (at most 65535). */
int pg_xcf_wick_work_bytes(pg_plan *plan, const pg_corr_params *params, int32_t max_pixels,
                           int32_t max_quasars, int64_t max_ctas, uint64_t *bytes);
int pg_xcf_wick(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *forests,
                const pg_forest_set *objs, const double *zw1, const double *zw_obj,
                const int64_t *x_offsets, const double *arena, const int32_t *item_forest,
                const int32_t *item_start, const int32_t *item_count, const int32_t *obj_index,
                const double *obj_angle, const int32_t *unit_slice, const int32_t *unit_slices,
                int64_t num_items, int32_t max_quasars, void *work, uint64_t work_bytes,
                const pg_wick_sums *out, void *stream);

/* Delta files (HOST memory; no device, no plan). pg_read_delta_file parses
 * one delta file, given its bytes (already gunzipped), in either layout: a
 * BINTABLE per line of sight (kept when z_min_qso < Z < z_max_qso) or the
 * image layout with a METADATA table (kept when z_min_qso <= Z <= z_max_qso,
 * pixels with weight > 0). Two passes: with out->los_id == NULL it only sets
 * num_los / num_pixels; then, with every array allocated, it fills them.
 * wave holds LOGLAM, or LAMBDA when wave_is_lambda (the caller takes log10).
 * DELTA_BLIND is read when the file is blinded. */
typedef struct pg_delta_arrays {
    int64_t num_los, num_pixels;   /* out */
    int32_t format;                /* out: 0 one table per line of sight, 1 image */
    int32_t wave_is_lambda;        /* out */
    int64_t *los_id, *plate, *mjd, *fiberid;  /* [num_los] */
    double *ra, *dec, *z_qso;                 /* [num_los] */
    int64_t *pix_offset;                      /* [num_los + 1] */
    double *wave, *delta, *weights, *cont;    /* [num_pixels] */
} pg_delta_arrays;

int pg_read_delta_file(const uint8_t *bytes, int64_t size, double z_min_qso, double z_max_qso,
                       pg_delta_arrays *out);

/* Delta.project of every line of sight (host arrays, in place): the
 * weighted mean of delta and, for order 1, its weighted linear trend in
 * log_lambda removed, with NumPy's summation order (bit-identical to the
 * reference). order[f] is 0 or 1; threads host threads. */
int pg_project_deltas(int64_t num_los, const int64_t *pix_offset, const double *log_lambda,
                      const double *weights, double *delta, const int32_t *order,
                      int32_t threads);

/* The same terms T1-T4 by factorisation, without the sweep over pairs of
 * listed pairs: T2 + T4 = U^T X1 U and T3 = W^T diag(zw1 / w1) W over the
 * forest's nonempty bins (U: per pixel and bin, the sum of the quasars'
 * zw_obj; W: of w1 w_obj), as FP64 GEMMs, with the same-quasar part T2
 * summed directly and T4 = U^T X1 U - T2. Same arguments as pg_xcf_wick
 * (item arrays on the device; no slices). Items run one after another on
 * `stream`, and the call waits for each item's bin count. work:
 * pg_xcf_wick_factored_work_bytes() bytes (4 max_pixels nb + 3 nb^2
 * doubles, nb = np nt). */
int pg_xcf_wick_factored_work_bytes(pg_plan *plan, const pg_corr_params *params,
                                    int32_t max_pixels, int32_t max_quasars, uint64_t *bytes);
int pg_xcf_wick_factored(pg_plan *plan, const pg_corr_params *params,
                         const pg_forest_set *forests, const pg_forest_set *objs,
                         const double *zw1, const double *zw_obj, const int64_t *x_offsets,
                         const double *arena, const int32_t *item_forest,
                         const int32_t *item_start, const int32_t *item_count,
                         const int32_t *obj_index, const double *obj_angle, int64_t num_items,
                         int32_t max_quasars, void *work, uint64_t work_bytes,
                         const pg_wick_sums *out, void *stream);

/* Fast metal distortion matrix (py/picca/bin/picca_fast_metal_dmat.py:30-251,
 * py/picca/bin/picca_fast_metal_xdmat.py:28-215): every pair (i, j) of two
 * pixel lists, side 1 the stacked deltas' wavelength grid, side 2 the same
 * grid (auto) or the quasars' redshift histogram (cross). Per pixel: the
 * comoving distance at the true absorber's redshift (r_in) and at the
 * assumed one's (r_out), the true redshift and the weight with its
 * redshift-evolution factor; a pair weighs weight_1 weight_2. */
typedef struct pg_fast_metal_side {
    const double *r_in, *r_out, *z_in, *weight;
    int64_t num;
} pg_fast_metal_side;

/* r_par edges: r_par_min + ((r_par_max - r_par_min) / num_bins_r_par) k.
 * num_ratio_bins: equal-width bins of the distance ratio (the reference
 * uses 4 (num_bins_r_trans + 1)). signed_r_par 0 folds r_par (|r1 - r2|,
 * the auto script), 1 keeps r1 - r2 (the cross script). near_r_par: the
 * ratio histogram keeps pairs with |r_par_in| < near_r_par (20 Mpc/h). */
typedef struct pg_fast_metal_params {
    double r_par_min, r_par_max, near_r_par;
    int32_t num_bins_r_par, num_ratio_bins, signed_r_par, reserved;
} pg_fast_metal_params;

/* Outputs (device, OVERWRITTEN): rp_dmat[num_bins_r_par^2] the histogram2d of
 * (r_par_out, r_par_in) (row: output bin), ratio_weights / ratio_edges the
 * ratio histogram and its edges (num_ratio_bins + 1, numpy's linspace over
 * the ratio's range), out_weight / out_weight_rp / out_weight_z the sums of
 * w, w r_par_out and w (z_in1 + z_in2) / 2 on the r_par_out bins. */
typedef struct pg_fast_metal_sums {
    double *rp_dmat, *ratio_weights, *ratio_edges;
    double *out_weight, *out_weight_rp, *out_weight_z;
} pg_fast_metal_sums;

int pg_fast_metal_dmat(pg_plan *plan, const pg_fast_metal_params *params,
                       const pg_fast_metal_side *s1, const pg_fast_metal_side *s2,
                       const pg_fast_metal_sums *out, void *stream);

/* Delta x quasar distortion matrix (py/picca/xcf.py:325-675,
 * py/picca/bin/picca_xdmat.py). A work item q is forest item_forest[q] of
 * `forests` with the quasars obj_index[item_start[q] .. item_start[q] +
 * item_count[q]) of `objs` (at most PG_XDMAT_MAX_OBJECTS; a forest's kept
 * quasars may be split over several items, their contributions add). The
 * caller makes the random rejection and drops forests without a kept
 * quasar (xcf.py:382-386). dparams->alpha2 is the quasars' redshift
 * evolution (alpha_obj). obj_angle (optional, aligned with obj_index)
 * overrides the angles computed from the unit vectors. r_par is signed;
 * there is no half-plate veto and no velocity cut in the reference's
 * kernel. */
#define PG_XDMAT_MAX_OBJECTS 256
int pg_xcf_dmat_work_bytes(pg_plan *plan, const pg_corr_params *params,
                           const pg_dmat_params *dparams, int32_t max_pixels, int64_t max_ctas,
                           uint64_t *bytes);
int pg_xcf_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                const pg_forest_set *forests, const pg_forest_set *objs, const double *log_lambda,
                const int32_t *order, const int32_t *item_forest, const int32_t *item_start,
                const int32_t *item_count, const int32_t *obj_index, const double *obj_angle,
                int64_t num_items, void *work, uint64_t work_bytes, const pg_dmat_sums *out,
                void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PICCA_GB300_H */
