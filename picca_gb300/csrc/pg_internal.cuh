// Internal definitions shared by the picca_gb300 CUDA translation units.
// The whole library is compiled with -fmad=false: every FP64 expression keeps
// the operation order of picca's numba kernels (no contraction), and the FP32
// kernels request fused multiply-adds explicitly with __fmaf_rn.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../../include/picca_gb300.h"

namespace pg {

constexpr double kSpeedLight = 299792.458;  // km/s (scipy.constants.c / 1000)
constexpr double kPi = 3.141592653589793;
// 2 arcsec in radians, py/picca/constants.py:16
constexpr double kSmallAngle = 2. / 3600. * 3.141592653589793 / 180.;

// Scratch owned by a plan (device memory, a few hundred bytes).
struct Scratch {
    int32_t work_counter;      // persistent-kernel work queue head
    int32_t status;            // first device-side error (0 = none)
    int32_t error_detail;
    int32_t pad;
    unsigned long long rechecked_pairs;
    unsigned long long recheck_overflows;
    unsigned long long work_items;
    unsigned long long visited_pairs;  // pixel-pair slots evaluated by the fast cf kernel
    unsigned long long gemm_macs;      // distortion matrix: multiply-adds of the U E^T products
    // ordered-integer encodings of FP64 data ranges (guard-band inputs)
    unsigned long long r_min_key, r_max_key, d_max_key;
    // fast metal matrix: range of the distance ratio (minimum as ~key)
    unsigned long long ratio_lo_inv_key, ratio_hi_key;
};

// Map a double to an unsigned key with the same ordering (for atomicMin/Max).
__host__ __device__ __forceinline__ unsigned long long order_key(double v) {
    unsigned long long bits;
    memcpy(&bits, &v, sizeof(bits));
    return (bits & 0x8000000000000000ull) ? ~bits : (bits | 0x8000000000000000ull);
}
__host__ __device__ __forceinline__ double order_value(unsigned long long key) {
    unsigned long long bits = (key & 0x8000000000000000ull) ? (key & 0x7FFFFFFFFFFFFFFFull) : ~key;
    double v;
    memcpy(&v, &bits, sizeof(v));
    return v;
}

// Device-side error report: first error wins, never traps.
__device__ __forceinline__ void report_error(Scratch *scratch, int32_t code, int32_t detail) {
    if (atomicCAS(&scratch->status, 0, code) == 0) scratch->error_detail = detail;
}

// Angular separation, scalar branch of QSO.get_angle_between
// (py/picca/data.py:143-161): arccos of the clipped dot product
// x2*x1 + y2*y1 + z2*z1 (evaluated left to right, no FMA), replaced by the
// flat-sky distance when |dRA| and |dDec| are both below 2 arcsec.
__device__ __forceinline__ double angle_between(double x1, double y1, double z1, double ra1,
                                                double dec1, double cos_dec1, double x2,
                                                double y2, double z2, double ra2, double dec2) {
    double cosang = __dadd_rn(__dadd_rn(__dmul_rn(x2, x1), __dmul_rn(y2, y1)), __dmul_rn(z2, z1));
    if (cosang >= 1.) cosang = 1.;
    else if (cosang <= -1.) cosang = -1.;
    double ang = acos(cosang);
    if (fabs(__dsub_rn(ra2, ra1)) < kSmallAngle && fabs(__dsub_rn(dec2, dec1)) < kSmallAngle) {
        double ddec = __dsub_rn(dec2, dec1);
        double dra = __dmul_rn(cos_dec1, __dsub_rn(ra2, ra1));
        ang = __dsqrt_rn(__dadd_rn(__dmul_rn(ddec, ddec), __dmul_rn(dra, dra)));
    }
    return ang;
}

// Per-launch constants of the binning, derived once on the host.
struct Binning {
    double r_par_min, r_par_max, r_trans_max;
    double r_par_range;          // r_par_max - r_par_min
    double half_plate_cut;       // (r_par_max - r_par_min) / num_bins_r_par
    double z_min, z_max;         // NaN: off
    double zerr_ang, zerr_kms;   // zerr_cut_deg * pi / 180, km/s; NaN: off
    int32_t np, nt, nbins;
    int32_t x_correlation, rmu, ang_corr, remove_shp;
    int32_t zmin_on, zmax_on, zerr_on;
};

inline Binning make_binning(const pg_corr_params &p) {
    Binning b;
    b.r_par_min = p.r_par_min;
    b.r_par_max = p.r_par_max;
    b.r_trans_max = p.r_trans_max;
    b.r_par_range = p.r_par_max - p.r_par_min;
    b.half_plate_cut = (p.r_par_max - p.r_par_min) / p.num_bins_r_par;
    b.z_min = p.z_min_pairs;
    b.z_max = p.z_max_pairs;
    b.zerr_ang = p.zerr_cut_deg * kPi / 180.0;
    b.zerr_kms = p.zerr_cut_kms;
    b.np = p.num_bins_r_par;
    b.nt = p.num_bins_r_trans;
    b.nbins = p.num_bins_r_par * p.num_bins_r_trans;
    b.x_correlation = p.x_correlation;
    b.rmu = p.rmu_binning;
    b.ang_corr = p.ang_correlation;
    b.remove_shp = p.remove_same_half_plate_close_pairs;
    b.zmin_on = !isnan(p.z_min_pairs);
    b.zmax_on = !isnan(p.z_max_pairs);
    b.zerr_on = !isnan(p.zerr_cut_deg) && !isnan(p.zerr_cut_kms);
    return b;
}

// Velocity veto of a pixel against the other line of sight's quasar
// (py/picca/cf.py:321-328 and :341-348): true when the pixel is dropped.
__device__ __forceinline__ bool zerr_veto(double z_pix, double z_qso, double kms) {
    double z_qf = __dmul_rn(0.5, __dadd_rn(z_pix, z_qso));
    double dv = fabs(__dsub_rn(z_pix, z_qso)) / __dadd_rn(1.0, z_qf);
    dv = __dmul_rn(dv, kSpeedLight);
    return dv < kms;
}

// Exact FP64 pair decision of cf.compute_xi_forest_pairs_fast
// (py/picca/cf.py:334-380) for pixels that already passed the weight and
// zerr tests. Returns the bin (>= 0) or -1 if the pair is rejected; writes
// r_par, r_trans and z as the reference computes them.
__device__ __forceinline__ int64_t cf_pair_bin(const Binning &b, double z1, double r1, double m1,
                                               double z2, double r2, double m2, double ang,
                                               double cos_half, double sin_half, bool shp,
                                               double &r_par_out, double &r_trans_out,
                                               double &z_out) {
    double z = __dadd_rn(z1, z2) / 2;
    if ((b.zmin_on && z < b.z_min) || (b.zmax_on && z > b.z_max)) return -1;
    double r_par, r_trans;
    if (b.ang_corr) {
        r_par = r1 / r2;
        if (!b.x_correlation && r_par < 1.0) r_par = 1.0 / r_par;
        r_trans = ang;
    } else {
        r_par = __dmul_rn(__dsub_rn(r1, r2), cos_half);
        r_trans = __dmul_rn(__dadd_rn(m1, m2), sin_half);
        if (b.rmu) {
            r_trans = __dsqrt_rn(__dadd_rn(__dmul_rn(r_trans, r_trans), __dmul_rn(r_par, r_par)));
            r_par = r_par / r_trans;
        }
        if (!b.x_correlation) r_par = fabs(r_par);
    }
    if (r_par >= b.r_par_max || r_trans >= b.r_trans_max || r_par < b.r_par_min) return -1;
    double bins_r_par = floor(__dmul_rn(__dsub_rn(r_par, b.r_par_min) / b.r_par_range, (double)b.np));
    double bins_r_trans = floor(__dmul_rn(r_trans / b.r_trans_max, (double)b.nt));
    if (b.remove_shp && shp && fabs(r_par) < b.half_plate_cut) return -1;
    r_par_out = r_par;
    r_trans_out = r_trans;
    z_out = z;
    return (int64_t)__dadd_rn(bins_r_trans, __dmul_rn((double)b.nt, bins_r_par));
}

// Exact FP64 pair decision of xcf.compute_xi_forest_pairs_fast
// (py/picca/xcf.py:286-317).
__device__ __forceinline__ int64_t xcf_pair_bin(const Binning &b, double z1, double r1, double m1,
                                                double zq, double rq, double mq, double ang,
                                                double cos_half, double sin_half,
                                                double &r_par_out, double &r_trans_out,
                                                double &z_out) {
    double z = __dadd_rn(z1, zq) / 2;
    if ((b.zmin_on && z < b.z_min) || (b.zmax_on && z > b.z_max)) return -1;
    double r_par, r_trans;
    if (b.ang_corr) {
        r_par = r1 / rq;
        r_trans = ang;
    } else {
        r_par = __dmul_rn(__dsub_rn(r1, rq), cos_half);
        r_trans = __dmul_rn(__dadd_rn(m1, mq), sin_half);
    }
    if (b.rmu) {
        r_trans = __dsqrt_rn(__dadd_rn(__dmul_rn(r_trans, r_trans), __dmul_rn(r_par, r_par)));
        r_par = r_par / r_trans;
    }
    if (r_par >= b.r_par_max || r_trans >= b.r_trans_max || r_par <= b.r_par_min) return -1;
    double bins_r_par = floor(__dmul_rn(__dsub_rn(r_par, b.r_par_min) / b.r_par_range, (double)b.np));
    double bins_r_trans = floor(__dmul_rn(r_trans / b.r_trans_max, (double)b.nt));
    r_par_out = r_par;
    r_trans_out = r_trans;
    z_out = z;
    return (int64_t)__dadd_rn(bins_r_trans, __dmul_rn((double)b.nt, bins_r_par));
}

// Host helpers (pg_api.cu)
int check_cuda(cudaError_t err);

// Launchers implemented in the kernel translation units.
int launch_cf_neighbours(const pg_corr_params &p, const pg_forest_set &s1, const pg_forest_set &s2,
                         bool auto_mode, const pg_nbr_groups *groups, int64_t *counts,
                         const int64_t *offsets, int32_t *index, cudaStream_t stream);
int launch_xcf_neighbours(const pg_corr_params &p, const pg_forest_set &forests,
                          const pg_forest_set &objs, const pg_nbr_groups *groups,
                          int64_t *counts, const int64_t *offsets, int32_t *index,
                          cudaStream_t stream);
int launch_cf_xi_fp64(const Binning &b, const pg_forest_set &s1, const pg_forest_set &s2,
                      const int64_t *nbr_offsets, const int32_t *nbr_index, const double *nbr_angle,
                      const int32_t *work_order, int64_t num_work, const pg_xi_rows &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream);
int launch_xcf_xi_fp64(const Binning &b, const pg_forest_set &forests, const pg_forest_set &objs,
                       const int64_t *nbr_offsets, const int32_t *nbr_index, const double *nbr_angle,
                       const int32_t *work_order, int64_t num_work, const pg_xi_rows &out,
                       Scratch *scratch, int num_sms, cudaStream_t stream);
// Size of the device buffer holding the precision-form constants.
size_t fast_const_bytes();
// Launch shape of the precision-form pair kernels: warps per CTA (the CTA
// size) and CTAs per SM (each CTA holds one copy of the shared histogram);
// 0 selects the default (the most warps shared memory allows, as many CTAs
// as fit).
struct LaunchTuning {
    int warps = 0;
    int blocks_per_sm = 0;
};
int launch_cf_xi_fast(const Binning &b, double ang_max, const pg_forest_set &s1,
                      const pg_forest_set &s2, const int64_t *nbr_offsets,
                      const int32_t *nbr_index, const double *nbr_angle,
                      const int32_t *work_order, int64_t num_work,
                      const pg_xi_rows &out, Scratch *scratch, void *fast_const, int num_sms,
                      cudaStream_t stream, LaunchTuning tuning = LaunchTuning());
int launch_xcf_xi_fast(const Binning &b, double ang_max, const pg_forest_set &forests,
                       const pg_forest_set &objs, const int64_t *nbr_offsets,
                       const int32_t *nbr_index, const double *nbr_angle,
                       const int32_t *work_order, int64_t num_work,
                       const pg_xi_rows &out, Scratch *scratch, void *fast_const, int num_sms,
                       cudaStream_t stream, LaunchTuning tuning = LaunchTuning());

// Distortion matrix (pg_dmat.cu). Default number of U and E rows a CTA keeps
// before the bins of one forest pair are split into chunks.
constexpr int64_t kDmatRowCapacity = 512;
struct DmatConstHost {
    size_t smem;
    int32_t p1, p2, mwords, dwords;
    int64_t list_doubles, work_doubles, cta_doubles;
    int max_grid;
    int split;
    int xcf;
};
// p1 / p2: pixel capacity of the two forests (cross: of the forest; the
// quasar capacity of a work item is fixed).
int dmat_config(const pg_corr_params &p, const pg_dmat_params &d, int p1, int p2, int num_sms,
                DmatConstHost &h, bool xcf);
int launch_xcf_dmat(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h,
                    const pg_forest_set &forests, const pg_forest_set &objs, const double *ll,
                    const int32_t *order, const int32_t *item_forest, const int32_t *item_start,
                    const int32_t *item_count, const int32_t *obj_index,
                    const double *obj_angle, int64_t num_items, double *work, int grid,
                    const pg_dmat_sums &out, Scratch *scratch, cudaStream_t stream);
int launch_cf_dmat(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h,
                   const pg_forest_set &s1, const pg_forest_set &s2, const double *ll1,
                   const double *ll2, const int32_t *order1, const int32_t *order2,
                   const int32_t *pair_first, const int32_t *pair_second,
                   const double *pair_angle, int64_t num_pairs, double *work, int grid,
                   const pg_dmat_sums &out, Scratch *scratch, cudaStream_t stream);

int launch_metal_dmat(const pg_corr_params &p, const pg_dmat_params &d, double zevol_den,
                      const pg_forest_set &s1, const pg_forest_set &s2,
                      const pg_metal_pixels &a1, const pg_metal_pixels &a2,
                      const int32_t *pair_first, const int32_t *pair_second,
                      const double *pair_angle, int64_t num_pairs, const pg_dmat_sums &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream, bool xcf);

int launch_wick_xmat(const pg_forest_set &s, const double *log_lambda, const double *variance,
                     const double *bounds, const double *values, int32_t num_values,
                     const int32_t *forests, int64_t num_forests, const int64_t *x_offsets,
                     double *arena, int num_sms, cudaStream_t stream);
int wick_t123_grid(int nb, int num_sms, int *grid);
int launch_wick_t123(const pg_corr_params &p, const pg_forest_set &s1, const pg_forest_set &s2,
                     const double *zw1, const double *zw2, const int64_t *xo1,
                     const double *xa1, const int64_t *xo2, const double *xa2,
                     const int32_t *pair_first, const int32_t *pair_second,
                     const double *pair_angle, const int32_t *unit_slice,
                     const int32_t *unit_slices, int64_t num_pairs, uint32_t *work,
                     int64_t cap, int grid, const pg_wick_sums &out, Scratch *scratch,
                     cudaStream_t stream);

int64_t xwick_cta_bytes(int64_t cap, int64_t max_quasars);
int xwick_grid(int nb, int num_sms, int *grid);
int launch_xwick(const pg_corr_params &p, const pg_forest_set &forests, const pg_forest_set &objs,
                 const double *zw1, const double *zw_obj, const int64_t *xo, const double *xa,
                 const int32_t *item_forest, const int32_t *item_start, const int32_t *item_count,
                 const int32_t *obj_index, const double *obj_angle, const int32_t *unit_slice,
                 const int32_t *unit_slices, int64_t num_items, char *work, int64_t cap,
                 int64_t max_quasars, int grid, const pg_wick_sums &out, Scratch *scratch,
                 cudaStream_t stream);

int read_delta_file(const uint8_t *buf, int64_t size, double z_min, double z_max,
                    pg_delta_arrays *out);
int project_deltas(int64_t num_los, const int64_t *pix_offset, const double *log_lambda,
                   const double *weights, double *delta, const int32_t *order, int threads);

uint64_t xwick_factored_bytes(int nb, int max_pixels, int max_quasars);
int run_xwick_factored(const pg_corr_params &p, const pg_forest_set &forests,
                       const pg_forest_set &objs, const double *zw1, const double *zw_obj,
                       const int64_t *xo_host, const double *xa, const int32_t *item_forest,
                       const int32_t *item_start, const int32_t *item_count,
                       const int32_t *obj_index, const double *obj_angle, int64_t num_items,
                       const int64_t *pix_offset_host, int max_pixels, int max_quasars,
                       char *work, const pg_wick_sums &out, Scratch *scratch, int num_sms,
                       cudaStream_t st);

int launch_fast_metal(const pg_fast_metal_params &p, const pg_fast_metal_side &a,
                      const pg_fast_metal_side &b, const pg_fast_metal_sums &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream);

int launch_cont_fit(const pg_spectra &sp, const pg_cont_model &m, const double *start,
                    const int32_t *index, int64_t count, int max_iter, double tol, int mode,
                    const pg_cont_fit &out, Scratch *scratch, int num_sms, cudaStream_t stream,
                    float cert_chi2 = 0.f, float cert_ab = 0.f);
int launch_cont_stacks(const pg_spectra &sp, const pg_cont_model &m, const pg_cont_fit &fit,
                       const pg_cont_stacks &st, Scratch *scratch, int num_sms,
                       cudaStream_t stream);
int launch_cont_deltas(const pg_spectra &sp, const pg_cont_model &m, const pg_cont_fit &fit,
                       double *delta, double *weights, int num_sms, cudaStream_t stream);
int64_t mlp_packed_elems();
int launch_mlp_pack(const uint16_t *params16, uint16_t *packed, cudaStream_t stream);
int launch_mlp_forward_tc(const uint16_t *packed, const float *params, const uint16_t *x, int64_t m,
                          int stride, float *y, Scratch *scratch, int num_sms,
                          cudaStream_t stream);
int launch_mlp_warm_start_tc(const pg_spectra &sp, const pg_cont_model &model,
                             const uint16_t *packed, const float *params, float *y, double *a0,
                             Scratch *scratch, int num_sms, cudaStream_t stream);
int launch_mlp_features(const pg_spectra &sp, const pg_cont_model &m, uint16_t *features,
                        int stride, double *a0, Scratch *scratch, int num_sms,
                        cudaStream_t stream);

}  // namespace pg
