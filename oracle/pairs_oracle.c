/*
 * CPU oracle for the pair-accumulation path. TEST INFRASTRUCTURE ONLY: this
 * file is compiled and called by tests/, by the package smoke check and by
 * bench.py's CPU-baseline leg, never by the library itself.
 *
 * It is a plain-C FP64 restatement of picca's numba kernels, keeping their
 * operation order (compile with -ffp-contract=off so no FMA is formed):
 *   - oracle_cf_forest_pair   <- cf.compute_xi_forest_pairs_fast
 *                                (py/picca/cf.py:250-387)
 *   - oracle_xcf_forest       <- xcf.compute_xi_forest_pairs_fast
 *                                (py/picca/xcf.py:223-322)
 *   - oracle_angle            <- QSO.get_angle_between, scalar branch
 *                                (py/picca/data.py:143-161)
 *   - oracle_cf_neighbours    <- cf.fill_neighs (py/picca/cf.py:82-135):
 *                                every forest of set 2 with angle < ang_max,
 *                                other thingid, and (auto) ra1 > ra2
 *   - oracle_xcf_neighbours   <- xcf.fill_neighs (py/picca/xcf.py:71-123)
 *   - oracle_cf_rows / oracle_xcf_rows <- the per-healpix loops of
 *                                cf.compute_xi (py/picca/cf.py:138-247) and
 *                                xcf.compute_xi (py/picca/xcf.py:126-220),
 *                                OpenMP over output rows (healpix).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_SPEED_LIGHT 299792.458           /* km/s, scipy.constants.c / 1000 */
#define ORACLE_SMALL_ANGLE (2. / 3600. * 3.141592653589793 / 180.)

typedef struct {
    double r_par_min, r_par_max, r_trans_max;
    int32_t num_bins_r_par, num_bins_r_trans;
    double z_min_pairs, z_max_pairs;    /* NaN: no cut */
    double zerr_cut_deg, zerr_cut_kms;  /* NaN: no cut */
    int32_t x_correlation, rmu_binning, ang_correlation;
    int32_t remove_same_half_plate_close_pairs;
} oracle_cf_params;

/* scalar angle between two unit vectors (data.py:143-161) */
double oracle_angle(double x1, double y1, double z1, double ra1, double dec1,
                    double cos_dec1, double x2, double y2, double z2,
                    double ra2, double dec2)
{
    double cosang = x2 * x1 + y2 * y1 + z2 * z1;
    if (cosang >= 1.) cosang = 1.;
    else if (cosang <= -1.) cosang = -1.;
    double ang = acos(cosang);
    if (fabs(ra2 - ra1) < ORACLE_SMALL_ANGLE && fabs(dec2 - dec1) < ORACLE_SMALL_ANGLE) {
        double ddec = dec2 - dec1;
        double dra = cos_dec1 * (ra2 - ra1);
        ang = sqrt(ddec * ddec + dra * dra);
    }
    return ang;
}

void oracle_cf_forest_pair(const oracle_cf_params *p,
                           const double *z1, const double *r_comov1,
                           const double *dist_m1, const double *weights1,
                           const double *delta1, int64_t n1, double z_qso_1,
                           const double *z2, const double *r_comov2,
                           const double *dist_m2, const double *weights2,
                           const double *delta2, int64_t n2, double z_qso_2,
                           double ang, int32_t same_half_plate,
                           double *rebin_weight, double *rebin_xi,
                           double *rebin_r_par, double *rebin_r_trans,
                           double *rebin_z, int64_t *rebin_num_pairs)
{
    const int zerr_on = !isnan(p->zerr_cut_deg) &&
                        (ang < p->zerr_cut_deg * 3.141592653589793 / 180.0);
    const int zmin_on = !isnan(p->z_min_pairs);
    const int zmax_on = !isnan(p->z_max_pairs);
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        if (zerr_on) {
            double z_qf = 0.5 * (z1[i] + z_qso_2);
            double dv_kms = fabs(z1[i] - z_qso_2) / (1 + z_qf);
            dv_kms *= ORACLE_SPEED_LIGHT;
            if (dv_kms < p->zerr_cut_kms) continue;
        }
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            double z = (z1[i] + z2[j]) / 2;
            if ((zmin_on && z < p->z_min_pairs) || (zmax_on && z > p->z_max_pairs)) continue;
            if (zerr_on) {
                double z_qf = 0.5 * (z2[j] + z_qso_1);
                double dv_kms = fabs(z2[j] - z_qso_1) / (1 + z_qf);
                dv_kms *= ORACLE_SPEED_LIGHT;
                if (dv_kms < p->zerr_cut_kms) continue;
            }
            double r_par, r_trans;
            if (p->ang_correlation) {
                r_par = r_comov1[i] / r_comov2[j];
                if (!p->x_correlation && r_par < 1.0) r_par = 1.0 / r_par;
                r_trans = ang;
            } else {
                r_par = (r_comov1[i] - r_comov2[j]) * cos(ang / 2);
                r_trans = (dist_m1[i] + dist_m2[j]) * sin(ang / 2);
                if (p->rmu_binning) {
                    r_trans = sqrt(r_trans * r_trans + r_par * r_par);
                    r_par /= r_trans;
                }
                if (!p->x_correlation) r_par = fabs(r_par);
            }
            if (r_par >= p->r_par_max || r_trans >= p->r_trans_max || r_par < p->r_par_min)
                continue;
            double dw1 = delta1[i] * weights1[i];
            double dw2 = delta2[j] * weights2[j];
            double dw12 = dw1 * dw2;
            double w12 = weights1[i] * weights2[j];
            double bins_r_par = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                      p->num_bins_r_par);
            double bins_r_trans = floor(r_trans / p->r_trans_max * p->num_bins_r_trans);
            int64_t bins = (int64_t)(bins_r_trans + p->num_bins_r_trans * bins_r_par);
            if (p->remove_same_half_plate_close_pairs && same_half_plate) {
                if (fabs(r_par) < (p->r_par_max - p->r_par_min) / p->num_bins_r_par) continue;
            }
            rebin_xi[bins] += dw12;
            rebin_weight[bins] += w12;
            rebin_r_par[bins] += r_par * w12;
            rebin_r_trans[bins] += r_trans * w12;
            rebin_z[bins] += z * w12;
            rebin_num_pairs[bins] += 1;
        }
    }
}

void oracle_xcf_forest(const oracle_cf_params *p,
                       const double *z1, const double *r_comov1, const double *dist_m1,
                       const double *weights1, const double *delta1, int64_t n1,
                       const double *z2, const double *r_comov2, const double *dist_m2,
                       const double *weights2, const double *ang, int64_t n2,
                       double *rebin_weight, double *rebin_xi, double *rebin_r_par,
                       double *rebin_r_trans, double *rebin_z, int64_t *rebin_num_pairs)
{
    const int zmin_on = !isnan(p->z_min_pairs);
    const int zmax_on = !isnan(p->z_max_pairs);
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            double z = (z1[i] + z2[j]) / 2;
            if ((zmin_on && z < p->z_min_pairs) || (zmax_on && z > p->z_max_pairs)) continue;
            double r_par, r_trans;
            if (p->ang_correlation) {
                r_par = r_comov1[i] / r_comov2[j];
                r_trans = ang[j];
            } else {
                r_par = (r_comov1[i] - r_comov2[j]) * cos(ang[j] / 2);
                r_trans = (dist_m1[i] + dist_m2[j]) * sin(ang[j] / 2);
            }
            if (p->rmu_binning) {
                r_trans = sqrt(r_trans * r_trans + r_par * r_par);
                r_par /= r_trans;
            }
            if (r_par >= p->r_par_max || r_trans >= p->r_trans_max || r_par <= p->r_par_min)
                continue;
            double delta_times_weight = delta1[i] * weights1[i] * weights2[j];
            double weights12 = weights1[i] * weights2[j];
            double bins_r_par = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                      p->num_bins_r_par);
            double bins_r_trans = floor(r_trans / p->r_trans_max * p->num_bins_r_trans);
            int64_t bins = (int64_t)(bins_r_trans + p->num_bins_r_trans * bins_r_par);
            rebin_xi[bins] += delta_times_weight;
            rebin_weight[bins] += weights12;
            rebin_r_par[bins] += r_par * weights12;
            rebin_r_trans[bins] += r_trans * weights12;
            rebin_z[bins] += z * weights12;
            rebin_num_pairs[bins] += 1;
        }
    }
}

/* Per-forest geometry of a set of lines of sight (structure of arrays). */
typedef struct {
    int64_t num;
    const int64_t *pix_offset;   /* [num + 1] into the pixel arrays */
    const double *z, *r_comov, *dist_m, *weights, *delta;   /* per pixel */
    const double *ra, *dec, *x_cart, *y_cart, *z_cart, *cos_dec, *z_qso;
    const double *obj_r_comov, *obj_dist_m, *obj_weight;    /* quasar sets only */
    const int64_t *thingid, *plate, *fiberid;
} oracle_set;

/* Neighbour counts (pass offsets == NULL) or lists for forests [f_begin, f_end)
 * of set 1 against set 2. auto_mode keeps ra1 > ra2 only (cf.py:129-135). */
int64_t oracle_cf_neighbours(const oracle_set *s1, const oracle_set *s2, int32_t auto_mode,
                             double ang_max, int64_t f_begin, int64_t f_end,
                             int64_t *counts, const int64_t *offsets, int64_t *index)
{
    int64_t total = 0;
    /* cheap pre-test standing in for healpy.query_disc: a pair whose dot
     * product is 1e-5 below cos(ang_max) is > 1e-4 rad beyond ang_max */
    const double dot_min = (ang_max < 1e-3 || ang_max >= 3.141592653589793) ? -2.0
                                                                               : cos(ang_max) - 1e-5;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
    for (int64_t f = f_begin; f < f_end; ++f) {
        int64_t n = 0;
        int64_t out = offsets ? offsets[f - f_begin] : 0;
        for (int64_t g = 0; g < s2->num; ++g) {
            if (s2->x_cart[g] * s1->x_cart[f] + s2->y_cart[g] * s1->y_cart[f] +
                    s2->z_cart[g] * s1->z_cart[f] < dot_min)
                continue;
            if (s1->thingid[f] == s2->thingid[g]) continue;
            double ang = oracle_angle(s1->x_cart[f], s1->y_cart[f], s1->z_cart[f], s1->ra[f],
                                      s1->dec[f], s1->cos_dec[f], s2->x_cart[g], s2->y_cart[g],
                                      s2->z_cart[g], s2->ra[g], s2->dec[g]);
            if (!(ang < ang_max)) continue;
            if (auto_mode && !(s1->ra[f] > s2->ra[g])) continue;
            if (offsets) index[out + n] = g;
            ++n;
        }
        if (counts) counts[f - f_begin] = n;
        total += n;
    }
    return total;
}

/* Quasar neighbours of forests (xcf.py:71-123): other thingid, angle <
 * ang_max, optional (zerr_cut_deg, zerr_cut_kms) quasar-pair veto, and the
 * first/last-pixel r_comov pre-cut (skipped in angular mode). */
int64_t oracle_xcf_neighbours(const oracle_set *forests, const oracle_set *objs,
                              const oracle_cf_params *p, double ang_max,
                              int64_t f_begin, int64_t f_end, int64_t *counts,
                              const int64_t *offsets, int64_t *index)
{
    int64_t total = 0;
    const double f = p->rmu_binning ? p->r_trans_max : 1;
    const double dot_min = (ang_max < 1e-3 || ang_max >= 3.141592653589793) ? -2.0
                                                                               : cos(ang_max) - 1e-5;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
    for (int64_t k = f_begin; k < f_end; ++k) {
        int64_t n = 0;
        int64_t out = offsets ? offsets[k - f_begin] : 0;
        int64_t p0 = forests->pix_offset[k], p1 = forests->pix_offset[k + 1];
        for (int64_t g = 0; g < objs->num; ++g) {
            if (objs->x_cart[g] * forests->x_cart[k] + objs->y_cart[g] * forests->y_cart[k] +
                    objs->z_cart[g] * forests->z_cart[k] < dot_min)
                continue;
            if (objs->thingid[g] == forests->thingid[k]) continue;
            double ang = oracle_angle(forests->x_cart[k], forests->y_cart[k], forests->z_cart[k],
                                      forests->ra[k], forests->dec[k], forests->cos_dec[k],
                                      objs->x_cart[g], objs->y_cart[g], objs->z_cart[g],
                                      objs->ra[g], objs->dec[g]);
            if (!(ang < ang_max)) continue;
            if (!isnan(p->zerr_cut_deg)) {
                double ang_deg = 180.0 / 3.141592653589793 * ang;
                double z_qq = 0.5 * (forests->z_qso[k] + objs->z_qso[g]);
                double dv = fabs(forests->z_qso[k] - objs->z_qso[g]) / (1 + z_qq);
                dv *= ORACLE_SPEED_LIGHT;
                if (ang_deg < p->zerr_cut_deg && dv < p->zerr_cut_kms) continue;
            }
            if (!p->ang_correlation) {
                double c = cos(ang / 2.);
                if (!((forests->r_comov[p0] - objs->obj_r_comov[g]) * c < p->r_par_max * f)) continue;
                if (!((forests->r_comov[p1 - 1] - objs->obj_r_comov[g]) * c > p->r_par_min * f)) continue;
            }
            if (offsets) index[out + n] = g;
            ++n;
        }
        if (counts) counts[k - f_begin] = n;
        total += n;
    }
    return total;
}

/* Accumulate rows: forest f of set 1 (f in [f_begin, f_end)) contributes to
 * row[f]; its neighbours are index[offsets[f-f_begin] .. offsets[f-f_begin+1]).
 * Rows must be ordered so that forests of one row are contiguous; each thread
 * owns whole rows, so no two threads write the same output row. */
void oracle_cf_rows(const oracle_set *s1, const oracle_set *s2, const oracle_cf_params *p,
                    int64_t f_begin, int64_t f_end, const int64_t *offsets,
                    const int64_t *index, const int32_t *row, int32_t num_rows,
                    double *we, double *xi, double *rp, double *rt, double *zz, int64_t *nb)
{
    const int64_t nbins = (int64_t)p->num_bins_r_par * p->num_bins_r_trans;
    /* row starts */
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (num_rows + 1));
    for (int32_t r = 0; r <= num_rows; ++r) start[r] = f_end;
    for (int64_t f = f_end - 1; f >= f_begin; --f) start[row[f]] = f;
    for (int32_t r = num_rows - 1; r >= 0; --r)
        if (start[r] > start[r + 1]) start[r] = start[r + 1];
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t r = 0; r < num_rows; ++r) {
        double *o_we = we + r * nbins, *o_xi = xi + r * nbins, *o_rp = rp + r * nbins;
        double *o_rt = rt + r * nbins, *o_z = zz + r * nbins;
        int64_t *o_nb = nb + r * nbins;
        for (int64_t f = start[r]; f < f_end && row[f] == r; ++f) {
            int64_t a0 = s1->pix_offset[f], a1 = s1->pix_offset[f + 1];
            for (int64_t k = offsets[f - f_begin]; k < offsets[f - f_begin + 1]; ++k) {
                int64_t g = index[k];
                int64_t b0 = s2->pix_offset[g], b1 = s2->pix_offset[g + 1];
                double ang = oracle_angle(s1->x_cart[f], s1->y_cart[f], s1->z_cart[f],
                                          s1->ra[f], s1->dec[f], s1->cos_dec[f],
                                          s2->x_cart[g], s2->y_cart[g], s2->z_cart[g],
                                          s2->ra[g], s2->dec[g]);
                int32_t shp = 0;
                if (p->remove_same_half_plate_close_pairs) {
                    shp = (s1->plate[f] == s2->plate[g]) &&
                          ((s1->fiberid[f] <= 500 && s2->fiberid[g] <= 500) ||
                           (s1->fiberid[f] > 500 && s2->fiberid[g] > 500));
                }
                oracle_cf_forest_pair(p, s1->z + a0, s1->r_comov + a0, s1->dist_m + a0,
                                      s1->weights + a0, s1->delta + a0, a1 - a0, s1->z_qso[f],
                                      s2->z + b0, s2->r_comov + b0, s2->dist_m + b0,
                                      s2->weights + b0, s2->delta + b0, b1 - b0, s2->z_qso[g],
                                      ang, shp, o_we, o_xi, o_rp, o_rt, o_z, o_nb);
            }
        }
    }
    free(start);
}

void oracle_xcf_rows(const oracle_set *forests, const oracle_set *objs,
                     const oracle_cf_params *p, int64_t f_begin, int64_t f_end,
                     const int64_t *offsets, const int64_t *index, const int32_t *row,
                     int32_t num_rows, double *we, double *xi, double *rp, double *rt,
                     double *zz, int64_t *nb)
{
    const int64_t nbins = (int64_t)p->num_bins_r_par * p->num_bins_r_trans;
    int64_t *start = (int64_t *)malloc(sizeof(int64_t) * (num_rows + 1));
    for (int32_t r = 0; r <= num_rows; ++r) start[r] = f_end;
    for (int64_t f = f_end - 1; f >= f_begin; --f) start[row[f]] = f;
    for (int32_t r = num_rows - 1; r >= 0; --r)
        if (start[r] > start[r + 1]) start[r] = start[r + 1];
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t r = 0; r < num_rows; ++r) {
        int64_t maxn = 0;
        for (int64_t f = start[r]; f < f_end && row[f] == r; ++f) {
            int64_t n = offsets[f - f_begin + 1] - offsets[f - f_begin];
            if (n > maxn) maxn = n;
        }
        double *buf = (double *)malloc(sizeof(double) * (5 * maxn + 1));
        double *zq = buf, *rq = buf + maxn, *mq = buf + 2 * maxn, *wq = buf + 3 * maxn;
        double *angs = buf + 4 * maxn;
        for (int64_t f = start[r]; f < f_end && row[f] == r; ++f) {
            int64_t k0 = offsets[f - f_begin], k1 = offsets[f - f_begin + 1];
            if (k1 == k0) continue;
            for (int64_t k = k0; k < k1; ++k) {
                int64_t g = index[k];
                zq[k - k0] = objs->z_qso[g];
                rq[k - k0] = objs->obj_r_comov[g];
                mq[k - k0] = objs->obj_dist_m[g];
                wq[k - k0] = objs->obj_weight[g];
                angs[k - k0] = oracle_angle(forests->x_cart[f], forests->y_cart[f],
                                            forests->z_cart[f], forests->ra[f], forests->dec[f],
                                            forests->cos_dec[f], objs->x_cart[g], objs->y_cart[g],
                                            objs->z_cart[g], objs->ra[g], objs->dec[g]);
            }
            int64_t a0 = forests->pix_offset[f], a1 = forests->pix_offset[f + 1];
            oracle_xcf_forest(p, forests->z + a0, forests->r_comov + a0, forests->dist_m + a0,
                              forests->weights + a0, forests->delta + a0, a1 - a0, zq, rq, mq,
                              wq, angs, k1 - k0, we + r * nbins, xi + r * nbins, rp + r * nbins,
                              rt + r * nbins, zz + r * nbins, nb + r * nbins);
        }
        free(buf);
    }
    free(start);
}
