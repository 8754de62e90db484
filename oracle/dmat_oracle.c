/* CPU oracle of picca's distortion matrix (TEST INFRASTRUCTURE ONLY).
 *
 * Plain-C restatement, FP64 with the operation order of picca's numba code,
 * of
 *   - oracle_dmat_forest_pair <- cf.compute_dmat_forest_pairs_fast
 *                                (py/picca/cf.py:519-887): the eta terms of
 *                                equations 6 and 21 of du Mas des Bourboux
 *                                et al. 2020 for one forest pair, added to
 *                                the distortion matrix and the effective
 *                                (r_par, r_trans, z, weight) of the model bins.
 *   - oracle_xdmat_forest     <- xcf.compute_dmat_forest_pairs_fast
 *                                (py/picca/xcf.py:427-675): the eta2 / eta4
 *                                terms of one forest and its kept objects.
 * The selection of forest pairs (the random rejection of cf.compute_dmat,
 * py/picca/cf.py:390-517, and xcf.compute_dmat, py/picca/xcf.py:325-424) is
 * made by the caller.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define DMAT_SPEED_LIGHT 299792.458 /* km/s */

typedef struct {
    double r_par_min, r_par_max, r_trans_max;
    int32_t num_bins_r_par, num_bins_r_trans;
    int32_t num_model_bins_r_par, num_model_bins_r_trans;
    double z_min_pairs, z_max_pairs;   /* NaN: no cut */
    double zerr_cut_deg, zerr_cut_kms; /* NaN: no cut */
    int32_t x_correlation, remove_same_half_plate_close_pairs;
    int32_t redshift_evolution;        /* redshift_evolution_in_distortion_matrix */
    double z_ref, alpha, alpha2;
    int32_t rmu_binning, pad;
} oracle_dmat_params;

/* Same pair selection as the first loop of cf.py:544-568: returns 1 when the
 * pair is inside the model range (r_par, r_trans computed like the
 * reference). */
static int in_range(const oracle_dmat_params *p, double r1, double r2, double d1, double d2,
                    double c, double s, double *r_par, double *r_trans)
{
    double rp = (r1 - r2) * c;
    double rt = (d1 + d2) * s;
    if (p->rmu_binning) {
        rt = sqrt(rt * rt + rp * rp);
        rp /= rt;
    }
    if (!p->x_correlation) rp = fabs(rp);
    *r_par = rp;
    *r_trans = rt;
    return !(rp >= p->r_par_max || rt >= p->r_trans_max || rp < p->r_par_min);
}

void oracle_dmat_forest_pair(const oracle_dmat_params *p,
                             const double *log_lambda1, const double *log_lambda2,
                             const double *r_comov1, const double *r_comov2,
                             const double *dist_m1, const double *dist_m2,
                             const double *z1, const double *z2,
                             const double *weights1, const double *weights2,
                             int64_t n1, int64_t n2, double z_qso_1, double z_qso_2,
                             double ang, int32_t same_half_plate, int32_t order1,
                             int32_t order2, double *weights_dmat, double *dmat,
                             double *r_par_eff, double *r_trans_eff, double *z_eff,
                             double *weight_eff)
{
    const double c = cos(ang / 2), s = sin(ang / 2);
    const int64_t nmp = p->num_model_bins_r_par, nmt = p->num_model_bins_r_trans;
    const int64_t nm = nmp * nmt;
    const int zerr_on = !isnan(p->zerr_cut_deg) &&
                        (ang < p->zerr_cut_deg * 3.141592653589793 / 180.0);
    const int zmin_on = !isnan(p->z_min_pairs), zmax_on = !isnan(p->z_max_pairs);

    /* first loop (cf.py:544-568): number of pairs in the model range */
    int64_t num_pairs = 0;
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            double rp, rt;
            if (!in_range(p, r_comov1[i], r_comov2[j], dist_m1[i], dist_m2[j], c, s, &rp, &rt))
                continue;
            if (p->remove_same_half_plate_close_pairs && same_half_plate &&
                fabs(rp) < (p->r_par_max - p->r_par_min) / p->num_bins_r_par)
                continue;
            ++num_pairs;
        }
    }
    if (num_pairs == 0) return;

    /* auxiliary sums (cf.py:573-595), left-to-right like numba */
    double sw1 = 0., sw2 = 0., sll1 = 0., sll2 = 0.;
    for (int64_t i = 0; i < n1; ++i) sw1 += weights1[i];
    for (int64_t j = 0; j < n2; ++j) sw2 += weights2[j];
    for (int64_t i = 0; i < n1; ++i) sll1 += log_lambda1[i] * weights1[i];
    for (int64_t j = 0; j < n2; ++j) sll2 += log_lambda2[j] * weights2[j];
    const double mean1 = sll1 / sw1, mean2 = sll2 / sw2;
    double *dll1 = (double *)malloc(sizeof(double) * (n1 > 0 ? n1 : 1));
    double *dll2 = (double *)malloc(sizeof(double) * (n2 > 0 ? n2 : 1));
    double swsll1 = 0., swsll2 = 0.;
    for (int64_t i = 0; i < n1; ++i) {
        dll1[i] = log_lambda1[i] - mean1;
        swsll1 += weights1[i] * (dll1[i] * dll1[i]);
    }
    for (int64_t j = 0; j < n2; ++j) {
        dll2[j] = log_lambda2[j] - mean2;
        swsll2 += weights2[j] * (dll2[j] * dll2[j]);
    }

    double *eta1 = (double *)calloc((size_t)(nm * n1), sizeof(double));
    double *eta2 = (double *)calloc((size_t)(nm * n2), sizeof(double));
    double *eta3 = (double *)calloc((size_t)(nm * n1), sizeof(double));
    double *eta4 = (double *)calloc((size_t)(nm * n2), sizeof(double));
    double *eta5 = (double *)calloc((size_t)nm, sizeof(double));
    double *eta6 = (double *)calloc((size_t)nm, sizeof(double));
    double *eta7 = (double *)calloc((size_t)nm, sizeof(double));
    double *eta8 = (double *)calloc((size_t)nm, sizeof(double));
    char *touched = (char *)calloc((size_t)nm, 1);
    int32_t *sel_model = (int32_t *)malloc(sizeof(int32_t) * num_pairs);
    int32_t *sel_data = (int32_t *)malloc(sizeof(int32_t) * num_pairs);
    int32_t *sel_i = (int32_t *)malloc(sizeof(int32_t) * num_pairs);
    int32_t *sel_j = (int32_t *)malloc(sizeof(int32_t) * num_pairs);
    int64_t num_sel = 0;

    /* second loop (cf.py:620-840) */
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        int i_selected = 1;
        if (zerr_on) {
            double z_qf = 0.5 * (z1[i] + z_qso_2);
            double dv = fabs(z1[i] - z_qso_2) / (1 + z_qf);
            dv *= DMAT_SPEED_LIGHT;
            if (dv < p->zerr_cut_kms) i_selected = 0;
        }
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            const double z = (z1[i] + z2[j]) / 2;
            int j_selected = 1;
            if ((zmin_on && z < p->z_min_pairs) || (zmax_on && z > p->z_max_pairs))
                j_selected = 0;
            if (zerr_on) {
                double z_qf = 0.5 * (z2[j] + z_qso_1);
                double dv = fabs(z2[j] - z_qso_1) / (1 + z_qf);
                dv *= DMAT_SPEED_LIGHT;
                if (dv < p->zerr_cut_kms) j_selected = 0;
            }
            double r_par, r_trans;
            if (!in_range(p, r_comov1[i], r_comov2[j], dist_m1[i], dist_m2[j], c, s, &r_par,
                          &r_trans))
                continue;
            if (p->remove_same_half_plate_close_pairs && same_half_plate &&
                fabs(r_par) < (p->r_par_max - p->r_par_min) / p->num_bins_r_par)
                j_selected = 0;
            const double w12 = weights1[i] * weights2[j];
            double zfac = 1.0;
            if (p->redshift_evolution)
                zfac = pow((1 + z1[i]) / (1 + p->z_ref), p->alpha - 1) *
                       pow((1 + z2[j]) / (1 + p->z_ref), p->alpha2 - 1);
            const double bp = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                    p->num_bins_r_par);
            const double bt = floor(r_trans / p->r_trans_max * p->num_bins_r_trans);
            const int32_t bins = (int32_t)(bt + p->num_bins_r_trans * bp);
            const double mp = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                    (double)nmp);
            const double mt = floor(r_trans / p->r_trans_max * (double)nmt);
            const int32_t mb = (int32_t)(mt + (double)nmt * mp);
            touched[mb] = 1;
            if (i_selected && j_selected) {
                sel_model[num_sel] = mb;
                sel_data[num_sel] = bins;
                sel_i[num_sel] = (int32_t)i;
                sel_j[num_sel] = (int32_t)j;
                ++num_sel;
                r_par_eff[mb] += w12 * r_par;
                r_trans_eff[mb] += w12 * r_trans;
                z_eff[mb] += w12 * z;
                weight_eff[mb] += w12;
                weights_dmat[bins] += w12;
            }
            eta1[i + n1 * mb] += zfac * weights2[j] / sw2;
            eta2[j + n2 * mb] += zfac * weights1[i] / sw1;
            eta5[mb] += zfac * w12 / sw1 / sw2;
            if (order2 == 1) {
                eta3[i + n1 * mb] += zfac * weights2[j] * dll2[j] / swsll2;
                eta6[mb] += zfac * weights1[i] / sw1 * (weights2[j] * dll2[j] / swsll2);
            }
            if (order1 == 1) {
                eta4[j + n2 * mb] += zfac * weights1[i] * dll1[i] / swsll1;
                eta7[mb] += zfac * weights2[j] / sw2 * (weights1[i] * dll1[i] / swsll1);
                if (order2 == 1)
                    eta8[mb] += zfac * weights1[i] * dll1[i] * weights2[j] * dll2[j] / swsll1 /
                                swsll2;
            }
        }
    }

    /* accumulation (cf.py:842-887) over the model bins touched by any pair,
     * ascending like np.unique(all_model_bins) */
    int64_t num_touched = 0;
    int32_t *touched_list = (int32_t *)malloc(sizeof(int32_t) * (nm > 0 ? nm : 1));
    for (int64_t k = 0; k < nm; ++k)
        if (touched[k]) touched_list[num_touched++] = (int32_t)k;
    for (int64_t q = 0; q < num_sel; ++q) {
        const int64_t i = sel_i[q], j = sel_j[q];
        const int64_t bins = sel_data[q];
        const double w12 = weights1[i] * weights2[j];
        double zfac = 1.0;
        if (p->redshift_evolution)
            zfac = pow((1 + z1[i]) / (1 + p->z_ref), p->alpha - 1) *
                   pow((1 + z2[j]) / (1 + p->z_ref), p->alpha2 - 1);
        dmat[sel_model[q] + nm * bins] += w12 * zfac;
        for (int64_t t = 0; t < num_touched; ++t) {
            const int64_t k = touched_list[t];
            dmat[k + nm * bins] +=
                w12 * (eta5[k] + eta6[k] * dll2[j] + eta7[k] * dll1[i] +
                       eta8[k] * dll1[i] * dll2[j] - eta1[i + n1 * k] - eta2[j + n2 * k] -
                       eta3[i + n1 * k] * dll2[j] - eta4[j + n2 * k] * dll1[i]);
        }
    }
    free(dll1); free(dll2);
    free(eta1); free(eta2); free(eta3); free(eta4);
    free(eta5); free(eta6); free(eta7); free(eta8);
    free(touched); free(touched_list); free(sel_model); free(sel_data); free(sel_i); free(sel_j);
}

/* xcf.compute_dmat_forest_pairs_fast (py/picca/xcf.py:427-675): one forest
 * and the n2 objects kept for it (per-object angle), FP64 in the reference's
 * operation order. p->alpha2 is alpha_obj; r_par is signed (no abs), no
 * half-plate or velocity cut. The first loop counts pairs with
 * r_par <= r_par_min as outside (xcf.py:466), the second with
 * r_par < r_par_min (xcf.py:521), as the reference does. */
void oracle_xdmat_forest(const oracle_dmat_params *p, const double *log_lambda1,
                         const double *r_comov1, const double *dist_m1, const double *z1,
                         const double *weights1, int64_t n1, const double *r_comov2,
                         const double *dist_m2, const double *z2, const double *weights2,
                         const double *ang, int64_t n2, int32_t order1, double *weights_dmat,
                         double *dmat, double *r_par_eff, double *r_trans_eff, double *z_eff,
                         double *weight_eff)
{
    const int64_t nmp = p->num_model_bins_r_par, nmt = p->num_model_bins_r_trans;
    const int64_t nm = nmp * nmt;
    const int zmin_on = !isnan(p->z_min_pairs), zmax_on = !isnan(p->z_max_pairs);
    int64_t num_pairs = 0;
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            double rp = (r_comov1[i] - r_comov2[j]) * cos(ang[j] / 2);
            double rt = (dist_m1[i] + dist_m2[j]) * sin(ang[j] / 2);
            if (p->rmu_binning) {
                rt = sqrt(rt * rt + rp * rp);
                rp /= rt;
            }
            if (rp >= p->r_par_max || rt >= p->r_trans_max || rp <= p->r_par_min) continue;
            ++num_pairs;
        }
    }
    if (num_pairs == 0) return;
    double sw1 = 0., sll1 = 0.;
    for (int64_t i = 0; i < n1; ++i) sw1 += weights1[i];
    for (int64_t i = 0; i < n1; ++i) sll1 += log_lambda1[i] * weights1[i];
    const double mean1 = sll1 / sw1;
    double *dll1 = (double *)malloc(sizeof(double) * (n1 > 0 ? n1 : 1));
    double swsll1 = 0.;
    for (int64_t i = 0; i < n1; ++i) {
        dll1[i] = log_lambda1[i] - mean1;
        swsll1 += weights1[i] * (dll1[i] * dll1[i]);
    }
    double *eta2 = (double *)calloc((size_t)(nm * n2), sizeof(double));
    double *eta4 = (double *)calloc((size_t)(nm * n2), sizeof(double));
    char *touched = (char *)calloc((size_t)nm, 1);
    const int64_t cap = n1 * n2 > 0 ? n1 * n2 : 1;
    int32_t *sel_model = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *sel_data = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *sel_i = (int32_t *)malloc(sizeof(int32_t) * cap);
    int32_t *sel_j = (int32_t *)malloc(sizeof(int32_t) * cap);
    int64_t num_sel = 0;
    for (int64_t i = 0; i < n1; ++i) {
        if (weights1[i] == 0) continue;
        for (int64_t j = 0; j < n2; ++j) {
            if (weights2[j] == 0) continue;
            const double z = (z1[i] + z2[j]) / 2;
            int j_selected = 1;
            if ((zmin_on && z < p->z_min_pairs) || (zmax_on && z > p->z_max_pairs)) j_selected = 0;
            double r_par = (r_comov1[i] - r_comov2[j]) * cos(ang[j] / 2);
            double r_trans = (dist_m1[i] + dist_m2[j]) * sin(ang[j] / 2);
            if (p->rmu_binning) {
                r_trans = sqrt(r_trans * r_trans + r_par * r_par);
                r_par /= r_trans;
            }
            if (r_par >= p->r_par_max || r_trans >= p->r_trans_max || r_par < p->r_par_min)
                continue;
            const double w12 = weights1[i] * weights2[j];
            double zfac = 1.0;
            if (p->redshift_evolution)
                zfac = pow((1 + z1[i]) / (1 + p->z_ref), p->alpha - 1) *
                       pow((1 + z2[j]) / (1 + p->z_ref), p->alpha2 - 1);
            const double bp = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                    p->num_bins_r_par);
            const double bt = floor(r_trans / p->r_trans_max * p->num_bins_r_trans);
            const int32_t bins = (int32_t)(bt + p->num_bins_r_trans * bp);
            const double mp = floor((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                    (double)nmp);
            const double mt = floor(r_trans / p->r_trans_max * (double)nmt);
            const int32_t mb = (int32_t)(mt + (double)nmt * mp);
            touched[mb] = 1;
            if (j_selected) {
                sel_model[num_sel] = mb;
                sel_data[num_sel] = bins;
                sel_i[num_sel] = (int32_t)i;
                sel_j[num_sel] = (int32_t)j;
                ++num_sel;
                r_par_eff[mb] += w12 * r_par;
                r_trans_eff[mb] += w12 * r_trans;
                z_eff[mb] += w12 * z;
                weight_eff[mb] += w12;
                weights_dmat[bins] += w12;
            }
            eta2[j + n2 * mb] += zfac * weights1[i] / sw1;
            if (order1 == 1)
                eta4[j + n2 * mb] += zfac * (weights1[i] * dll1[i] / swsll1);
        }
    }
    int64_t num_touched = 0;
    int32_t *touched_list = (int32_t *)malloc(sizeof(int32_t) * (nm > 0 ? nm : 1));
    for (int64_t k = 0; k < nm; ++k)
        if (touched[k]) touched_list[num_touched++] = (int32_t)k;
    for (int64_t q = 0; q < num_sel; ++q) {
        const int64_t i = sel_i[q], j = sel_j[q];
        const int64_t bins = sel_data[q];
        const double w12 = weights1[i] * weights2[j];
        double zfac = 1.0;
        if (p->redshift_evolution)
            zfac = pow((1 + z1[i]) / (1 + p->z_ref), p->alpha - 1) *
                   pow((1 + z2[j]) / (1 + p->z_ref), p->alpha2 - 1);
        dmat[sel_model[q] + nm * bins] += zfac * w12;
        for (int64_t t = 0; t < num_touched; ++t) {
            const int64_t k = touched_list[t];
            dmat[k + nm * bins] += w12 * (-eta2[j + n2 * k] - eta4[j + n2 * k] * dll1[i]);
        }
    }
    free(dll1); free(eta2); free(eta4); free(touched); free(touched_list);
    free(sel_model); free(sel_data); free(sel_i); free(sel_j);
}
