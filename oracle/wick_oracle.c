/* CPU oracle of picca's Wick covariance terms T1-T3 (TEST INFRASTRUCTURE ONLY).
 *
 * Restates cf.compute_wickT123_pairs (py/picca/cf.py:1498-1626) for one
 * forest pair: the kept pixel pairs in the reference's order (pixel of
 * forest 2 outer, pixel of forest 1 inner, py/picca/cf.py:1558-1599), then
 * every pair of kept pixel pairs (a < b) adding to T2 when they share a
 * pixel and to T3 otherwise, symmetrically (:1601-1624). FP64 throughout,
 * compiled without FMA contraction so each expression rounds as numba's.
 * The weighted 1D correlation matrices X1, X2 (n x n, row-major) are the
 * caller's, formed as the reference does at py/picca/cf.py:1392-1418.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct {
    double r_par_min, r_par_max, r_trans_max;
    int32_t num_bins_r_par, num_bins_r_trans;
    int32_t x_correlation;
    int32_t pad;
} oracle_wick_params;

void oracle_wick_t123(const oracle_wick_params *p, const double *r1, const double *w1,
                      const double *zw1, const double *x1, int64_t n1, const double *r2,
                      const double *w2, const double *zw2, const double *x2, int64_t n2,
                      double ang, double *weights_wick, int64_t *num_pairs_wick, double *t1,
                      double *t2, double *t3) {
    const int64_t nb = (int64_t)p->num_bins_r_par * p->num_bins_r_trans;
    const double c = cos(ang / 2), s = sin(ang / 2);
    int64_t cap = n1 * n2, k = 0;
    int64_t *pi = malloc(sizeof(int64_t) * (cap ? cap : 1));
    int64_t *pj = malloc(sizeof(int64_t) * (cap ? cap : 1));
    int64_t *pb = malloc(sizeof(int64_t) * (cap ? cap : 1));
    for (int64_t j = 0; j < n2; ++j) {
        for (int64_t i = 0; i < n1; ++i) {
            double r_par = (r1[i] - r2[j]) * c;
            if (!p->x_correlation) r_par = fabs(r_par);
            const double r_trans = (r1[i] + r2[j]) * s;
            if (!(r_par < p->r_par_max && r_trans < p->r_trans_max && r_par >= p->r_par_min))
                continue;
            const int64_t bp = (int64_t)((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                         p->num_bins_r_par);
            const int64_t bt = (int64_t)(r_trans / p->r_trans_max * p->num_bins_r_trans);
            pi[k] = i;
            pj[k] = j;
            pb[k] = bt + p->num_bins_r_trans * bp;
            ++k;
        }
    }
    for (int64_t a = 0; a < k; ++a) {
        const int64_t pa = pb[a], ia = pi[a], ja = pj[a];
        const double w12 = w1[ia] * w2[ja];
        weights_wick[pa] += w12;
        num_pairs_wick[pa] += 1;
        t1[pa * nb + pa] += w12 * (zw1[ia] * zw2[ja]);
        for (int64_t b = a + 1; b < k; ++b) {
            const int64_t q = pb[b], ib = pi[b], jb = pj[b];
            double prod;
            double *t;
            if (ia == ib) {
                prod = x2[ja * n2 + jb] * w1[ia] * zw1[ia];
                t = t2;
            } else if (ja == jb) {
                prod = x1[ia * n1 + ib] * w2[jb] * zw2[ja];
                t = t2;
            } else {
                prod = x1[ia * n1 + ib] * x2[ja * n2 + jb];
                t = t3;
            }
            t[pa * nb + q] += prod;
            t[q * nb + pa] += prod;
        }
    }
    free(pi);
    free(pj);
    free(pb);
}

/* xcf.compute_wickT1234_pairs (py/picca/xcf.py:1220-1351) for one forest and
 * its neighbouring quasars (the objects of xcf.fill_neighs, each with its own
 * angle): pixel pairs listed quasar outer, pixel inner (:1280-1316), r_par
 * signed; then every pair of listed pairs (a < b): same quasar adds
 * X1[i_a, i_b] zw2^2 to T2, same pixel adds w12_a w12_b / w1 zw1 to T3, and
 * otherwise X1[i_a, i_b] zw2_a zw2_b goes to T4 (:1318-1350). */
void oracle_xwick_t1234(const oracle_wick_params *p, const double *r1, const double *w1,
                        const double *zw1, const double *x1, int64_t n1, const double *r2,
                        const double *w2, const double *zw2, const double *ang, int64_t n2,
                        double *weights_wick, int64_t *num_pairs_wick, double *t1, double *t2,
                        double *t3, double *t4) {
    const int64_t nb = (int64_t)p->num_bins_r_par * p->num_bins_r_trans;
    int64_t cap = n1 * n2, k = 0;
    int64_t *pi = malloc(sizeof(int64_t) * (cap ? cap : 1));
    int64_t *pj = malloc(sizeof(int64_t) * (cap ? cap : 1));
    int64_t *pb = malloc(sizeof(int64_t) * (cap ? cap : 1));
    double *pw = malloc(sizeof(double) * (cap ? cap : 1));
    for (int64_t j = 0; j < n2; ++j) {
        const double c = cos(ang[j] / 2), s = sin(ang[j] / 2);
        for (int64_t i = 0; i < n1; ++i) {
            const double r_par = (r1[i] - r2[j]) * c;
            const double r_trans = (r1[i] + r2[j]) * s;
            if (!(r_par < p->r_par_max && r_trans < p->r_trans_max && r_par >= p->r_par_min))
                continue;
            const int64_t bp = (int64_t)((r_par - p->r_par_min) / (p->r_par_max - p->r_par_min) *
                                         p->num_bins_r_par);
            const int64_t bt = (int64_t)(r_trans / p->r_trans_max * p->num_bins_r_trans);
            pi[k] = i;
            pj[k] = j;
            pb[k] = bt + p->num_bins_r_trans * bp;
            pw[k] = w1[i] * w2[j];
            ++k;
        }
    }
    for (int64_t a = 0; a < k; ++a) {
        const int64_t pa = pb[a], ia = pi[a], ja = pj[a];
        weights_wick[pa] += pw[a];
        num_pairs_wick[pa] += 1;
        t1[pa * nb + pa] += pw[a] * pw[a] / w1[ia] * zw1[ia];
        for (int64_t b = a + 1; b < k; ++b) {
            const int64_t q = pb[b], ib = pi[b], jb = pj[b];
            double prod;
            double *t;
            if (ja == jb) {
                prod = x1[ia * n1 + ib] * (zw2[ja] * zw2[ja]);
                t = t2;
            } else if (ia == ib) {
                prod = pw[a] * pw[b] / w1[ia] * zw1[ia];
                t = t3;
            } else {
                prod = x1[ia * n1 + ib] * zw2[ja] * zw2[jb];
                t = t4;
            }
            t[pa * nb + q] += prod;
            t[q * nb + pa] += prod;
        }
    }
    free(pi);
    free(pj);
    free(pb);
    free(pw);
}
