// Neighbour search: cf.fill_neighs (py/picca/cf.py:82-135) and
// xcf.fill_neighs (py/picca/xcf.py:71-123).
//
// The reference asks healpy.query_disc for candidate healpix and then keeps
// objects with angle < ang_max; the result is exactly "every object of the
// other set within ang_max" (plus the thingid / RA-order / zerr / r_comov
// filters). Here each thread owns one query forest and streams the other set
// through shared memory in tiles. A cheap FP32 dot-product test discards
// pairs whose cosine is more than 1e-5 below cos(ang_max) (FP32 unit-vector
// dot products are accurate to ~4e-7, so no true neighbour is lost); the
// survivors are decided exactly in FP64 with the reference's formula.
#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kNbrBlock = 256;
constexpr int kNbrTile = 1024;

struct NbrArgs {
    // query set
    int64_t n1;
    const double *x1, *y1, *z1, *ra1, *dec1, *cosdec1, *zq1, *rfirst1, *rlast1;
    const int64_t *id1;
    // other set
    int64_t n2;
    const double *x2, *y2, *z2, *ra2, *dec2, *zq2, *robj2;
    const int64_t *id2;
    double ang_max;
    float dot_threshold;
    // xcf filters
    double zerr_deg, zerr_kms, r_par_min_f, r_par_max_f;
    int32_t zerr_on, precut_on;
};

template <int MODE>  // 0: cf cross (two sets), 1: cf auto, 2: xcf
__global__ void __launch_bounds__(kNbrBlock) neighbours_kernel(NbrArgs a, int64_t *counts,
                                                                const int64_t *offsets,
                                                                int32_t *index) {
    __shared__ float4 tile[kNbrTile];
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = f < a.n1;
    double qx = 0, qy = 0, qz = 0, qra = 0, qdec = 0, qcos = 1, qzq = 0, qrf = 0, qrl = 0;
    int64_t qid = 0;
    if (active) {
        qx = a.x1[f]; qy = a.y1[f]; qz = a.z1[f];
        qra = a.ra1[f]; qdec = a.dec1[f]; qcos = a.cosdec1[f];
        qid = a.id1[f];
        if (MODE == 2) {
            qzq = a.zq1[f];
            qrf = a.rfirst1[f];
            qrl = a.rlast1[f];
        }
    }
    const float fx = (float)qx, fy = (float)qy, fz = (float)qz;
    int64_t n = 0;
    const int64_t out = (active && offsets) ? offsets[f] : 0;
    for (int64_t t0 = 0; t0 < a.n2; t0 += kNbrTile) {
        const int tn = (int)min((int64_t)kNbrTile, a.n2 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < tn; k += blockDim.x) {
            tile[k] = make_float4((float)a.x2[t0 + k], (float)a.y2[t0 + k], (float)a.z2[t0 + k], 0.f);
        }
        __syncthreads();
        if (!active) continue;
        for (int k = 0; k < tn; ++k) {
            const float4 t = tile[k];
            const float dot = __fmaf_rn(fz, t.z, __fmaf_rn(fy, t.y, fx * t.x));
            if (dot <= a.dot_threshold) continue;
            const int64_t g = t0 + k;
            if (a.id2[g] == qid) continue;
            const double ang = angle_between(qx, qy, qz, qra, qdec, qcos, a.x2[g], a.y2[g],
                                             a.z2[g], a.ra2[g], a.dec2[g]);
            if (!(ang < a.ang_max)) continue;
            if (MODE == 1 && !(qra > a.ra2[g])) continue;
            if (MODE == 2) {
                if (a.zerr_on) {
                    const double ang_deg = __dmul_rn(180.0 / kPi, ang);
                    const double zq = a.zq2[g];
                    const double z_qq = __dmul_rn(0.5, __dadd_rn(qzq, zq));
                    double dv = fabs(__dsub_rn(qzq, zq)) / __dadd_rn(1.0, z_qq);
                    dv = __dmul_rn(dv, kSpeedLight);
                    if (ang_deg < a.zerr_deg && dv < a.zerr_kms) continue;
                }
                if (a.precut_on) {
                    const double c = cos(ang / 2.);
                    const double robj = a.robj2[g];
                    if (!(__dmul_rn(__dsub_rn(qrf, robj), c) < a.r_par_max_f)) continue;
                    if (!(__dmul_rn(__dsub_rn(qrl, robj), c) > a.r_par_min_f)) continue;
                }
            }
            if (offsets) index[out + n] = (int32_t)g;
            ++n;
        }
    }
    if (active && !offsets) counts[f] = n;
}

float dot_threshold(double ang_max) {
    // below ~1e-3 rad the 1e-5 cosine margin is no longer small; test all
    if (ang_max < 1e-3 || ang_max >= kPi) return -2.0f;
    return (float)cos(ang_max) - 1e-5f;
}

}  // namespace

int launch_cf_neighbours(const pg_corr_params &p, const pg_forest_set &s1, const pg_forest_set &s2,
                         bool auto_mode, int64_t *counts, const int64_t *offsets, int32_t *index,
                         cudaStream_t stream) {
    NbrArgs a{};
    a.n1 = s1.num;
    a.x1 = s1.x_cart; a.y1 = s1.y_cart; a.z1 = s1.z_cart;
    a.ra1 = s1.ra; a.dec1 = s1.dec; a.cosdec1 = s1.cos_dec; a.id1 = s1.thingid;
    a.n2 = s2.num;
    a.x2 = s2.x_cart; a.y2 = s2.y_cart; a.z2 = s2.z_cart;
    a.ra2 = s2.ra; a.dec2 = s2.dec; a.id2 = s2.thingid;
    a.ang_max = p.ang_max;
    a.dot_threshold = dot_threshold(p.ang_max);
    if (a.n1 == 0) return PG_OK;
    const dim3 grid((unsigned)((a.n1 + kNbrBlock - 1) / kNbrBlock));
    if (auto_mode)
        neighbours_kernel<1><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    else
        neighbours_kernel<0><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    return check_cuda(cudaGetLastError());
}

int launch_xcf_neighbours(const pg_corr_params &p, const pg_forest_set &forests,
                          const pg_forest_set &objs, int64_t *counts, const int64_t *offsets,
                          int32_t *index, cudaStream_t stream) {
    NbrArgs a{};
    a.n1 = forests.num;
    a.x1 = forests.x_cart; a.y1 = forests.y_cart; a.z1 = forests.z_cart;
    a.ra1 = forests.ra; a.dec1 = forests.dec; a.cosdec1 = forests.cos_dec;
    a.zq1 = forests.z_qso; a.rfirst1 = forests.r_first; a.rlast1 = forests.r_last;
    a.id1 = forests.thingid;
    a.n2 = objs.num;
    a.x2 = objs.x_cart; a.y2 = objs.y_cart; a.z2 = objs.z_cart;
    a.ra2 = objs.ra; a.dec2 = objs.dec; a.zq2 = objs.z_qso; a.robj2 = objs.obj_r_comov;
    a.id2 = objs.thingid;
    a.ang_max = p.ang_max;
    a.dot_threshold = dot_threshold(p.ang_max);
    a.zerr_on = !isnan(p.zerr_cut_deg) && !isnan(p.zerr_cut_kms);
    a.zerr_deg = p.zerr_cut_deg;
    a.zerr_kms = p.zerr_cut_kms;
    a.precut_on = !p.ang_correlation;
    const double f = p.rmu_binning ? p.r_trans_max : 1;
    a.r_par_max_f = p.r_par_max * f;
    a.r_par_min_f = p.r_par_min * f;
    if (a.n1 == 0) return PG_OK;
    const dim3 grid((unsigned)((a.n1 + kNbrBlock - 1) / kNbrBlock));
    neighbours_kernel<2><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
