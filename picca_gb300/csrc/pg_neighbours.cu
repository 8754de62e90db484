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
    float dot_threshold;  // below: certainly farther than ang_max
    float dot_sure;       // above: certainly closer than ang_max
    // xcf filters
    double zerr_deg, zerr_kms, r_par_min_f, r_par_max_f;
    int32_t zerr_on, precut_on;
};

// One query against one candidate g of the other set (after the FP32
// prefilter): thingid, exact FP64 angle with the reference's formula, and
// the mode's filters. True when g is a neighbour.
struct Query {
    double x, y, z, ra, dec, cosdec, zq, rfirst, rlast;
    int64_t id;
};

// The FP64 angle (and, for the xcf pre-cut, cos(ang / 2)) is formed only
// where a decision needs it: a pair whose FP32 cosine is above dot_sure is
// within ang_max whatever the rounding, and a pre-cut whose FP32 estimate is
// farther than its error bound from the limit has the exact outcome. Both
// shortcuts give the FP64 decision itself, so the lists are unchanged; they
// remove the FP64 trigonometry that otherwise runs for almost every
// candidate (a warp executes it when any of its lanes needs it).
template <int MODE>
__device__ __forceinline__ bool is_neighbour(const NbrArgs &a, const Query &q, int64_t g,
                                             float dot) {
    if (a.id2[g] == q.id) return false;
    double ang = -1.0;
    auto exact_angle = [&]() {
        if (ang < 0.0)
            ang = angle_between(q.x, q.y, q.z, q.ra, q.dec, q.cosdec, a.x2[g], a.y2[g], a.z2[g],
                                a.ra2[g], a.dec2[g]);
        return ang;
    };
    if (!(dot > a.dot_sure) && !(exact_angle() < a.ang_max)) return false;
    if (MODE == 1 && !(q.ra > a.ra2[g])) return false;
    if (MODE == 2) {
        if (a.zerr_on) {
            const double ang_deg = __dmul_rn(180.0 / kPi, exact_angle());
            const double zq = a.zq2[g];
            const double z_qq = __dmul_rn(0.5, __dadd_rn(q.zq, zq));
            double dv = fabs(__dsub_rn(q.zq, zq)) / __dadd_rn(1.0, z_qq);
            dv = __dmul_rn(dv, kSpeedLight);
            if (ang_deg < a.zerr_deg && dv < a.zerr_kms) return false;
        }
        if (a.precut_on) {
            const double robj = a.robj2[g];
            const double u1 = __dsub_rn(q.rfirst, robj), u2 = __dsub_rn(q.rlast, robj);
            // cos(ang / 2) = sqrt(x), x = (1 + cos ang) / 2, from the FP32
            // cosine (within 4e-7): for x >= 1/4 (ang <= 120 deg) its
            // relative error is below 1e-6, and a limit farther than 4e-6
            // of |u| from the product is decided from it; otherwise (and
            // for wider angles) the FP64 cos(ang / 2) decides
            const float xh = 0.5f * (1.f + dot);
            const bool est = xh >= 0.25f;
            const float ch = sqrtf(fmaxf(xh, 0.f));
            const double e1 = fabs(u1) * 4e-6 + 1e-9, e2 = fabs(u2) * 4e-6 + 1e-9;
            const double p1 = u1 * (double)ch, p2 = u2 * (double)ch;
            bool lo_ok, hi_ok;
            if (est && p1 < a.r_par_max_f - e1) hi_ok = true;
            else if (est && p1 > a.r_par_max_f + e1) hi_ok = false;
            else hi_ok = __dmul_rn(u1, cos(exact_angle() / 2.)) < a.r_par_max_f;
            if (!hi_ok) return false;
            if (est && p2 > a.r_par_min_f + e2) lo_ok = true;
            else if (est && p2 < a.r_par_min_f - e2) lo_ok = false;
            else lo_ok = __dmul_rn(u2, cos(exact_angle() / 2.)) > a.r_par_min_f;
            if (!lo_ok) return false;
        }
    }
    return true;
}

template <int MODE>
__device__ __forceinline__ Query load_query(const NbrArgs &a, int64_t f, bool active) {
    Query q{0, 0, 0, 0, 0, 1, 0, 0, 0, 0};
    if (active) {
        q.x = a.x1[f]; q.y = a.y1[f]; q.z = a.z1[f];
        q.ra = a.ra1[f]; q.dec = a.dec1[f]; q.cosdec = a.cosdec1[f];
        q.id = a.id1[f];
        if (MODE == 2) {
            q.zq = a.zq1[f];
            q.rfirst = a.rfirst1[f];
            q.rlast = a.rlast1[f];
        }
    }
    return q;
}

// Tests the query against objects [t0, t0 + tn) staged in the tile (FP32 unit
// vectors); appends neighbours in increasing index order.
template <int MODE>
__device__ __forceinline__ void scan_tile(const NbrArgs &a, const Query &q, float fx, float fy,
                                          float fz, const float4 *tile, int64_t t0, int tn,
                                          int64_t out, const int64_t *offsets, int32_t *index,
                                          int64_t &n) {
    for (int k = 0; k < tn; ++k) {
        const float4 t = tile[k];
        const float dot = __fmaf_rn(fz, t.z, __fmaf_rn(fy, t.y, fx * t.x));
        if (dot <= a.dot_threshold) continue;
        const int64_t g = t0 + k;
        if (!is_neighbour<MODE>(a, q, g, dot)) continue;
        if (offsets) index[out + n] = (int32_t)g;
        ++n;
    }
}

template <int MODE>  // 0: cf cross (two sets), 1: cf auto, 2: xcf
__global__ void __launch_bounds__(kNbrBlock) neighbours_kernel(NbrArgs a, int64_t *counts,
                                                                const int64_t *offsets,
                                                                int32_t *index) {
    __shared__ float4 tile[kNbrTile];
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = f < a.n1;
    const Query q = load_query<MODE>(a, f, active);
    const float fx = (float)q.x, fy = (float)q.y, fz = (float)q.z;
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
        scan_tile<MODE>(a, q, fx, fy, fz, tile, t0, tn, out, offsets, index, n);
    }
    if (active && !offsets) counts[f] = n;
}

// Grouped search: a block takes up to kNbrBlock queries of one group of the
// query set and scans only the candidate groups of the other set (object
// ranges, ascending), so neighbours still come out in increasing index
// order. The candidate lists are a superset (bounding caps), the tests per
// object are those of the brute-force kernel.
template <int MODE>
__global__ void __launch_bounds__(kNbrBlock) neighbours_grouped_kernel(
    NbrArgs a, pg_nbr_groups gr, int64_t *counts, const int64_t *offsets, int32_t *index) {
    __shared__ float4 tile[kNbrTile];
    const int grp = gr.block_group[blockIdx.x];
    const int64_t f = gr.block_first[blockIdx.x] + threadIdx.x;
    const bool active = f < gr.block_end[blockIdx.x];
    const Query q = load_query<MODE>(a, f, active);
    const float fx = (float)q.x, fy = (float)q.y, fz = (float)q.z;
    int64_t n = 0;
    const int64_t out = (active && offsets) ? offsets[f] : 0;
    for (int c = gr.cand_offsets[grp]; c < gr.cand_offsets[grp + 1]; ++c) {
        const int g2 = gr.cand_groups[c];
        const int64_t lo = gr.start2[g2], hi = gr.start2[g2 + 1];
        for (int64_t t0 = lo; t0 < hi; t0 += kNbrTile) {
            const int tn = (int)min((int64_t)kNbrTile, hi - t0);
            __syncthreads();
            for (int k = threadIdx.x; k < tn; k += blockDim.x)
                tile[k] = make_float4((float)a.x2[t0 + k], (float)a.y2[t0 + k],
                                      (float)a.z2[t0 + k], 0.f);
            __syncthreads();
            if (active) scan_tile<MODE>(a, q, fx, fy, fz, tile, t0, tn, out, offsets, index, n);
        }
    }
    if (active && !offsets) counts[f] = n;
}

float dot_threshold(double ang_max) {
    // below ~1e-3 rad the 1e-5 cosine margin is no longer small; test all
    if (ang_max < 1e-3 || ang_max >= kPi) return -2.0f;
    return (float)cos(ang_max) - 1e-5f;
}

// FP32 unit-vector cosines are accurate to ~4e-7: above this value the FP64
// angle is below ang_max (2 = never: decide every pair in FP64)
float dot_sure(double ang_max) {
    if (ang_max < 1e-3 || ang_max >= kPi) return 2.0f;
    return (float)cos(ang_max) + 1e-5f;
}

}  // namespace

int launch_cf_neighbours(const pg_corr_params &p, const pg_forest_set &s1, const pg_forest_set &s2,
                         bool auto_mode, const pg_nbr_groups *groups, int64_t *counts,
                         const int64_t *offsets, int32_t *index, cudaStream_t stream) {
    NbrArgs a{};
    a.n1 = s1.num;
    a.x1 = s1.x_cart; a.y1 = s1.y_cart; a.z1 = s1.z_cart;
    a.ra1 = s1.ra; a.dec1 = s1.dec; a.cosdec1 = s1.cos_dec; a.id1 = s1.thingid;
    a.n2 = s2.num;
    a.x2 = s2.x_cart; a.y2 = s2.y_cart; a.z2 = s2.z_cart;
    a.ra2 = s2.ra; a.dec2 = s2.dec; a.id2 = s2.thingid;
    a.ang_max = p.ang_max;
    a.dot_threshold = dot_threshold(p.ang_max);
    a.dot_sure = dot_sure(p.ang_max);
    if (a.n1 == 0) return PG_OK;
    if (groups) {
        if (groups->num_blocks <= 0) return PG_OK;
        const dim3 grid((unsigned)groups->num_blocks);
        if (auto_mode)
            neighbours_grouped_kernel<1><<<grid, kNbrBlock, 0, stream>>>(a, *groups, counts,
                                                                         offsets, index);
        else
            neighbours_grouped_kernel<0><<<grid, kNbrBlock, 0, stream>>>(a, *groups, counts,
                                                                         offsets, index);
        return check_cuda(cudaGetLastError());
    }
    const dim3 grid((unsigned)((a.n1 + kNbrBlock - 1) / kNbrBlock));
    if (auto_mode)
        neighbours_kernel<1><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    else
        neighbours_kernel<0><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    return check_cuda(cudaGetLastError());
}

int launch_xcf_neighbours(const pg_corr_params &p, const pg_forest_set &forests,
                          const pg_forest_set &objs, const pg_nbr_groups *groups,
                          int64_t *counts, const int64_t *offsets, int32_t *index,
                          cudaStream_t stream) {
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
    a.dot_sure = dot_sure(p.ang_max);
    a.zerr_on = !isnan(p.zerr_cut_deg) && !isnan(p.zerr_cut_kms);
    a.zerr_deg = p.zerr_cut_deg;
    a.zerr_kms = p.zerr_cut_kms;
    a.precut_on = !p.ang_correlation;
    const double f = p.rmu_binning ? p.r_trans_max : 1;
    a.r_par_max_f = p.r_par_max * f;
    a.r_par_min_f = p.r_par_min * f;
    if (a.n1 == 0) return PG_OK;
    if (groups) {
        if (groups->num_blocks <= 0) return PG_OK;
        neighbours_grouped_kernel<2><<<(unsigned)groups->num_blocks, kNbrBlock, 0, stream>>>(
            a, *groups, counts, offsets, index);
        return check_cuda(cudaGetLastError());
    }
    const dim3 grid((unsigned)((a.n1 + kNbrBlock - 1) / kNbrBlock));
    neighbours_kernel<2><<<grid, kNbrBlock, 0, stream>>>(a, counts, offsets, index);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
