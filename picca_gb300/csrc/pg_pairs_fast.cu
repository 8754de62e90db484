// Precision-form pair accumulation: FP32 geometry with an FP64 bin-edge
// guard, compensated FP32 shared-memory block sums, FP64 rows.
//
// Same persistent structure as the FP64 kernels (one work item = one forest
// of set 1 with all its neighbours; warps take neighbour forests; lanes own
// forest-2 pixels in registers and loop over the forest-1 pixels staged in
// shared memory). For every pixel pair the kernel evaluates, in FP32,
//     p = cp*((r1h - r2h) + (r1l - r2l))   (= r_par * np/(r_par_max - r_par_min))
//     x_par = |p| - r_par_min*inv_p       (p itself for signed, cross correlations)
//     x_tr  = st*d1 + st*d2               (= r_trans * nt/r_trans_max)
// with cp = cos(theta/2) * inv_p, st = sin(theta/2) * inv_t, and the comoving
// distance carried as an FP32 pair r = rh + rl, so that r1 - r2 is exact to
// ~1e-7 of itself (not of r). The bin index of py/picca/cf.py:372-376 is floor(x). It is taken with
// one round-toward-minus-infinity add: y = x + (2^23 + 1) rounded down is
// 2^23 + 1 + floor(x) for every x >= -1, so floor(x) = bits(y) - bits(2^23)
// - 1 and x - (y - (2^23 + 1)) is the fractional part. A pair whose
// fractional part is within a guard band g of 0 or 1 in either coordinate
// (bin edges and the r_par / r_trans acceptance limits), or within a guard
// of the half-plate r_par cut or the z-pair cuts, is queued and re-decided
// in FP64 with the reference's operation order (cf_pair_bin /
// xcf_pair_bin), so every accepted pair, bin index and pair count equals
// the FP64 reference. g exceeds the worst-case FP32 error (make_fast_const).
//
// Sums: per-CTA FP32 histograms of xi, w, p*w, x_tr*w, (z1+z2)*w and an
// int32 count. xi (products of signed deltas, strongly cancelling) and w
// (the normalisation) are accumulated error-free: the atomic add returns the
// previous value, Knuth's TwoSum recovers the exact rounding error of the add
// and a second histogram collects it. After each work item the partials are
// added to the FP64 rows and mapped back to picca's units (r_par = p/inv_p,
// r_trans = x_tr/inv_t, z = (z1+z2)/2).
#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr float kFloorMagic = 8388609.0f;  // 2^23 + 1, exact in FP32
constexpr int kFloorBits = 0x4B000001;     // bits of 2^23 + 1
constexpr int kQueue = 128;                // recheck entries per warp
constexpr int kCfP = 4;                    // forest-2 pixels per lane per pass
constexpr int kXcfP = 2;                   // quasars per lane per pass
constexpr int kCfBlock = 384;              // cf threads per CTA (2 CTAs per SM)

struct FastConst {
    double inv_p, inv_t;
    float pmin;             // r_par_min * inv_p
    float g_par, g_tr;      // guard bands (fraction of a bin)
    float one_m_g_par, one_m_g_tr;
    float guard_v;          // half-plate cut guard (in units of p)
    float guard_z;          // guard on z1 + z2
    float zmin2, zmax2;     // 2 z_min, 2 z_max
    unsigned np, nt;
    int nbins;
    int hstride;            // histogram array stride (nbins rounded up to 4)
    int lower_exact;        // auto-correlation with r_par_min = 0: x_par = |p| >= 0, so
                            // the lower edge of bin 0 can never be crossed
};

enum {
    H_XI = 0, H_XIL, H_WE, H_WEL, H_PW, H_TW, H_ZW, H_NB, H_COUNT
};

__device__ __forceinline__ void two_sum_add(float *hi, float *lo, float v) {
    const float old = atomicAdd(hi, v);
    const float s = old + v;
    const float bb = s - old;
    atomicAdd(lo, (old - (s - bb)) + (v - bb));
}

__device__ __forceinline__ void acc_pair(float *h, int hs, int bin, float xi, float w, float pw,
                                         float tw, float zw) {
    float *hx = h + bin;
    two_sum_add(hx + H_XI * hs, hx + H_XIL * hs, xi);
    two_sum_add(hx + H_WE * hs, hx + H_WEL * hs, w);
    atomicAdd(hx + H_PW * hs, pw);
    atomicAdd(hx + H_TW * hs, tw);
    atomicAdd(hx + H_ZW * hs, zw);
    atomicAdd(reinterpret_cast<int *>(hx + H_NB * hs), 1);
}

// FP32 value of a weight that stays nonzero when the FP64 weight is nonzero
// (a weight below the FP32 range still counts its pairs, as in FP64).
__device__ __forceinline__ float weight32(double w) {
    const float f = (float)w;
    if (f == 0.f && w != 0.) return w > 0 ? 1.401298464e-45f : -1.401298464e-45f;
    return f;
}

// floor(x) (as unsigned, x >= -1) and the fractional part x - floor(x).
__device__ __forceinline__ unsigned floor_frac(float x, float &frac) {
    const float y = __fadd_rd(x, kFloorMagic);
    frac = x - (y - kFloorMagic);
    return (unsigned)(__float_as_int(y) - kFloorBits);
}

__device__ __forceinline__ void flush_rows(float *h, const FastConst &fc, const pg_xi_rows &out,
                                           int32_t row) {
    const int nbins = fc.nbins, hs = fc.hstride;
    const size_t o = (size_t)row * nbins;
    int *hnb = reinterpret_cast<int *>(h + H_NB * hs);
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        const int nb = hnb[b];
        if (nb == 0) continue;
        atomicAdd(&out.weights[o + b], (double)h[H_WE * hs + b] + (double)h[H_WEL * hs + b]);
        atomicAdd(&out.xi[o + b], (double)h[H_XI * hs + b] + (double)h[H_XIL * hs + b]);
        atomicAdd(&out.r_par[o + b], (double)h[H_PW * hs + b] / fc.inv_p);
        atomicAdd(&out.r_trans[o + b], (double)h[H_TW * hs + b] / fc.inv_t);
        atomicAdd(&out.z[o + b], 0.5 * (double)h[H_ZW * hs + b]);
        atomicAdd((unsigned long long *)&out.num_pairs[o + b], (unsigned long long)nb);
#pragma unroll
        for (int k = 0; k < H_NB; ++k) h[k * hs + b] = 0.f;
        hnb[b] = 0;
    }
}

__device__ __forceinline__ void zero_all(float *h, int hs) {
    for (int b = threadIdx.x; b < H_COUNT * hs; b += blockDim.x) h[b] = 0.f;
}

__device__ __forceinline__ int next_item(Scratch *scratch, int *slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(&scratch->work_counter, 1);
    __syncthreads();
    return *slot;
}

// ---------------------------------------------------------------------------
// cf
// ---------------------------------------------------------------------------
struct CfPairCtx {
    int64_t a0, b0;
    double ang, c, s;
    bool shp;
};

// FP64 re-decision of queued (i, j) pairs, then FP32 accumulation.
__device__ __forceinline__ void cf_drain(const Binning &b, const FastConst *__restrict__ fcp,
                                      const pg_forest_set &s1, const pg_forest_set &s2,
                                      CfPairCtx ctx, const uint32_t *queue, int count, float *h,
                                      Scratch *scratch) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const int hs = fcp->hstride;
    for (int e = lane; e < count; e += 32) {
        const uint32_t entry = queue[e];
        const int64_t ia = ctx.a0 + (entry >> 16), jb = ctx.b0 + (entry & 0xFFFF);
        const double z1 = s1.z[ia], z2 = s2.z[jb];
        double r_par, r_trans, z;
        const int64_t bin = cf_pair_bin(b, z1, s1.r_comov[ia], s1.dist_m[ia], z2, s2.r_comov[jb],
                                        s2.dist_m[jb], ctx.ang, ctx.c, ctx.s, ctx.shp, r_par,
                                        r_trans, z);
        if (bin < 0) continue;
        if (bin >= b.nbins) {
            report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bin);
            continue;
        }
        const double w1 = s1.weights[ia], w2 = s2.weights[jb];
        const float w12 = weight32(w1) * weight32(w2);
        const float dw12 = (float)(s1.delta[ia] * w1) * (float)(s2.delta[jb] * w2);
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)z2;
        acc_pair(h, hs, (int)bin, dw12, w12, pv * w12, tv * w12, zs * w12);
    }
    __syncwarp();
}

// EXTRA: half-plate veto, z-pair cuts or zerr cut may be active.
template <bool AUTO, bool EXTRA>
__global__ void __launch_bounds__(kCfBlock, 2) cf_xi_fast_kernel(
    const __grid_constant__ Binning b, const FastConst *__restrict__ fcp,
    const __grid_constant__ pg_forest_set s1, const __grid_constant__ pg_forest_set s2,
    const int64_t *__restrict__ nbr_offsets, const int32_t *__restrict__ nbr_index,
    const double *__restrict__ nbr_angle, const int32_t *__restrict__ work_order,
    int64_t num_work, const __grid_constant__ pg_xi_rows out, Scratch *scratch, int max_pix1) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int hs = fcp->hstride;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pmin = fcp->pmin;
    const float g_par = fcp->g_par, g_tr = fcp->g_tr;
    const float omg_par = fcp->one_m_g_par, omg_tr = fcp->one_m_g_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    const bool lower_exact = AUTO && fcp->lower_exact;
    float *h = reinterpret_cast<float *>(smem);
    float4 *p1 = reinterpret_cast<float4 *>(h + H_COUNT * hs);
    float2 *p2 = reinterpret_cast<float2 *>(p1 + max_pix1);
    uint32_t *queue = reinterpret_cast<uint32_t *>(p2 + max_pix1) + warp * kQueue;
    __shared__ long long nbr_next;
    zero_all(h, hs);
    unsigned long long rechecks = 0, overflows = 0;

    for (;;) {
        const int item = next_item(scratch, &item_slot);
        if (item >= num_work) break;
        const int64_t f1 = work_order ? work_order[item] : item;
        const int32_t row = s1.row[f1];
        const int64_t a0 = s1.pix_offset[f1];
        const int64_t n1_64 = s1.pix_offset[f1 + 1] - a0;
        if (n1_64 > max_pix1 || n1_64 > 65535) {
            if (threadIdx.x == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)f1);
            continue;
        }
        const int n1 = (int)n1_64;
        // stage forest 1 in FP32: r as (hi, lo), dist_m, z; (w, delta*w)
        for (int i = threadIdx.x; i < n1; i += blockDim.x) {
            const double w = s1.weights[a0 + i];
            const double r = s1.r_comov[a0 + i];
            const float rh = (float)r;
            p1[i] = make_float4(rh, (float)(r - (double)rh), (float)s1.dist_m[a0 + i],
                                (float)s1.z[a0 + i]);
            p2[i] = make_float2(weight32(w), (float)(s1.delta[a0 + i] * w));
        }
        const double x1 = s1.x_cart[f1], y1 = s1.y_cart[f1], zc1 = s1.z_cart[f1];
        const double ra1 = s1.ra[f1], dec1 = s1.dec[f1], cd1 = s1.cos_dec[f1];
        const double zq1 = s1.z_qso[f1];
        const int64_t k0 = nbr_offsets[f1], k1 = nbr_offsets[f1 + 1];
        if (threadIdx.x == 0) nbr_next = k0;
        __syncthreads();
        for (;;) {
            // warps take neighbour forests dynamically (balances uneven lengths)
            int64_t k = 0;
            if (lane == 0) k = (int64_t)atomicAdd((unsigned long long *)&nbr_next, 1ull);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= k1) break;
            CfPairCtx ctx;
            const int64_t g = nbr_index[k];
            ctx.a0 = a0;
            ctx.b0 = s2.pix_offset[g];
            const int64_t n2_64 = s2.pix_offset[g + 1] - ctx.b0;
            if (n2_64 > 65535) {
                if (lane == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)g);
                continue;
            }
            const int n2 = (int)n2_64;
            ctx.ang = nbr_angle ? nbr_angle[k]
                                : angle_between(x1, y1, zc1, ra1, dec1, cd1, s2.x_cart[g],
                                                s2.y_cart[g], s2.z_cart[g], s2.ra[g], s2.dec[g]);
            ctx.c = cos(ctx.ang / 2);
            ctx.s = sin(ctx.ang / 2);
            ctx.shp = false;
            bool zerr_pair = false;
            double zq2 = 0.;
            if (EXTRA) {
                if (b.remove_shp) {
                    const int64_t fb1 = s1.fiberid[f1], fb2 = s2.fiberid[g];
                    ctx.shp = (s1.plate[f1] == s2.plate[g]) &&
                              ((fb1 <= 500 && fb2 <= 500) || (fb1 > 500 && fb2 > 500));
                }
                zerr_pair = b.zerr_on && (ctx.ang < b.zerr_ang);
                zq2 = s2.z_qso[g];
            }
            const float cp = (float)(ctx.c * inv_p);
            const float st = (float)(ctx.s * inv_t);
            int qn = 0;
            for (int jb = 0; jb < n2; jb += 32 * kCfP) {
                float rh[kCfP], rl[kCfP], t[kCfP], zv[kCfP], wv[kCfP], dv[kCfP];
                unsigned vmask = 0;
#pragma unroll
                for (int p = 0; p < kCfP; ++p) {
                    const int j = jb + lane + 32 * p;
                    rh[p] = 0.f; rl[p] = 0.f; t[p] = 0.f; zv[p] = 0.f; wv[p] = 0.f; dv[p] = 0.f;
                    if (j < n2) {
                        const int64_t jj = ctx.b0 + j;
                        const double w2 = s2.weights[jj];
                        bool ok = w2 != 0;
                        if (EXTRA && zerr_pair && ok) ok = !zerr_veto(s2.z[jj], zq1, b.zerr_kms);
                        if (ok) {
                            vmask |= 1u << p;
                            const double r = s2.r_comov[jj];
                            rh[p] = (float)r;
                            rl[p] = (float)(r - (double)rh[p]);
                            t[p] = st * (float)s2.dist_m[jj];
                            zv[p] = (float)s2.z[jj];
                            wv[p] = weight32(w2);
                            dv[p] = (float)(s2.delta[jj] * w2);
                        }
                    }
                }
                if (__ballot_sync(0xffffffffu, vmask != 0) == 0) continue;
                for (int i = 0; i < n1; ++i) {
                    const float2 qw = p2[i];
                    if (qw.x == 0.f) continue;  // zero-weight pixel (warp-uniform)
                    if (EXTRA && zerr_pair && zerr_veto(s1.z[a0 + i], zq2, b.zerr_kms)) continue;
                    const float4 q = p1[i];
                    const float dw1 = qw.y;
                    const float ui = st * q.z;
                    unsigned near_mask = 0;
#pragma unroll
                    for (int p = 0; p < kCfP; ++p) {
                        const float diff = cp * ((q.x - rh[p]) + (q.y - rl[p]));
                        const float v = fabsf(diff);
                        const float pv = AUTO ? v : diff;
                        const float tv = ui + t[p];
                        float fp, ft;
                        const unsigned ip = floor_frac(pv - pmin, fp);
                        const unsigned it = floor_frac(tv, ft);
                        bool near = ((fp < g_par) & ((ip != 0u) | !lower_exact)) | (fp > omg_par) |
                                    (ft < g_tr) | (ft > omg_tr);
                        bool ok = (ip < np) & (it < nt);
                        const float zs = q.w + zv[p];
                        if (EXTRA) {
                            if (ctx.shp) {
                                near |= fabsf(v - 1.f) < fcp->guard_v;
                                ok &= !(v < 1.f);
                            }
                            if (b.zmin_on) {
                                near |= fabsf(zs - fcp->zmin2) < fcp->guard_z;
                                ok &= !(zs < fcp->zmin2);
                            }
                            if (b.zmax_on) {
                                near |= fabsf(zs - fcp->zmax2) < fcp->guard_z;
                                ok &= !(zs > fcp->zmax2);
                            }
                        }
                        const bool valid = (vmask >> p) & 1u;
                        near_mask |= (unsigned)(near & valid) << p;
                        if (ok & valid & !near) {
                            const float w12 = qw.x * wv[p];
                            acc_pair(h, hs, (int)(ip * nt + it), dw1 * dv[p], w12, pv * w12,
                                     tv * w12, zs * w12);
                        }
                    }
                    if (__any_sync(0xffffffffu, near_mask != 0)) {
                        // rare path: queue the pairs near an edge for FP64 re-decision
#pragma unroll
                        for (int p = 0; p < kCfP; ++p) {
                            const bool near = (near_mask >> p) & 1u;
                            const unsigned nmask = __ballot_sync(0xffffffffu, near);
                            if (!nmask) continue;
                            const int cnt = __popc(nmask);
                            if (qn + cnt > kQueue) {
                                cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
                                rechecks += qn;
                                ++overflows;
                                qn = 0;
                            }
                            if (near) {
                                const int pos = qn + __popc(nmask & ((1u << lane) - 1u));
                                queue[pos] = ((uint32_t)i << 16) | (uint32_t)(jb + lane + 32 * p);
                            }
                            qn += cnt;
                        }
                    }
                }
            }
            if (qn) {
                cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
                rechecks += qn;
            }
        }
        __syncthreads();
        flush_rows(h, *fcp, out, row);
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
    if (lane == 0) {
        // per-warp counters are warp-uniform
        atomicAdd(&scratch->rechecked_pairs, rechecks);
        atomicAdd(&scratch->recheck_overflows, overflows);
    }
}

// ---------------------------------------------------------------------------
// xcf
// ---------------------------------------------------------------------------
struct XcfCtx {
    int64_t a0, k0;
    double x1, y1, zc1, ra1, dec1, cd1;
};

__device__ __forceinline__ void xcf_drain(const Binning &b, const FastConst *__restrict__ fcp,
                                       const pg_forest_set &fs, const pg_forest_set &objs,
                                       const int32_t *__restrict__ nbr_index,
                                       const double *__restrict__ nbr_angle, XcfCtx ctx,
                                       const uint32_t *queue, int count, float *h,
                                       Scratch *scratch) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const int hs = fcp->hstride;
    for (int e = lane; e < count; e += 32) {
        const uint32_t entry = queue[e];
        const int64_t ia = ctx.a0 + (entry >> 16);
        const int64_t kabs = ctx.k0 + (entry & 0xFFFF);
        const int64_t g = nbr_index[kabs];
        const double ang = nbr_angle ? nbr_angle[kabs]
                                     : angle_between(ctx.x1, ctx.y1, ctx.zc1, ctx.ra1, ctx.dec1,
                                                     ctx.cd1, objs.x_cart[g], objs.y_cart[g],
                                                     objs.z_cart[g], objs.ra[g], objs.dec[g]);
        const double z1 = fs.z[ia], zq = objs.z_qso[g];
        double r_par, r_trans, z;
        const int64_t bin = xcf_pair_bin(b, z1, fs.r_comov[ia], fs.dist_m[ia], zq,
                                         objs.obj_r_comov[g], objs.obj_dist_m[g], ang,
                                         cos(ang / 2), sin(ang / 2), r_par, r_trans, z);
        if (bin < 0) continue;
        if (bin >= b.nbins) {
            report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bin);
            continue;
        }
        const double w1 = fs.weights[ia], wq = objs.obj_weight[g];
        const float w12 = weight32(w1) * weight32(wq);
        const float dw = (float)(fs.delta[ia] * w1) * weight32(wq);
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)zq;
        acc_pair(h, hs, (int)bin, dw, w12, pv * w12, tv * w12, zs * w12);
    }
    __syncwarp();
}

template <bool EXTRA>
__global__ void __launch_bounds__(512, 1) xcf_xi_fast_kernel(
    const __grid_constant__ Binning b, const FastConst *__restrict__ fcp,
    const __grid_constant__ pg_forest_set fs, const __grid_constant__ pg_forest_set objs,
    const int64_t *__restrict__ nbr_offsets, const int32_t *__restrict__ nbr_index,
    const double *__restrict__ nbr_angle, const int32_t *__restrict__ work_order,
    int64_t num_work, const __grid_constant__ pg_xi_rows out, Scratch *scratch, int max_pix1) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int hs = fcp->hstride;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pmin = fcp->pmin;
    const float g_par = fcp->g_par, g_tr = fcp->g_tr;
    const float omg_par = fcp->one_m_g_par, omg_tr = fcp->one_m_g_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    float *h = reinterpret_cast<float *>(smem);
    float4 *p1 = reinterpret_cast<float4 *>(h + H_COUNT * hs);
    float2 *p2 = reinterpret_cast<float2 *>(p1 + max_pix1);
    uint32_t *queue = reinterpret_cast<uint32_t *>(p2 + max_pix1) + warp * kQueue;
    zero_all(h, hs);
    unsigned long long rechecks = 0, overflows = 0;

    for (;;) {
        const int item = next_item(scratch, &item_slot);
        if (item >= num_work) break;
        const int64_t f = work_order ? work_order[item] : item;
        const int32_t row = fs.row[f];
        XcfCtx ctx;
        ctx.a0 = fs.pix_offset[f];
        const int64_t n1_64 = fs.pix_offset[f + 1] - ctx.a0;
        const int64_t nq_64 = nbr_offsets[f + 1] - nbr_offsets[f];
        if (n1_64 > max_pix1 || n1_64 > 65535 || nq_64 > 65535) {
            if (threadIdx.x == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)f);
            continue;
        }
        const int n1 = (int)n1_64;
        for (int i = threadIdx.x; i < n1; i += blockDim.x) {
            const double w = fs.weights[ctx.a0 + i];
            const double r = fs.r_comov[ctx.a0 + i];
            const float rh = (float)r;
            p1[i] = make_float4(rh, (float)(r - (double)rh), (float)fs.dist_m[ctx.a0 + i],
                                (float)fs.z[ctx.a0 + i]);
            p2[i] = make_float2(weight32(w), (float)(fs.delta[ctx.a0 + i] * w));
        }
        __syncthreads();
        ctx.x1 = fs.x_cart[f]; ctx.y1 = fs.y_cart[f]; ctx.zc1 = fs.z_cart[f];
        ctx.ra1 = fs.ra[f]; ctx.dec1 = fs.dec[f]; ctx.cd1 = fs.cos_dec[f];
        ctx.k0 = nbr_offsets[f];
        const int nq = (int)nq_64;
        for (int kb = warp * 32 * kXcfP; kb < nq; kb += nwarps * 32 * kXcfP) {
            float cp[kXcfP], st[kXcfP], rh[kXcfP], rl[kXcfP], t[kXcfP], zv[kXcfP], wv[kXcfP];
            unsigned vmask = 0;
#pragma unroll
            for (int p = 0; p < kXcfP; ++p) {
                const int kk = kb + lane + 32 * p;
                cp[p] = 0.f; st[p] = 0.f; rh[p] = 0.f; rl[p] = 0.f; t[p] = 0.f; zv[p] = 0.f;
                wv[p] = 0.f;
                if (kk < nq) {
                    const int64_t g = nbr_index[ctx.k0 + kk];
                    const double wq = objs.obj_weight[g];
                    if (wq != 0) {
                        vmask |= 1u << p;
                        const double ang =
                            nbr_angle ? nbr_angle[ctx.k0 + kk]
                                      : angle_between(ctx.x1, ctx.y1, ctx.zc1, ctx.ra1, ctx.dec1,
                                                      ctx.cd1, objs.x_cart[g], objs.y_cart[g],
                                                      objs.z_cart[g], objs.ra[g], objs.dec[g]);
                        cp[p] = (float)(cos(ang / 2) * inv_p);
                        st[p] = (float)(sin(ang / 2) * inv_t);
                        const double r = objs.obj_r_comov[g];
                        rh[p] = (float)r;
                        rl[p] = (float)(r - (double)rh[p]);
                        t[p] = st[p] * (float)objs.obj_dist_m[g];
                        zv[p] = (float)objs.z_qso[g];
                        wv[p] = weight32(wq);
                    }
                }
            }
            if (__ballot_sync(0xffffffffu, vmask != 0) == 0) continue;
            int qn = 0;
            for (int i = 0; i < n1; ++i) {
                const float2 qw = p2[i];
                if (qw.x == 0.f) continue;
                const float4 q = p1[i];
                const float dw1 = qw.y;
                unsigned near_mask = 0;
#pragma unroll
                for (int p = 0; p < kXcfP; ++p) {
                    const float pv = cp[p] * ((q.x - rh[p]) + (q.y - rl[p]));
                    const float tv = __fmaf_rn(st[p], q.z, t[p]);
                    float fp, ft;
                    const unsigned ip = floor_frac(pv - pmin, fp);
                    const unsigned it = floor_frac(tv, ft);
                    bool near = (fp < g_par) | (fp > omg_par) | (ft < g_tr) | (ft > omg_tr);
                    bool ok = (ip < np) & (it < nt);
                    const float zs = q.w + zv[p];
                    if (EXTRA) {
                        if (b.zmin_on) {
                            near |= fabsf(zs - fcp->zmin2) < fcp->guard_z;
                            ok &= !(zs < fcp->zmin2);
                        }
                        if (b.zmax_on) {
                            near |= fabsf(zs - fcp->zmax2) < fcp->guard_z;
                            ok &= !(zs > fcp->zmax2);
                        }
                    }
                    const bool valid = (vmask >> p) & 1u;
                    near_mask |= (unsigned)(near & valid) << p;
                    if (ok & valid & !near) {
                        const float w12 = qw.x * wv[p];
                        acc_pair(h, hs, (int)(ip * nt + it), dw1 * wv[p], w12, pv * w12,
                                 tv * w12, zs * w12);
                    }
                }
                if (__any_sync(0xffffffffu, near_mask != 0)) {
#pragma unroll
                    for (int p = 0; p < kXcfP; ++p) {
                        const bool near = (near_mask >> p) & 1u;
                        const unsigned nmask = __ballot_sync(0xffffffffu, near);
                        if (!nmask) continue;
                        const int cnt = __popc(nmask);
                        if (qn + cnt > kQueue) {
                            xcf_drain(b, fcp, fs, objs, nbr_index, nbr_angle, ctx, queue, qn, h,
                                      scratch);
                            rechecks += qn;
                            ++overflows;
                            qn = 0;
                        }
                        if (near) {
                            const int pos = qn + __popc(nmask & ((1u << lane) - 1u));
                            queue[pos] = ((uint32_t)i << 16) | (uint32_t)(kb + lane + 32 * p);
                        }
                        qn += cnt;
                    }
                }
            }
            if (qn) {
                xcf_drain(b, fcp, fs, objs, nbr_index, nbr_angle, ctx, queue, qn, h, scratch);
                rechecks += qn;
            }
        }
        __syncthreads();
        flush_rows(h, *fcp, out, row);
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
    if (lane == 0) {
        atomicAdd(&scratch->rechecked_pairs, rechecks);
        atomicAdd(&scratch->recheck_overflows, overflows);
    }
}

// Guard bands. Let u = 2^-24. r is carried as rh + rl with |r - rh - rl|
// <= u^2 r (negligible), so r1 - r2 = (r1h - r2h) + (r1l - r2l) is formed
// with two roundings of size u |r1 - r2| and u |r1l - r2l|; the product with
// cp (itself rounded, relative u) and the subtraction of pmin add u |p| and
// u |x|. Altogether |x_par(FP32) - x_par| <= 6 u (|x| + |pmin| + 1). For
// x_tr = st d1 + st d2 the FP32 rounding of d1 and d2 (relative u), of the
// two products, of st and of the sum give <= 5 u |x_tr|. Only pairs whose
// exact x lies in [-1, n + 1] matter (the others are rejected either way),
// so with a factor > 2 of margin
//   g = 16 u (n + |pmin| + 2) + 1e-6.
// The reference's own FP64 evaluation is within 1e-12 of the exact value,
// far inside these bands.
FastConst make_fast_const(const Binning &b) {
    FastConst fc{};
    const double u = 1.0 / 16777216.0;
    fc.inv_p = (double)b.np / b.r_par_range;
    fc.inv_t = (double)b.nt / b.r_trans_max;
    fc.pmin = (float)(b.r_par_min * fc.inv_p);
    double g_par = 16 * u * (b.np + fabs(b.r_par_min * fc.inv_p) + 2) + 1e-6;
    double g_tr = 16 * u * (b.nt + 2) + 1e-6;
    if (!(g_par < 0.05)) g_par = 0.05;  // absurd bin counts: almost everything is re-decided
    if (!(g_tr < 0.05)) g_tr = 0.05;
    fc.g_par = (float)g_par;
    fc.g_tr = (float)g_tr;
    fc.one_m_g_par = (float)(1.0 - g_par);
    fc.one_m_g_tr = (float)(1.0 - g_tr);
    fc.guard_v = (float)g_par;
    fc.guard_z = 1e-5f;  // z1 + z2 < 20: FP32 error below 5e-6
    fc.zmin2 = (float)(2 * b.z_min);
    fc.zmax2 = (float)(2 * b.z_max);
    fc.np = (unsigned)b.np;
    fc.nt = (unsigned)b.nt;
    fc.nbins = b.nbins;
    fc.hstride = (b.nbins + 3) & ~3;
    fc.lower_exact = (!b.x_correlation && b.r_par_min == 0.0) ? 1 : 0;
    return fc;
}

// Writes the constants into the plan's device buffer in stream order.
__global__ void store_const_kernel(FastConst value, FastConst *dst) { *dst = value; }

size_t fast_smem_bytes(int hstride, int max_pix1, int nwarps) {
    return (size_t)hstride * H_COUNT * 4 + (size_t)max_pix1 * 24 + (size_t)nwarps * kQueue * 4;
}

template <typename K>
int persistent_grid(K kernel, int block, size_t smem, int num_sms, int64_t num_work, int *grid) {
    cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (err != cudaSuccess) return check_cuda(err);
    if (per_sm < 1) return PG_ERR_UNSUPPORTED;
    int64_t g = (int64_t)num_sms * per_sm;
    if (g > num_work) g = num_work;
    *grid = (int)(g < 1 ? 1 : g);
    return PG_OK;
}

int prepare_fast(const Binning &b, FastConst *fc, cudaStream_t stream) {
    store_const_kernel<<<1, 1, 0, stream>>>(make_fast_const(b), fc);
    return check_cuda(cudaGetLastError());
}

}  // namespace

size_t fast_const_bytes() { return (sizeof(FastConst) + 255) & ~(size_t)255; }

int launch_cf_xi_fast(const Binning &b, double ang_max, const pg_forest_set &s1,
                      const pg_forest_set &s2, const int64_t *nbr_offsets,
                      const int32_t *nbr_index, const double *nbr_angle,
                      const int32_t *work_order, int64_t num_work,
                      const pg_xi_rows &out, Scratch *scratch, void *fast_const, int num_sms,
                      cudaStream_t stream) {
    if (num_work <= 0) return PG_OK;
    FastConst *fc = static_cast<FastConst *>(fast_const);
    const int block = kCfBlock;
    const int max_pix1 = s1.max_pixels;
    const size_t smem = fast_smem_bytes((b.nbins + 3) & ~3, max_pix1, block / 32);
    if (smem > 227 * 1024) return PG_ERR_UNSUPPORTED;
    (void)ang_max;
    int rc = prepare_fast(b, fc, stream);
    if (rc) return rc;
    const bool extra = b.remove_shp || b.zmin_on || b.zmax_on || b.zerr_on;
    const bool autoc = !b.x_correlation;
    int grid = 0;
#define PG_LAUNCH_CF(A, E)                                                                     \
    rc = persistent_grid(cf_xi_fast_kernel<A, E>, block, smem, num_sms, num_work, &grid);      \
    if (rc) return rc;                                                                         \
    cf_xi_fast_kernel<A, E><<<grid, block, smem, stream>>>(b, fc, s1, s2, nbr_offsets,         \
                                                           nbr_index, nbr_angle, work_order,   \
                                                           num_work, out, scratch, max_pix1);
    if (autoc && !extra) { PG_LAUNCH_CF(true, false) }
    else if (autoc && extra) { PG_LAUNCH_CF(true, true) }
    else if (!autoc && !extra) { PG_LAUNCH_CF(false, false) }
    else { PG_LAUNCH_CF(false, true) }
#undef PG_LAUNCH_CF
    return check_cuda(cudaGetLastError());
}

int launch_xcf_xi_fast(const Binning &b, double ang_max, const pg_forest_set &forests,
                       const pg_forest_set &objs, const int64_t *nbr_offsets,
                       const int32_t *nbr_index, const double *nbr_angle,
                       const int32_t *work_order, int64_t num_work,
                       const pg_xi_rows &out, Scratch *scratch, void *fast_const, int num_sms,
                       cudaStream_t stream) {
    if (num_work <= 0) return PG_OK;
    FastConst *fc = static_cast<FastConst *>(fast_const);
    const int block = 512;
    const int max_pix1 = forests.max_pixels;
    const size_t smem = fast_smem_bytes((b.nbins + 3) & ~3, max_pix1, block / 32);
    if (smem > 227 * 1024) return PG_ERR_UNSUPPORTED;
    (void)ang_max;
    int rc = prepare_fast(b, fc, stream);
    if (rc) return rc;
    const bool extra = b.zmin_on || b.zmax_on;
    int grid = 0;
    if (extra) {
        rc = persistent_grid(xcf_xi_fast_kernel<true>, block, smem, num_sms, num_work, &grid);
        if (rc) return rc;
        xcf_xi_fast_kernel<true><<<grid, block, smem, stream>>>(
            b, fc, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out,
            scratch, max_pix1);
    } else {
        rc = persistent_grid(xcf_xi_fast_kernel<false>, block, smem, num_sms, num_work, &grid);
        if (rc) return rc;
        xcf_xi_fast_kernel<false><<<grid, block, smem, stream>>>(
            b, fc, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out,
            scratch, max_pix1);
    }
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
