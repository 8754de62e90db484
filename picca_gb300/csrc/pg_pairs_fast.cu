// Precision-form pair accumulation: FP32 geometry with an FP64 bin-edge
// guard, double-float xi terms, compensated FP32 shared-memory block sums,
// FP64 rows.
//
// Persistent structure: one work item = one forest of set 1 with all its
// neighbours; the forest-1 pixels are staged in shared memory and warps take
// neighbours dynamically. The auto-correlation sweeps each forest pair
// along diagonals (cf_xi_diag_kernel), the cross-correlation each quasar
// along the forest (xcf_xi_fast_kernel); both sum runs of consecutive pairs
// of one bin in registers.
//
// Geometry. Comoving distances are taken relative to R, the distance of the
// middle pixel of forest 1 (one FP64 subtraction per pixel, exact), and
// rounded to FP32: rho = r - R, |rho| of the order of a forest's length
// rather than of r (~4000 Mpc/h). Per forest pair and forest-2 pixel the
// lane holds nB = -cp*rho2 (cp = cos(theta/2) * inv_p), so that for every
// pixel pair one FFMA gives
//     p   = cp*rho1 + nB                 (= r_par * np/(r_par_max - r_par_min))
//     x'  = |p| - (r_par_min*inv_p + 1/2)  (p itself for signed, cross correlations)
//     xt' = st*d1 + (st*d2 - 1/2)         (= r_trans * nt/r_trans_max - 1/2)
// with st = sin(theta/2) * inv_t. The bin index of py/picca/cf.py:372-376 is
// floor(x) = round(x'), taken with one round-to-nearest add of 1.5 * 2^23:
// y = x' + 1.5*2^23 is an integer for |x'| < 2^22, so round(x') is the bit
// pattern of y minus that of 1.5*2^23 and f = x' - (y - 1.5*2^23), in
// [-1/2, 1/2], is exact. A pair with |f| > 1/2 - g in either coordinate (a bin
// edge or an acceptance limit within the guard band g), or within a guard
// of the half-plate r_par cut or the z-pair cuts, is queued and re-decided
// in FP64 with the reference's operation order (cf_pair_bin /
// xcf_pair_bin), so every accepted pair, bin index and pair count equals
// the FP64 reference. g exceeds the worst-case FP32 error; its r_par part
// grows with the largest |rho1| of the work item (make_fast_const, and the
// per-item band computed after staging).
// Forest-2 slots past the end of the forest or with zero weight carry
// nB = t = z = 1e30 (and cp = 1 for quasars), which lands far outside every
// bin, edge and cut, so such a slot is neither accepted nor queued.
//
// xi terms. delta*w of every pixel is formed in FP64 and carried as an FP32
// pair (hi, lo) with hi + lo = delta*w to 2^-48. The product of two such
// pairs is hi1*hi2 (rounded) plus a low part: the exact rounding error of
// hi1*hi2 (one FMA) and the cross terms hi1*lo2 + lo1*hi2; the lost lo1*lo2
// is below 2^-48 of the term. Runs of accepted pairs of one lane in one bin
// sum the high parts with Knuth's TwoSum, its error going to the run's low
// part, so a run reaches the histogram as (hi, lo) with an error of order
// 2^-46 of its terms.
//
// Sums: per-CTA FP32 shared-memory histograms of xi, w, p*w, x_tr*w,
// (z1+z2)*w and an int32 count. xi (products of signed deltas, strongly
// cancelling) and w (the normalisation) are summed error-free: the atomic add
// returns the previous value, TwoSum recovers the exact rounding error of
// the add and a second histogram collects it together with the run's low
// part. Accepted pairs first go to a per-warp ring, and the warp applies
// them 32 at a time, so the eight atomic adds of a pair run with every lane
// active instead of in the divergent branch of each pair. After each work
// item the histograms are added to the FP64 rows and mapped back to picca's
// units (r_par = p/inv_p, r_trans = x_tr/inv_t, z = (z1+z2)/2).
#include <type_traits>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr float kMagic = 12582912.0f;        // 1.5 * 2^23
constexpr unsigned kMagicBits = 0x4B400000u;  // bits of 1.5 * 2^23
constexpr float kFar = 1e30f;                 // nB, t and z of an empty slot
// cos(1e-3): above it (angles below 1e-3 rad, and the reference's flat-sky
// branch below 2 arcsec) the pair kernels take cos and sin of half the angle
// from the angle itself, not from the half-angle identities
constexpr double kCosHalfAngleForm = 0.9999995;
constexpr int kQueue = 256;                   // FP64 recheck entries per warp (cross)
constexpr int kCfQueue = 128;                 // FP64 recheck entries per warp (auto)
constexpr int kAccQ = 64;                     // run ring per warp (<= 31 + 32 entries held)
constexpr int kChunk = 128;                   // forest-2 pixels staged per warp at a time
constexpr int kRunMax = 64;                   // pairs summed in FP32 registers per run
constexpr int kCfBlock = 640;
constexpr int kXcfBlock = 512;

struct FastConst {
    double inv_p, inv_t;    // histogram scales: r_par (mu with r-mu bins) and r_trans (r)
    double geom_p;          // scale of the staged r_par geometry (inv_p; the r scale with
                            // r-mu bins, where both coordinates are in r-bin units)
    float pc;               // r_par_min * inv_p + 1/2
    float g0_par;           // guard band of x' without the |rho1| term
    float g_rho;            // guard band of x' per unit of the work item's max |rho1|
    float h_tr;             // 1/2 - g_tr: |f| above this is near an r_trans edge
    float guard_z;          // guard on z1 + z2
    float zmin2, zmax2;     // 2 z_min, 2 z_max
    unsigned np, nt;
    int nbins;
    int hstride;            // histogram array stride (nbins rounded up to 4)
    int lower_exact;        // auto-correlation with r_par_min = 0: x = |p| >= 0, so
                            // the lower edge of bin 0 can never be crossed
    // r-mu binning: mu = r_par / r in bins of inv_mu = np / (mu_max - mu_min)
    float inv_mu, mu_off;   // mu_off = mu_min * inv_mu + 1/2
    float g_mu0;            // guard of x_mu without the r_par error term
};

// Guard of the r_par coordinate of one work item (see make_fast_const).
struct ParGuard {
    float h_par;      // 1/2 - g
    float low_clamp;  // -1/2 + 2 g (auto-correlation with r_par_min = 0)
    float guard_v;    // half-plate cut guard (in units of p)
};

__device__ __forceinline__ ParGuard par_guard(const FastConst *fcp, float max_rho) {
    float g = fcp->g0_par + fcp->g_rho * max_rho;
    if (!(g < 0.05f)) g = 0.05f;  // absurd bin counts: almost everything is re-decided
    ParGuard pg;
    pg.h_par = 0.5f - g;
    pg.low_clamp = -0.5f + 2.f * g;
    pg.guard_v = g;
    return pg;
}

// ---------------------------------------------------------------------------
// shared-memory histograms: H_COUNT float arrays of stride hstride
// ---------------------------------------------------------------------------
enum { H_XI = 0, H_XIL, H_WE, H_WEL, H_PW, H_TW, H_ZW, H_NB, H_COUNT };

// One run of pairs into the histograms. xi (given as hi + lo) and w are
// compensated: the atomic add returns the previous value, Knuth's TwoSum of
// it and the term gives the exact rounding error of the add, which goes to
// the error histogram together with xi's low part. The two adds whose
// previous value is needed go first, so that their round trips overlap the
// four plain adds.
__device__ __forceinline__ void hist_add(float *h, int hs, unsigned bin, float xi, float xil,
                                         float w, float pw, float tw, float zw, int count) {
    float *hx = h + bin;
    const float oxi = atomicAdd(hx + H_XI * hs, xi);
    const float owe = atomicAdd(hx + H_WE * hs, w);
    atomicAdd(hx + H_PW * hs, pw);
    atomicAdd(hx + H_TW * hs, tw);
    atomicAdd(hx + H_ZW * hs, zw);
    atomicAdd(reinterpret_cast<int *>(hx + H_NB * hs), count);
    float sum = oxi + xi, bb = sum - oxi;
    atomicAdd(hx + H_XIL * hs, ((oxi - (sum - bb)) + (xi - bb)) + xil);
    sum = owe + w;
    bb = sum - owe;
    atomicAdd(hx + H_WEL * hs, (owe - (sum - bb)) + (w - bb));
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

__device__ __forceinline__ void zero_all(float *h, int n) {
    for (int b = threadIdx.x; b < n; b += blockDim.x) h[b] = 0.f;
}

// Next work item of the persistent CTA; also clears the work item's
// max |rho1| (written by the staging loop after the second barrier).
__device__ __forceinline__ int next_item(Scratch *scratch, int *slot, unsigned *max_rho_bits) {
    __syncthreads();
    if (threadIdx.x == 0) {
        *slot = atomicAdd(&scratch->work_counter, 1);
        *max_rho_bits = 0u;
    }
    __syncthreads();
    return *slot;
}

// FP32 value of a weight that stays nonzero when the FP64 weight is nonzero
// (a weight below the FP32 range still counts its pairs, as in FP64).
__device__ __forceinline__ float weight32(double w) {
    const float f = (float)w;
    if (f == 0.f && w != 0.) return w > 0 ? 1.401298464e-45f : -1.401298464e-45f;
    return f;
}

// x as an FP32 pair hi + lo (equal to x to about 2^-48 of |x|).
__device__ __forceinline__ float2 split2(double x) {
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// (ah + al) * (bh + bl) = ph + pl: ph the rounded product of the high
// parts, pl its exact rounding error (one FMA) plus the cross terms.
__device__ __forceinline__ void two_prod(float ah, float al, float bh, float bl, float &ph,
                                         float &pl) {
    ph = __fmul_rn(ah, bh);
    pl = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, __fmaf_rn(ah, bh, -ph)));
}

// s + x with TwoSum: s becomes the rounded sum, its exact error goes to lo.
__device__ __forceinline__ void two_sum_into(float &s, float &lo, float x) {
    const float t = s + x;
    const float bb = t - s;
    lo += (s - (t - bb)) + (x - bb);
    s = t;
}

// round(x) (as unsigned; negative results wrap to large values) and the
// remainder x - round(x) in [-1/2, 1/2].
__device__ __forceinline__ unsigned round_rem(float x, float &rem) {
    const float y = x + kMagic;
    rem = x - (y - kMagic);
    return __float_as_uint(y) - kMagicBits;
}

// Shared-memory layout of the cross-correlation kernel (byte offsets from
// the start). p1: float4 (rho, dist_m, z, w) per forest pixel; p2: float4
// (delta*w hi, lo, rho lo, 0); queue: the FP64 re-decision entries.
struct SmemLayout {
    size_t cells, p1, p2, acc0, acc1, queue, order, buckets, total;
};

// The cross-correlation kernel visits a forest's quasars in order of
// distance (kXcfBuckets buckets of kXcfBucketMpc along the line of sight,
// relative to the forest's middle pixel) when it has at most kXcfOrderMax.
constexpr int kXcfOrderMax = 4096;
constexpr int kXcfBuckets = 128;
constexpr float kXcfBucketMpc = 8.f;

__host__ __device__ inline SmemLayout smem_layout(int nbins, int max_pix1, int nwarps,
                                                  bool acc_queue) {
    SmemLayout l;
    const size_t mp = (size_t)((max_pix1 + 1) & ~1);
    l.cells = 0;
    l.p1 = l.cells + (size_t)((nbins + 3) & ~3) * H_COUNT * 4;
    l.p2 = l.p1 + mp * 16;
    l.acc0 = l.p2 + mp * 16;
    l.acc1 = l.acc0 + (acc_queue ? (size_t)nwarps * kAccQ * 16 : 0);
    l.queue = l.acc1 + (acc_queue ? (size_t)nwarps * kAccQ * 16 : 0);
    l.order = l.queue + (size_t)nwarps * kQueue * 4;
    l.buckets = l.order + (acc_queue ? (size_t)kXcfOrderMax * 2 : 0);
    l.total = l.buckets + (acc_queue ? (size_t)kXcfBuckets * 4 : 0);
    return l;
}

// Stages a forest of set 1 (n1 pixels from a0) in shared memory relative to
// r_ref: p1 = (rho, dist_m, z, w), p2 = (delta*w hi, lo, rho lo, 0) with
// rho + rho lo = r - r_ref to 2^-48 (the low part sharpens the r_par that is
// summed, not the bin decision). Records the largest |rho| in *max_rho_bits
// (a non-negative float's bits order as unsigned). Returns whether rho and
// dist_m are non-decreasing along the forest (block-wide, after a barrier).
__device__ __forceinline__ bool stage_forest1(const pg_forest_set &s1, int64_t a0, int n1,
                                              double r_ref, float4 *p1, float4 *p2,
                                              unsigned *max_rho_bits) {
    bool ordered = true;
    float local_max = 0.f;
    for (int i = threadIdx.x; i < n1; i += blockDim.x) {
        const double w = s1.weights[a0 + i];
        const double rho_d = s1.r_comov[a0 + i] - r_ref;
        const float rho = (float)rho_d;
        const float d = (float)s1.dist_m[a0 + i];
        p1[i] = make_float4(rho, d, (float)s1.z[a0 + i], weight32(w));
        const float2 dw = split2(s1.delta[a0 + i] * w);
        p2[i] = make_float4(dw.x, dw.y, (float)(rho_d - (double)rho), 0.f);
        local_max = fmaxf(local_max, fabsf(rho));
        if (i + 1 < n1)
            ordered &= (float)(s1.r_comov[a0 + i + 1] - r_ref) >= rho &&
                       (float)s1.dist_m[a0 + i + 1] >= d;
    }
    if (local_max > 0.f) atomicMax(max_rho_bits, __float_as_uint(local_max));
    return __syncthreads_and(ordered) != 0;
}

// ---------------------------------------------------------------------------
// cf
// ---------------------------------------------------------------------------
struct CfPairCtx {
    int64_t a0, b0;
    double ang, c, s, zq2;
    bool shp;
};

// FP64 re-decision of queued (i, j) pairs, then accumulation.
__device__ __forceinline__ void cf_drain(const Binning &b, const FastConst *__restrict__ fcp,
                                      const pg_forest_set &s1, const pg_forest_set &s2,
                                      const CfPairCtx &ctx, const uint32_t *queue, int count,
                                      float *h, Scratch *scratch) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
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
        // delta_times_weight1 * delta_times_weight2 (py/picca/cf.py:367-369)
        const float2 dw12 = split2((s1.delta[ia] * w1) * (s2.delta[jb] * w2));
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)z2;
        hist_add(h, fcp->hstride, (unsigned)bin, dw12.x, dw12.y, w12, pv * w12, tv * w12,
                 zs * w12, 1);
    }
    if (lane == 0) atomicAdd(&scratch->rechecked_pairs, (unsigned long long)count);
    __syncwarp();
}

// Applies n (<= 32) ring entries starting at position head. An entry is a
// run of accepted pairs of one lane in one bin (consecutive pairs of one
// diagonal): {sum dw1 dw2 (hi, lo), sum w1 w2, sum p w} and {sum x_tr w,
// sum (z1 + z2) w, bin, pairs}.
template <bool FULL>
__device__ __forceinline__ void apply_runs(const float4 *acc0, const float4 *acc1, int head,
                                           int n, float *h, int hs) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    if (FULL || lane < n) {  // FULL: n = 32, no divergence
        const int e = (head + lane) & (kAccQ - 1);
        const float4 v = acc0[e];
        const float4 u = acc1[e];
        hist_add(h, hs, __float_as_uint(u.z), v.x, v.y, v.z, v.w, u.x, u.y,
                 (int)__float_as_uint(u.w));
    }
    __syncwarp();
}

// Number of leading entries of a non-increasing sequence x[0..n) (the .x
// field of the staged forest-2 records) above v (OR_EQUAL: not below v).
template <bool OR_EQUAL>
__device__ __forceinline__ int count_leading(const float4 *x, int n, float v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float y = x[mid].x;
        if (OR_EQUAL ? y >= v : y > v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Shared-memory layout of the auto-correlation kernel (byte offsets):
// block histograms; forest 1 as float4 (rho, dist_m, z, w) and float4
// (delta*w hi, lo, rho lo, 0); then per warp the staged forest-2 chunk as
// float4 (nB, t, z, w) and float4 (delta*w hi, lo, nB lo, 0), the run ring
// (two float4 per entry), the FP64 re-decision queue and the forest-1 zerr
// veto bits.
struct CfSmem {
    size_t cells, p1, p1x, warps, per_warp, buf, bufx, acc0, acc1, queue, veto, total;
};

__host__ __device__ inline CfSmem cf_smem(int nbins, int max_pix1, int nwarps) {
    CfSmem l;
    const size_t mp = (size_t)((max_pix1 + 1) & ~1);
    l.cells = 0;
    l.p1 = (size_t)((nbins + 3) & ~3) * H_COUNT * 4;
    l.p1x = l.p1 + mp * 16;
    l.warps = l.p1x + mp * 16;
    l.buf = 0;
    l.bufx = l.buf + (size_t)kChunk * 16;
    l.acc0 = l.bufx + (size_t)kChunk * 16;
    l.acc1 = l.acc0 + (size_t)kAccQ * 16;
    l.queue = l.acc1 + (size_t)kAccQ * 16;
    l.veto = l.queue + (size_t)kCfQueue * 4;
    l.per_warp = (l.veto + ((mp + 31) / 32) * 4 + 15) & ~(size_t)15;
    l.total = l.warps + (size_t)nwarps * l.per_warp;
    return l;
}

// The auto-correlation (and the correlation of two delta fields) as sweeps
// along diagonals. For a forest pair the pixel pairs (i, j) with j - i = d
// form diagonal d; along it r1 - r2 and d1 + d2 change slowly (pixels on the
// same wavelength grid), so consecutive pairs of a diagonal share their bin
// for tens of steps. A lane owns one diagonal of a group of 32 consecutive
// ones and steps along it with the others, two pairs per step: the lanes
// share the forest-2 pixel j of the warp's staged chunk (a broadcast read of
// shared memory) and each reads its own forest-1 pixel i = j - d, so that
// the group's ranges share the chunk's ends. Consecutive accepted pairs of
// one bin are summed in registers (a run); a run goes to the block
// histogram only when its bin changes, through a ring that applies 32 runs
// with every lane active.
//
// Work skipped, every skip exact: forest 2 is staged in chunks of kChunk
// pixels; per chunk, binary searches give for every forest-1 pixel i the
// forest-2 pixels whose p = cp*rho1 + nB lies within one bin of the
// accepted r_par range, hence the band of diagonals [D_lo, D_hi) holding
// every such pair (requires rho non-decreasing along both forests, checked;
// otherwise every diagonal is swept). Along a diagonal x_tr' = st d1 + t is
// non-decreasing (d non-decreasing, checked), so a binary search ends each
// lane's sweep at the first pair with x_tr' >= nt + 1. Skipped pairs are at
// least one bin outside the accepted ranges, so the reference rejects them
// too.
//
// EXTRA: half-plate veto, z-pair cuts or zerr cut may be active.
// LOWX: auto-correlation with r_par_min = 0 (lower edge of bin 0 exempt).
// RMU: r-mu bins (--rmu-binning, py/picca/cf.py:354-358; not with EXTRA):
// both coordinates are staged in r-bin units, so that per pair
// r = sqrt(p^2 + t^2) (one FMA and a reciprocal square root) and
// mu = |p| / r (p / r for two fields); the guard of mu grows as the absolute
// error of p over r, and pairs at r ~ 0 (or whose mu guard exceeds 1/4) are
// re-decided in FP64. Runs along diagonals work as before: r and mu change
// slowly along a diagonal. The r_par histogram sums mu w, the r_trans one
// r w in r-bin units.
template <bool AUTO, bool EXTRA, bool LOWX, bool RMU>
__global__ void __launch_bounds__(kCfBlock, 1) cf_xi_diag_kernel(
    const __grid_constant__ Binning b, const FastConst *__restrict__ fcp,
    const __grid_constant__ pg_forest_set s1, const __grid_constant__ pg_forest_set s2,
    const int64_t *__restrict__ nbr_offsets, const int32_t *__restrict__ nbr_index,
    const double *__restrict__ nbr_angle, const int32_t *__restrict__ work_order,
    int64_t num_work, const __grid_constant__ pg_xi_rows out, Scratch *scratch, int max_pix1) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    __shared__ unsigned max_rho_bits;
    __shared__ long long nbr_next;
    __shared__ double f1_geom[7];  // x, y, z, ra, dec, cos dec, z_qso of forest 1
    __shared__ CfPairCtx pair_ctx[kCfBlock / 32];
    __shared__ unsigned long long visited[kCfBlock / 32];  // pair steps swept per warp
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nbins = fcp->nbins;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pc = fcp->pc;
    const float pmin_f = fcp->pc - 0.5f;
    const float h_tr = fcp->h_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    const float t_end = (float)nt + 1.f;  // x_tr' at or above this: rejected, a bin of margin
    // accepted range of p with one bin of margin each side: x = p - pmin in
    // [-1, np + 1]; |p| <= np + 1 for auto-correlations
    const float p_lo = RMU ? -(float)(nt + 1u) : (AUTO ? -(float)(np + 1u) : pmin_f - 1.f);
    const float p_hi = RMU ? (float)(nt + 1u) : (AUTO ? (float)(np + 1u) : pmin_f + (float)np + 1.f);
    const float inv_mu = fcp->inv_mu, mu_off = fcp->mu_off, g_mu0 = fcp->g_mu0;
    const int hs = fcp->hstride;
    const CfSmem L = cf_smem(nbins, max_pix1, nwarps);
    float *h = reinterpret_cast<float *>(smem + L.cells);
    const float4 *p1 = reinterpret_cast<const float4 *>(smem + L.p1);
    const float4 *p1x = reinterpret_cast<const float4 *>(smem + L.p1x);
    unsigned char *wbase = smem + L.warps + (size_t)warp * L.per_warp;
    float4 *buf = reinterpret_cast<float4 *>(wbase + L.buf);
    float4 *bufx = reinterpret_cast<float4 *>(wbase + L.bufx);
    float4 *acc0 = reinterpret_cast<float4 *>(wbase + L.acc0);
    float4 *acc1 = reinterpret_cast<float4 *>(wbase + L.acc1);
    uint32_t *queue = reinterpret_cast<uint32_t *>(wbase + L.queue);
    uint32_t *veto1 = reinterpret_cast<uint32_t *>(wbase + L.veto);
    zero_all(h, H_COUNT * hs);
    CfPairCtx &ctx = pair_ctx[warp];
    if (lane == 0) visited[warp] = 0ull;

    for (;;) {
        const int item = next_item(scratch, &item_slot, &max_rho_bits);
        if (item >= num_work) break;
        const int64_t f1 = work_order ? work_order[item] : item;
        const int32_t row = s1.row[f1];
        const int64_t a0 = s1.pix_offset[f1];
        const int64_t n1_64 = s1.pix_offset[f1 + 1] - a0;
        if (n1_64 > max_pix1 || n1_64 > 65535 || n1_64 < 1) {
            if (threadIdx.x == 0 && n1_64 > 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)f1);
            continue;
        }
        const int n1 = (int)n1_64;
        // forest 1 in FP32 relative to the distance of its middle pixel
        const double r_ref = s1.r_comov[a0 + n1 / 2];
        if (threadIdx.x == 0) {
            f1_geom[0] = s1.x_cart[f1]; f1_geom[1] = s1.y_cart[f1]; f1_geom[2] = s1.z_cart[f1];
            f1_geom[3] = s1.ra[f1]; f1_geom[4] = s1.dec[f1]; f1_geom[5] = s1.cos_dec[f1];
            f1_geom[6] = s1.z_qso[f1];
            nbr_next = nbr_offsets[f1];
        }
        const bool sorted1 = stage_forest1(s1, a0, n1, r_ref, const_cast<float4 *>(p1),
                                           const_cast<float4 *>(p1x), &max_rho_bits);
        const ParGuard pg = par_guard(fcp, __uint_as_float(max_rho_bits));
        const float h_par = pg.h_par, low_clamp = pg.low_clamp;
        // r-mu: r carries the errors of both staged coordinates
        const float g_pp = pg.guard_v;
        const float h_r = h_tr - g_pp;
        const int64_t k1 = nbr_offsets[f1 + 1];
        int head = 0, tail = 0;  // run ring of this warp (warp-uniform)
        int qn = 0;              // FP64 re-decision queue of this warp
        for (;;) {
            // warps take neighbour forests dynamically (balances uneven lengths)
            int64_t k = 0;
            if (lane == 0) k = (int64_t)atomicAdd((unsigned long long *)&nbr_next, 1ull);
            k = __shfl_sync(0xffffffffu, k, 0);
            if (k >= k1) break;
            const int64_t g = nbr_index[k];
            const int64_t b0 = s2.pix_offset[g];
            const int64_t n2_64 = s2.pix_offset[g + 1] - b0;
            if (n2_64 > 65535) {
                if (lane == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)g);
                continue;
            }
            const int n2 = (int)n2_64;
            // cos and sin of half the angle: from the half-angle identities
            // on the FP64 dot product (one square root each; the FP64
            // rounding of the dot moves 1 - cos by a few 1e-16, below 1e-9
            // of it above 1e-3 rad), else from the angle itself. The angle
            // is needed only by the zerr cut (the angular binning never
            // runs here)
            double ang = 0.0, chalf, shalf;
            const double x2 = s2.x_cart[g], y2 = s2.y_cart[g], z2 = s2.z_cart[g];
            const double cosang =
                __dadd_rn(__dadd_rn(__dmul_rn(x2, f1_geom[0]), __dmul_rn(y2, f1_geom[1])),
                          __dmul_rn(z2, f1_geom[2]));
            if (!nbr_angle && !(EXTRA && b.zerr_on) && cosang < kCosHalfAngleForm) {
                const double cc = fmax(cosang, -1.0);
                chalf = __dsqrt_rn(__dmul_rn(0.5, __dadd_rn(1.0, cc)));
                shalf = __dsqrt_rn(__dmul_rn(0.5, __dsub_rn(1.0, cc)));
            } else {
                ang = nbr_angle ? nbr_angle[k]
                                : angle_between(f1_geom[0], f1_geom[1], f1_geom[2], f1_geom[3],
                                                f1_geom[4], f1_geom[5], x2, y2, z2, s2.ra[g],
                                                s2.dec[g]);
                chalf = cos(ang / 2);
                shalf = sin(ang / 2);
            }
            bool shp = false, zerr_pair = false;
            if (EXTRA) {
                if (b.remove_shp) {
                    const int64_t fb1 = s1.fiberid[f1], fb2 = s2.fiberid[g];
                    shp = (s1.plate[f1] == s2.plate[g]) &&
                          ((fb1 <= 500 && fb2 <= 500) || (fb1 > 500 && fb2 > 500));
                }
                zerr_pair = b.zerr_on && (ang < b.zerr_ang);
            }
            if (qn) {  // the queue holds the previous pair's entries
                cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
                qn = 0;
            }
            __syncwarp();
            if (lane == 0) {
                ctx.a0 = a0;
                ctx.b0 = b0;
                ctx.ang = ang;
                ctx.c = chalf;
                ctx.s = shalf;
                ctx.shp = shp;
                ctx.zq2 = EXTRA ? s2.z_qso[g] : 0.;
            }
            if (EXTRA && zerr_pair) {
                // forest-1 pixels vetoed against quasar 2 (py/picca/cf.py:321-328)
                const double zq2 = s2.z_qso[g];
                for (int i0 = 0; i0 < n1; i0 += 32) {
                    const int i = i0 + lane;
                    const bool v = i < n1 && zerr_veto(s1.z[a0 + i], zq2, b.zerr_kms);
                    const unsigned m = __ballot_sync(0xffffffffu, v);
                    if (lane == 0) veto1[i0 >> 5] = m;
                }
            }
            __syncwarp();
            const float cp = (float)(chalf * (RMU ? fcp->geom_p : inv_p));
            const float st = (float)(shalf * inv_t);
            for (int jc = 0; jc < n2; jc += kChunk) {
                const int jn = min(kChunk, n2 - jc);
                // stage the chunk: nB = -cp rho2, t = st d2 - 1/2; a pixel
                // without weight or vetoed against quasar 1 gets w = 0 (and
                // t = kFar), which removes its pairs in the sweep
                bool ordered2 = true, valid2 = true;
                __syncwarp();
                for (int jl = lane; jl < jn; jl += 32) {
                    const int64_t jj = b0 + jc + jl;
                    const double w2 = s2.weights[jj];
                    bool ok = w2 != 0;
                    if (EXTRA && zerr_pair && ok)
                        ok = !zerr_veto(s2.z[jj], f1_geom[6], b.zerr_kms);
                    const double rho2_d = s2.r_comov[jj] - r_ref;
                    const float rho2 = (float)rho2_d;
                    const float d2 = (float)s2.dist_m[jj];
                    // nB = -cp rho2 as hi + lo (exact to 2^-48): hi decides,
                    // hi + lo enters the summed r_par
                    const double nb_d = -((double)cp * rho2_d);
                    const float nb_h = -__fmul_rn(cp, rho2);
                    buf[jl] = make_float4(nb_h, ok ? __fmaf_rn(st, d2, RMU ? 0.f : -0.5f) : kFar,
                                          (float)s2.z[jj], ok ? weight32(w2) : 0.f);
                    const float2 dw = split2(s2.delta[jj] * w2);
                    bufx[jl] = make_float4(dw.x, dw.y, (float)(nb_d - (double)nb_h), 0.f);
                    valid2 &= ok;
                    if (jl + 1 < jn)
                        ordered2 &= (float)(s2.r_comov[jj + 1] - r_ref) >= rho2 &&
                                    (float)s2.dist_m[jj + 1] >= d2;
                }
                ordered2 = __all_sync(0xffffffffu, ordered2);
                valid2 = __all_sync(0xffffffffu, valid2);
                __syncwarp();
                // the band of diagonals [d_lo, d_hi) holding every pair within
                // one bin of the accepted r_par range
                int d_lo = jc - (n1 - 1), d_hi = jc + jn;
                if (sorted1 && ordered2) {
                    int lo = INT_MAX, hi = INT_MIN;
                    for (int i = lane; i < n1; i += 32) {
                        const float a = __fmul_rn(cp, p1[i].x);
                        const int j1 = count_leading<false>(buf, jn, p_hi - a);
                        const int j2 = count_leading<true>(buf, jn, p_lo - a);
                        if (j1 < j2) {
                            lo = min(lo, jc + j1 - i);
                            hi = max(hi, jc + j2 - i);
                        }
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
                    }
                    d_lo = lo;
                    d_hi = hi;
                }
                // along a diagonal x_tr' is non-decreasing: trim at t_end
                const bool t_trim = sorted1 && ordered2 && valid2 && st > 0.f;
                for (int d0 = d_lo; d0 < d_hi; d0 += 32) {
                    const int d = d0 + lane;
                    // this lane's pairs: j = i + d in the chunk, i in forest 1
                    int ia = max(0, jc - d), ib = min(n1, jc + jn - d);
                    if (d >= d_hi) ib = ia;
                    const int joff = d - jc;  // chunk index of pixel i's partner
                    if (t_trim && ia < ib) {
                        int lo = ia, hi = ib;
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            const float x = __fmaf_rn(st, p1[mid].y, buf[mid + joff].y);
                            if (x < t_end) lo = mid + 1;
                            else hi = mid;
                        }
                        ib = lo;
                    }
                    // the lanes step the chunk's pixel together (s = j - jc, a
                    // broadcast read) and each its own forest-1 pixel
                    // i = s - joff: their ranges of s share the chunk's ends
                    // and differ only where forest 1 ends or the sweep is
                    // trimmed
                    const int sa = ia + joff, sb = ib + joff;  // empty when ia >= ib
                    int g_lo = ia < ib ? sa : INT_MAX, g_hi = ia < ib ? sb : INT_MIN;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        g_lo = min(g_lo, __shfl_xor_sync(0xffffffffu, g_lo, o));
                        g_hi = max(g_hi, __shfl_xor_sync(0xffffffffu, g_hi, o));
                    }
                    if (g_lo >= g_hi) continue;
                    if (lane == 0) visited[warp] += (unsigned long long)(g_hi - g_lo) * 32u;
                    // the lane's run: bin, pairs and sums
                    unsigned run_bin = 0xFFFFFFFFu;
                    int run_n = 0;
                    float r_xi = 0.f, r_xil = 0.f, r_w = 0.f, r_pw = 0.f, r_tw = 0.f, r_zw = 0.f;
                    // stores the runs of the lanes in `flag` into the ring
                    auto store_runs = [&](bool flag) {
                        const unsigned m = __ballot_sync(0xffffffffu, flag);
                        const int pos = (tail + __popc(m & lt_mask)) & (kAccQ - 1);
                        if (flag) {
                            acc0[pos] = make_float4(r_xi, r_xil, r_w, r_pw);
                            acc1[pos] = make_float4(r_tw, r_zw, __uint_as_float(run_bin),
                                                    __uint_as_float((unsigned)run_n));
                        }
                        tail += __popc(m);
                    };
                    // one pair of the lane's diagonal: its bin and whether it
                    // is accepted or queued (the geometry of two consecutive
                    // pairs is evaluated before either enters the run, so
                    // that their dependency chains overlap)
                    struct PairEval {
                        unsigned bin;
                        int i;
                        float pp, xt, zs, w12;
                        bool acc, near;
                    };
                    auto eval = [&](int js, PairEval &e) {
                        bool in = (js >= sa) & (js < sb);
                        const int i = in ? js - joff : 0;
                        if (EXTRA && zerr_pair && in) in = ((veto1[i >> 5] >> (i & 31)) & 1u) == 0u;
                        // js <= g_hi <= jn: the clamp keeps the (unused) read
                        // one past the group's range inside the chunk
                        const float4 q1 = p1[i];
                        const float4 q2 = buf[min(js, jn - 1)];
                        const float pp = __fmaf_rn(cp, q1.x, q2.x);
                        const float v = fabsf(pp);
                        const float pv = AUTO ? v : pp;
                        const float xt = __fmaf_rn(st, q1.y, q2.y);
                        float fp, ft;
                        unsigned ip, it;
                        bool near;
                        if (RMU) {
                            const float r2 = __fmaf_rn(pp, pp, xt * xt);
                            const float sinv = rsqrtf(r2);
                            const float ru = r2 * sinv;
                            const float mu = pv * sinv;
                            float xm = __fmaf_rn(mu, inv_mu, -mu_off);
                            if (LOWX) xm = fmaxf(xm, low_clamp);
                            ip = round_rem(xm, fp);
                            it = round_rem(ru - 0.5f, ft);
                            const float gm = __fmaf_rn(g_pp * sinv, inv_mu, g_mu0);
                            near = !(gm < 0.25f) | (fabsf(fp) > 0.5f - gm) | (fabsf(ft) > h_r);
                        } else {
                            const float xp = LOWX ? fmaxf(pv - pc, low_clamp) : pv - pc;
                            ip = round_rem(xp, fp);
                            it = round_rem(xt, ft);
                            near = (fabsf(fp) > h_par) | (fabsf(ft) > h_tr);
                        }
                        // a pixel without weight or vetoed (w staged as 0) pairs
                        // with nothing: neither accepted nor queued
                        in &= (q1.w != 0.f) & (q2.w != 0.f);
                        bool ok = (ip < np) & (it < nt);
                        const float zs = q1.z + q2.z;
                        if (EXTRA) {
                            if (shp) {
                                near |= fabsf(v - 1.f) < pg.guard_v;
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
                        near &= in;
                        e.acc = in & ok & !near;
                        e.near = near;
                        e.bin = ip * nt + it;
                        e.i = i;
                        e.pp = pp;
                        e.xt = xt;
                        e.zs = zs;
                        e.w12 = q1.w * q2.w;
                    };
                    // the pair enters the lane's run (a new run when its bin
                    // differs or the run is full)
                    auto take = [&](const PairEval &e, int js) {
                        const bool brk = e.acc & ((e.bin != run_bin) | (run_n >= kRunMax));
                        const bool flush = brk & (run_n > 0);
                        if (__any_sync(0xffffffffu, flush)) {
                            store_runs(flush);
                            if (flush) {
                                run_n = 0;
                                r_xi = r_xil = r_w = r_pw = r_tw = r_zw = 0.f;
                            }
                            if (tail - head >= 32) {
                                apply_runs<true>(acc0, acc1, head, 32, h, hs);
                                head += 32;
                            }
                        }
                        if (brk) run_bin = e.bin;
                        if (e.acc) {
                            const float4 x1 = p1x[e.i];
                            const float4 x2 = bufx[js];
                            const float w12 = e.w12;
                            float th, tl;
                            two_prod(x1.x, x1.y, x2.x, x2.y, th, tl);
                            two_sum_into(r_xi, r_xil, th);
                            r_xil += tl;
                            r_w += w12;
                            // r_par (bin units) from the hi + lo distances:
                            // relative precision for the summed r_par
                            const float pp_s = e.pp + __fmaf_rn(cp, x1.z, x2.z);
                            if (RMU) {
                                // r and mu from the hi + lo distances: the
                                // staged r_par carries an absolute error that
                                // is large relative to a small r
                                const float r2s = __fmaf_rn(pp_s, pp_s, e.xt * e.xt);
                                const float ss = rsqrtf(r2s);
                                r_pw = __fmaf_rn((AUTO ? fabsf(pp_s) : pp_s) * ss, w12, r_pw);
                                r_tw = __fmaf_rn(r2s * ss, w12, r_tw);
                            } else {
                                r_pw = __fmaf_rn(AUTO ? fabsf(pp_s) : pp_s, w12, r_pw);
                                r_tw = __fmaf_rn(e.xt + 0.5f, w12, r_tw);
                            }
                            r_zw = __fmaf_rn(e.zs, w12, r_zw);
                            ++run_n;
                        }
                    };
                    for (int js = g_lo; js < g_hi; js += 2) {
                        PairEval ea, eb;
                        eval(js, ea);
                        eval(js + 1, eb);  // js + 1 = g_hi: outside every lane's range
                        take(ea, js);
                        take(eb, js + 1);
                        if (__any_sync(0xffffffffu, ea.near | eb.near)) {
                            // rare path: queue the pairs near an edge for FP64 re-decision
                            if (qn > kCfQueue - 64) {
                                cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
                                if (lane == 0) atomicAdd(&scratch->recheck_overflows, 1ull);
                                qn = 0;
                            }
                            unsigned nmask = __ballot_sync(0xffffffffu, ea.near);
                            if (ea.near)
                                queue[qn + __popc(nmask & lt_mask)] =
                                    ((uint32_t)ea.i << 16) | (uint32_t)(ea.i + d);
                            qn += __popc(nmask);
                            nmask = __ballot_sync(0xffffffffu, eb.near);
                            if (eb.near)
                                queue[qn + __popc(nmask & lt_mask)] =
                                    ((uint32_t)eb.i << 16) | (uint32_t)(eb.i + d);
                            qn += __popc(nmask);
                        }
                    }
                    store_runs(run_n > 0);
                    while (tail - head >= 32) {
                        apply_runs<true>(acc0, acc1, head, 32, h, hs);
                        head += 32;
                    }
                }
            }
        }
        if (qn) cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
        if (tail != head) apply_runs<false>(acc0, acc1, head, tail - head, h, hs);
        __syncthreads();
        flush_rows(h, *fcp, out, row);
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
    if (lane == 0) atomicAdd(&scratch->visited_pairs, visited[warp]);
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
        // delta1[i] * weights1[i] * weights2[j] (py/picca/xcf.py:308)
        const float2 dw = split2(fs.delta[ia] * w1 * wq);
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)zq;
        hist_add(h, fcp->hstride, (unsigned)bin, dw.x, dw.y, w12, pv * w12, tv * w12, zs * w12, 1);
    }
    __syncwarp();
}

// The cross-correlation as runs along the forest. A lane owns one quasar of
// a group of 32 neighbours and steps the forest pixels i with the others
// (pixel i is a broadcast read of shared memory); along the forest r_par and
// r_trans change slowly, so consecutive accepted pairs of a lane share their
// bin for several steps and are summed in registers as a run, which goes to
// the block histogram through the warp's ring when the bin changes (as in
// cf_xi_diag_kernel). Binary searches on the staged forest give each lane
// the pixels whose p = cp*rho1 + nB lies within one bin of the accepted
// r_par range and whose x_tr' is below the end of the r_trans range
// (requires rho and dist_m non-decreasing along the forest, checked;
// otherwise every pixel is swept); the skipped pairs are at least one bin
// outside the accepted ranges, so the reference rejects them too. Pairs
// within the guard band of an edge or a cut are re-decided in FP64
// (xcf_drain).
template <bool EXTRA>
__global__ void __launch_bounds__(kXcfBlock, 1) xcf_xi_fast_kernel(
    const __grid_constant__ Binning b, const FastConst *__restrict__ fcp,
    const __grid_constant__ pg_forest_set fs, const __grid_constant__ pg_forest_set objs,
    const int64_t *__restrict__ nbr_offsets, const int32_t *__restrict__ nbr_index,
    const double *__restrict__ nbr_angle, const int32_t *__restrict__ work_order,
    int64_t num_work, const __grid_constant__ pg_xi_rows out, Scratch *scratch, int max_pix1) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    __shared__ unsigned max_rho_bits;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nbins = fcp->nbins;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pc = fcp->pc;
    const float h_tr = fcp->h_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    const int hs = fcp->hstride;
    // accepted range of p with one bin of margin each side, and of x_tr'
    const float p_lo = (pc - 0.5f) - 1.f, p_hi = (pc - 0.5f) + (float)np + 1.f;
    const float t_end = (float)nt + 1.f;
    const SmemLayout L = smem_layout(nbins, max_pix1, nwarps, true);
    float *h = reinterpret_cast<float *>(smem + L.cells);
    float4 *p1 = reinterpret_cast<float4 *>(smem + L.p1);
    float4 *p2 = reinterpret_cast<float4 *>(smem + L.p2);
    float4 *acc0 = reinterpret_cast<float4 *>(smem + L.acc0) + (size_t)warp * kAccQ;
    float4 *acc1 = reinterpret_cast<float4 *>(smem + L.acc1) + (size_t)warp * kAccQ;
    uint32_t *queue = reinterpret_cast<uint32_t *>(smem + L.queue) + warp * kQueue;
    uint16_t *qorder = reinterpret_cast<uint16_t *>(smem + L.order);
    int *buckets = reinterpret_cast<int *>(smem + L.buckets);
    zero_all(h, H_COUNT * hs);
    unsigned long long rechecks = 0, overflows = 0;

    for (;;) {
        const int item = next_item(scratch, &item_slot, &max_rho_bits);
        if (item >= num_work) break;
        const int64_t f = work_order ? work_order[item] : item;
        const int32_t row = fs.row[f];
        XcfCtx ctx;
        ctx.a0 = fs.pix_offset[f];
        const int64_t n1_64 = fs.pix_offset[f + 1] - ctx.a0;
        const int64_t nq_64 = nbr_offsets[f + 1] - nbr_offsets[f];
        if (n1_64 > max_pix1 || n1_64 > 65535 || nq_64 > 65535 || n1_64 < 1) {
            if (threadIdx.x == 0 && n1_64 > 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)f);
            continue;
        }
        const int n1 = (int)n1_64;
        const double r_ref = fs.r_comov[ctx.a0 + n1 / 2];
        const bool sorted1 = stage_forest1(fs, ctx.a0, n1, r_ref, p1, p2, &max_rho_bits);
        const ParGuard pg = par_guard(fcp, __uint_as_float(max_rho_bits));
        const float h_par = pg.h_par;
        ctx.x1 = fs.x_cart[f]; ctx.y1 = fs.y_cart[f]; ctx.zc1 = fs.z_cart[f];
        ctx.ra1 = fs.ra[f]; ctx.dec1 = fs.dec[f]; ctx.cd1 = fs.cos_dec[f];
        ctx.k0 = nbr_offsets[f];
        const int nq = (int)nq_64;
        // the quasars in order of distance (a counting sort into buckets),
        // so that the 32 quasars of a pass cover nearby stretches of the
        // forest and the passes over quasars that pair with nothing end at
        // their empty ranges
        const bool by_distance = nq <= kXcfOrderMax;
        if (by_distance) {
            for (int e = threadIdx.x; e < kXcfBuckets; e += blockDim.x) buckets[e] = 0;
            __syncthreads();
            auto bucket_of = [&](int k) {
                const double rq = objs.obj_r_comov[nbr_index[ctx.k0 + k]] - r_ref;
                const int e = __float2int_rd((float)rq * (1.f / kXcfBucketMpc)) + kXcfBuckets / 2;
                return e < 0 ? 0 : (e >= kXcfBuckets ? kXcfBuckets - 1 : e);
            };
            for (int k = threadIdx.x; k < nq; k += blockDim.x) atomicAdd(&buckets[bucket_of(k)], 1);
            __syncthreads();
            if (warp == 0) {  // exclusive prefix sum of the bucket counts
                int carry = 0;
                for (int e0 = 0; e0 < kXcfBuckets; e0 += 32) {
                    const int c = buckets[e0 + lane];
                    int incl = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int t2 = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= o) incl += t2;
                    }
                    buckets[e0 + lane] = carry + incl - c;
                    carry += __shfl_sync(0xffffffffu, incl, 31);
                }
            }
            __syncthreads();
            for (int k = threadIdx.x; k < nq; k += blockDim.x)
                qorder[atomicAdd(&buckets[bucket_of(k)], 1)] = (uint16_t)k;
            __syncthreads();
        }
        int head = 0, tail = 0;  // run ring of this warp (warp-uniform)
        int qn = 0;              // FP64 re-decision queue of this warp
        for (int kb = warp * 32; kb < nq; kb += nwarps * 32) {
            const int kk = kb + lane < nq ? (by_distance ? (int)qorder[kb + lane] : kb + lane) : nq;
            float cp = 1.f, st = 0.f, nb = kFar, nbl = 0.f, t = kFar, zv = kFar;
            float wvh = 0.f, wvl = 0.f;
            bool valid = false;
            if (kk < nq) {
                const int64_t g = nbr_index[ctx.k0 + kk];
                const double wq = objs.obj_weight[g];
                if (wq != 0) {
                    valid = true;
                    // cos and sin of half the angle, needed here to FP32
                    // accuracy only (the FP64 re-decision forms its own)
                    double chalf, shalf;
                    const double x2 = objs.x_cart[g], y2 = objs.y_cart[g], z2 = objs.z_cart[g];
                    const double cosang = __dadd_rn(
                        __dadd_rn(__dmul_rn(x2, ctx.x1), __dmul_rn(y2, ctx.y1)),
                        __dmul_rn(z2, ctx.zc1));
                    if (!nbr_angle && cosang < kCosHalfAngleForm) {
                        // half-angle identities on the clipped dot product: its
                        // FP64 rounding moves 1 - cos by a few 1e-16, below
                        // 1e-9 of it above 1e-3 rad; one square root each
                        // instead of arccos, cos and sin
                        const double cc = fmax(cosang, -1.0);
                        chalf = __dsqrt_rn(__dmul_rn(0.5, __dadd_rn(1.0, cc)));
                        shalf = __dsqrt_rn(__dmul_rn(0.5, __dsub_rn(1.0, cc)));
                    } else {
                        const double ang =
                            nbr_angle ? nbr_angle[ctx.k0 + kk]
                                      : angle_between(ctx.x1, ctx.y1, ctx.zc1, ctx.ra1,
                                                      ctx.dec1, ctx.cd1, x2, y2, z2, objs.ra[g],
                                                      objs.dec[g]);
                        chalf = cos(ang / 2);
                        shalf = sin(ang / 2);
                    }
                    cp = (float)(chalf * inv_p);
                    st = (float)(shalf * inv_t);
                    const double rho_d = objs.obj_r_comov[g] - r_ref;
                    const float rho_q = (float)rho_d;
                    nb = -__fmul_rn(cp, rho_q);
                    nbl = (float)(-((double)cp * rho_d) - (double)nb);
                    t = __fmaf_rn(st, (float)objs.obj_dist_m[g], -0.5f);
                    zv = (float)objs.z_qso[g];
                    wvh = weight32(wq);
                    wvl = (float)(wq - (double)wvh);
                }
            }
            // this lane's pixels [ia, ib): p and x_tr' are non-decreasing
            // along a sorted forest
            int ia = 0, ib = valid ? n1 : 0;
            if (sorted1 && valid) {
                int lo = 0, hi = n1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__fmaf_rn(cp, p1[mid].x, nb) < p_lo) lo = mid + 1;
                    else hi = mid;
                }
                ia = lo;
                hi = n1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__fmaf_rn(cp, p1[mid].x, nb) <= p_hi) lo = mid + 1;
                    else hi = mid;
                }
                ib = lo;
                lo = ia;
                hi = ib;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__fmaf_rn(st, p1[mid].y, t) < t_end) lo = mid + 1;
                    else hi = mid;
                }
                ib = lo;
            }
            int g_lo = ia < ib ? ia : INT_MAX, g_hi = ia < ib ? ib : INT_MIN;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                g_lo = min(g_lo, __shfl_xor_sync(0xffffffffu, g_lo, o));
                g_hi = max(g_hi, __shfl_xor_sync(0xffffffffu, g_hi, o));
            }
            if (g_lo >= g_hi) continue;
            unsigned run_bin = 0xFFFFFFFFu;
            int run_n = 0;
            float r_xi = 0.f, r_xil = 0.f, r_w = 0.f, r_pw = 0.f, r_tw = 0.f, r_zw = 0.f;
            auto store_runs = [&](bool flag) {
                const unsigned m = __ballot_sync(0xffffffffu, flag);
                const int pos = (tail + __popc(m & lt_mask)) & (kAccQ - 1);
                if (flag) {
                    acc0[pos] = make_float4(r_xi, r_xil, r_w, r_pw);
                    acc1[pos] = make_float4(r_tw, r_zw, __uint_as_float(run_bin),
                                            __uint_as_float((unsigned)run_n));
                }
                tail += __popc(m);
            };
            // one forest pixel against this lane's quasar; two consecutive
            // pixels are evaluated before either enters the run, so that
            // their dependency chains overlap
            struct PairEval {
                unsigned bin;
                float pv, xt, zs, w;
                bool acc, near;
            };
            auto eval = [&](int i, PairEval &e) {
                // i <= g_hi <= n1: the clamp keeps the (unused) read one
                // past the group's range inside the forest
                const float4 q = p1[min(i, n1 - 1)];
                const bool in = (i >= ia) & (i < ib) & (q.w != 0.f);
                const float pv = __fmaf_rn(cp, q.x, nb);
                const float xt = __fmaf_rn(st, q.y, t);
                float fp, ft;
                const unsigned ip = round_rem(pv - pc, fp);
                const unsigned it = round_rem(xt, ft);
                bool near = (fabsf(fp) > h_par) | (fabsf(ft) > h_tr);
                bool ok = (ip < np) & (it < nt);
                const float zs = q.z + zv;
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
                near &= in;
                e.acc = in & ok & !near;
                e.near = near;
                e.bin = ip * nt + it;
                e.pv = pv;
                e.xt = xt;
                e.zs = zs;
                e.w = q.w;
            };
            auto take = [&](const PairEval &e, int i) {
                const bool brk = e.acc & ((e.bin != run_bin) | (run_n >= kRunMax));
                const bool flush = brk & (run_n > 0);
                if (__any_sync(0xffffffffu, flush)) {
                    store_runs(flush);
                    if (flush) {
                        run_n = 0;
                        r_xi = r_xil = r_w = r_pw = r_tw = r_zw = 0.f;
                    }
                    if (tail - head >= 32) {
                        apply_runs<true>(acc0, acc1, head, 32, h, hs);
                        head += 32;
                    }
                }
                if (brk) run_bin = e.bin;
                if (e.acc) {
                    const float4 qd = p2[i];
                    const float w12 = e.w * wvh;
                    float th, tl;
                    // delta1 w1 * w2 (py/picca/xcf.py:308) as hi + lo
                    two_prod(qd.x, qd.y, wvh, wvl, th, tl);
                    two_sum_into(r_xi, r_xil, th);
                    r_xil += tl;
                    r_w += w12;
                    // summed r_par from the hi + lo distances
                    const float pv_s = e.pv + __fmaf_rn(cp, qd.z, nbl);
                    r_pw = __fmaf_rn(pv_s, w12, r_pw);
                    r_tw = __fmaf_rn(e.xt + 0.5f, w12, r_tw);
                    r_zw = __fmaf_rn(e.zs, w12, r_zw);
                    ++run_n;
                }
            };
            for (int i = g_lo; i < g_hi; i += 2) {
                PairEval ea, eb;
                eval(i, ea);
                eval(i + 1, eb);  // i + 1 = g_hi: outside every lane's range
                take(ea, i);
                take(eb, i + 1);
                if (__any_sync(0xffffffffu, ea.near | eb.near)) {
                    if (qn > kQueue - 64) {
                        xcf_drain(b, fcp, fs, objs, nbr_index, nbr_angle, ctx, queue, qn, h,
                                  scratch);
                        rechecks += qn;
                        ++overflows;
                        qn = 0;
                    }
                    unsigned nmask = __ballot_sync(0xffffffffu, ea.near);
                    if (ea.near)
                        queue[qn + __popc(nmask & lt_mask)] = ((uint32_t)i << 16) | (uint32_t)kk;
                    qn += __popc(nmask);
                    nmask = __ballot_sync(0xffffffffu, eb.near);
                    if (eb.near)
                        queue[qn + __popc(nmask & lt_mask)] =
                            ((uint32_t)(i + 1) << 16) | (uint32_t)kk;
                    qn += __popc(nmask);
                }
            }
            store_runs(run_n > 0);
            while (tail - head >= 32) {
                apply_runs<true>(acc0, acc1, head, 32, h, hs);
                head += 32;
            }
        }
        if (qn) {
            xcf_drain(b, fcp, fs, objs, nbr_index, nbr_angle, ctx, queue, qn, h, scratch);
            rechecks += qn;
        }
        if (tail != head) apply_runs<false>(acc0, acc1, head, tail - head, h, hs);
        __syncthreads();
        flush_rows(h, *fcp, out, row);
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
    if (lane == 0) {
        atomicAdd(&scratch->rechecked_pairs, rechecks);
        atomicAdd(&scratch->recheck_overflows, overflows);
    }
}

// Guard bands. Let u = 2^-24 (the unit roundoff of FP32). For r_par: rho1
// and rho2 are the FP64 differences r - R (exact) rounded to FP32 (errors
// u|rho1|, u|rho2|); cp carries a relative error u, nB = -cp*rho2 another
// u|cp rho2|, and the FMA p = cp*rho1 + nB rounds once (u|p|). For a pair
// whose exact x lies in [-1, n + 1] (the others are rejected either way),
// |rho2| <= |rho1| + (n + 1)/cp, so p is within 4u(n + 1) + 3u cp|rho1| of
// the exact value; the rounding of pc = pmin + 1/2 and of the subtraction add
// u(|pmin| + 1/2) and u|x'|. With cp <= inv_p and a factor 2 of margin
//   g_par = 16 u (n + |pmin| + 2) + 8 u inv_p max|rho1| + 1e-6,
// the last term taken per work item (R is the middle pixel of forest 1, so
// max|rho1| is about half the forest's length). For x_tr the FP32 rounding
// of d1 and d2 (relative u), of st, of t = st*d2 - 1/2 (one FMA) and of the
// FMA st*d1 + t give <= 6u(|x_tr| + 1), and
//   g_tr = 16 u (n + 2) + 1e-6.
// round(x') and the remainder are exact (the magic-number add rounds to an
// integer and the subtraction is exact). The reference's own FP64 evaluation
// is within 1e-12 of the exact value, far inside these bands. With
// r_par_min = 0 in an auto-correlation x = |p| >= 0 and the lower edge of bin
// 0 cannot be crossed: x' is clamped from below at -1/2 + 2g, which keeps
// pairs with |p| < 2g (same-wavelength pixels give p = 0 exactly) in bin 0
// without flagging them.
FastConst make_fast_const(const Binning &b) {
    FastConst fc{};
    const double u = 1.0 / 16777216.0;
    fc.inv_p = (double)b.np / b.r_par_range;
    fc.inv_t = (double)b.nt / b.r_trans_max;
    fc.geom_p = fc.inv_p;
    const double pmin = b.r_par_min * fc.inv_p;
    fc.pc = (float)(pmin + 0.5);
    fc.g0_par = (float)(16 * u * (b.np + fabs(pmin) + 2) + 1e-6);
    fc.g_rho = (float)(8 * u * fc.inv_p);
    if (b.rmu) {
        // r-mu bins (py/picca/cf.py:354-358): r_par and r_trans are staged in
        // r-bin units, r = sqrt(r_par^2 + r_trans^2) and mu = r_par / r per
        // pair; the r_par histogram holds mu (scale 1). g0_par and g_rho
        // bound the absolute error of the staged r_par in r-bin units.
        fc.geom_p = fc.inv_t;
        fc.inv_p = 1.0;
        fc.pc = 0.5f;
        fc.g0_par = (float)(16 * u * (b.nt + 2) + 1e-6);
        fc.g_rho = (float)(8 * u * fc.inv_t);
        fc.inv_mu = (float)((double)b.np / b.r_par_range);
        fc.mu_off = (float)(b.r_par_min * (double)b.np / b.r_par_range + 0.5);
        fc.g_mu0 = (float)(16 * u * (b.np + fabs(b.r_par_min * b.np / b.r_par_range) + 2) + 1e-6);
    }
    double g_tr = 16 * u * (b.nt + 2) + 1e-6;
    // r-mu: r also carries the reciprocal square root and the sum of squares
    if (b.rmu) g_tr = 32 * u * (b.nt + 2) + 1e-6;
    if (!(g_tr < 0.05)) g_tr = 0.05;
    fc.h_tr = (float)(0.5 - g_tr);
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

template <typename K>
int persistent_grid(K kernel, int block, size_t smem, int num_sms, int64_t num_work, int *grid,
                    int blocks_per_sm = 0) {
    cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (err != cudaSuccess) return check_cuda(err);
    if (per_sm < 1) return PG_ERR_UNSUPPORTED;
    if (blocks_per_sm > 0 && blocks_per_sm < per_sm) per_sm = blocks_per_sm;
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
                      cudaStream_t stream, LaunchTuning tuning) {
    if (num_work <= 0) return PG_OK;
    FastConst *fc = static_cast<FastConst *>(fast_const);
    const int max_pix1 = s1.max_pixels;
    // as many warps (up to kCfBlock / 32, or the tuned count) as shared
    // memory leaves room for
    int nwarps = kCfBlock / 32;
    if (tuning.warps > 0 && tuning.warps < nwarps) nwarps = tuning.warps;
    while (nwarps > 1 && cf_smem(b.nbins, max_pix1, nwarps).total > 227 * 1024) --nwarps;
    const int block = nwarps * 32;
    const size_t smem = cf_smem(b.nbins, max_pix1, nwarps).total;
    if (smem > 227 * 1024) return PG_ERR_UNSUPPORTED;
    (void)ang_max;
    int rc = prepare_fast(b, fc, stream);
    if (rc) return rc;
    const bool extra = b.remove_shp || b.zmin_on || b.zmax_on || b.zerr_on;
    if (b.rmu && extra) return PG_ERR_UNSUPPORTED;  // callers use the FP64 kernel
    const bool autoc = !b.x_correlation;
    const bool lowx = autoc && b.r_par_min == 0.0;
    int grid = 0;
#define PG_LAUNCH_CF(A, E, L, R)                                                               \
    rc = persistent_grid(cf_xi_diag_kernel<A, E, L, R>, block, smem, num_sms, num_work, &grid, \
                         tuning.blocks_per_sm);                                                \
    if (rc) return rc;                                                                         \
    cf_xi_diag_kernel<A, E, L, R><<<grid, block, smem, stream>>>(b, fc, s1, s2, nbr_offsets,   \
                                                                 nbr_index, nbr_angle,         \
                                                                 work_order, num_work, out,    \
                                                                 scratch, max_pix1);
    if (b.rmu) {
        if (autoc && lowx) { PG_LAUNCH_CF(true, false, true, true) }
        else if (autoc) { PG_LAUNCH_CF(true, false, false, true) }
        else { PG_LAUNCH_CF(false, false, false, true) }
    }
    else if (autoc && lowx && !extra) { PG_LAUNCH_CF(true, false, true, false) }
    else if (autoc && lowx && extra) { PG_LAUNCH_CF(true, true, true, false) }
    else if (autoc && !extra) { PG_LAUNCH_CF(true, false, false, false) }
    else if (autoc && extra) { PG_LAUNCH_CF(true, true, false, false) }
    else if (!extra) { PG_LAUNCH_CF(false, false, false, false) }
    else { PG_LAUNCH_CF(false, true, false, false) }
#undef PG_LAUNCH_CF
    return check_cuda(cudaGetLastError());
}

int launch_xcf_xi_fast(const Binning &b, double ang_max, const pg_forest_set &forests,
                       const pg_forest_set &objs, const int64_t *nbr_offsets,
                       const int32_t *nbr_index, const double *nbr_angle,
                       const int32_t *work_order, int64_t num_work,
                       const pg_xi_rows &out, Scratch *scratch, void *fast_const, int num_sms,
                       cudaStream_t stream, LaunchTuning tuning) {
    if (num_work <= 0) return PG_OK;
    FastConst *fc = static_cast<FastConst *>(fast_const);
    const int max_pix1 = forests.max_pixels;
    // as many warps (up to kXcfBlock / 32, or the tuned count) as shared
    // memory leaves room for (histograms, forest, per-warp rings and queues)
    int nwarps = kXcfBlock / 32;
    if (tuning.warps > 0 && tuning.warps < nwarps) nwarps = tuning.warps;
    while (nwarps > 1 && smem_layout(b.nbins, max_pix1, nwarps, true).total > 227 * 1024) --nwarps;
    const int block = nwarps * 32;
    const size_t smem = smem_layout(b.nbins, max_pix1, nwarps, true).total;
    if (smem > 227 * 1024) return PG_ERR_UNSUPPORTED;
    (void)ang_max;
    int rc = prepare_fast(b, fc, stream);
    if (rc) return rc;
    const bool extra = b.zmin_on || b.zmax_on;
    int grid = 0;
    if (extra) {
        rc = persistent_grid(xcf_xi_fast_kernel<true>, block, smem, num_sms, num_work, &grid,
                             tuning.blocks_per_sm);
        if (rc) return rc;
        xcf_xi_fast_kernel<true><<<grid, block, smem, stream>>>(
            b, fc, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out,
            scratch, max_pix1);
    } else {
        rc = persistent_grid(xcf_xi_fast_kernel<false>, block, smem, num_sms, num_work, &grid,
                             tuning.blocks_per_sm);
        if (rc) return rc;
        xcf_xi_fast_kernel<false><<<grid, block, smem, stream>>>(
            b, fc, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out,
            scratch, max_pix1);
    }
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
