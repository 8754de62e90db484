// Precision-form pair accumulation: FP32 geometry with an FP64 bin-edge
// guard, compensated FP32 shared-memory block sums, FP64 rows.
//
// Persistent structure: one work item = one forest of set 1 with all its
// neighbours; the forest-1 pixels are staged in shared memory, warps take
// neighbour forests dynamically, and each lane holds P consecutive forest-2
// pixels in registers while it loops over the forest-1 pixels. For every
// pixel pair the kernel evaluates, in FP32,
//     p   = cp*((r1h - r2h) + (r1l - r2l))   (= r_par * np/(r_par_max - r_par_min))
//     x'  = |p| - (r_par_min*inv_p + 1/2)   (p itself for signed, cross correlations)
//     xt' = st*d1 + (st*d2 - 1/2)           (= r_trans * nt/r_trans_max - 1/2)
// with cp = cos(theta/2) * inv_p, st = sin(theta/2) * inv_t, and the comoving
// distance carried as an FP32 pair r = rh + rl, so that r1 - r2 is exact to
// ~1e-7 of itself (not of r). The bin index of py/picca/cf.py:372-376 is
// floor(x) = round(x'), taken with one round-to-nearest add of 1.5 * 2^23:
// y = x' + 1.5*2^23 is an integer for |x'| < 2^22, so round(x') is the bit
// pattern of y minus that of 1.5*2^23 and f = x' - (y - 1.5*2^23), in
// [-1/2, 1/2], is exact. A pair with |f| > 1/2 - g in either coordinate (a bin
// edge or an acceptance limit within the guard band g), or within a guard
// of the half-plate r_par cut or the z-pair cuts, is queued and re-decided
// in FP64 with the reference's operation order (cf_pair_bin /
// xcf_pair_bin), so every accepted pair, bin index and pair count equals
// the FP64 reference. g exceeds the worst-case FP32 error (make_fast_const).
// Forest-2 slots past the end of the forest or with zero weight carry
// r = t = z = 1e30 (and cp = 1 for quasars), which lands far outside every
// bin, edge and cut, so such a slot is neither accepted nor queued.
//
// Sums: per-CTA FP32 shared-memory histograms of xi, w, p*w, x_tr*w,
// (z1+z2)*w and an int32 count. xi (products of signed deltas, strongly
// cancelling) and w (the normalisation) are summed error-free: the atomic add
// returns the previous value, Knuth's TwoSum recovers the exact rounding
// error of the add and a second histogram collects it. Accepted pairs first
// go to a per-warp ring, and the warp applies them 32 at a time, so the
// eight atomic adds of a pair run with every lane active instead of in the
// divergent branch of each pair. After each work item the histograms are
// added to the FP64 rows and mapped back to picca's units (r_par =
// p/inv_p, r_trans = x_tr/inv_t, z = (z1+z2)/2).
#include <type_traits>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr float kMagic = 12582912.0f;        // 1.5 * 2^23
constexpr unsigned kMagicBits = 0x4B400000u;  // bits of 1.5 * 2^23
constexpr float kFar = 1e30f;                 // r and t of an empty slot
constexpr int kQueue = 256;                   // FP64 recheck entries per warp
constexpr int kAccQ = 128;                    // accepted-pair ring per warp
constexpr int kCfP = 4;                       // forest-2 pixels per lane (full passes)
constexpr int kXcfP = 2;                      // quasars per lane per pass
constexpr int kCfBlock = 768;
constexpr int kXcfBlock = 512;

struct FastConst {
    double inv_p, inv_t;
    float pc;               // r_par_min * inv_p + 1/2
    float low_clamp;        // -1/2 + 2 g_par (auto-correlation with r_par_min = 0)
    float h_par, h_tr;      // 1/2 - g: |f| above this is near an edge
    float guard_v;          // half-plate cut guard (in units of p)
    float guard_z;          // guard on z1 + z2
    float zmin2, zmax2;     // 2 z_min, 2 z_max
    unsigned np, nt;
    int nbins;
    int hstride;            // histogram array stride (nbins rounded up to 4)
    int lower_exact;        // auto-correlation with r_par_min = 0: x = |p| >= 0, so
                            // the lower edge of bin 0 can never be crossed
};

// ---------------------------------------------------------------------------
// shared-memory histograms: H_COUNT float arrays of stride hstride
// ---------------------------------------------------------------------------
enum { H_XI = 0, H_XIL, H_WE, H_WEL, H_PW, H_TW, H_ZW, H_NB, H_COUNT };

// One pair into the histograms. xi and w are compensated: the atomic add
// returns the previous value, Knuth's TwoSum of it and the term gives the
// exact rounding error of the add, which goes to the error histogram. The two
// adds whose previous value is needed go first, so that their round trips
// overlap the four plain adds.
__device__ __forceinline__ void hist_add(float *h, int hs, unsigned bin, float xi, float w,
                                         float pw, float tw, float zw, int count) {
    float *hx = h + bin;
    const float oxi = atomicAdd(hx + H_XI * hs, xi);
    const float owe = atomicAdd(hx + H_WE * hs, w);
    atomicAdd(hx + H_PW * hs, pw);
    atomicAdd(hx + H_TW * hs, tw);
    atomicAdd(hx + H_ZW * hs, zw);
    atomicAdd(reinterpret_cast<int *>(hx + H_NB * hs), count);
    float sum = oxi + xi, bb = sum - oxi;
    atomicAdd(hx + H_XIL * hs, (oxi - (sum - bb)) + (xi - bb));
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

__device__ __forceinline__ int next_item(Scratch *scratch, int *slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(&scratch->work_counter, 1);
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

// round(x) (as unsigned; negative results wrap to large values) and the
// remainder x - round(x) in [-1/2, 1/2].
__device__ __forceinline__ unsigned round_rem(float x, float &rem) {
    const float y = x + kMagic;
    rem = x - (y - kMagic);
    return __float_as_uint(y) - kMagicBits;
}

// Shared-memory layout of both kernels (offsets in bytes from the start).
struct SmemLayout {
    size_t cells, p1, p2, acc0, acc1, queue, total;
};

__host__ __device__ inline SmemLayout smem_layout(int nbins, int max_pix1, int nwarps,
                                                  bool acc_queue) {
    SmemLayout l;
    const size_t mp = (size_t)((max_pix1 + 1) & ~1);
    l.cells = 0;
    l.p1 = l.cells + (size_t)((nbins + 3) & ~3) * H_COUNT * 4;
    l.p2 = l.p1 + mp * 16;
    l.acc0 = l.p2 + mp * 8;
    l.acc1 = l.acc0 + (acc_queue ? (size_t)nwarps * kAccQ * 16 : 0);
    l.queue = l.acc1 + (acc_queue ? (size_t)nwarps * kAccQ * 8 : 0);
    l.total = l.queue + (size_t)nwarps * kQueue * 4;
    return l;
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
        const float dw12 = (float)(s1.delta[ia] * w1) * (float)(s2.delta[jb] * w2);
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)z2;
        hist_add(h, fcp->hstride, (unsigned)bin, dw12, w12, pv * w12, tv * w12, zs * w12, 1);
    }
    if (lane == 0) atomicAdd(&scratch->rechecked_pairs, (unsigned long long)count);
    __syncwarp();
}

// Applies n (<= 32) queued entries starting at ring position head. An entry
// is a run of accepted pairs of one lane in one bin (consecutive forest-2
// pixels against one forest-1 pixel): {sum dw1 dw2, sum w1 w2, sum p w,
// sum x_tr w} and {sum (z1 + z2) w, bin * 8 + pairs}.
template <bool FULL>
__device__ __forceinline__ void apply_accepted(const float4 *acc0, const float2 *acc1, int head,
                                               int n, float *h, int hs) {
    __syncwarp();
    const int lane = threadIdx.x & 31;
    if (FULL || lane < n) {  // FULL: n = 32, no divergence
        const int e = (head + lane) & (kAccQ - 1);
        const float4 v = acc0[e];
        const float2 u = acc1[e];
        const unsigned key = __float_as_uint(u.y);
        hist_add(h, hs, key >> 3, v.x, v.y, v.z, v.w, u.x, (int)(key & 7u));
    }
    __syncwarp();
}

// Number of leading forest-1 pixels whose field (0: r, 1: dist_m) is below v
// (UPPER: not above v), for pixels in increasing order of that field.
template <int FIELD, bool UPPER>
__device__ __forceinline__ int count_below(const float4 *p1, int n, float v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float4 q = p1[mid];
        const float x = FIELD == 0 ? q.x : q.z;
        if (UPPER ? x <= v : x < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Forest-1 pixel range [i_lo, i_hi) that can pair with this warp's
// forest-2 block, for forest-1 pixels in increasing r and dist_m. Pairs
// outside it have x = p - pmin more than one bin outside [0, np] (r1 beyond
// the block's r range +- the offsets) or x_tr' = st d1 + t above nt + 1
// (d1 beyond (nt + 1 - min t) / st); their FP32 values are then far from
// every bin and edge, so the FP32 test would reject them without queueing.
template <int P>
__device__ __forceinline__ void window(const float4 *p1, int n1, const float (&rh)[P],
                                       const float (&t)[P], float st, float lo_off,
                                       float hi_off, float t_end, int &i_lo, int &i_hi) {
    float rmin = kFar, rmax = -kFar, tmin = kFar;
#pragma unroll
    for (int p = 0; p < P; ++p) {
        if (rh[p] < 0.5f * kFar) {
            rmin = fminf(rmin, rh[p]);
            rmax = fmaxf(rmax, rh[p]);
            tmin = fminf(tmin, t[p]);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        rmin = fminf(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
        rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        tmin = fminf(tmin, __shfl_xor_sync(0xffffffffu, tmin, o));
    }
    i_lo = count_below<0, false>(p1, n1, rmin + lo_off);
    i_hi = count_below<0, true>(p1, n1, rmax + hi_off);
    if (st > 0.f) {
        const int it_end = count_below<1, false>(p1, n1, (t_end - tmin) / st);
        if (it_end < i_hi) i_hi = it_end;
    }
}

// EXTRA: half-plate veto, z-pair cuts or zerr cut may be active.
// LOWX: auto-correlation with r_par_min = 0 (lower edge of bin 0 exempt).
template <bool AUTO, bool EXTRA, bool LOWX>
__global__ void __launch_bounds__(kCfBlock, 1) cf_xi_fast_kernel(
    const __grid_constant__ Binning b, const FastConst *__restrict__ fcp,
    const __grid_constant__ pg_forest_set s1, const __grid_constant__ pg_forest_set s2,
    const int64_t *__restrict__ nbr_offsets, const int32_t *__restrict__ nbr_index,
    const double *__restrict__ nbr_angle, const int32_t *__restrict__ work_order,
    int64_t num_work, const __grid_constant__ pg_xi_rows out, Scratch *scratch, int max_pix1) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    __shared__ long long nbr_next;
    // state read only off the hot loop lives in shared memory, which keeps
    // the registers for the pixel pairs (and 24 warps per SM resident)
    __shared__ double f1_geom[7];  // x, y, z, ra, dec, cos dec, z_qso of forest 1
    __shared__ CfPairCtx pair_ctx[kCfBlock / 32];
    __shared__ unsigned long long visited[kCfBlock / 32];  // forest-1 pixel steps per warp
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nbins = fcp->nbins;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pc = fcp->pc, low_clamp = fcp->low_clamp;
    const float pmin_f = fcp->pc - 0.5f;
    const float h_par = fcp->h_par, h_tr = fcp->h_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    const float t_end = (float)nt + 1.f;  // x_tr' above this: rejected with a bin of margin
    const int hs = fcp->hstride;
    const SmemLayout L = smem_layout(nbins, max_pix1, nwarps, true);
    float *h = reinterpret_cast<float *>(smem + L.cells);
    float4 *p1 = reinterpret_cast<float4 *>(smem + L.p1);
    float2 *p2 = reinterpret_cast<float2 *>(smem + L.p2);
    float4 *acc0 = reinterpret_cast<float4 *>(smem + L.acc0) + warp * kAccQ;
    float2 *acc1 = reinterpret_cast<float2 *>(smem + L.acc1) + warp * kAccQ;
    uint32_t *queue = reinterpret_cast<uint32_t *>(smem + L.queue) + warp * kQueue;
    zero_all(h, H_COUNT * hs);
    CfPairCtx &ctx = pair_ctx[warp];
    if (lane == 0) visited[warp] = 0ull;

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
        bool ordered = true;
        for (int i = threadIdx.x; i < n1; i += blockDim.x) {
            const double w = s1.weights[a0 + i];
            const double r = s1.r_comov[a0 + i];
            const float rh = (float)r;
            p1[i] = make_float4(rh, (float)(r - (double)rh), (float)s1.dist_m[a0 + i],
                                (float)s1.z[a0 + i]);
            p2[i] = make_float2(weight32(w), (float)(s1.delta[a0 + i] * w));
            if (i + 1 < n1)
                ordered &= (float)s1.r_comov[a0 + i + 1] >= rh &&
                           (float)s1.dist_m[a0 + i + 1] >= (float)s1.dist_m[a0 + i];
        }
        // forest-1 pixels in increasing distance: each forest-2 block only
        // visits the forest-1 pixels that can pair with it (see below)
        if (threadIdx.x == 0) {
            f1_geom[0] = s1.x_cart[f1]; f1_geom[1] = s1.y_cart[f1]; f1_geom[2] = s1.z_cart[f1];
            f1_geom[3] = s1.ra[f1]; f1_geom[4] = s1.dec[f1]; f1_geom[5] = s1.cos_dec[f1];
            f1_geom[6] = s1.z_qso[f1];
            nbr_next = nbr_offsets[f1];
        }
        const bool sorted1 = __syncthreads_and(ordered) != 0;
        const int64_t k1 = nbr_offsets[f1 + 1];
        int head = 0, tail = 0;  // accepted-pair ring of this warp (warp-uniform)
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
            const double ang = nbr_angle ? nbr_angle[k]
                                         : angle_between(f1_geom[0], f1_geom[1], f1_geom[2],
                                                         f1_geom[3], f1_geom[4], f1_geom[5],
                                                         s2.x_cart[g], s2.y_cart[g],
                                                         s2.z_cart[g], s2.ra[g], s2.dec[g]);
            const double chalf = cos(ang / 2), shalf = sin(ang / 2);
            bool shp = false, zerr_pair = false;
            if (EXTRA) {
                if (b.remove_shp) {
                    const int64_t fb1 = s1.fiberid[f1], fb2 = s2.fiberid[g];
                    shp = (s1.plate[f1] == s2.plate[g]) &&
                          ((fb1 <= 500 && fb2 <= 500) || (fb1 > 500 && fb2 > 500));
                }
                zerr_pair = b.zerr_on && (ang < b.zerr_ang);
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
            __syncwarp();
            const float cp = (float)(chalf * inv_p);
            const float st = (float)(shalf * inv_t);
            // r1 - r2 limits of pairs that can land in a bin, one bin of margin
            // each side: x = p - pmin in [-1, np + 1], |p| for auto-correlations
            const float lo_off = AUTO ? -(float)(np + 1u) / cp : (pmin_f - 1.f) / cp;
            const float hi_off = AUTO ? (float)(np + 1u) / cp : (pmin_f + (float)np + 1.f) / cp;
            int qn = 0;
            // One pass over forest-2 pixels [jb, jb + 32 P): lane l holds pixels
            // jb + P l + p, p < P. The forest is covered with P = 4 passes and
            // a last pass of P = 2 or 1 for a short remainder, so that few
            // slots are empty.
            auto pass = [&](auto p_const, const int jb) {
              constexpr int P = decltype(p_const)::value;
              // The FP64 re-decision queue is drained between passes over the
              // forest-1 pixels, outside the pixel loop, so that its FP64 code
              // does not hold registers in the loop; a pass stops early when
              // one more pixel could overflow the queue, and the next pass
              // reloads the forest-2 slots and resumes at that pixel.
              int i_next = -1, i_end = n1;
              for (;;) {
                // lane owns pixels jb + kCfP*lane + p (consecutive pixels, so the
                // lanes of a warp mostly fall in different r_par bins)
                float rh[P], rl[P], t[P], zv[P], wv[P], dv[P];
                bool any = false;
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    const int j = jb + P * lane + p;
                    rh[p] = kFar; rl[p] = 0.f; t[p] = kFar; zv[p] = kFar; wv[p] = 0.f; dv[p] = 0.f;
                    if (j < n2) {
                        const int64_t jj = b0 + j;
                        const double w2 = s2.weights[jj];
                        bool ok = w2 != 0;
                        if (EXTRA && zerr_pair && ok)
                            ok = !zerr_veto(s2.z[jj], f1_geom[6], b.zerr_kms);
                        if (ok) {
                            any = true;
                            const double r = s2.r_comov[jj];
                            rh[p] = (float)r;
                            rl[p] = (float)(r - (double)rh[p]);
                            t[p] = st * (float)s2.dist_m[jj] - 0.5f;
                            zv[p] = (float)s2.z[jj];
                            wv[p] = weight32(w2);
                            dv[p] = (float)(s2.delta[jj] * w2);
                        }
                    }
                }
                if (!__any_sync(0xffffffffu, any)) break;
                if (i_next < 0) {
                    int i_lo = 0, i_hi = n1;
                    if (sorted1)
                        window<P>(p1, n1, rh, t, st, lo_off, hi_off, t_end, i_lo, i_hi);
                    i_next = i_lo;
                    i_end = i_hi;
                }
                int i = i_next;

                for (; i < i_end; ++i) {
                    if (qn > kQueue - 32 * P) break;  // drain first (below)
                    const float2 qw = p2[i];
                    const float4 q = p1[i];
                    if (qw.x == 0.f) continue;  // zero-weight pixel (warp-uniform)
                    if (EXTRA && zerr_pair && zerr_veto(s1.z[a0 + i], ctx.zq2, b.zerr_kms))
                        continue;
                    const float ui = st * q.z;
                    unsigned near_mask = 0;
                    // Accepted pairs of this lane's consecutive slots that fall in
                    // the same bin are summed in registers (a run) and go to the
                    // ring as one entry, which halves the shared-memory atomics.
                    unsigned run_bin = 0u;
                    int run_n = 0;
                    float r_xi = 0.f, r_w = 0.f, r_pw = 0.f, r_tw = 0.f, r_zw = 0.f;
                    // stores the runs of the lanes in `flag` into the ring
                    auto store_runs = [&](bool flag) {
                        const unsigned m = __ballot_sync(0xffffffffu, flag);
                        const int pos = (tail + __popc(m & lt_mask)) & (kAccQ - 1);
                        if (flag) {
                            acc0[pos] = make_float4(r_xi, r_w, r_pw, r_tw);
                            acc1[pos] = make_float2(r_zw, __uint_as_float((run_bin << 3) |
                                                                          (unsigned)run_n));
                        }
                        tail += __popc(m);
                    };
#pragma unroll
                    for (int p = 0; p < P; ++p) {
                        const float pp = cp * ((q.x - rh[p]) + (q.y - rl[p]));
                        const float v = fabsf(pp);
                        const float pv = AUTO ? v : pp;
                        const float xp = LOWX ? fmaxf(pv - pc, low_clamp) : pv - pc;
                        const float xt = ui + t[p];
                        float fp, ft;
                        const unsigned ip = round_rem(xp, fp);
                        const unsigned it = round_rem(xt, ft);
                        bool near = (fabsf(fp) > h_par) | (fabsf(ft) > h_tr);
                        bool ok = (ip < np) & (it < nt);
                        const float zs = q.w + zv[p];
                        if (EXTRA) {
                            if (shp) {
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
                        near_mask |= (unsigned)near << p;
                        const bool acc = ok & !near;
                        const unsigned bin = ip * nt + it;
                        const bool extend = acc & (run_n > 0) & (bin == run_bin);
                        // a pair that starts a new run stores the previous one
                        store_runs(acc & (run_n > 0) & !extend);
                        if (acc) {
                            if (!extend) {
                                run_bin = bin;
                                run_n = 0;
                                r_xi = r_w = r_pw = r_tw = r_zw = 0.f;
                            }
                            const float w12 = qw.x * wv[p];
                            r_xi += qw.y * dv[p];
                            r_w += w12;
                            r_pw += pv * w12;
                            r_tw += (xt + 0.5f) * w12;
                            r_zw += zs * w12;
                            ++run_n;
                        }
                        if (p & 1) {
                            // at most 64 entries since the last check: the ring
                            // (kAccQ = 128 > 31 + 64) never overflows
                            while (tail - head >= 32) {
                                apply_accepted<true>(acc0, acc1, head, 32, h, hs);
                                head += 32;
                            }
                        }
                    }
                    store_runs(run_n > 0);
                    while (tail - head >= 32) {
                        apply_accepted<true>(acc0, acc1, head, 32, h, hs);
                        head += 32;
                    }
                    if (__any_sync(0xffffffffu, near_mask != 0)) {
                        // rare path: queue the pairs near an edge for FP64 re-decision
#pragma unroll
                        for (int p = 0; p < P; ++p) {
                            const bool near = (near_mask >> p) & 1u;
                            const unsigned nmask = __ballot_sync(0xffffffffu, near);
                            if (!nmask) continue;
                            const int cnt = __popc(nmask);
                            if (near) {
                                const int pos = qn + __popc(nmask & lt_mask);
                                queue[pos] = ((uint32_t)i << 16) | (uint32_t)(jb + P * lane + p);
                            }
                            qn += cnt;
                        }
                    }
                }
                if (lane == 0) visited[warp] += (unsigned long long)(i - i_next) * (32u * P);
                if (i >= i_end) break;
                cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
                if (lane == 0) atomicAdd(&scratch->recheck_overflows, 1ull);
                qn = 0;
                i_next = i;
              }
            };
            for (int jb = 0; jb < n2;) {
                const int rem = n2 - jb;
                if (rem > 64) {
                    pass(std::integral_constant<int, 4>{}, jb);
                    jb += 128;
                } else if (rem > 32) {
                    pass(std::integral_constant<int, 2>{}, jb);
                    jb += 64;
                } else {
                    pass(std::integral_constant<int, 1>{}, jb);
                    jb += 32;
                }
            }
            if (qn) cf_drain(b, fcp, s1, s2, ctx, queue, qn, h, scratch);
        }
        if (tail != head) apply_accepted<false>(acc0, acc1, head, tail - head, h, hs);
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
        const float dw = (float)(fs.delta[ia] * w1) * weight32(wq);
        const float pv = (float)(r_par * inv_p);
        const float tv = (float)(r_trans * inv_t);
        const float zs = (float)z1 + (float)zq;
        hist_add(h, fcp->hstride, (unsigned)bin, dw, w12, pv * w12, tv * w12, zs * w12, 1);
    }
    __syncwarp();
}

template <bool EXTRA>
__global__ void __launch_bounds__(kXcfBlock, 1) xcf_xi_fast_kernel(
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
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nbins = fcp->nbins;
    const double inv_p = fcp->inv_p, inv_t = fcp->inv_t;
    const float pc = fcp->pc;
    const float h_par = fcp->h_par, h_tr = fcp->h_tr;
    const unsigned np = fcp->np, nt = fcp->nt;
    const int hs = fcp->hstride;
    const SmemLayout L = smem_layout(nbins, max_pix1, nwarps, false);
    float *h = reinterpret_cast<float *>(smem + L.cells);
    float4 *p1 = reinterpret_cast<float4 *>(smem + L.p1);
    float2 *p2 = reinterpret_cast<float2 *>(smem + L.p2);
    uint32_t *queue = reinterpret_cast<uint32_t *>(smem + L.queue) + warp * kQueue;
    zero_all(h, H_COUNT * hs);
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
            bool any = false;
#pragma unroll
            for (int p = 0; p < kXcfP; ++p) {
                const int kk = kb + lane + 32 * p;
                cp[p] = 1.f; st[p] = 0.f; rh[p] = kFar; rl[p] = 0.f; t[p] = kFar; zv[p] = kFar;
                wv[p] = 0.f;
                if (kk < nq) {
                    const int64_t g = nbr_index[ctx.k0 + kk];
                    const double wq = objs.obj_weight[g];
                    if (wq != 0) {
                        any = true;
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
                        t[p] = st[p] * (float)objs.obj_dist_m[g] - 0.5f;
                        zv[p] = (float)objs.z_qso[g];
                        wv[p] = weight32(wq);
                    }
                }
            }
            if (!__any_sync(0xffffffffu, any)) continue;
            int qn = 0;
            for (int i = 0; i < n1; ++i) {
                const float2 qw = p2[i];
                if (qw.x == 0.f) continue;
                const float4 q = p1[i];
                unsigned near_mask = 0;
#pragma unroll
                for (int p = 0; p < kXcfP; ++p) {
                    const float pv = cp[p] * ((q.x - rh[p]) + (q.y - rl[p]));
                    const float xt = __fmaf_rn(st[p], q.z, t[p]);
                    float fp, ft;
                    const unsigned ip = round_rem(pv - pc, fp);
                    const unsigned it = round_rem(xt, ft);
                    bool near = (fabsf(fp) > h_par) | (fabsf(ft) > h_tr);
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
                    near_mask |= (unsigned)near << p;
                    if (ok & !near) {
                        const float w12 = qw.x * wv[p];
                        const unsigned bin = ip * nt + it;
                        hist_add(h, hs, bin, qw.y * wv[p], w12, pv * w12, (xt + 0.5f) * w12,
                                 zs * w12, 1);
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
                            const int pos = qn + __popc(nmask & lt_mask);
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
// cp (itself rounded, relative u), the rounding of pc = pmin + 1/2 and the
// subtraction add u |p|, u (|pmin| + 1/2) and u |x'|. Altogether the FP32 x'
// is within 6 u (|x| + |pmin| + 1) of the exact x - 1/2. For x_tr the FP32
// rounding of d1 and d2 (relative u), of st, of the two products, of the
// shift by 1/2 and of the sum give <= 6 u (|x_tr| + 1). round(x') and the
// remainder are exact (the magic-number add rounds to an integer and the
// subtraction is exact). Only pairs whose exact x lies in [-1, n + 1] matter
// (the others are rejected either way), so with a factor > 2 of margin
//   g = 16 u (n + |pmin| + 2) + 1e-6.
// The reference's own FP64 evaluation is within 1e-12 of the exact value,
// far inside these bands. With r_par_min = 0 in an auto-correlation x = |p|
// >= 0 and the lower edge of bin 0 cannot be crossed: x' is clamped from
// below at -1/2 + 2g, which keeps pairs with |p| < 2g (same-wavelength pixels
// give p = 0 exactly) in bin 0 without flagging them.
FastConst make_fast_const(const Binning &b) {
    FastConst fc{};
    const double u = 1.0 / 16777216.0;
    fc.inv_p = (double)b.np / b.r_par_range;
    fc.inv_t = (double)b.nt / b.r_trans_max;
    const double pmin = b.r_par_min * fc.inv_p;
    fc.pc = (float)(pmin + 0.5);
    double g_par = 16 * u * (b.np + fabs(pmin) + 2) + 1e-6;
    double g_tr = 16 * u * (b.nt + 2) + 1e-6;
    if (!(g_par < 0.05)) g_par = 0.05;  // absurd bin counts: almost everything is re-decided
    if (!(g_tr < 0.05)) g_tr = 0.05;
    fc.h_par = (float)(0.5 - g_par);
    fc.h_tr = (float)(0.5 - g_tr);
    fc.low_clamp = (float)(-0.5 + 2 * g_par);
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
    const int max_pix1 = s1.max_pixels;
    // as many warps (up to kCfBlock / 32) as the per-warp queues leave room for
    int nwarps = kCfBlock / 32;
    while (nwarps > 1 && smem_layout(b.nbins, max_pix1, nwarps, true).total > 227 * 1024)
        --nwarps;
    const int block = nwarps * 32;
    const size_t smem = smem_layout(b.nbins, max_pix1, nwarps, true).total;
    if (smem > 227 * 1024) return PG_ERR_UNSUPPORTED;
    (void)ang_max;
    int rc = prepare_fast(b, fc, stream);
    if (rc) return rc;
    const bool extra = b.remove_shp || b.zmin_on || b.zmax_on || b.zerr_on;
    const bool autoc = !b.x_correlation;
    const bool lowx = autoc && b.r_par_min == 0.0;
    int grid = 0;
#define PG_LAUNCH_CF(A, E, L)                                                                  \
    rc = persistent_grid(cf_xi_fast_kernel<A, E, L>, block, smem, num_sms, num_work, &grid);   \
    if (rc) return rc;                                                                         \
    cf_xi_fast_kernel<A, E, L><<<grid, block, smem, stream>>>(b, fc, s1, s2, nbr_offsets,      \
                                                              nbr_index, nbr_angle,            \
                                                              work_order, num_work, out,       \
                                                              scratch, max_pix1);
    if (autoc && lowx && !extra) { PG_LAUNCH_CF(true, false, true) }
    else if (autoc && lowx && extra) { PG_LAUNCH_CF(true, true, true) }
    else if (autoc && !extra) { PG_LAUNCH_CF(true, false, false) }
    else if (autoc && extra) { PG_LAUNCH_CF(true, true, false) }
    else if (!extra) { PG_LAUNCH_CF(false, false, false) }
    else { PG_LAUNCH_CF(false, true, false) }
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
    const int block = kXcfBlock;
    const int max_pix1 = forests.max_pixels;
    const size_t smem = smem_layout(b.nbins, max_pix1, block / 32, false).total;
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
