// Distortion matrix of the auto-correlation: cf.compute_dmat
// (py/picca/cf.py:390-517) and cf.compute_dmat_forest_pairs_fast
// (py/picca/cf.py:519-887).
//
// One CTA per selected forest pair (a persistent kernel over a cost-ordered
// pair list). The reference adds, for every selected pixel pair q = (i, j)
// in data bin b and every model bin k touched by the forest pair,
//   w12 * (eta5[k] + eta6[k] dll2_j + eta7[k] dll1_i + eta8[k] dll1_i dll2_j
//          - eta1[i,k] - eta2[j,k] - eta3[i,k] dll2_j - eta4[j,k] dll1_i)
// to dmat[b, k]. Summed over the pairs of one data bin this is a dense
// product D[b, k] = sum_kappa U[b, kappa] E[k, kappa] over
//   kappa = i    : U = sum_j w12              E = -eta1[i, k]
//   kappa = j    : U = sum_i w12              E = -eta2[j, k]
//   kappa = i'   : U = sum_j w12 dll2_j       E = -eta3[i, k]   (order2 == 1)
//   kappa = j'   : U = sum_i w12 dll1_i       E = -eta4[j, k]   (order1 == 1)
//   four rows    : U = (A, B, C, D)_b         E = eta5..eta8
// with A = sum w12, B = sum w12 dll2, C = sum w12 dll1, D = sum w12 dll1 dll2
// over the selected pairs of the bin. The kernel therefore
//   1. classifies every pixel pair (bitmaps of the touched model bins and of
//      the data bins of selected pairs; the reference's early return when no
//      pair counts),
//   2. builds U (data bins x kappa) and E (model bins x kappa) in per-CTA
//      global scratch with a row sweep (a thread per pixel of forest 1) and a
//      column sweep (a thread per pixel of forest 2), merging runs of equal
//      bins in registers; the row sweep also adds the Kronecker term
//      w12 * zfac and the effective (r_par, r_trans, z, weight) sums,
//   3. reduces the four rank rows,
//   4. multiplies U by E^T in 32 x 32 FP64 tiles and adds the tile to the
//      global matrix with atomics.
// All arithmetic is FP64 (the library is compiled with -fmad=false); sums
// are reassociated with respect to the reference, so results agree to a few
// ulp of the summed magnitudes, not bit for bit.
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kDmBlock = 256;
constexpr int kDmWarps = kDmBlock / 32;
constexpr int kTile = 32;   // GEMM output tile edge (data bins x model bins)
constexpr int kSlab = 16;   // GEMM reduction step
constexpr int kTilePad = kTile + 1;

struct DmatConst {
    Binning b;
    int32_t nmp, nmt, nm;    // model bins along r_par, r_trans, total
    int32_t redshift_evolution;
    double z_ref, alpha, alpha2;
    double inv_r_par_range, inv_r_trans_max;  // reciprocals for the bin estimate
    int32_t p1, p2;          // pixel capacity of the shared-memory forest slots
    int32_t mwords, dwords;  // bitmap words (model, data)
    int64_t list_doubles;    // per-CTA scratch: bin lists (nm + nb int32), in doubles
    int64_t work_doubles;    // per-CTA scratch: U and E rows
    int64_t cta_doubles;     // list_doubles + work_doubles
};

// Shared-memory layout (bytes), identical on host and device.
struct DmSmem {
    size_t f1, f2, flags1, flags2, mbits, mpref, dbits, dpref, tile_a, tile_b, total;
};

__host__ __device__ inline size_t dm_align(size_t v, size_t a) { return (v + a - 1) / a * a; }

__host__ __device__ inline DmSmem dm_smem(int p1, int p2, int mwords, int dwords) {
    DmSmem s;
    size_t o = 0;
    s.f1 = o; o += sizeof(double) * 6 * (size_t)p1;
    s.f2 = o; o += sizeof(double) * 6 * (size_t)p2;
    s.flags1 = o; o = dm_align(o + (size_t)p1, 8);
    s.flags2 = o; o = dm_align(o + (size_t)p2, 8);
    s.mbits = o; o += sizeof(uint32_t) * (size_t)mwords;
    s.mpref = o; o += sizeof(int32_t) * (size_t)mwords;
    s.dbits = o; o += sizeof(uint32_t) * (size_t)dwords;
    s.dpref = o; o += sizeof(int32_t) * (size_t)dwords;
    o = dm_align(o, 16);
    s.tile_a = o; o += sizeof(double) * kSlab * kTilePad;
    s.tile_b = o; o += sizeof(double) * kSlab * kTilePad;
    s.total = dm_align(o, 16);
    return s;
}

struct DmPair {
    double rp, rt, z;
    int32_t db, mb;
    bool counted;  // passes the same-half-plate veto (the reference's num_pairs)
    bool zsel;     // passes the z_min / z_max cut
};

// floor(x * n) of the reference for x = num / den, from an estimate
// x' = num * (1 / den) (a few ulp from x): the estimate decides unless
// x' * n is within 1e-9 of an integer, where the exact quotient is formed.
__device__ __forceinline__ double dm_floor_bin(double est, double num, double den, int32_t n) {
    const double y = __dmul_rn(est, (double)n);
    const double f = floor(y);
    if (__dsub_rn(y, f) > 1e-9 && __dsub_rn(__dadd_rn(f, 1.), y) > 1e-9) return f;
    return floor(__dmul_rn(num / den, (double)n));
}

// Pixel-pair decision and bins of compute_dmat_forest_pairs_fast
// (py/picca/cf.py:544-568 and :620-700), in the reference's operation order;
// the bin quotients (r_par - r_par_min) / (r_par_max - r_par_min) and
// r_trans / r_trans_max are estimated with reciprocals and formed exactly
// only next to a bin edge (dm_floor_bin).
__device__ __forceinline__ bool dm_pair(const DmatConst &c, double r1, double m1, double z1,
                                        double r2, double m2, double z2, double cc, double ss,
                                        bool shp, DmPair &o) {
    double rp = __dmul_rn(__dsub_rn(r1, r2), cc);
    double rt = __dmul_rn(__dadd_rn(m1, m2), ss);
    if (c.b.rmu) {
        rt = __dsqrt_rn(__dadd_rn(__dmul_rn(rt, rt), __dmul_rn(rp, rp)));
        rp = rp / rt;
    }
    if (!c.b.x_correlation) rp = fabs(rp);
    if (rp >= c.b.r_par_max || rt >= c.b.r_trans_max || rp < c.b.r_par_min) return false;
    const double np_num = __dsub_rn(rp, c.b.r_par_min);
    const double fp = __dmul_rn(np_num, c.inv_r_par_range);
    const double ft = __dmul_rn(rt, c.inv_r_trans_max);
    const double bp = dm_floor_bin(fp, np_num, c.b.r_par_range, c.b.np);
    const double bt = dm_floor_bin(ft, rt, c.b.r_trans_max, c.b.nt);
    o.db = (int32_t)__dadd_rn(bt, __dmul_rn((double)c.b.nt, bp));
    const double mp = dm_floor_bin(fp, np_num, c.b.r_par_range, c.nmp);
    const double mt = dm_floor_bin(ft, rt, c.b.r_trans_max, c.nmt);
    o.mb = (int32_t)__dadd_rn(mt, __dmul_rn((double)c.nmt, mp));
    o.z = __dadd_rn(z1, z2) / 2;
    o.counted = !(c.b.remove_shp && shp && fabs(rp) < c.b.half_plate_cut);
    o.zsel = !((c.b.zmin_on && o.z < c.b.z_min) || (c.b.zmax_on && o.z > c.b.z_max));
    o.rp = rp;
    o.rt = rt;
    return true;
}

__device__ __forceinline__ int dm_rank(const uint32_t *bits, const int32_t *pref, int32_t bin) {
    const int w = bin >> 5;
    const uint32_t below = bits[w] & ((1u << (bin & 31)) - 1u);
    return pref[w] + __popc(below);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum (every thread gets the result). Uses red[kDmWarps].
__device__ double dm_block_sum(double v, double *red) {
    v = warp_sum(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.;
    for (int k = 0; k < kDmWarps; ++k) t += red[k];
    return t;
}

// Exclusive prefix of popcounts over a bitmap; returns the total.
__device__ int dm_scan_bits(const uint32_t *bits, int32_t *pref, int words, int *red_int) {
    const int per = (words + kDmBlock - 1) / kDmBlock;
    const int w0 = min(words, (int)threadIdx.x * per), w1 = min(words, w0 + per);
    int local = 0;
    for (int w = w0; w < w1; ++w) local += __popc(bits[w]);
    // inclusive scan of the per-thread totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();
    if (lane == 31) red_int[warp] = incl;
    __syncthreads();
    int base = 0, total = 0;
    for (int k = 0; k < kDmWarps; ++k) {
        if (k < warp) base += red_int[k];
        total += red_int[k];
    }
    int run = base + incl - local;
    for (int w = w0; w < w1; ++w) {
        pref[w] = run;
        run += __popc(bits[w]);
    }
    __syncthreads();
    return total;
}

struct DmItem {
    int32_t n1, n2;
    double cc, ss;
    double sw1, sw2, swsll1, swsll2;
    double inv_sw1, inv_sw2, inv_q1, inv_q2;  // reciprocals of the four sums
    int32_t order1, order2;
    bool shp;
};

__global__ void __launch_bounds__(kDmBlock)
    cf_dmat_kernel(DmatConst c, pg_forest_set s1, pg_forest_set s2, const double *ll1,
                   const double *ll2, const int32_t *order1g, const int32_t *order2g,
                   const int32_t *pair_first, const int32_t *pair_second,
                   const double *pair_angle, int64_t num_pairs, pg_dmat_sums out,
                   double *work, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const DmSmem L = dm_smem(c.p1, c.p2, c.mwords, c.dwords);
    double *f1 = reinterpret_cast<double *>(smem + L.f1);
    double *f2 = reinterpret_cast<double *>(smem + L.f2);
    double *r1s = f1, *m1s = f1 + c.p1, *z1s = f1 + 2 * c.p1, *w1s = f1 + 3 * c.p1,
           *d1s = f1 + 4 * c.p1, *zf1s = f1 + 5 * c.p1;
    double *r2s = f2, *m2s = f2 + c.p2, *z2s = f2 + 2 * c.p2, *w2s = f2 + 3 * c.p2,
           *d2s = f2 + 4 * c.p2, *zf2s = f2 + 5 * c.p2;
    unsigned char *sel1 = smem + L.flags1, *sel2 = smem + L.flags2;
    uint32_t *mbits = reinterpret_cast<uint32_t *>(smem + L.mbits);
    int32_t *mpref = reinterpret_cast<int32_t *>(smem + L.mpref);
    uint32_t *dbits = reinterpret_cast<uint32_t *>(smem + L.dbits);
    int32_t *dpref = reinterpret_cast<int32_t *>(smem + L.dpref);
    double (*ta)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_a);
    double (*tb)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_b);
    __shared__ double red[kDmWarps];
    __shared__ int red_int[kDmWarps];
    __shared__ int s_item;
    __shared__ int s_count;

    const int tid = threadIdx.x;
    const int nb = c.b.nbins, nm = c.nm;
    double *cta = work + (int64_t)blockIdx.x * c.cta_doubles;
    int32_t *dlist = reinterpret_cast<int32_t *>(cta);  // [nb]
    int32_t *mlist = dlist + nb;                         // [nm]
    double *rows = cta + c.list_doubles;

    for (;;) {
        if (tid == 0) s_item = atomicAdd(&scratch->work_counter, 1);
        __syncthreads();
        const int64_t q = s_item;
        if (q >= num_pairs) break;
        const int f = pair_first[q], g = pair_second[q];
        DmItem it;
        const int64_t o1 = s1.pix_offset[f], o2 = s2.pix_offset[g];
        it.n1 = (int32_t)(s1.pix_offset[f + 1] - o1);
        it.n2 = (int32_t)(s2.pix_offset[g + 1] - o2);
        if (it.n1 > c.p1 || it.n2 > c.p2) {
            if (tid == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)q);
            __syncthreads();
            continue;
        }
        const double ang = pair_angle ? pair_angle[q]
                                      : angle_between(s1.x_cart[f], s1.y_cart[f], s1.z_cart[f],
                                                      s1.ra[f], s1.dec[f], s1.cos_dec[f],
                                                      s2.x_cart[g], s2.y_cart[g], s2.z_cart[g],
                                                      s2.ra[g], s2.dec[g]);
        it.cc = cos(ang / 2);
        it.ss = sin(ang / 2);
        it.order1 = order1g[f];
        it.order2 = order2g[g];
        it.shp = false;
        if (c.b.remove_shp && s1.plate[f] == s2.plate[g]) {
            const int64_t a = s1.fiberid[f], b2 = s2.fiberid[g];
            it.shp = (a <= 500 && b2 <= 500) || (a > 500 && b2 > 500);
        }
        const bool zerr_on = c.b.zerr_on && ang < c.b.zerr_ang;
        const double zq1 = s1.z_qso[f], zq2 = s2.z_qso[g];

        // stage the pixels
        for (int t = tid; t < it.n1; t += kDmBlock) {
            r1s[t] = s1.r_comov[o1 + t];
            m1s[t] = s1.dist_m[o1 + t];
            z1s[t] = s1.z[o1 + t];
            w1s[t] = s1.weights[o1 + t];
            d1s[t] = ll1[o1 + t];
            sel1[t] = !(zerr_on && zerr_veto(z1s[t], zq2, c.b.zerr_kms));
        }
        for (int t = tid; t < it.n2; t += kDmBlock) {
            r2s[t] = s2.r_comov[o2 + t];
            m2s[t] = s2.dist_m[o2 + t];
            z2s[t] = s2.z[o2 + t];
            w2s[t] = s2.weights[o2 + t];
            d2s[t] = ll2[o2 + t];
            sel2[t] = !(zerr_on && zerr_veto(z2s[t], zq1, c.b.zerr_kms));
        }
        for (int t = tid; t < c.mwords; t += kDmBlock) mbits[t] = 0u;
        for (int t = tid; t < c.dwords; t += kDmBlock) dbits[t] = 0u;
        if (tid == 0) s_count = 0;
        __syncthreads();

        // 1. classification: touched model bins, data bins of selected pairs
        {
            const int warp = tid >> 5, lane = tid & 31;
            int counted = 0;
            for (int i = warp; i < it.n1; i += kDmWarps) {
                const double r1 = r1s[i], m1 = m1s[i], z1 = z1s[i];
                if (w1s[i] == 0.) continue;
                for (int j = lane; j < it.n2; j += 32) {
                    if (w2s[j] == 0.) continue;
                    DmPair o;
                    if (!dm_pair(c, r1, m1, z1, r2s[j], m2s[j], z2s[j], it.cc, it.ss, it.shp, o))
                        continue;
                    if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) {
                        report_error(scratch, PG_ERR_BIN_RANGE, o.mb);
                        continue;
                    }
                    counted += o.counted;
                    const uint32_t mbit = 1u << (o.mb & 31);
                    if (!(mbits[o.mb >> 5] & mbit)) atomicOr(&mbits[o.mb >> 5], mbit);
                    if (o.counted && o.zsel && sel1[i] && sel2[j]) {
                        const uint32_t dbit = 1u << (o.db & 31);
                        if (!(dbits[o.db >> 5] & dbit)) atomicOr(&dbits[o.db >> 5], dbit);
                    }
                }
            }
            for (int o = 16; o > 0; o >>= 1) counted += __shfl_xor_sync(0xffffffffu, counted, o);
            if (lane == 0 && counted) atomicAdd(&s_count, counted);
        }
        __syncthreads();
        if (s_count == 0) {
            __syncthreads();
            continue;
        }
        const int nmt = dm_scan_bits(mbits, mpref, c.mwords, red_int);
        const int nbt = dm_scan_bits(dbits, dpref, c.dwords, red_int);
        if (nbt == 0) {  // no selected pair: nothing reaches the matrix
            __syncthreads();
            continue;
        }
        if (tid == 0) atomicAdd(&scratch->work_items, 1ull);
        for (int w = tid; w < c.mwords; w += kDmBlock) {
            uint32_t bits = mbits[w];
            int k = mpref[w];
            while (bits) {
                const int bit = __ffs(bits) - 1;
                mlist[k++] = w * 32 + bit;
                bits &= bits - 1u;
            }
        }
        for (int w = tid; w < c.dwords; w += kDmBlock) {
            uint32_t bits = dbits[w];
            int k = dpref[w];
            while (bits) {
                const int bit = __ffs(bits) - 1;
                dlist[k++] = w * 32 + bit;
                bits &= bits - 1u;
            }
        }

        // auxiliary sums (py/picca/cf.py:573-595)
        double lw = 0., lsw = 0.;
        for (int t = tid; t < it.n1; t += kDmBlock) {
            lw += w1s[t];
            lsw += __dmul_rn(d1s[t], w1s[t]);
        }
        it.sw1 = dm_block_sum(lw, red);
        const double sll1 = dm_block_sum(lsw, red);
        lw = 0.;
        lsw = 0.;
        for (int t = tid; t < it.n2; t += kDmBlock) {
            lw += w2s[t];
            lsw += __dmul_rn(d2s[t], w2s[t]);
        }
        it.sw2 = dm_block_sum(lw, red);
        const double sll2 = dm_block_sum(lsw, red);
        const double mean1 = sll1 / it.sw1, mean2 = sll2 / it.sw2;
        double q1 = 0., q2 = 0.;
        for (int t = tid; t < it.n1; t += kDmBlock) {
            const double d = __dsub_rn(d1s[t], mean1);
            d1s[t] = d;
            q1 += __dmul_rn(w1s[t], __dmul_rn(d, d));
            zf1s[t] = c.redshift_evolution
                          ? pow(__dadd_rn(1., z1s[t]) / __dadd_rn(1., c.z_ref),
                                __dsub_rn(c.alpha, 1.))
                          : 1.;
        }
        for (int t = tid; t < it.n2; t += kDmBlock) {
            const double d = __dsub_rn(d2s[t], mean2);
            d2s[t] = d;
            q2 += __dmul_rn(w2s[t], __dmul_rn(d, d));
            zf2s[t] = c.redshift_evolution
                          ? pow(__dadd_rn(1., z2s[t]) / __dadd_rn(1., c.z_ref),
                                __dsub_rn(c.alpha2, 1.))
                          : 1.;
        }
        it.swsll1 = dm_block_sum(q1, red);
        it.swsll2 = dm_block_sum(q2, red);
        it.inv_sw1 = 1. / it.sw1;
        it.inv_sw2 = 1. / it.sw2;
        it.inv_q1 = 1. / it.swsll1;
        it.inv_q2 = 1. / it.swsll2;

        // kappa layout of the U and E rows
        const int n1 = it.n1, n2 = it.n2;
        const int kU = 0, kX = n1, kV = n1 + n2;
        const int kY = kV + (it.order2 == 1 ? n1 : 0);
        const int kR = kY + (it.order1 == 1 ? n2 : 0);
        const int kst = (int)dm_align((size_t)kR + 4, kSlab);
        const int64_t cap = c.work_doubles / kst;
        int dc = nbt, mc = nmt;
        if ((int64_t)nbt + nmt > cap) {
            dc = (int)min((int64_t)nbt, cap / 2);
            mc = (int)(cap - dc);
        }
        const bool ord1 = it.order1 == 1, ord2 = it.order2 == 1;

        for (int d0 = 0; d0 < nbt; d0 += dc) {
            const int dcc = min(dc, nbt - d0);
            for (int m0 = 0; m0 < nmt; m0 += mc) {
                const int mcc = min(mc, nmt - m0);
                const bool first = d0 == 0 && m0 == 0;
                double *U = rows;
                double *E = rows + (int64_t)dcc * kst;
                {
                    const int64_t n = (int64_t)(dcc + mcc) * kst / 2;
                    double2 *p = reinterpret_cast<double2 *>(rows);
                    for (int64_t t = tid; t < n; t += kDmBlock) p[t] = make_double2(0., 0.);
                }
                __syncthreads();

                // 2a. row sweep: a thread per pixel i of forest 1
                for (int i = tid; i < n1; i += kDmBlock) {
                    const double w1 = w1s[i];
                    if (w1 == 0.) continue;
                    const double r1 = r1s[i], m1 = m1s[i], z1 = z1s[i], zf1 = zf1s[i];
                    const bool ok1 = sel1[i];
                    int run_m = -1, run_d = -1;
                    double e1 = 0., e3 = 0., u = 0., v = 0.;
                    int64_t run_k = -1;
                    int32_t k_db = 0, k_mb = 0;
                    double k_dm = 0., k_w = 0., k_rp = 0., k_rt = 0., k_z = 0.;
                    for (int j = 0; j < n2; ++j) {
                        const double w2 = w2s[j];
                        if (w2 == 0.) continue;
                        DmPair o;
                        if (!dm_pair(c, r1, m1, z1, r2s[j], m2s[j], z2s[j], it.cc, it.ss, it.shp,
                                     o))
                            continue;
                        if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) continue;
                        const double zfac = c.redshift_evolution ? __dmul_rn(zf1, zf2s[j]) : 1.;
                        const int ml = dm_rank(mbits, mpref, o.mb) - m0;
                        if (ml >= 0 && ml < mcc) {
                            if (ml != run_m) {
                                if (run_m >= 0) {
                                    E[(int64_t)run_m * kst + kU + i] -= e1;
                                    if (ord2) E[(int64_t)run_m * kst + kV + i] -= e3;
                                }
                                run_m = ml;
                                e1 = 0.;
                                e3 = 0.;
                            }
                            e1 += __dmul_rn(__dmul_rn(zfac, w2), it.inv_sw2);
                            if (ord2) e3 += __dmul_rn(__dmul_rn(__dmul_rn(zfac, w2), d2s[j]), it.inv_q2);
                        }
                        if (o.counted && o.zsel && ok1 && sel2[j]) {
                            const double w12 = __dmul_rn(w1, w2);
                            const int dl = dm_rank(dbits, dpref, o.db) - d0;
                            if (dl >= 0 && dl < dcc) {
                                if (dl != run_d) {
                                    if (run_d >= 0) {
                                        U[(int64_t)run_d * kst + kU + i] += u;
                                        if (ord2) U[(int64_t)run_d * kst + kV + i] += v;
                                    }
                                    run_d = dl;
                                    u = 0.;
                                    v = 0.;
                                }
                                u += w12;
                                if (ord2) v += __dmul_rn(w12, d2s[j]);
                            }
                            if (first) {
                                const int64_t key = (int64_t)o.db * nm + o.mb;
                                if (key != run_k) {
                                    if (run_k >= 0) {
                                        atomicAdd(&out.dmat[run_k], k_dm);
                                        atomicAdd(&out.weights_dmat[k_db], k_w);
                                        atomicAdd(&out.r_par_eff[k_mb], k_rp);
                                        atomicAdd(&out.r_trans_eff[k_mb], k_rt);
                                        atomicAdd(&out.z_eff[k_mb], k_z);
                                        atomicAdd(&out.weight_eff[k_mb], k_w);
                                    }
                                    run_k = key;
                                    k_db = o.db;
                                    k_mb = o.mb;
                                    k_dm = k_w = k_rp = k_rt = k_z = 0.;
                                }
                                k_dm += __dmul_rn(w12, zfac);
                                k_w += w12;
                                k_rp += __dmul_rn(w12, o.rp);
                                k_rt += __dmul_rn(w12, o.rt);
                                k_z += __dmul_rn(w12, o.z);
                            }
                        }
                    }
                    if (run_m >= 0) {
                        E[(int64_t)run_m * kst + kU + i] -= e1;
                        if (ord2) E[(int64_t)run_m * kst + kV + i] -= e3;
                    }
                    if (run_d >= 0) {
                        U[(int64_t)run_d * kst + kU + i] += u;
                        if (ord2) U[(int64_t)run_d * kst + kV + i] += v;
                    }
                    if (run_k >= 0) {
                        atomicAdd(&out.dmat[run_k], k_dm);
                        atomicAdd(&out.weights_dmat[k_db], k_w);
                        atomicAdd(&out.r_par_eff[k_mb], k_rp);
                        atomicAdd(&out.r_trans_eff[k_mb], k_rt);
                        atomicAdd(&out.z_eff[k_mb], k_z);
                        atomicAdd(&out.weight_eff[k_mb], k_w);
                    }
                }

                // 2b. column sweep: a thread per pixel j of forest 2
                for (int j = tid; j < n2; j += kDmBlock) {
                    const double w2 = w2s[j];
                    if (w2 == 0.) continue;
                    const double r2 = r2s[j], m2 = m2s[j], z2 = z2s[j], zf2 = zf2s[j];
                    const bool ok2 = sel2[j];
                    int run_m = -1, run_d = -1;
                    double e2 = 0., e4 = 0., x = 0., y = 0.;
                    for (int i = 0; i < n1; ++i) {
                        const double w1 = w1s[i];
                        if (w1 == 0.) continue;
                        DmPair o;
                        if (!dm_pair(c, r1s[i], m1s[i], z1s[i], r2, m2, z2, it.cc, it.ss, it.shp,
                                     o))
                            continue;
                        if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) continue;
                        const double zfac = c.redshift_evolution ? __dmul_rn(zf1s[i], zf2) : 1.;
                        const int ml = dm_rank(mbits, mpref, o.mb) - m0;
                        if (ml >= 0 && ml < mcc) {
                            if (ml != run_m) {
                                if (run_m >= 0) {
                                    E[(int64_t)run_m * kst + kX + j] -= e2;
                                    if (ord1) E[(int64_t)run_m * kst + kY + j] -= e4;
                                }
                                run_m = ml;
                                e2 = 0.;
                                e4 = 0.;
                            }
                            e2 += __dmul_rn(__dmul_rn(zfac, w1), it.inv_sw1);
                            if (ord1) e4 += __dmul_rn(__dmul_rn(__dmul_rn(zfac, w1), d1s[i]), it.inv_q1);
                        }
                        if (o.counted && o.zsel && ok2 && sel1[i]) {
                            const double w12 = __dmul_rn(w1, w2);
                            const int dl = dm_rank(dbits, dpref, o.db) - d0;
                            if (dl >= 0 && dl < dcc) {
                                if (dl != run_d) {
                                    if (run_d >= 0) {
                                        U[(int64_t)run_d * kst + kX + j] += x;
                                        if (ord1) U[(int64_t)run_d * kst + kY + j] += y;
                                    }
                                    run_d = dl;
                                    x = 0.;
                                    y = 0.;
                                }
                                x += w12;
                                if (ord1) y += __dmul_rn(w12, d1s[i]);
                            }
                        }
                    }
                    if (run_m >= 0) {
                        E[(int64_t)run_m * kst + kX + j] -= e2;
                        if (ord1) E[(int64_t)run_m * kst + kY + j] -= e4;
                    }
                    if (run_d >= 0) {
                        U[(int64_t)run_d * kst + kX + j] += x;
                        if (ord1) U[(int64_t)run_d * kst + kY + j] += y;
                    }
                }
                __syncthreads();

                // 3. rank rows: (A, B, C, D) per data bin, eta5..eta8 per model bin
                {
                    const int warp = tid >> 5, lane = tid & 31;
                    for (int r = warp; r < dcc + mcc; r += kDmWarps) {
                        double s0 = 0., s1v = 0., s2v = 0., s3 = 0.;
                        if (r < dcc) {
                            const double *row = U + (int64_t)r * kst;
                            for (int i = lane; i < n1; i += 32) {
                                const double a = row[kU + i];
                                s0 += a;
                                s2v += __dmul_rn(d1s[i], a);
                                if (ord1 && ord2) s3 += __dmul_rn(d1s[i], row[kV + i]);
                            }
                            for (int j = lane; j < n2; j += 32) s1v += __dmul_rn(d2s[j], row[kX + j]);
                        } else {
                            const double *row = E + (int64_t)(r - dcc) * kst;
                            for (int i = lane; i < n1; i += 32) {
                                const double a1 = __dmul_rn(w1s[i], it.inv_sw1);
                                const double e1 = row[kU + i];
                                s0 -= __dmul_rn(a1, e1);
                                if (ord2) s1v -= __dmul_rn(a1, row[kV + i]);
                                if (ord1) {
                                    const double a7 = __dmul_rn(__dmul_rn(w1s[i], d1s[i]), it.inv_q1);
                                    s2v -= __dmul_rn(a7, e1);
                                    if (ord2) s3 -= __dmul_rn(a7, row[kV + i]);
                                }
                            }
                        }
                        s0 = warp_sum(s0);
                        s1v = warp_sum(s1v);
                        s2v = warp_sum(s2v);
                        s3 = warp_sum(s3);
                        if (lane == 0) {
                            double *row = (r < dcc ? U + (int64_t)r * kst : E + (int64_t)(r - dcc) * kst);
                            row[kR + 0] = s0;
                            row[kR + 1] = s1v;
                            row[kR + 2] = s2v;
                            row[kR + 3] = s3;
                        }
                    }
                }
                __syncthreads();

                // 4. D = U E^T in 32 x 32 tiles, added to the global matrix
                if (tid == 0)
                    atomicAdd(&scratch->gemm_macs,
                              (unsigned long long)dcc * (unsigned long long)mcc * (kR + 4));
                const int tx = tid & 15, ty = tid >> 4;
                for (int td = 0; td < dcc; td += kTile) {
                    for (int tm = 0; tm < mcc; tm += kTile) {
                        double acc[2][2];
#pragma unroll
                        for (int a = 0; a < 2; ++a)
#pragma unroll
                            for (int b2 = 0; b2 < 2; ++b2) acc[a][b2] = 0.;
                        for (int k0 = 0; k0 < kst; k0 += kSlab) {
                            for (int e = tid; e < kTile * kSlab; e += kDmBlock) {
                                const int rr = e / kSlab, kk = e % kSlab;
                                ta[kk][rr] = (td + rr < dcc) ? U[(int64_t)(td + rr) * kst + k0 + kk] : 0.;
                                tb[kk][rr] = (tm + rr < mcc) ? E[(int64_t)(tm + rr) * kst + k0 + kk] : 0.;
                            }
                            __syncthreads();
#pragma unroll
                            for (int kk = 0; kk < kSlab; ++kk) {
                                double av[2], bv[2];
#pragma unroll
                                for (int a = 0; a < 2; ++a) av[a] = ta[kk][ty + 16 * a];
#pragma unroll
                                for (int b2 = 0; b2 < 2; ++b2) bv[b2] = tb[kk][tx + 16 * b2];
#pragma unroll
                                for (int a = 0; a < 2; ++a)
#pragma unroll
                                    for (int b2 = 0; b2 < 2; ++b2)
                                        acc[a][b2] = __fma_rn(av[a], bv[b2], acc[a][b2]);
                            }
                            __syncthreads();
                        }
#pragma unroll
                        for (int a = 0; a < 2; ++a) {
                            const int dl = td + ty + 16 * a;
                            if (dl >= dcc) continue;
                            const int64_t base = (int64_t)dlist[d0 + dl] * nm;
#pragma unroll
                            for (int b2 = 0; b2 < 2; ++b2) {
                                const int ml = tm + tx + 16 * b2;
                                if (ml < mcc && acc[a][b2] != 0.)
                                    atomicAdd(&out.dmat[base + mlist[m0 + ml]], acc[a][b2]);
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
}

}  // namespace

int dmat_config(const pg_corr_params &p, const pg_dmat_params &d, int p1, int p2, int num_sms,
                DmatConstHost &h) {
    if (d.num_model_bins_r_par <= 0 || d.num_model_bins_r_trans <= 0) return PG_ERR_INVALID_ARGUMENT;
    if (p1 <= 0 || p2 <= 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t nm = (int64_t)d.num_model_bins_r_par * d.num_model_bins_r_trans;
    const int64_t nb = (int64_t)p.num_bins_r_par * p.num_bins_r_trans;
    if (nm > (1 << 26) || nb > (1 << 26)) return PG_ERR_UNSUPPORTED;
    const int mwords = (int)((nm + 31) / 32), dwords = (int)((nb + 31) / 32);
    const DmSmem s = dm_smem(p1, p2, mwords, dwords);
    if (s.total > 200 * 1024) return PG_ERR_UNSUPPORTED;
    h.smem = s.total;
    h.p1 = p1;
    h.p2 = p2;
    h.mwords = mwords;
    h.dwords = dwords;
    const int64_t kcap = (int64_t)dm_align((size_t)2 * p1 + 2 * p2 + 4, kSlab);
    if (d.row_capacity < 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t wanted = d.row_capacity > 0 ? std::max<int64_t>(d.row_capacity, 2)
                                              : kDmatRowCapacity;
    const int64_t rows = std::min<int64_t>(nb + nm, wanted);
    h.list_doubles = (int64_t)dm_align((size_t)(nb + nm), 32) / 2;
    h.work_doubles = rows * kcap;
    h.cta_doubles = (int64_t)dm_align((size_t)(h.list_doubles + h.work_doubles), 32);
    int occ = 0;
    if (cudaFuncSetAttribute(cf_dmat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)s.total) != cudaSuccess)
        return PG_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cf_dmat_kernel, kDmBlock, s.total) !=
            cudaSuccess ||
        occ < 1)
        return PG_ERR_CUDA;
    h.max_grid = num_sms * occ;
    return PG_OK;
}

int launch_cf_dmat(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h,
                   const pg_forest_set &s1, const pg_forest_set &s2, const double *ll1,
                   const double *ll2, const int32_t *order1, const int32_t *order2,
                   const int32_t *pair_first, const int32_t *pair_second,
                   const double *pair_angle, int64_t num_pairs, double *work, int grid,
                   const pg_dmat_sums &out, Scratch *scratch, cudaStream_t stream) {
    if (num_pairs == 0) return PG_OK;
    DmatConst c;
    c.b = make_binning(p);
    c.nmp = d.num_model_bins_r_par;
    c.nmt = d.num_model_bins_r_trans;
    c.nm = c.nmp * c.nmt;
    c.redshift_evolution = d.redshift_evolution;
    c.z_ref = d.z_ref;
    c.alpha = d.alpha;
    c.alpha2 = d.alpha2;
    c.inv_r_par_range = 1. / c.b.r_par_range;
    c.inv_r_trans_max = 1. / c.b.r_trans_max;
    c.p1 = h.p1;
    c.p2 = h.p2;
    c.mwords = h.mwords;
    c.dwords = h.dwords;
    c.list_doubles = h.list_doubles;
    c.work_doubles = h.work_doubles;
    c.cta_doubles = h.cta_doubles;
    cf_dmat_kernel<<<grid, kDmBlock, h.smem, stream>>>(c, s1, s2, ll1, ll2, order1, order2,
                                                       pair_first, pair_second, pair_angle,
                                                       num_pairs, out, work, scratch);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
