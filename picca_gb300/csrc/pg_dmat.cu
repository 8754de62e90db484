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
//      pair counts). The geometry runs in FP32 (r as an FP32 hi/lo pair) with
//      guard bands that bound its distance to the reference's FP64 values;
//      pairs inside a guard band (a range limit, a bin edge, the half-plate
//      cut) are decided in FP64 with the reference's expressions, so every
//      decision and bin is the reference's,
//   2. builds U (data bins x kappa) and E (model bins x kappa) in per-CTA
//      global scratch with a row sweep (a thread per pixel of forest 1) and a
//      column sweep (a thread per pixel of forest 2), merging runs of equal
//      bins in registers; the row sweep also adds the Kronecker term
//      w12 * zfac and the effective (r_par, r_trans, z, weight) sums,
//   3. reduces the four rank rows,
//   4. multiplies U by E^T in 32 x 32 FP64 tiles and adds the tile to the
//      global matrix with atomics.
// Sums are FP64 (the library is compiled with -fmad=false) and reassociated
// with respect to the reference (run sums of per-pixel factors, scaled once
// per run), so results agree to a few ulp of the summed magnitudes, not bit
// for bit; the product is FP64 on the CUDA cores or exact 8-bit digit
// products on the tensor cores (PG_DMAT_SPLIT_BF16).
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kDmBlock = 256;
constexpr int kDmWarps = kDmBlock / 32;
constexpr int kTile = 32;   // GEMM output tile edge (data bins x model bins)
constexpr int kSlab = 16;   // GEMM reduction step
constexpr int kTilePad = kTile + 1;
// Tensor-core form of the product (PG_DMAT_SPLIT_BF16): each FP64 row is
// scaled by a power of two to |x| < 1/2, rounded to 48 fractional bits and
// written as six signed digits of at most 128 in magnitude (exact in bf16).
// Products of digits are exact in the FP32 accumulators of mma.sync
// m16n8k16; the 21 digit pairs with p + q <= 5 (0-based) are summed per
// level p + q over 32 reduction steps (|sum| < 2^22), moved into 32-bit
// integer level sums (exact) and combined in FP64 at the end.
constexpr int kSlices = 6;
constexpr int kTcM = 32, kTcN = 32, kTcK = 32;
constexpr int kTcRow = kTcK + 8;  // bf16 per staged row (pad: conflict-free fragments)

struct DmatConst {
    Binning b;
    int32_t nmp, nmt, nm;    // model bins along r_par, r_trans, total
    int32_t redshift_evolution;
    double z_ref, alpha, alpha2;
    double inv_r_par_range, inv_r_trans_max;  // reciprocals for the bin estimate
    double sp, smp, st, smt;  // bins per unit: np / range, nmp / range, nt / rt_max, nmt / rt_max
    float f_rpmin, f_rpmax, f_rtmax, f_hpc;   // FP32 limits and half-plate cut
    float f_sp, f_smp, f_st, f_smt;
    int32_t p1, p2;          // pixel capacity of the shared-memory forest slots
    int32_t mwords, dwords;  // bitmap words (model, data)
    int64_t list_doubles;    // per-CTA scratch: bin lists (nm + nb int32), in doubles
    int64_t work_doubles;    // per-CTA scratch: U and E rows
    int64_t cta_doubles;     // list_doubles + work_doubles (+ digits and exponents)
    int32_t split;           // 1: tensor-core product (PG_DMAT_SPLIT_BF16)
    int32_t xcf;             // 1: delta x quasar layout (forest, quasar slots)
};

// Shared-memory layout (bytes), identical on host and device.
struct DmSmem {
    size_t f1, f2, flags1, flags2, mbits, mpref, dbits, dpref, tile_a, tile_b, total;
};

__host__ __device__ inline size_t dm_align(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Slot bytes per pixel: forest 1 of the auto-correlation (9 FP64 + 3 FP32
// arrays), forest 2 and the forest of the cross (12 + 3), quasars (7 + 5).
constexpr size_t kPix1Bytes = sizeof(double) * 9 + sizeof(float) * 3;
constexpr size_t kPix2Bytes = sizeof(double) * 12 + sizeof(float) * 3;
constexpr size_t kObjBytes = sizeof(double) * 7 + sizeof(float) * 5;
constexpr int kXdObjects = PG_XDMAT_MAX_OBJECTS;  // quasars of one xcf work item

__host__ __device__ inline DmSmem dm_smem(int p1, int p2, int mwords, int dwords, int split,
                                          int xcf = 0) {
    DmSmem s;
    size_t o = 0;
    s.f1 = o; o += (xcf ? kPix2Bytes : kPix1Bytes) * (size_t)p1;
    o = dm_align(o, 16);
    s.f2 = o; o += (xcf ? kObjBytes : kPix2Bytes) * (size_t)p2;
    s.flags1 = o; o = dm_align(o + (size_t)p1, 8);
    s.flags2 = o; o = dm_align(o + (size_t)p2, 8);
    s.mbits = o; o += sizeof(uint32_t) * (size_t)mwords;
    s.mpref = o; o += sizeof(int32_t) * (size_t)mwords;
    s.dbits = o; o += sizeof(uint32_t) * (size_t)dwords;
    s.dpref = o; o += sizeof(int32_t) * (size_t)dwords;
    o = dm_align(o, 16);
    if (split) {  // two staging buffers per operand
        s.tile_a = o; o += 2 * sizeof(uint16_t) * kSlices * kTcM * kTcRow;
        s.tile_b = o; o += 2 * sizeof(uint16_t) * kSlices * kTcN * kTcRow;
    } else {
        s.tile_a = o; o += sizeof(double) * kSlab * kTilePad;
        s.tile_b = o; o += sizeof(double) * kSlab * kTilePad;
    }
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

// round(x * 2^(48 - e)) for |x| < 2^e (zero and subnormal x give 0).
__device__ __forceinline__ long long dm_fixed48(double x, int e) {
    const long long bits = __double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    if (ex == 0) return 0;
    const long long man = (bits & 0xFFFFFFFFFFFFFLL) | 0x10000000000000LL;
    const int sh = 1075 - 48 + e - ex;  // right shift (>= 5 for |x| < 2^e)
    const long long m = sh >= 63 ? 0 : (man + (1LL << (sh - 1))) >> sh;
    return bits < 0 ? -m : m;
}

// bf16 bits of a small integer |v| <= 256 (exact).
__device__ __forceinline__ uint32_t dm_bf16_small(int v) {
    const float f = __int_as_float(0x4B400000 + v) - 12582912.f;
    return __float_as_uint(f) >> 16;
}

__device__ __forceinline__ void dm_mma(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
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

// D = U E^T of one chunk on the tensor cores (see kSlices), added to the
// global matrix: dmat[dlist[dl] * nm + mlist[ml]] += D[dl][ml]. U is
// [dcc][kst], E is [mcc][kst] (FP64, zero-padded to kst, a multiple of 16).
__device__ __forceinline__ void dm_ldsm4(uint32_t r[4], const uint16_t *p) {
    const unsigned addr = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

// 16-byte asynchronous copy global -> shared; valid = false writes zeros.
__device__ __forceinline__ void dm_cp16(uint16_t *dst, const uint16_t *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n"
                 :
                 : "r"(d), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}

__device__ __forceinline__ void dm_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void dm_cp_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void dm_cp_wait_0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// D = U E^T of one chunk on the tensor cores (see kSlices), added to the
// global matrix: dmat[dlist[dl] * nm + mlist[ml]] += D[dl][ml]. U is
// [dcc][kst], E is [mcc][kst] (FP64, zero-padded to kst, a multiple of 16).
// sa / sb: two staging buffers of kSlices x 32 rows x kTcRow bf16 each.
__device__ void dm_product_split(const double *U, const double *E, int dcc, int mcc, int kst,
                                 uint16_t *digits, int32_t *rexp, uint16_t *sa, uint16_t *sb,
                                 const int32_t *dlist, const int32_t *mlist, int nm,
                                 double *dmat) {
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // row exponents and digits (a warp per row): rows are scaled to |x| < 1/2
    // so every digit is at most 128 in magnitude
    for (int r = warp; r < dcc + mcc; r += kDmWarps) {
        const double *row = r < dcc ? U + (int64_t)r * kst : E + (int64_t)(r - dcc) * kst;
        double mx = 0.;
        for (int k = lane; k < kst; k += 32) mx = fmax(mx, fabs(__ldcg(row + k)));
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        const int ex = (int)((__double_as_longlong(mx) >> 52) & 0x7FF);
        const int e = (ex == 0 ? -1022 : ex - 1022) + 1;  // |x| <= mx < 2^(e - 1)
        if (lane == 0) rexp[r] = e;
        uint16_t *dst = digits + (int64_t)r * kSlices * kst;
        for (int k = lane; k < kst; k += 32) {
            long long m = dm_fixed48(__ldcg(row + k), e);
#pragma unroll
            for (int p = 0; p < kSlices; ++p) {
                const int sh = 8 * (kSlices - 1 - p);
                const long long d = sh ? (m + (1LL << (sh - 1))) >> sh : m;
                m -= d << sh;
                dst[(int64_t)p * kst + k] = (uint16_t)dm_bf16_small((int)d);
            }
        }
    }
    __syncthreads();
    const int group = lane >> 2, tig = lane & 3;
    const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, 16 x 8 each
    constexpr int kParts = kTcK / 8;
    constexpr int kOne = kSlices * kTcM * kParts;    // 16-byte copies per operand
    constexpr int kBuf = kSlices * kTcM * kTcRow;    // bf16 per operand buffer
    for (int td = 0; td < dcc; td += kTcM) {
        for (int tm = 0; tm < mcc; tm += kTcN) {
            // stage the digits of rows [td, td + 32) of U and [tm, tm + 32) of
            // E for reduction steps [k0, k0 + 32) into buffer b
            auto stage = [&](int b, int k0) {
                for (int e = tid; e < 2 * kOne; e += kDmBlock) {
                    const bool isa = e < kOne;
                    const int f = isa ? e : e - kOne;
                    const int part = f % kParts;
                    const int r = (f / kParts) % kTcM;
                    const int p = f / (kParts * kTcM);
                    const int grow = (isa ? td : tm) + r;
                    const int kk = k0 + part * 8;
                    const bool valid = grow < (isa ? dcc : mcc) && kk < kst;
                    const int64_t src_row = isa ? grow : dcc + grow;
                    const uint16_t *src =
                        valid ? digits + (src_row * kSlices + p) * (int64_t)kst + kk : digits;
                    dm_cp16((isa ? sa : sb) + b * kBuf + (p * kTcM + r) * kTcRow + part * 8, src,
                            valid);
                }
                dm_cp_commit();
            };
            uint32_t lev[kSlices][4];
#pragma unroll
            for (int l = 0; l < kSlices; ++l)
#pragma unroll
                for (int q = 0; q < 4; ++q) lev[l][q] = 0u;
            uint32_t drains = 0;
            stage(0, 0);
            int b = 0;
            for (int k0 = 0; k0 < kst; k0 += kTcK) {
                if (k0 + kTcK < kst) {
                    stage(b ^ 1, k0 + kTcK);
                    dm_cp_wait_1();
                } else {
                    dm_cp_wait_0();
                }
                __syncthreads();
                const uint16_t *A = sa + b * kBuf, *B = sb + b * kBuf;
                // digit products: |digit| <= 128, so a level (p + q fixed, at
                // most 6 pairs) summed over 32 reduction steps stays below
                // 6 * 32 * 2^14 < 2^22 and is an exact FP32 integer
                float acc[kSlices][4];
#pragma unroll
                for (int l = 0; l < kSlices; ++l)
#pragma unroll
                    for (int q = 0; q < 4; ++q) acc[l][q] = 0.f;
#pragma unroll
                for (int ks = 0; ks < kTcK; ks += 16) {
                    if (k0 + ks >= kst) break;
                    uint32_t af[kSlices][4], bf[kSlices][2];
#pragma unroll
                    for (int p = 0; p < kSlices; ++p)
                        dm_ldsm4(af[p], A + (p * kTcM + wm * 16 + (lane & 15)) * kTcRow + ks +
                                            (lane >> 4) * 8);
#pragma unroll
                    for (int p = 0; p < kSlices; p += 2) {
                        uint32_t t[4];
                        dm_ldsm4(t, B + ((p + (lane >> 4)) * kTcN + wn * 8 + (lane & 7)) * kTcRow +
                                        ks + ((lane >> 3) & 1) * 8);
                        bf[p][0] = t[0];
                        bf[p][1] = t[1];
                        bf[p + 1][0] = t[2];
                        bf[p + 1][1] = t[3];
                    }
#pragma unroll
                    for (int l = 0; l < kSlices; ++l)
#pragma unroll
                        for (int p = 0; p <= l; ++p) dm_mma(acc[l], af[p], bf[l - p]);
                }
                // bits of v + 1.5 * 2^23 carry the exact integer v (|v| < 2^22)
#pragma unroll
                for (int l = 0; l < kSlices; ++l)
#pragma unroll
                    for (int q = 0; q < 4; ++q) lev[l][q] += __float_as_uint(acc[l][q] + 12582912.f);
                ++drains;
                __syncthreads();
                b ^= 1;
            }
            const uint32_t bias = drains * 0x4B400000u;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int dl = td + wm * 16 + group + ((q >> 1) << 3);
                const int ml = tm + wn * 8 + tig * 2 + (q & 1);
                if (dl >= dcc || ml >= mcc) continue;
                double v = 0.;
#pragma unroll
                for (int l = kSlices - 1; l >= 0; --l)
                    v = __fma_rn(v, 0.00390625, (double)(int32_t)(lev[l][q] - bias));
                // v = sum_l lev_l 2^(-8 l); the level l product carries 2^(-8 (l + 2))
                v = ldexp(v, rexp[dl] + rexp[dcc + ml] - 16);
                if (v != 0.) atomicAdd(&dmat[(int64_t)dlist[dl] * nm + mlist[ml]], v);
            }
        }
    }
}

// D = U E^T of one chunk in FP64 on the CUDA cores (32 x 32 tiles), added to
// the global matrix like dm_product_split.
__device__ void dm_product_fp64(const double *U, const double *E, int dcc, int mcc, int kst,
                                double (*ta)[kTilePad], double (*tb)[kTilePad],
                                const int32_t *dlist, const int32_t *mlist, int nm,
                                double *dmat) {
    const int tid = threadIdx.x;
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
                    ta[kk][rr] = (td + rr < dcc) ? __ldcg(U + (int64_t)(td + rr) * kst + k0 + kk) : 0.;
                    tb[kk][rr] = (tm + rr < mcc) ? __ldcg(E + (int64_t)(tm + rr) * kst + k0 + kk) : 0.;
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
                const int64_t base = (int64_t)dlist[dl] * nm;
#pragma unroll
                for (int b2 = 0; b2 < 2; ++b2) {
                    const int ml = tm + tx + 16 * b2;
                    if (ml < mcc && acc[a][b2] != 0.)
                        atomicAdd(&dmat[base + mlist[ml]], acc[a][b2]);
                }
            }
        }
    }
}

struct DmItem {
    int32_t n1, n2;
    double cc, ss;
    double sw1, sw2, swsll1, swsll2;
    double inv_sw1, inv_sw2, inv_q1, inv_q2;  // reciprocals of the four sums
    int32_t order1, order2;
    bool shp;
};

// FP32 form of the pixel-pair geometry of one forest pair, with guard bands
// that bound its distance to the FP64 computation of the reference.
struct DmGuard {
    float cc, ss;             // cos, sin of half the angle
    float gp, gt;             // |r_par - r_par(FP64)|, |r_trans - r_trans(FP64)| bounds
    float gyp, gyt, gymp, gymt;  // the same bounds in units of the four bin widths
};

// Per-pixel slots of the two forests in shared memory (FP64 unless noted).
struct DmPix {
    double *r, *m, *z, *w, *dll, *zf;
    double *a;    // zf w / sum(w)
    double *b;    // zf w dll / sum(w dll^2)
    double *wd;   // w dll
    double *wz;   // w zf       (forest 2 only)
    double *wzz;  // w z        (forest 2 only)
    double *wm;   // w dist_m   (forest 2 only)
    float *rh, *rl, *mf;  // FP32: r = rh + rl, dist_m
};

__device__ __forceinline__ DmPix dm_pix(unsigned char *base, int p, bool second) {
    DmPix x;
    double *d = reinterpret_cast<double *>(base);
    x.r = d; x.m = d + p; x.z = d + 2 * p; x.w = d + 3 * p; x.dll = d + 4 * p; x.zf = d + 5 * p;
    x.a = d + 6 * p; x.b = d + 7 * p; x.wd = d + 8 * p;
    const int nd = second ? 12 : 9;
    x.wz = second ? d + 9 * p : nullptr;
    x.wzz = second ? d + 10 * p : nullptr;
    x.wm = second ? d + 11 * p : nullptr;
    float *f = reinterpret_cast<float *>(d + nd * p);
    x.rh = f; x.rl = f + p; x.mf = f + 2 * p;
    return x;
}

// FP32 decision of a pixel pair: 0 outside the model range, 1 inside with
// the bins and the half-plate flag set, 2 too close to a range limit, a bin
// edge or the half-plate cut for FP32 to decide (the caller uses dm_pair).
__device__ __forceinline__ int dm_pair_f32(const DmatConst &c, const DmGuard &g, float r1h,
                                           float r1l, float m1, float r2h, float r2l, float m2,
                                           bool shp, DmPair &o) {
    const float d = __fadd_rn(__fsub_rn(r1h, r2h), __fsub_rn(r1l, r2l));
    float rp = __fmul_rn(d, g.cc);
    if (!c.b.x_correlation) rp = fabsf(rp);
    const float rt = __fmul_rn(__fadd_rn(m1, m2), g.ss);
    if (rp >= c.f_rpmax + g.gp || rt >= c.f_rtmax + g.gt || rp < c.f_rpmin - g.gp) return 0;
    if (rp > c.f_rpmax - g.gp || rt > c.f_rtmax - g.gt || rp < c.f_rpmin + g.gp) return 2;
    o.counted = true;
    if (c.b.remove_shp && shp) {
        const float a = fabsf(rp);
        if (fabsf(__fsub_rn(a, c.f_hpc)) <= g.gp) return 2;
        o.counted = a >= c.f_hpc;
    }
    const float xp = __fsub_rn(rp, c.f_rpmin);
    const float yp = __fmul_rn(xp, c.f_sp), ymp = __fmul_rn(xp, c.f_smp);
    const float yt = __fmul_rn(rt, c.f_st), ymt = __fmul_rn(rt, c.f_smt);
    const float bp = floorf(yp), bt = floorf(yt), mp = floorf(ymp), mt = floorf(ymt);
    if (yp - bp <= g.gyp || bp + 1.f - yp <= g.gyp || yt - bt <= g.gyt ||
        bt + 1.f - yt <= g.gyt || ymp - mp <= g.gymp || mp + 1.f - ymp <= g.gymp ||
        ymt - mt <= g.gymt || mt + 1.f - ymt <= g.gymt)
        return 2;
    o.db = (int32_t)bt + c.b.nt * (int32_t)bp;
    o.mb = (int32_t)mt + c.nmt * (int32_t)mp;
    return 1;
}

// Decision of pixel pair (i, j): 0 outside, 1 inside (FP32 form; o.rp,
// o.rt not set), 2 inside (FP64 form, dm_pair: o.rp, o.rt, o.z set). o.zsel
// is set in both inside cases.
__device__ __forceinline__ int dm_decide(const DmatConst &c, const DmGuard &g, const DmItem &it,
                                         const DmPix &p1, const DmPix &p2, int i, int j,
                                         DmPair &o) {
    int st = c.b.rmu ? 2
                     : dm_pair_f32(c, g, p1.rh[i], p1.rl[i], p1.mf[i], p2.rh[j], p2.rl[j],
                                   p2.mf[j], it.shp, o);
    if (st == 0) return 0;
    if (st == 2)
        return dm_pair(c, p1.r[i], p1.m[i], p1.z[i], p2.r[j], p2.m[j], p2.z[j], it.cc, it.ss,
                       it.shp, o) ? 2 : 0;
    o.zsel = true;
    if (c.b.zmin_on || c.b.zmax_on) {
        const double z = __dadd_rn(p1.z[i], p2.z[j]) / 2;
        o.zsel = !((c.b.zmin_on && z < c.b.z_min) || (c.b.zmax_on && z > c.b.z_max));
    }
    return 1;
}

__global__ void __launch_bounds__(kDmBlock, 2)
    cf_dmat_kernel(DmatConst c, pg_forest_set s1, pg_forest_set s2, const double *ll1,
                   const double *ll2, const int32_t *order1g, const int32_t *order2g,
                   const int32_t *pair_first, const int32_t *pair_second,
                   const double *pair_angle, int64_t num_pairs, pg_dmat_sums out,
                   double *work, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const DmSmem L = dm_smem(c.p1, c.p2, c.mwords, c.dwords, c.split);
    const DmPix P1 = dm_pix(smem + L.f1, c.p1, false);
    const DmPix P2 = dm_pix(smem + L.f2, c.p2, true);
    unsigned char *sel1 = smem + L.flags1, *sel2 = smem + L.flags2;
    uint32_t *mbits = reinterpret_cast<uint32_t *>(smem + L.mbits);
    int32_t *mpref = reinterpret_cast<int32_t *>(smem + L.mpref);
    uint32_t *dbits = reinterpret_cast<uint32_t *>(smem + L.dbits);
    int32_t *dpref = reinterpret_cast<int32_t *>(smem + L.dpref);
    double (*ta)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_a);
    double (*tb)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_b);
    uint16_t *ta_raw = reinterpret_cast<uint16_t *>(smem + L.tile_a);
    uint16_t *tb_raw = reinterpret_cast<uint16_t *>(smem + L.tile_b);
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
    // tensor-core form: digits [rows][kSlices][kst] bf16, then row exponents
    uint16_t *digits = reinterpret_cast<uint16_t *>(rows + c.work_doubles);
    int32_t *rexp = reinterpret_cast<int32_t *>(digits + (c.work_doubles * kSlices));

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
        double lmax = 0., lmmax = 0.;
        for (int t = tid; t < it.n1; t += kDmBlock) {
            const double r = s1.r_comov[o1 + t], m = s1.dist_m[o1 + t];
            P1.r[t] = r;
            P1.m[t] = m;
            P1.z[t] = s1.z[o1 + t];
            P1.w[t] = s1.weights[o1 + t];
            P1.dll[t] = ll1[o1 + t];
            const float rh = (float)r;
            P1.rh[t] = rh;
            P1.rl[t] = (float)__dsub_rn(r, (double)rh);
            P1.mf[t] = (float)m;
            lmax = fmax(lmax, fabs(r));
            lmmax = fmax(lmmax, fabs(m));
            sel1[t] = !(zerr_on && zerr_veto(P1.z[t], zq2, c.b.zerr_kms));
        }
        for (int t = tid; t < it.n2; t += kDmBlock) {
            const double r = s2.r_comov[o2 + t], m = s2.dist_m[o2 + t];
            P2.r[t] = r;
            P2.m[t] = m;
            P2.z[t] = s2.z[o2 + t];
            P2.w[t] = s2.weights[o2 + t];
            P2.dll[t] = ll2[o2 + t];
            const float rh = (float)r;
            P2.rh[t] = rh;
            P2.rl[t] = (float)__dsub_rn(r, (double)rh);
            P2.mf[t] = (float)m;
            lmax = fmax(lmax, fabs(r));
            lmmax = fmax(lmmax, fabs(m));
            sel2[t] = !(zerr_on && zerr_veto(P2.z[t], zq1, c.b.zerr_kms));
        }
        for (int t = tid; t < c.mwords; t += kDmBlock) mbits[t] = 0u;
        for (int t = tid; t < c.dwords; t += kDmBlock) dbits[t] = 0u;
        // guard bands of the FP32 geometry: |r_par error| <= 2^-23 max|r| +
        // 3 2^-24 |r_par| / cos, |r_trans error| <= 2^-22 max|dist_m| sin +
        // 2^-23 r_trans (rounding of the inputs, the difference or sum, the
        // half-angle trig and the products), doubled
        for (int o = 16; o > 0; o >>= 1) {
            lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
            lmmax = fmax(lmmax, __shfl_xor_sync(0xffffffffu, lmmax, o));
        }
        if ((tid & 31) == 0) {
            red[tid >> 5] = lmax;
            red_int[tid >> 5] = 0;
        }
        __syncthreads();
        double rmax = 0.;
        for (int k = 0; k < kDmWarps; ++k) rmax = fmax(rmax, red[k]);
        __syncthreads();
        if ((tid & 31) == 0) red[tid >> 5] = lmmax;
        if (tid == 0) s_count = 0;
        __syncthreads();
        double mmax = 0.;
        for (int k = 0; k < kDmWarps; ++k) mmax = fmax(mmax, red[k]);
        DmGuard gd;
        {
            const double u = 5.9604644775390625e-8;  // 2^-24
            const double rlim = fmax(fabs(c.b.r_par_max), fabs(c.b.r_par_min));
            const double gp = 2. * (2. * u * rmax + 3. * u * (rlim + 1.) / fmax(it.cc, 1e-6));
            const double gt = 2. * (4. * u * mmax * it.ss + 2. * u * c.b.r_trans_max);
            const double ey = 8. * u;  // relative error of the bin coordinate itself
            gd.cc = (float)it.cc;
            gd.ss = (float)it.ss;
            gd.gp = (float)gp;
            gd.gt = (float)gt;
            gd.gyp = (float)(gp * c.sp + ey * (c.b.np + 1));
            gd.gymp = (float)(gp * c.smp + ey * (c.nmp + 1));
            gd.gyt = (float)(gt * c.st + ey * (c.b.nt + 1));
            gd.gymt = (float)(gt * c.smt + ey * (c.nmt + 1));
        }
        __syncthreads();

        // 1. classification: touched model bins, data bins of selected pairs
        {
            const int warp = tid >> 5, lane = tid & 31;
            int counted = 0;
            for (int i = warp; i < it.n1; i += kDmWarps) {
                if (P1.w[i] == 0.) continue;
                for (int j = lane; j < it.n2; j += 32) {
                    if (P2.w[j] == 0.) continue;
                    DmPair o;
                    if (!dm_decide(c, gd, it, P1, P2, i, j, o)) continue;
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
            lw += P1.w[t];
            lsw += __dmul_rn(P1.dll[t], P1.w[t]);
        }
        it.sw1 = dm_block_sum(lw, red);
        const double sll1 = dm_block_sum(lsw, red);
        lw = 0.;
        lsw = 0.;
        for (int t = tid; t < it.n2; t += kDmBlock) {
            lw += P2.w[t];
            lsw += __dmul_rn(P2.dll[t], P2.w[t]);
        }
        it.sw2 = dm_block_sum(lw, red);
        const double sll2 = dm_block_sum(lsw, red);
        const double mean1 = sll1 / it.sw1, mean2 = sll2 / it.sw2;
        double q1 = 0., q2 = 0.;
        for (int t = tid; t < it.n1; t += kDmBlock) {
            const double d = __dsub_rn(P1.dll[t], mean1);
            P1.dll[t] = d;
            q1 += __dmul_rn(P1.w[t], __dmul_rn(d, d));
            P1.zf[t] = c.redshift_evolution
                           ? pow(__dadd_rn(1., P1.z[t]) / __dadd_rn(1., c.z_ref),
                                 __dsub_rn(c.alpha, 1.))
                           : 1.;
        }
        for (int t = tid; t < it.n2; t += kDmBlock) {
            const double d = __dsub_rn(P2.dll[t], mean2);
            P2.dll[t] = d;
            q2 += __dmul_rn(P2.w[t], __dmul_rn(d, d));
            P2.zf[t] = c.redshift_evolution
                           ? pow(__dadd_rn(1., P2.z[t]) / __dadd_rn(1., c.z_ref),
                                 __dsub_rn(c.alpha2, 1.))
                           : 1.;
        }
        it.swsll1 = dm_block_sum(q1, red);
        it.swsll2 = dm_block_sum(q2, red);
        it.inv_sw1 = 1. / it.sw1;
        it.inv_sw2 = 1. / it.sw2;
        it.inv_q1 = 1. / it.swsll1;
        it.inv_q2 = 1. / it.swsll2;
        const bool ord1 = it.order1 == 1, ord2 = it.order2 == 1;
        if ((ord1 && !(it.swsll1 != 0.)) || (ord2 && !(it.swsll2 != 0.))) {
            // the reference divides by zero here (a forest without spread in
            // log lambda); the pair is reported and skipped
            if (tid == 0) report_error(scratch, PG_ERR_INVALID_ARGUMENT, (int32_t)q);
            __syncthreads();
            continue;
        }
        // per-pixel factors of the eta terms and of the effective sums
        for (int t = tid; t < it.n1; t += kDmBlock) {
            const double wz = __dmul_rn(P1.w[t], P1.zf[t]);
            P1.a[t] = __dmul_rn(wz, it.inv_sw1);
            P1.b[t] = __dmul_rn(__dmul_rn(wz, P1.dll[t]), it.inv_q1);
            P1.wd[t] = __dmul_rn(P1.w[t], P1.dll[t]);
        }
        for (int t = tid; t < it.n2; t += kDmBlock) {
            const double wz = __dmul_rn(P2.w[t], P2.zf[t]);
            P2.a[t] = __dmul_rn(wz, it.inv_sw2);
            P2.b[t] = __dmul_rn(__dmul_rn(wz, P2.dll[t]), it.inv_q2);
            P2.wd[t] = __dmul_rn(P2.w[t], P2.dll[t]);
            P2.wz[t] = wz;
            P2.wzz[t] = __dmul_rn(P2.w[t], P2.z[t]);
            P2.wm[t] = __dmul_rn(P2.w[t], P2.m[t]);
        }
        __syncthreads();

        // kappa layout of the U and E rows
        const int n1 = it.n1, n2 = it.n2;
        const int kU = 0, kX = n1, kV = n1 + n2;
        const int kY = kV + (ord2 ? n1 : 0);
        const int kR = kY + (ord1 ? n2 : 0);
        const int kst = (int)dm_align((size_t)kR + 4, kSlab);
        const int64_t cap = c.work_doubles / kst;
        int dc = nbt, mc = nmt;
        if ((int64_t)nbt + nmt > cap) {
            dc = (int)min((int64_t)nbt, cap / 2);
            mc = (int)(cap - dc);
        }

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

                // Rows are accumulated with non-returning atomic adds (a row
                // entry belongs to one thread, so they never contend) and read
                // back through L2 (__ldcg) after the barrier.
                // 2a. row sweep: a thread per pixel i of forest 1. Run sums are
                // per-pixel factors of forest 2, scaled by those of pixel i at
                // the flush (zfac = zf1 zf2, w12 = w1 w2, z = (z1 + z2) / 2,
                // r_trans = (dist_m1 + dist_m2) sin)
                for (int i = tid; i < n1; i += kDmBlock) {
                    const double w1 = P1.w[i];
                    if (w1 == 0.) continue;
                    const double zf1 = P1.zf[i], r1 = P1.r[i];
                    const bool ok1 = sel1[i];
                    int run_m = -1, run_d = -1;
                    double e1 = 0., e3 = 0., u = 0., v = 0.;
                    int64_t run_k = -1;
                    int32_t k_db = 0, k_mb = 0;
                    double k_dm = 0., k_w = 0., k_rp = 0., k_rt = 0., k_z = 0.;
                    auto flush_k = [&]() {
                        const double w1zf = __dmul_rn(w1, zf1);
                        atomicAdd(&out.dmat[run_k], __dmul_rn(w1zf, k_dm));
                        atomicAdd(&out.weights_dmat[k_db], __dmul_rn(w1, k_w));
                        atomicAdd(&out.r_par_eff[k_mb], __dmul_rn(w1, k_rp));
                        const double rt = c.b.rmu ? k_rt
                                                  : __dmul_rn(__dadd_rn(__dmul_rn(P1.m[i], k_w),
                                                                        k_rt), it.ss);
                        atomicAdd(&out.r_trans_eff[k_mb], __dmul_rn(w1, rt));
                        atomicAdd(&out.z_eff[k_mb],
                                  __dmul_rn(w1, __dmul_rn(0.5, __dadd_rn(__dmul_rn(P1.z[i], k_w),
                                                                         k_z))));
                        atomicAdd(&out.weight_eff[k_mb], __dmul_rn(w1, k_w));
                    };
                    for (int j = 0; j < n2; ++j) {
                        if (P2.w[j] == 0.) continue;
                        DmPair o;
                        const int st = dm_decide(c, gd, it, P1, P2, i, j, o);
                        if (!st) continue;
                        if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) continue;
                        const int ml = dm_rank(mbits, mpref, o.mb) - m0;
                        if (ml >= 0 && ml < mcc) {
                            if (ml != run_m) {
                                if (run_m >= 0) {
                                    atomicAdd(&E[(int64_t)run_m * kst + kU + i], -__dmul_rn(zf1, e1));
                                    if (ord2) atomicAdd(&E[(int64_t)run_m * kst + kV + i], -__dmul_rn(zf1, e3));
                                }
                                run_m = ml;
                                e1 = 0.;
                                e3 = 0.;
                            }
                            e1 += P2.a[j];
                            if (ord2) e3 += P2.b[j];
                        }
                        if (o.counted && o.zsel && ok1 && sel2[j]) {
                            const int dl = dm_rank(dbits, dpref, o.db) - d0;
                            if (dl >= 0 && dl < dcc) {
                                if (dl != run_d) {
                                    if (run_d >= 0) {
                                        atomicAdd(&U[(int64_t)run_d * kst + kU + i], __dmul_rn(w1, u));
                                        if (ord2) atomicAdd(&U[(int64_t)run_d * kst + kV + i], __dmul_rn(w1, v));
                                    }
                                    run_d = dl;
                                    u = 0.;
                                    v = 0.;
                                }
                                u += P2.w[j];
                                if (ord2) v += P2.wd[j];
                            }
                            if (first) {
                                const int64_t key = (int64_t)o.db * nm + o.mb;
                                if (key != run_k) {
                                    if (run_k >= 0) flush_k();
                                    run_k = key;
                                    k_db = o.db;
                                    k_mb = o.mb;
                                    k_dm = k_w = k_rp = k_rt = k_z = 0.;
                                }
                                const double w2 = P2.w[j];
                                k_dm += P2.wz[j];
                                k_w += w2;
                                k_z += P2.wzz[j];
                                if (st == 2) {
                                    k_rp += __dmul_rn(w2, o.rp);
                                    if (c.b.rmu) k_rt += __dmul_rn(w2, o.rt);
                                    else k_rt += P2.wm[j];
                                } else {
                                    double rp = __dmul_rn(__dsub_rn(r1, P2.r[j]), it.cc);
                                    if (!c.b.x_correlation) rp = fabs(rp);
                                    k_rp += __dmul_rn(w2, rp);
                                    k_rt += P2.wm[j];
                                }
                            }
                        }
                    }
                    if (run_m >= 0) {
                        atomicAdd(&E[(int64_t)run_m * kst + kU + i], -__dmul_rn(zf1, e1));
                        if (ord2) atomicAdd(&E[(int64_t)run_m * kst + kV + i], -__dmul_rn(zf1, e3));
                    }
                    if (run_d >= 0) {
                        atomicAdd(&U[(int64_t)run_d * kst + kU + i], __dmul_rn(w1, u));
                        if (ord2) atomicAdd(&U[(int64_t)run_d * kst + kV + i], __dmul_rn(w1, v));
                    }
                    if (run_k >= 0) flush_k();
                }

                // 2b. column sweep: a thread per pixel j of forest 2
                for (int j = tid; j < n2; j += kDmBlock) {
                    const double w2 = P2.w[j];
                    if (w2 == 0.) continue;
                    const double zf2 = P2.zf[j];
                    const bool ok2 = sel2[j];
                    int run_m = -1, run_d = -1;
                    double e2 = 0., e4 = 0., x = 0., y = 0.;
                    for (int i = 0; i < n1; ++i) {
                        if (P1.w[i] == 0.) continue;
                        DmPair o;
                        if (!dm_decide(c, gd, it, P1, P2, i, j, o)) continue;
                        if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) continue;
                        const int ml = dm_rank(mbits, mpref, o.mb) - m0;
                        if (ml >= 0 && ml < mcc) {
                            if (ml != run_m) {
                                if (run_m >= 0) {
                                    atomicAdd(&E[(int64_t)run_m * kst + kX + j], -__dmul_rn(zf2, e2));
                                    if (ord1) atomicAdd(&E[(int64_t)run_m * kst + kY + j], -__dmul_rn(zf2, e4));
                                }
                                run_m = ml;
                                e2 = 0.;
                                e4 = 0.;
                            }
                            e2 += P1.a[i];
                            if (ord1) e4 += P1.b[i];
                        }
                        if (o.counted && o.zsel && ok2 && sel1[i]) {
                            const int dl = dm_rank(dbits, dpref, o.db) - d0;
                            if (dl >= 0 && dl < dcc) {
                                if (dl != run_d) {
                                    if (run_d >= 0) {
                                        atomicAdd(&U[(int64_t)run_d * kst + kX + j], __dmul_rn(w2, x));
                                        if (ord1) atomicAdd(&U[(int64_t)run_d * kst + kY + j], __dmul_rn(w2, y));
                                    }
                                    run_d = dl;
                                    x = 0.;
                                    y = 0.;
                                }
                                x += P1.w[i];
                                if (ord1) y += P1.wd[i];
                            }
                        }
                    }
                    if (run_m >= 0) {
                        atomicAdd(&E[(int64_t)run_m * kst + kX + j], -__dmul_rn(zf2, e2));
                        if (ord1) atomicAdd(&E[(int64_t)run_m * kst + kY + j], -__dmul_rn(zf2, e4));
                    }
                    if (run_d >= 0) {
                        atomicAdd(&U[(int64_t)run_d * kst + kX + j], __dmul_rn(w2, x));
                        if (ord1) atomicAdd(&U[(int64_t)run_d * kst + kY + j], __dmul_rn(w2, y));
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
                                const double a = __ldcg(row + kU + i);
                                s0 += a;
                                s2v += __dmul_rn(P1.dll[i], a);
                                if (ord1 && ord2) s3 += __dmul_rn(P1.dll[i], __ldcg(row + kV + i));
                            }
                            for (int j = lane; j < n2; j += 32)
                                s1v += __dmul_rn(P2.dll[j], __ldcg(row + kX + j));
                        } else {
                            const double *row = E + (int64_t)(r - dcc) * kst;
                            for (int i = lane; i < n1; i += 32) {
                                const double a1 = __dmul_rn(P1.w[i], it.inv_sw1);
                                const double e1 = __ldcg(row + kU + i);
                                s0 -= __dmul_rn(a1, e1);
                                if (ord2) s1v -= __dmul_rn(a1, __ldcg(row + kV + i));
                                if (ord1) {
                                    const double a7 = __dmul_rn(__dmul_rn(P1.w[i], P1.dll[i]), it.inv_q1);
                                    s2v -= __dmul_rn(a7, e1);
                                    if (ord2) s3 -= __dmul_rn(a7, __ldcg(row + kV + i));
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
                if (c.split)
                    dm_product_split(U, E, dcc, mcc, kst, digits, rexp, ta_raw, tb_raw,
                                     dlist + d0, mlist + m0, nm, out.dmat);
                else
                    dm_product_fp64(U, E, dcc, mcc, kst, ta, tb, dlist + d0, mlist + m0, nm,
                                    out.dmat);
                __syncthreads();
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Delta x quasar distortion matrix: xcf.compute_dmat (py/picca/xcf.py:325-424)
// and xcf.compute_dmat_forest_pairs_fast (py/picca/xcf.py:427-675). A work
// item is one forest with up to kXdObjects of its kept quasars. Only the
// forest's continuum is projected out, so the product has the two kappa
// blocks of the quasars: U = (sum_i w12, sum_i w12 dll1_i) per data bin and
// E = -(eta2, eta4) per model bin; contributions of different quasars add,
// so a forest's quasars may be split over items.

// Per-quasar shared slots.
struct DmObj {
    double *r, *m, *z, *w, *zf, *cc, *ss;
    float *rh, *rl, *mf, *ccf, *ssf;
};

__device__ __forceinline__ DmObj dm_obj(unsigned char *base, int n) {
    DmObj x;
    double *d = reinterpret_cast<double *>(base);
    x.r = d; x.m = d + n; x.z = d + 2 * n; x.w = d + 3 * n; x.zf = d + 4 * n;
    x.cc = d + 5 * n; x.ss = d + 6 * n;
    float *f = reinterpret_cast<float *>(d + 7 * n);
    x.rh = f; x.rl = f + n; x.mf = f + 2 * n; x.ccf = f + 3 * n; x.ssf = f + 4 * n;
    return x;
}

// Decision of pixel i and quasar j: 0 outside, 1 inside (FP32 form), 2
// inside (FP64 form, o.rp / o.rt / o.z set). r_par is signed.
__device__ __forceinline__ int dm_decide_x(const DmatConst &c, const DmGuard &g, const DmPix &f,
                                           const DmObj &q, int i, int j, DmPair &o) {
    int st = 2;
    if (!c.b.rmu) {
        DmGuard gj = g;
        gj.cc = q.ccf[j];
        gj.ss = q.ssf[j];
        st = dm_pair_f32(c, gj, f.rh[i], f.rl[i], f.mf[i], q.rh[j], q.rl[j], q.mf[j], false, o);
    }
    if (st == 0) return 0;
    if (st == 2)
        return dm_pair(c, f.r[i], f.m[i], f.z[i], q.r[j], q.m[j], q.z[j], q.cc[j], q.ss[j],
                       false, o) ? 2 : 0;
    o.zsel = true;
    if (c.b.zmin_on || c.b.zmax_on) {
        const double z = __dadd_rn(f.z[i], q.z[j]) / 2;
        o.zsel = !((c.b.zmin_on && z < c.b.z_min) || (c.b.zmax_on && z > c.b.z_max));
    }
    return 1;
}

__global__ void __launch_bounds__(kDmBlock, 2)
    xcf_dmat_kernel(DmatConst c, pg_forest_set fs, pg_forest_set qs, const double *ll,
                    const int32_t *order, const int32_t *item_forest, const int32_t *item_start,
                    const int32_t *item_count, const int32_t *obj_index,
                    const double *obj_angle, int64_t num_items, pg_dmat_sums out, double *work,
                    Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const DmSmem L = dm_smem(c.p1, c.p2, c.mwords, c.dwords, c.split, 1);
    const DmPix F = dm_pix(smem + L.f1, c.p1, true);
    const DmObj Q = dm_obj(smem + L.f2, c.p2);
    uint32_t *mbits = reinterpret_cast<uint32_t *>(smem + L.mbits);
    int32_t *mpref = reinterpret_cast<int32_t *>(smem + L.mpref);
    uint32_t *dbits = reinterpret_cast<uint32_t *>(smem + L.dbits);
    int32_t *dpref = reinterpret_cast<int32_t *>(smem + L.dpref);
    double (*ta)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_a);
    double (*tb)[kTilePad] = reinterpret_cast<double (*)[kTilePad]>(smem + L.tile_b);
    uint16_t *ta_raw = reinterpret_cast<uint16_t *>(smem + L.tile_a);
    uint16_t *tb_raw = reinterpret_cast<uint16_t *>(smem + L.tile_b);
    __shared__ double red[kDmWarps];
    __shared__ int red_int[kDmWarps];
    __shared__ int s_item;
    __shared__ int s_count;

    const int tid = threadIdx.x;
    const int nb = c.b.nbins, nm = c.nm;
    double *cta = work + (int64_t)blockIdx.x * c.cta_doubles;
    int32_t *dlist = reinterpret_cast<int32_t *>(cta);
    int32_t *mlist = dlist + nb;
    double *rows = cta + c.list_doubles;
    uint16_t *digits = reinterpret_cast<uint16_t *>(rows + c.work_doubles);
    int32_t *rexp = reinterpret_cast<int32_t *>(digits + (c.work_doubles * kSlices));

    for (;;) {
        if (tid == 0) s_item = atomicAdd(&scratch->work_counter, 1);
        __syncthreads();
        const int64_t q = s_item;
        if (q >= num_items) break;
        const int f = item_forest[q];
        const int o0 = item_start[q];
        const int n2 = item_count[q];
        const int64_t p0 = fs.pix_offset[f];
        const int n1 = (int)(fs.pix_offset[f + 1] - p0);
        if (n1 > c.p1 || n2 > c.p2 || n2 < 0) {
            if (tid == 0) report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)q);
            __syncthreads();
            continue;
        }
        const int ord1 = order[f] == 1;
        // stage the forest and its quasars
        double lmax = 0., lmmax = 0., lss = 0., lcc = 1.;
        for (int t = tid; t < n1; t += kDmBlock) {
            const double r = fs.r_comov[p0 + t], m = fs.dist_m[p0 + t];
            F.r[t] = r;
            F.m[t] = m;
            F.z[t] = fs.z[p0 + t];
            F.w[t] = fs.weights[p0 + t];
            F.dll[t] = ll[p0 + t];
            const float rh = (float)r;
            F.rh[t] = rh;
            F.rl[t] = (float)__dsub_rn(r, (double)rh);
            F.mf[t] = (float)m;
            lmax = fmax(lmax, fabs(r));
            lmmax = fmax(lmmax, fabs(m));
        }
        for (int t = tid; t < n2; t += kDmBlock) {
            const int g = obj_index[o0 + t];
            const double r = qs.obj_r_comov[g], m = qs.obj_dist_m[g];
            const double ang =
                obj_angle ? obj_angle[o0 + t]
                          : angle_between(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                          fs.dec[f], fs.cos_dec[f], qs.x_cart[g], qs.y_cart[g],
                                          qs.z_cart[g], qs.ra[g], qs.dec[g]);
            const double cc = cos(ang / 2), ss = sin(ang / 2);
            Q.r[t] = r;
            Q.m[t] = m;
            Q.z[t] = qs.z_qso[g];
            Q.w[t] = qs.obj_weight[g];
            Q.cc[t] = cc;
            Q.ss[t] = ss;
            const float rh = (float)r;
            Q.rh[t] = rh;
            Q.rl[t] = (float)__dsub_rn(r, (double)rh);
            Q.mf[t] = (float)m;
            Q.ccf[t] = (float)cc;
            Q.ssf[t] = (float)ss;
            Q.zf[t] = c.redshift_evolution
                          ? pow(__dadd_rn(1., Q.z[t]) / __dadd_rn(1., c.z_ref),
                                __dsub_rn(c.alpha2, 1.))
                          : 1.;
            lmax = fmax(lmax, fabs(r));
            lmmax = fmax(lmmax, fabs(m));
            lss = fmax(lss, ss);
            lcc = fmin(lcc, cc);
        }
        for (int t = tid; t < c.mwords; t += kDmBlock) mbits[t] = 0u;
        for (int t = tid; t < c.dwords; t += kDmBlock) dbits[t] = 0u;
        // guard bands as in the auto-correlation, with the extreme half-angles
        double rmax, mmax, ssmax, ccmin;
        {
            for (int o = 16; o > 0; o >>= 1) {
                lmax = fmax(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
                lmmax = fmax(lmmax, __shfl_xor_sync(0xffffffffu, lmmax, o));
                lss = fmax(lss, __shfl_xor_sync(0xffffffffu, lss, o));
                lcc = fmin(lcc, __shfl_xor_sync(0xffffffffu, lcc, o));
            }
            double v[4] = {lmax, lmmax, lss, -lcc};
            double res[4];
            for (int k = 0; k < 4; ++k) {
                __syncthreads();
                if ((tid & 31) == 0) red[tid >> 5] = v[k];
                __syncthreads();
                double mx = -1e300;
                for (int w = 0; w < kDmWarps; ++w) mx = fmax(mx, red[w]);
                res[k] = mx;
            }
            rmax = res[0];
            mmax = res[1];
            ssmax = res[2];
            ccmin = -res[3];
        }
        DmGuard gd;
        {
            const double u = 5.9604644775390625e-8;  // 2^-24
            const double rlim = fmax(fabs(c.b.r_par_max), fabs(c.b.r_par_min));
            const double gp = 2. * (2. * u * rmax + 3. * u * (rlim + 1.) / fmax(ccmin, 1e-6));
            const double gt = 2. * (4. * u * mmax * ssmax + 2. * u * c.b.r_trans_max);
            const double ey = 8. * u;
            gd.cc = 1.f;
            gd.ss = 0.f;
            gd.gp = (float)gp;
            gd.gt = (float)gt;
            gd.gyp = (float)(gp * c.sp + ey * (c.b.np + 1));
            gd.gymp = (float)(gp * c.smp + ey * (c.nmp + 1));
            gd.gyt = (float)(gt * c.st + ey * (c.b.nt + 1));
            gd.gymt = (float)(gt * c.smt + ey * (c.nmt + 1));
        }
        if (tid == 0) s_count = 0;
        __syncthreads();

        // 1. classification over (pixel, quasar)
        {
            int counted = 0;
            for (int e = tid; e < n1 * n2; e += kDmBlock) {
                const int j = e / n1, i = e - j * n1;
                if (F.w[i] == 0. || Q.w[j] == 0.) continue;
                DmPair o;
                if (!dm_decide_x(c, gd, F, Q, i, j, o)) continue;
                if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) {
                    report_error(scratch, PG_ERR_BIN_RANGE, o.mb);
                    continue;
                }
                ++counted;
                const uint32_t mbit = 1u << (o.mb & 31);
                if (!(mbits[o.mb >> 5] & mbit)) atomicOr(&mbits[o.mb >> 5], mbit);
                if (o.zsel) {
                    const uint32_t dbit = 1u << (o.db & 31);
                    if (!(dbits[o.db >> 5] & dbit)) atomicOr(&dbits[o.db >> 5], dbit);
                }
            }
            for (int o = 16; o > 0; o >>= 1) counted += __shfl_xor_sync(0xffffffffu, counted, o);
            if ((tid & 31) == 0 && counted) atomicAdd(&s_count, counted);
        }
        __syncthreads();
        if (s_count == 0) {
            __syncthreads();
            continue;
        }
        const int nmt = dm_scan_bits(mbits, mpref, c.mwords, red_int);
        const int nbt = dm_scan_bits(dbits, dpref, c.dwords, red_int);
        if (nbt == 0) {
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
        // forest sums (py/picca/xcf.py:470-487) and per-pixel factors
        double lw = 0., lsw = 0.;
        for (int t = tid; t < n1; t += kDmBlock) {
            lw += F.w[t];
            lsw += __dmul_rn(F.dll[t], F.w[t]);
        }
        const double sw1 = dm_block_sum(lw, red);
        const double sll1 = dm_block_sum(lsw, red);
        const double mean1 = sll1 / sw1;
        double q1 = 0.;
        for (int t = tid; t < n1; t += kDmBlock) {
            const double d = __dsub_rn(F.dll[t], mean1);
            F.dll[t] = d;
            q1 += __dmul_rn(F.w[t], __dmul_rn(d, d));
            F.zf[t] = c.redshift_evolution
                          ? pow(__dadd_rn(1., F.z[t]) / __dadd_rn(1., c.z_ref),
                                __dsub_rn(c.alpha, 1.))
                          : 1.;
        }
        const double swsll1 = dm_block_sum(q1, red);
        if (ord1 && !(swsll1 != 0.)) {
            if (tid == 0) report_error(scratch, PG_ERR_INVALID_ARGUMENT, (int32_t)q);
            __syncthreads();
            continue;
        }
        const double inv_sw1 = 1. / sw1, inv_q1 = 1. / swsll1;
        for (int t = tid; t < n1; t += kDmBlock) {
            const double wz = __dmul_rn(F.w[t], F.zf[t]);
            F.a[t] = __dmul_rn(wz, inv_sw1);
            F.b[t] = __dmul_rn(__dmul_rn(wz, F.dll[t]), inv_q1);
            F.wd[t] = __dmul_rn(F.w[t], F.dll[t]);
            F.wz[t] = wz;
            F.wzz[t] = __dmul_rn(F.w[t], F.z[t]);
            F.wm[t] = __dmul_rn(F.w[t], F.m[t]);
        }
        __syncthreads();

        const int kX = 0, kY = n2;
        const int kR = n2 + (ord1 ? n2 : 0);
        const int kst = (int)dm_align((size_t)max(kR, 1), kSlab);
        const int64_t cap = c.work_doubles / kst;
        int dc = nbt, mc = nmt;
        if ((int64_t)nbt + nmt > cap) {
            dc = (int)min((int64_t)nbt, cap / 2);
            mc = (int)(cap - dc);
        }
        // the sweep runs over (quasar, pixel segment): segs segments per quasar
        const int segs = max(1, min(kDmBlock / max(n2, 1), (n1 + 7) / 8));
        const int seg_len = (n1 + segs - 1) / segs;
        for (int d0 = 0; d0 < nbt; d0 += dc) {
            const int dcc = min(dc, nbt - d0);
            for (int m0 = 0; m0 < nmt; m0 += mc) {
                const int mcc = min(mc, nmt - m0);
                const bool first = d0 == 0 && m0 == 0;
                double *U = rows;
                double *E = rows + (int64_t)dcc * kst;
                {
                    const int64_t n = (int64_t)(dcc + mcc) * kst / 2;
                    double2 *pz = reinterpret_cast<double2 *>(rows);
                    for (int64_t t = tid; t < n; t += kDmBlock) pz[t] = make_double2(0., 0.);
                }
                __syncthreads();
                for (int e = tid; e < n2 * segs; e += kDmBlock) {
                    const int j = e / segs, sg = e - j * segs;
                    const int i0 = sg * seg_len, i1 = min(n1, i0 + seg_len);
                    const double w2 = Q.w[j];
                    if (w2 == 0.) continue;
                    const double zf2 = Q.zf[j];
                    int run_m = -1, run_d = -1;
                    double e2 = 0., e4 = 0., x = 0., y = 0.;
                    int64_t run_k = -1;
                    int32_t k_db = 0, k_mb = 0;
                    double k_dm = 0., k_w = 0., k_rp = 0., k_rt = 0., k_z = 0.;
                    auto flush_k = [&]() {
                        const double w2zf = __dmul_rn(w2, zf2);
                        atomicAdd(&out.dmat[run_k], __dmul_rn(w2zf, k_dm));
                        atomicAdd(&out.weights_dmat[k_db], __dmul_rn(w2, k_w));
                        atomicAdd(&out.r_par_eff[k_mb], __dmul_rn(w2, k_rp));
                        const double rt = c.b.rmu ? k_rt
                                                  : __dmul_rn(__dadd_rn(k_rt,
                                                                        __dmul_rn(Q.m[j], k_w)),
                                                              Q.ss[j]);
                        atomicAdd(&out.r_trans_eff[k_mb], __dmul_rn(w2, rt));
                        atomicAdd(&out.z_eff[k_mb],
                                  __dmul_rn(w2, __dmul_rn(0.5, __dadd_rn(k_z,
                                                                         __dmul_rn(Q.z[j], k_w)))));
                        atomicAdd(&out.weight_eff[k_mb], __dmul_rn(w2, k_w));
                    };
                    for (int i = i0; i < i1; ++i) {
                        const double w1 = F.w[i];
                        if (w1 == 0.) continue;
                        DmPair o;
                        const int st = dm_decide_x(c, gd, F, Q, i, j, o);
                        if (!st) continue;
                        if (o.db < 0 || o.db >= nb || o.mb < 0 || o.mb >= nm) continue;
                        const int ml = dm_rank(mbits, mpref, o.mb) - m0;
                        if (ml >= 0 && ml < mcc) {
                            if (ml != run_m) {
                                if (run_m >= 0) {
                                    atomicAdd(&E[(int64_t)run_m * kst + kX + j], -__dmul_rn(zf2, e2));
                                    if (ord1) atomicAdd(&E[(int64_t)run_m * kst + kY + j], -__dmul_rn(zf2, e4));
                                }
                                run_m = ml;
                                e2 = 0.;
                                e4 = 0.;
                            }
                            e2 += F.a[i];
                            if (ord1) e4 += F.b[i];
                        }
                        if (o.zsel) {
                            const int dl = dm_rank(dbits, dpref, o.db) - d0;
                            if (dl >= 0 && dl < dcc) {
                                if (dl != run_d) {
                                    if (run_d >= 0) {
                                        atomicAdd(&U[(int64_t)run_d * kst + kX + j], __dmul_rn(w2, x));
                                        if (ord1) atomicAdd(&U[(int64_t)run_d * kst + kY + j], __dmul_rn(w2, y));
                                    }
                                    run_d = dl;
                                    x = 0.;
                                    y = 0.;
                                }
                                x += w1;
                                if (ord1) y += F.wd[i];
                            }
                            if (first) {
                                const int64_t key = (int64_t)o.db * nm + o.mb;
                                if (key != run_k) {
                                    if (run_k >= 0) flush_k();
                                    run_k = key;
                                    k_db = o.db;
                                    k_mb = o.mb;
                                    k_dm = k_w = k_rp = k_rt = k_z = 0.;
                                }
                                k_dm += F.wz[i];
                                k_w += w1;
                                k_z += F.wzz[i];
                                if (st == 2) {
                                    k_rp += __dmul_rn(w1, o.rp);
                                    if (c.b.rmu) k_rt += __dmul_rn(w1, o.rt);
                                    else k_rt += F.wm[i];
                                } else {
                                    k_rp += __dmul_rn(w1, __dmul_rn(__dsub_rn(F.r[i], Q.r[j]),
                                                                    Q.cc[j]));
                                    k_rt += F.wm[i];
                                }
                            }
                        }
                    }
                    if (run_m >= 0) {
                        atomicAdd(&E[(int64_t)run_m * kst + kX + j], -__dmul_rn(zf2, e2));
                        if (ord1) atomicAdd(&E[(int64_t)run_m * kst + kY + j], -__dmul_rn(zf2, e4));
                    }
                    if (run_d >= 0) {
                        atomicAdd(&U[(int64_t)run_d * kst + kX + j], __dmul_rn(w2, x));
                        if (ord1) atomicAdd(&U[(int64_t)run_d * kst + kY + j], __dmul_rn(w2, y));
                    }
                    if (run_k >= 0) flush_k();
                }
                __syncthreads();
                if (tid == 0)
                    atomicAdd(&scratch->gemm_macs,
                              (unsigned long long)dcc * (unsigned long long)mcc * kR);
                if (c.split)
                    dm_product_split(U, E, dcc, mcc, kst, digits, rexp, ta_raw, tb_raw,
                                     dlist + d0, mlist + m0, nm, out.dmat);
                else
                    dm_product_fp64(U, E, dcc, mcc, kst, ta, tb, dlist + d0, mlist + m0, nm,
                                    out.dmat);
                __syncthreads();
            }
        }
    }
}

}  // namespace

int dmat_config(const pg_corr_params &p, const pg_dmat_params &d, int p1, int p2, int num_sms,
                DmatConstHost &h, bool xcf) {
    if (xcf) p2 = kXdObjects;
    if (d.num_model_bins_r_par <= 0 || d.num_model_bins_r_trans <= 0) return PG_ERR_INVALID_ARGUMENT;
    if (p1 <= 0 || p2 <= 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t nm = (int64_t)d.num_model_bins_r_par * d.num_model_bins_r_trans;
    const int64_t nb = (int64_t)p.num_bins_r_par * p.num_bins_r_trans;
    if (nm > (1 << 26) || nb > (1 << 26)) return PG_ERR_UNSUPPORTED;
    const int mwords = (int)((nm + 31) / 32), dwords = (int)((nb + 31) / 32);
    if (d.product != PG_DMAT_FP64 && d.product != PG_DMAT_SPLIT_BF16) return PG_ERR_INVALID_ARGUMENT;
    const int split = d.product == PG_DMAT_SPLIT_BF16;
    const DmSmem s = dm_smem(p1, p2, mwords, dwords, split, xcf);
    if (s.total > 220 * 1024) return PG_ERR_UNSUPPORTED;
    h.smem = s.total;
    h.p1 = p1;
    h.p2 = p2;
    h.mwords = mwords;
    h.dwords = dwords;
    const int64_t kcap = xcf ? (int64_t)dm_align((size_t)2 * p2, kSlab)
                             : (int64_t)dm_align((size_t)2 * p1 + 2 * p2 + 4, kSlab);
    if (d.row_capacity < 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t wanted = d.row_capacity > 0 ? std::max<int64_t>(d.row_capacity, 2)
                                              : kDmatRowCapacity;
    const int64_t rows = std::min<int64_t>(nb + nm, wanted);
    h.list_doubles = (int64_t)dm_align((size_t)(nb + nm), 32) / 2;
    h.work_doubles = rows * kcap;
    // tensor-core form: six bf16 digits per element and one exponent per row
    const int64_t extra = split ? h.work_doubles * kSlices / 4 + h.work_doubles / 32 : 0;
    h.split = split;
    h.cta_doubles = (int64_t)dm_align((size_t)(h.list_doubles + h.work_doubles + extra), 32);
    h.xcf = xcf;
    int occ = 0;
    const void *fn = xcf ? (const void *)xcf_dmat_kernel : (const void *)cf_dmat_kernel;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.total) !=
        cudaSuccess)
        return PG_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kDmBlock, s.total) !=
            cudaSuccess ||
        occ < 1)
        return PG_ERR_CUDA;
    h.max_grid = num_sms * occ;
    return PG_OK;
}

static DmatConst dmat_const(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h) {
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
    c.sp = c.b.np / c.b.r_par_range;
    c.smp = c.nmp / c.b.r_par_range;
    c.st = c.b.nt / c.b.r_trans_max;
    c.smt = c.nmt / c.b.r_trans_max;
    c.f_rpmin = (float)c.b.r_par_min;
    c.f_rpmax = (float)c.b.r_par_max;
    c.f_rtmax = (float)c.b.r_trans_max;
    c.f_hpc = (float)c.b.half_plate_cut;
    c.f_sp = (float)c.sp;
    c.f_smp = (float)c.smp;
    c.f_st = (float)c.st;
    c.f_smt = (float)c.smt;
    c.p1 = h.p1;
    c.p2 = h.p2;
    c.mwords = h.mwords;
    c.dwords = h.dwords;
    c.list_doubles = h.list_doubles;
    c.work_doubles = h.work_doubles;
    c.cta_doubles = h.cta_doubles;
    c.split = h.split;
    c.xcf = h.xcf;
    return c;
}

int launch_cf_dmat(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h,
                   const pg_forest_set &s1, const pg_forest_set &s2, const double *ll1,
                   const double *ll2, const int32_t *order1, const int32_t *order2,
                   const int32_t *pair_first, const int32_t *pair_second,
                   const double *pair_angle, int64_t num_pairs, double *work, int grid,
                   const pg_dmat_sums &out, Scratch *scratch, cudaStream_t stream) {
    if (num_pairs == 0) return PG_OK;
    const DmatConst c = dmat_const(p, d, h);
    cf_dmat_kernel<<<grid, kDmBlock, h.smem, stream>>>(c, s1, s2, ll1, ll2, order1, order2,
                                                       pair_first, pair_second, pair_angle,
                                                       num_pairs, out, work, scratch);
    return check_cuda(cudaGetLastError());
}

int launch_xcf_dmat(const pg_corr_params &p, const pg_dmat_params &d, const DmatConstHost &h,
                    const pg_forest_set &forests, const pg_forest_set &objs, const double *ll,
                    const int32_t *order, const int32_t *item_forest, const int32_t *item_start,
                    const int32_t *item_count, const int32_t *obj_index,
                    const double *obj_angle, int64_t num_items, double *work, int grid,
                    const pg_dmat_sums &out, Scratch *scratch, cudaStream_t stream) {
    if (num_items == 0) return PG_OK;
    DmatConst c = dmat_const(p, d, h);
    c.b.x_correlation = 1;  // r_par is signed in the cross-correlation
    c.b.remove_shp = 0;
    c.b.zerr_on = 0;
    xcf_dmat_kernel<<<grid, kDmBlock, h.smem, stream>>>(c, forests, objs, ll, order, item_forest,
                                                        item_start, item_count, obj_index,
                                                        obj_angle, num_items, out, work,
                                                        scratch);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
