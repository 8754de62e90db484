// Device helpers shared by the continuum kernels and the fused warm-start
// network kernel: FP64 inputs converted on the integer pipe, the mixed fit's
// shared-memory model tables, warp sums (internal linkage in each
// translation unit that includes this file).
#pragma once

#include "pg_internal.cuh"

namespace pg {
namespace {

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}


// ---- FP64 inputs on the integer pipe -------------------------------------
// GB300's FP64 pipe is narrow (1/64 of FP32). The mixed fit converts its FP64
// inputs with integer operations on the bit patterns and forms the one
// difference that needs more than FP32 (L - Lmin) from two-float parts.

// v rounded to FP32 (round half away from zero on the dropped bits: equal to
// round-to-nearest-even except on exact ties). Integer operations only:
// magnitudes below the FP32 normal range give a signed zero (flush to zero),
// above it a signed infinity; NaN stays NaN.
__device__ __forceinline__ float f64_to_f32(double v) {
    const unsigned hw = (unsigned)__double2hiint(v), lw = (unsigned)__double2loint(v);
    const unsigned sign = hw & 0x80000000u;
    const unsigned e = (hw >> 20) & 0x7FFu;
    const unsigned mag = ((((hw & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lw >> 29)) +
                         ((lw >> 28) & 1u);
    const bool nan = e == 0x7FFu && ((hw & 0xFFFFFu) | lw) != 0u;
    const unsigned bits = e < 897u ? 0u : (e > 1150u ? (nan ? 0x7FC00000u : 0x7F800000u) : mag);
    return __uint_as_float(sign | bits);
}

// v = hi + lo: hi is v truncated to 24 significant bits, lo the remaining 29
// bits rounded to FP32 (|v - hi - lo| <= 2^-48 |v|) for 2^-74 <= |v| < 2^127;
// outside that range hi = f64_to_f32(v) and lo = 0. Integer operations only.
__device__ __forceinline__ float2 split_f64(double v) {
    const unsigned hw = (unsigned)__double2hiint(v), lw = (unsigned)__double2loint(v);
    const unsigned e = (hw >> 20) & 0x7FFu;
    const unsigned sign = hw & 0x80000000u;
    const float hi =
        __uint_as_float(sign | ((((hw & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lw >> 29)));
    const unsigned rem = lw & 0x1FFFFFFFu;
    // the 29-bit remainder as (6 bits) 2^23 + (23 bits), each exact in FP32
    const float r_lo = __uint_as_float(0x4B000000u | (rem & 0x7FFFFFu)) - 8388608.f;
    const float r_hi = __uint_as_float(0x4B000000u | (rem >> 23)) - 8388608.f;
    const float r = fmaf(r_hi, 8388608.f, r_lo) * __uint_as_float(((e - 948u) & 0xFFu) << 23);
    const bool normal = e - 949u <= 200u;
    return make_float2(normal ? hi : f64_to_f32(v),
                       normal ? __uint_as_float(__float_as_uint(r) | sign) : 0.f);
}

// x exactly in FP64 (integer operations; FP32 subnormals give a signed zero)
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned sign = u & 0x80000000u;
    const unsigned ex = (u >> 23) & 0xFFu;
    const unsigned hw_n = sign | (((u & 0x7FFFFFFFu) >> 3) + (896u << 20));
    const unsigned hw_s = sign | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3);  // inf, NaN
    const unsigned hw = ex == 0u ? sign : (ex == 0xFFu ? hw_s : hw_n);
    return __hiloint2double((int)hw, ex == 0u ? 0 : (int)(u << 29));
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// a b - c d with one rounding's accuracy (Kahan's difference of products)
__device__ __forceinline__ float diff_prod(float a, float b, float c, float d) {
    const float w = c * d;
    const float e = fmaf(-c, d, w);
    return fmaf(a, b, -w) + e;
}

// ---- model tables of the mixed fit (shared memory) ----------------------
// Mean continuum nodes as FP32 offsets from the rest-frame grid start (the
// pixels' rest-frame coordinate is formed as L - Lmin, exact in FP32 to its
// last bit); variance functions as FP32 cubics, the three functions of an
// interval interleaved (eta, var_lss, fudge: c3 c2 c1 c0 each). Uniformly
// spaced nodes or breaks (the usual case) are found by one multiply and a
// correction step, others by bisection.
struct FitTables {
    const float *mc_off, *mc_y, *mc_slope, *brk;
    const float4 *coef;
    int nmc, m;
    float mc_off0, mc_inv_step, brk0, brk_inv_step;
    bool mc_uniform, brk_uniform;
};

__host__ __device__ inline size_t fit_smem_bytes(int nmc, int m) {
    return (size_t)(3 * nmc + m + 8) * 4 + 16 + (size_t)3 * m * 16 + 16;
}

__device__ FitTables load_fit_tables(const pg_cont_model &m, unsigned char *smem) {
    __shared__ int s_uniform[2];
    FitTables t;
    const int nmc = m.num_mean_cont, mi = m.use_constant_weight ? 0 : m.num_var_intervals;
    float4 *coef = reinterpret_cast<float4 *>(smem);
    float *mc_off = reinterpret_cast<float *>(coef + 3 * mi);
    float *mc_y = mc_off + nmc;
    float *mc_slope = mc_y + nmc;
    float *brk = mc_slope + nmc;
    if (threadIdx.x == 0) s_uniform[0] = s_uniform[1] = 1;
    __syncthreads();
    const double rest_min = m.log_lambda_rest_min;
    const double mc_step = nmc > 1 ? (m.mean_cont_x[nmc - 1] - m.mean_cont_x[0]) / (nmc - 1) : 1.;
    for (int i = threadIdx.x; i < nmc; i += blockDim.x) {
        const double x = m.mean_cont_x[i], y = m.mean_cont_y[i];
        mc_off[i] = (float)(x - rest_min);
        mc_y[i] = (float)y;
        mc_slope[i] = i + 1 < nmc ? (float)((m.mean_cont_y[i + 1] - y) / (m.mean_cont_x[i + 1] - x))
                                  : 0.f;
        if (fabs(x - m.mean_cont_x[0] - i * mc_step) > 1e-3 * mc_step) s_uniform[0] = 0;
    }
    const double brk_step = mi > 0 ? (m.var_breaks[mi] - m.var_breaks[0]) / mi : 1.;
    for (int i = threadIdx.x; i <= mi; i += blockDim.x) {
        brk[i] = (float)m.var_breaks[i];
        if (fabs(m.var_breaks[i] - m.var_breaks[0] - i * brk_step) > 1e-3 * brk_step)
            s_uniform[1] = 0;
    }
    for (int i = threadIdx.x; i < mi; i += blockDim.x) {
        coef[3 * i] = make_float4((float)m.eta_coef[i], (float)m.eta_coef[mi + i],
                                  (float)m.eta_coef[2 * mi + i], (float)m.eta_coef[3 * mi + i]);
        coef[3 * i + 1] =
            make_float4((float)m.var_lss_coef[i], (float)m.var_lss_coef[mi + i],
                        (float)m.var_lss_coef[2 * mi + i], (float)m.var_lss_coef[3 * mi + i]);
        coef[3 * i + 2] =
            make_float4((float)m.fudge_coef[i], (float)m.fudge_coef[mi + i],
                        (float)m.fudge_coef[2 * mi + i], (float)m.fudge_coef[3 * mi + i]);
    }
    __syncthreads();
    t.mc_off = mc_off; t.mc_y = mc_y; t.mc_slope = mc_slope; t.brk = brk; t.coef = coef;
    t.nmc = nmc; t.m = mi;
    t.mc_off0 = nmc > 0 ? mc_off[0] : 0.f;
    t.mc_inv_step = (float)(1.0 / mc_step);
    t.mc_uniform = s_uniform[0] != 0 && nmc > 2;
    t.brk0 = mi > 0 ? brk[0] : 0.f;
    t.brk_inv_step = (float)(1.0 / brk_step);
    t.brk_uniform = s_uniform[1] != 0 && mi > 1;
    return t;
}

// mean continuum at rest-frame offset u = L - Lmin (linear interpolation
// with extrapolation, interp_linear's intervals)
__device__ __forceinline__ float fit_mean_cont(const FitTables &t, float u) {
    int i;
    const int top = t.nmc - 2;
    if (t.mc_uniform) {
        i = __float2int_rd((u - t.mc_off0) * t.mc_inv_step);
        i = i < 0 ? 0 : (i > top ? top : i);
        if (i > 0 && u < t.mc_off[i]) --i;
        else if (i < top && u >= t.mc_off[i + 1]) ++i;
    } else {
        int lo = 0, hi = t.nmc;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (t.mc_off[mid] < u) lo = mid + 1;
            else hi = mid;
        }
        i = lo < 1 ? 0 : (lo > t.nmc - 1 ? t.nmc - 2 : lo - 1);
    }
    return fmaf(t.mc_slope[i], u - t.mc_off[i], t.mc_y[i]);
}

// eta, var_lss and fudge at observed log lambda v (eval_ppoly's intervals)
__device__ __forceinline__ void fit_var_funcs(const FitTables &t, float v, float &eta,
                                              float &var_lss, float &fudge) {
    int i;
    const int top = t.m - 1;
    if (t.brk_uniform) {
        i = __float2int_rd((v - t.brk0) * t.brk_inv_step);
        i = i < 0 ? 0 : (i > top ? top : i);
        if (i > 0 && v < t.brk[i]) --i;
        else if (i < top && v >= t.brk[i + 1]) ++i;
    } else {
        int lo = 0, hi = t.m + 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (t.brk[mid] <= v) lo = mid + 1;
            else hi = mid;
        }
        i = lo - 1;
        i = i < 0 ? 0 : (i > top ? top : i);
    }
    const float dx = v - t.brk[i];
    const float4 ce = t.coef[3 * i], cv = t.coef[3 * i + 1], cf = t.coef[3 * i + 2];
    eta = fmaf(fmaf(fmaf(ce.x, dx, ce.y), dx, ce.z), dx, ce.w);
    var_lss = fmaf(fmaf(fmaf(cv.x, dx, cv.y), dx, cv.z), dx, cv.w);
    fudge = fmaf(fmaf(fmaf(cf.x, dx, cf.y), dx, cf.z), dx, cf.w);
}

// ---- warm-start network inputs ------------------------------------------
// 64 rest-frame bins of f / mean continuum (ivar-weighted, normalised by
// a0 = sum f ivar / sum ivar, minus 1; empty bins 0), z_qso - 3 and the log
// of the mean f sqrt(ivar), in FP32 per pixel.
constexpr int kFeatBins = 64;
constexpr int kFeatUsed = kFeatBins + 2;

struct FeatScalars {
    float a0, zfeat, snrfeat;
};

// Lmin = rest-frame grid start + log10(1 + z_qso) of forest f as two floats
__device__ __forceinline__ float2 forest_lmin(const pg_spectra &sp, const pg_cont_model &m,
                                              int64_t f) {
    return split_f64(m.log_lambda_rest_min + log10(1. + sp.z_qso[f]));
}

// Sums of forest f's rest-frame bins into sums[0][bin] (sum f/mc ivar) and
// sums[1][bin] (sum ivar), zeroed here, and its scalar inputs; the whole warp
// calls it. Consecutive pixels fall in runs of one bin across the lanes: a
// segmented scan over the maximal runs of equal bins leaves each run's sum
// at its last lane, which alone adds it to the bin.
__device__ FeatScalars forest_feature_sums(const pg_spectra &sp, const FitTables &tab, int64_t f,
                                           float lmh, float lml, float bins_per_span,
                                           float (*sums)[kFeatBins], int lane) {
    for (int k = lane; k < kFeatBins; k += 32) {
        sums[0][k] = 0.f;
        sums[1][k] = 0.f;
    }
    __syncwarp();
    const int64_t off = sp.pix_offset[f];
    const int64_t n = sp.pix_offset[f + 1] - off;
    float sfi = 0.f, si = 0.f, snr = 0.f, cnt = 0.f;
    for (int64_t base = 0; base < n; base += 32) {
        const int64_t p = base + lane;
        int bin = -1;
        float num = 0.f, den = 0.f;
        if (p < n) {
            const float fl = f64_to_f32(sp.flux[off + p]);
            const float iv = f64_to_f32(sp.ivar[off + p]);
            sfi = fmaf(fl, iv, sfi);
            si += iv;
            if (iv > 0.f) {
                snr = fmaf(fl, sqrtf(iv), snr);
                cnt += 1.f;
                const float2 ll = split_f64(sp.log_lambda[off + p]);
                const float u = (ll.x - lmh) + (ll.y - lml);  // L - Lmin
                const float mc =
                    fit_mean_cont(tab, u) * f64_to_f32(sp.transmission_correction[off + p]);
                if (mc != 0.f) {
                    bin = __float2int_rd(u * bins_per_span);
                    bin = bin < 0 ? 0 : (bin >= kFeatBins ? kFeatBins - 1 : bin);
                    num = __fdividef(fl, mc) * iv;
                    den = iv;
                }
            }
        }
        const int prev = __shfl_up_sync(0xffffffffu, bin, 1);
        const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != bin);
        const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
        const int start = 31 - __clz(heads & upto);  // first lane of this run
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float tn = __shfl_up_sync(0xffffffffu, num, o);
            const float td = __shfl_up_sync(0xffffffffu, den, o);
            if (lane - o >= start) {
                num += tn;
                den += td;
            }
        }
        const int next = __shfl_down_sync(0xffffffffu, bin, 1);
        if (bin >= 0 && (lane == 31 || next != bin)) {
            atomicAdd(&sums[0][bin], num);
            atomicAdd(&sums[1][bin], den);
        }
    }
    sfi = warp_sum_f(sfi);
    si = warp_sum_f(si);
    snr = warp_sum_f(snr);
    cnt = warp_sum_f(cnt);
    __syncwarp();
    FeatScalars fs;
    fs.a0 = si > 0.f ? sfi / si : 0.f;
    fs.zfeat = f64_to_f32(sp.z_qso[f]) - 3.f;
    fs.snrfeat = logf(fmaxf(cnt > 0.f ? snr / cnt : 0.f, 1e-3f));
    return fs;
}

// feature k of a forest from its sums (k >= kFeatUsed: 0, the padding)
__device__ __forceinline__ float forest_feature(const float (*sums)[kFeatBins],
                                                const FeatScalars &fs, int k) {
    if (k < kFeatBins) {
        const float w = sums[1][k];
        return (w > 0.f && fs.a0 != 0.f) ? sums[0][k] / w / fs.a0 - 1.f : 0.f;
    }
    if (k == kFeatBins) return fs.zfeat;
    if (k == kFeatBins + 1) return fs.snrfeat;
    return 0.f;
}

}  // namespace
}  // namespace pg
