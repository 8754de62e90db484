// Batched Dr16 continuum fit (delta_extraction/expected_fluxes/utils.py:12-136
// and least_squares/least_squares_cont_model.py:65-197, paths under
// py/picca), the per-iteration histograms of Dr16ExpectedFlux and the final
// delta extraction.
//
// One warp fits one forest: every lane holds up to K pixels in registers as
// the coefficients of
//     C = (a + b x) mc,      x = (L - Lmin)/(Lmax - Lmin),
//     D = eta/ivar + var_lss C^2 + fudge ivar C^4,
//     chi2 = sum (f - C)^2 / D + sum log D
// (the reference's chi2 - sum log w with w = 1/D), evaluates chi2, its
// gradient and Hessian in (a, b) in one pass, reduces them in FP64 with warp
// shuffles and takes a damped Newton step solved in FP64 (backtracking
// Armijo line search). The per-pixel terms are FP64 (PG_FIT_FP64) or FP32
// (PG_FIT_MIXED); the reported chi2 is always re-evaluated in FP64.
// The reference minimises the same function with iminuit's MIGRAD.
#include <cuda_bf16.h>

#include "pg_cont_common.cuh"
#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kContBlock = 256;
constexpr int kContK = 7;  // pixels per lane held in registers (forests <= 224 pixels)
constexpr int kVarBins = 100;
constexpr double kVarPipeMin = -5.0;                  // log10(1e-5)
constexpr double kVarPipeMax = 0.30102999566398120;   // log10(2)

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// scipy interp1d(kind="linear", fill_value="extrapolate"): searchsorted
// (left) clipped to [1, n-1], then slope * (v - x_lo) + y_lo.
__device__ double interp_linear(const double *__restrict__ x, const double *__restrict__ y, int n,
                                double v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    int idx = lo < 1 ? 1 : (lo > n - 1 ? n - 1 : lo);
    const double xl = x[idx - 1], xh = x[idx], yl = y[idx - 1], yh = y[idx];
    const double slope = (yh - yl) / (xh - xl);
    return __dadd_rn(__dmul_rn(slope, __dsub_rn(v, xl)), yl);
}

// Piecewise cubic (highest power first), extrapolated with the end pieces.
__device__ double eval_ppoly(const double *__restrict__ brk, const double *__restrict__ coef, int m,
                             double v) {
    int lo = 0, hi = m + 1;  // searchsorted right over the m + 1 breakpoints
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (brk[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > m - 1 ? m - 1 : i);
    const double dx = v - brk[i];
    return ((coef[i] * dx + coef[m + i]) * dx + coef[2 * m + i]) * dx + coef[3 * m + i];
}

// scipy interp1d(kind="nearest"): index of the nearest stack point.
__device__ double interp_nearest(const double *__restrict__ x, const double *__restrict__ y, int n,
                                 double v) {
    // midpoints x_bds[i] = (x[i] + x[i+1]) / 2; idx = searchsorted(x_bds, v, "left")
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double bd = (x[mid] + x[mid + 1]) / 2.0;
        if (bd < v) lo = mid + 1;
        else hi = mid;
    }
    return y[lo];
}

struct ModelEval {
    double mc, eta, var_lss, fudge;
};

__device__ __forceinline__ ModelEval eval_model(const pg_cont_model &m, double ll, double zp1,
                                                double tc) {
    ModelEval e;
    e.mc = interp_linear(m.mean_cont_x, m.mean_cont_y, m.num_mean_cont, ll - zp1) * tc;
    if (m.use_constant_weight) {
        e.eta = 0.;
        e.var_lss = 1.;
        e.fudge = 0.;
    } else {
        e.eta = eval_ppoly(m.var_breaks, m.eta_coef, m.num_var_intervals, ll);
        e.var_lss = eval_ppoly(m.var_breaks, m.var_lss_coef, m.num_var_intervals, ll);
        e.fudge = eval_ppoly(m.var_breaks, m.fudge_coef, m.num_var_intervals, ll);
    }
    return e;
}

template <typename T>
struct PixelTerms {
    T ja[kContK], jb[kContK], f[kContK], q[kContK], vl[kContK], fi[kContK];
    unsigned valid;
};

// chi2 / 2 and its derivatives of one lane's pixels (accumulated in T,
// returned in FP64); constant weights use q = 1, vl = fi = 0 with no log.
// U is the arithmetic type of the per-pixel terms (T or FP64).
template <typename U, typename T, typename O, typename A>
__device__ __forceinline__ void lane_terms(const PixelTerms<T> &px, A a, A b, bool const_w,
                                           O s[6]) {
    U val = 0, ga = 0, gb = 0, haa = 0, hab = 0, hbb = 0;
    const U ua = (U)a, ub = (U)b;
#pragma unroll
    for (int k = 0; k < kContK; ++k) {
        if (!((px.valid >> k) & 1u)) continue;
        const U ja = (U)px.ja[k], jb = (U)px.jb[k];
        const U q = (U)px.q[k], vl = (U)px.vl[k], fi = (U)px.fi[k];
        const U c = ua * ja + ub * jb;
        const U c2 = c * c;
        const U d = q + vl * c2 + fi * c2 * c2;
        const U dd = (U)2 * vl * c + (U)4 * fi * c2 * c;
        const U d2d = (U)2 * vl + (U)12 * fi * c2;
        const U r = (U)px.f[k] - c;
        const U id = (U)1 / d;
        const U rid = r * id;
        const U ddid = dd * id;
        val += r * rid + (const_w ? (U)0 : log(d));
        const U g = (U)-2 * rid - rid * rid * dd + ddid;
        const U h = (U)2 * id + (U)4 * rid * ddid + (U)2 * rid * rid * dd * ddid - rid * rid * d2d
                    + d2d * id - ddid * ddid;
        ga += g * ja;
        gb += g * jb;
        haa += h * ja * ja;
        hab += h * ja * jb;
        hbb += h * jb * jb;
    }
    s[0] = (O)val; s[1] = (O)ga; s[2] = (O)gb;
    s[3] = (O)haa; s[4] = (O)hab; s[5] = (O)hbb;
}

template <typename U, typename T>
__device__ __forceinline__ void eval_all(const PixelTerms<T> &px, double a, double b, bool const_w,
                                         double s[6]) {
    lane_terms<U, T, double, double>(px, a, b, const_w, s);
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k] = warp_sum(s[k]);
}

template <typename T>
__global__ void __launch_bounds__(kContBlock) cont_fit_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const double *__restrict__ start, const int32_t *__restrict__ index, int64_t count,
    int max_iter, double tol, const __grid_constant__ pg_cont_fit out, Scratch *scratch) {
    const int lane = threadIdx.x & 31;
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool const_w = m.use_constant_weight != 0;
    for (int64_t w = warp_global; w < count; w += nwarps) {
        const int64_t f = index ? (int64_t)index[w] : w;
        const int64_t off = sp.pix_offset[f];
        const int64_t n64 = sp.pix_offset[f + 1] - off;
        if (n64 > 32 * kContK) continue;  // a long forest: cont_fit_long_kernel
        if (n64 <= 0) {
            if (lane == 0) {
                out.zero_point[f] = NAN;
                out.slope[f] = NAN;
                out.chi2[f] = NAN;
                out.ndata[f] = 0;
                out.status[f] = 1;
                out.iterations[f] = 0;
            }
            continue;
        }
        const int n = (int)n64;
        const double zp1 = log10(1 + sp.z_qso[f]);
        const double ll_min = m.log_lambda_rest_min + zp1;
        const double ll_max = m.log_lambda_rest_max + zp1;
        PixelTerms<T> px;
        px.valid = 0;
        double sfi = 0., si = 0.;
#pragma unroll
        for (int k = 0; k < kContK; ++k) {
            const int p = lane + 32 * k;
            px.ja[k] = px.jb[k] = px.f[k] = px.q[k] = px.vl[k] = px.fi[k] = (T)0;
            if (p < n) {
                const double ll = sp.log_lambda[off + p], fl = sp.flux[off + p];
                const double iv = sp.ivar[off + p];
                sfi += fl * iv;
                si += iv;
                if (iv > 0) {
                    const ModelEval e = eval_model(m, ll, zp1, sp.transmission_correction[off + p]);
                    const double x = (ll - ll_min) / (ll_max - ll_min);
                    px.ja[k] = (T)e.mc;
                    px.jb[k] = (T)(x * e.mc);
                    px.f[k] = (T)fl;
                    px.q[k] = (T)(const_w ? 1. : e.eta / iv);
                    px.vl[k] = (T)(const_w ? 0. : e.var_lss);
                    px.fi[k] = (T)(const_w ? 0. : e.fudge * iv);
                    px.valid |= 1u << k;
                }
            }
        }
        sfi = warp_sum(sfi);
        si = warp_sum(si);
        const double a0 = sfi / si;  // utils.py:92
        // ndata: pixels with a positive weight at the reference's starting
        // point (a0, 0) (cont_model.py:88-92)
        int nd = 0;
#pragma unroll
        for (int k = 0; k < kContK; ++k) {
            if ((px.valid >> k) & 1u) {
                const double c = a0 * (double)px.ja[k];
                const double d = (double)px.q[k] + (double)px.vl[k] * c * c +
                                 (double)px.fi[k] * c * c * c * c;
                nd += (d > 0.) ? 1 : 0;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
        double a = a0, b = 0.;
        if (start) {
            a = start[2 * f];
            b = m.order == 0 ? 0. : start[2 * f + 1];
        }

        double s[6];
        eval_all<T>(px, a, b, const_w, s);
        int it = 0;
        // max_iter == 0 with a start: evaluate the model at the given (a, b)
        bool converged = max_iter == 0 && start != nullptr;
        for (; it < max_iter; ++it) {
            double da, db;
            if (m.order == 0) {
                da = s[3] > 0 ? -s[1] / s[3] : -s[1];
                db = 0.;
            } else {
                const double det = s[3] * s[5] - s[4] * s[4];
                if (det > 0 && s[3] > 0) {
                    da = -(s[5] * s[1] - s[4] * s[2]) / det;
                    db = -(s[3] * s[2] - s[4] * s[1]) / det;
                } else {
                    const double scale = fmax(fabs(s[3]), fabs(s[5]));
                    da = -s[1] / (scale > 0 ? scale : 1.);
                    db = -s[2] / (scale > 0 ? scale : 1.);
                }
                if (da * s[1] + db * s[2] >= 0) {  // not a descent direction
                    const double scale = fmax(fabs(s[3]), fabs(s[5]));
                    da = -s[1] / (scale > 0 ? scale : 1.);
                    db = -s[2] / (scale > 0 ? scale : 1.);
                }
            }
            const double slope_dir = da * s[1] + db * s[2];
            double t = 1.;
            double trial[6];
            bool accepted = false;
            for (int ls = 0; ls < 40; ++ls) {
                eval_all<T>(px, a + t * da, b + t * db, const_w, trial);
                if (isfinite(trial[0]) && trial[0] <= s[0] + 1e-4 * t * slope_dir) {
                    accepted = true;
                    break;
                }
                t *= 0.5;
            }
            if (!accepted) {
                converged = fabs(s[1]) + fabs(s[2]) < 1e-6 * fmax(1., fabs(s[0]));
                break;
            }
            a += t * da;
            b += t * db;
#pragma unroll
            for (int k = 0; k < 6; ++k) s[k] = trial[k];
            if (fabs(t * da) < tol * fmax(1., fmax(fabs(a), fabs(b))) &&
                fabs(t * db) < tol * fmax(1., fmax(fabs(a), fabs(b)))) {
                converged = true;
                ++it;
                break;
            }
        }
        // chi2 at the solution in FP64, and the continuum with the
        // reference's operation order (cont_model.py:138-144)
        double fin[6];
        eval_all<double>(px, a, b, const_w, fin);
        bool negative = false, all_zero = true;
        for (int p = lane; p < n; p += 32) {
            const double ll = sp.log_lambda[off + p];
            const double mc = interp_linear(m.mean_cont_x, m.mean_cont_y, m.num_mean_cont,
                                            ll - zp1) * sp.transmission_correction[off + p];
            const double line = b * (ll - ll_min) / (ll_max - ll_min) + a;
            const double c = line * mc;
            if (out.continuum) out.continuum[off + p] = c;
            negative |= c < 0;
            all_zero &= c == 0;
        }
        negative = __any_sync(0xffffffffu, negative);
        all_zero = __all_sync(0xffffffffu, all_zero);
        if (lane == 0) {
            int status = converged ? 0 : 1;
            if (negative) status = 2;
            if (all_zero) status = 3;
            out.zero_point[f] = status == 0 ? a : NAN;
            out.slope[f] = status == 0 ? b : NAN;
            out.chi2[f] = status == 0 ? fin[0] : NAN;
            out.ndata[f] = nd;
            out.status[f] = status;
            out.iterations[f] = it;
        }
    }
}

// ---------------------------------------------------------------------------
// Long forests (more than 32 * kContK pixels, up to 32 * kLongK: the linear
// 0.8 Angstrom grid reaches about 1,000 pixels). Same fit as cont_fit_kernel
// in FP64 (damped Newton with Armijo backtracking, the same status codes),
// with the per-pixel terms in the warp's shared-memory slab instead of
// registers: term t of pixel k*32 + lane at slab[t * 32 * kLongK + k * 32 +
// lane] (consecutive lanes, consecutive banks). Forests of at most
// 32 * kContK pixels are left to the register kernels.
// ---------------------------------------------------------------------------
constexpr int kLongK = 32;
constexpr int kLongWarps = 4;  // 4 x 48 KB slabs per block

__device__ __forceinline__ void long_terms(const double *slab, unsigned valid, int nk, double a,
                                           double b, bool const_w, double s[6]) {
    const int lane = threadIdx.x & 31;
    double val = 0, ga = 0, gb = 0, haa = 0, hab = 0, hbb = 0;
    constexpr int S = 32 * kLongK;
    for (int k = 0; k < nk; ++k) {
        if (!((valid >> k) & 1u)) continue;
        const int e = k * 32 + lane;
        const double ja = slab[e], jb = slab[S + e], fl = slab[2 * S + e];
        const double q = slab[3 * S + e], vl = slab[4 * S + e], fi = slab[5 * S + e];
        const double c = a * ja + b * jb;
        const double c2 = c * c;
        const double d = q + vl * c2 + fi * c2 * c2;
        const double dd = 2. * vl * c + 4. * fi * c2 * c;
        const double d2d = 2. * vl + 12. * fi * c2;
        const double r = fl - c;
        const double id = 1. / d;
        const double rid = r * id;
        const double ddid = dd * id;
        val += r * rid + (const_w ? 0. : log(d));
        const double g = -2. * rid - rid * rid * dd + ddid;
        const double h = 2. * id + 4. * rid * ddid + 2. * rid * rid * dd * ddid - rid * rid * d2d +
                         d2d * id - ddid * ddid;
        ga += g * ja;
        gb += g * jb;
        haa += h * ja * ja;
        hab += h * ja * jb;
        hbb += h * jb * jb;
    }
    s[0] = warp_sum(val); s[1] = warp_sum(ga); s[2] = warp_sum(gb);
    s[3] = warp_sum(haa); s[4] = warp_sum(hab); s[5] = warp_sum(hbb);
}

__global__ void __launch_bounds__(32 * kLongWarps) cont_fit_long_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const double *__restrict__ start, const int32_t *__restrict__ index, int64_t count,
    int max_iter, double tol, const __grid_constant__ pg_cont_fit out, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    double *slab = reinterpret_cast<double *>(smem) + (size_t)(threadIdx.x >> 5) * 6 * 32 * kLongK;
    constexpr int S = 32 * kLongK;
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool const_w = m.use_constant_weight != 0;
    // lanes test 32 forests at a time; the warp fits the long ones among them
    for (int64_t base = warp_global * 32; base < count; base += nwarps * 32) {
        int64_t lane_f = -1;
        bool is_long = false;
        if (base + lane < count) {
            lane_f = index ? (int64_t)index[base + lane] : base + lane;
            is_long = sp.pix_offset[lane_f + 1] - sp.pix_offset[lane_f] > 32 * kContK;
        }
        unsigned todo = __ballot_sync(0xffffffffu, is_long);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int64_t f = __shfl_sync(0xffffffffu, lane_f, src);
            const int64_t off = sp.pix_offset[f];
            const int64_t n64 = sp.pix_offset[f + 1] - off;
            if (n64 <= 32 * kContK) continue;  // the register kernels' forests
            if (n64 > 32 * kLongK) {
                if (lane == 0) {
                    report_error(scratch, PG_ERR_UNSUPPORTED, (int32_t)f);
                    out.zero_point[f] = NAN;
                    out.slope[f] = NAN;
                    out.chi2[f] = NAN;
                    out.ndata[f] = 0;
                    out.status[f] = 1;
                    out.iterations[f] = 0;
                }
                continue;
            }
            const int n = (int)n64;
            const int nk = (n + 31) / 32;
            const double zp1 = log10(1 + sp.z_qso[f]);
            const double ll_min = m.log_lambda_rest_min + zp1;
            const double ll_max = m.log_lambda_rest_max + zp1;
            unsigned valid = 0;
            double sfi = 0., si = 0.;
            __syncwarp();
            for (int k = 0; k < nk; ++k) {
                const int p = lane + 32 * k;
                const int e = k * 32 + lane;
                double ja = 0, jb = 0, fl = 0, q = 0, vl = 0, fi = 0;
                if (p < n) {
                    const double ll = sp.log_lambda[off + p];
                    fl = sp.flux[off + p];
                    const double iv = sp.ivar[off + p];
                    sfi += fl * iv;
                    si += iv;
                    if (iv > 0) {
                        const ModelEval ev = eval_model(m, ll, zp1, sp.transmission_correction[off + p]);
                        const double x = (ll - ll_min) / (ll_max - ll_min);
                        ja = ev.mc;
                        jb = x * ev.mc;
                        q = const_w ? 1. : ev.eta / iv;
                        vl = const_w ? 0. : ev.var_lss;
                        fi = const_w ? 0. : ev.fudge * iv;
                        valid |= 1u << k;
                    }
                }
                slab[e] = ja; slab[S + e] = jb; slab[2 * S + e] = fl;
                slab[3 * S + e] = q; slab[4 * S + e] = vl; slab[5 * S + e] = fi;
            }
            __syncwarp();
            sfi = warp_sum(sfi);
            si = warp_sum(si);
            const double a0 = sfi / si;  // utils.py:92
            int nd = 0;
            for (int k = 0; k < nk; ++k) {
                if ((valid >> k) & 1u) {
                    const int e = k * 32 + lane;
                    const double c = a0 * slab[e];
                    const double d = slab[3 * S + e] + slab[4 * S + e] * c * c +
                                     slab[5 * S + e] * c * c * c * c;
                    nd += (d > 0.) ? 1 : 0;
                }
            }
    #pragma unroll
            for (int o = 16; o > 0; o >>= 1) nd += __shfl_xor_sync(0xffffffffu, nd, o);
            double a = a0, b = 0.;
            if (start) {
                a = start[2 * f];
                b = m.order == 0 ? 0. : start[2 * f + 1];
            }
            double s[6];
            long_terms(slab, valid, nk, a, b, const_w, s);
            int it = 0;
            bool converged = max_iter == 0 && start != nullptr;
            for (; it < max_iter; ++it) {
                double da, db;
                if (m.order == 0) {
                    da = s[3] > 0 ? -s[1] / s[3] : -s[1];
                    db = 0.;
                } else {
                    const double det = s[3] * s[5] - s[4] * s[4];
                    if (det > 0 && s[3] > 0) {
                        da = -(s[5] * s[1] - s[4] * s[2]) / det;
                        db = -(s[3] * s[2] - s[4] * s[1]) / det;
                    } else {
                        const double scale = fmax(fabs(s[3]), fabs(s[5]));
                        da = -s[1] / (scale > 0 ? scale : 1.);
                        db = -s[2] / (scale > 0 ? scale : 1.);
                    }
                    if (da * s[1] + db * s[2] >= 0) {  // not a descent direction
                        const double scale = fmax(fabs(s[3]), fabs(s[5]));
                        da = -s[1] / (scale > 0 ? scale : 1.);
                        db = -s[2] / (scale > 0 ? scale : 1.);
                    }
                }
                const double slope_dir = da * s[1] + db * s[2];
                double t = 1.;
                double trial[6];
                bool accepted = false;
                for (int ls = 0; ls < 40; ++ls) {
                    long_terms(slab, valid, nk, a + t * da, b + t * db, const_w, trial);
                    if (isfinite(trial[0]) && trial[0] <= s[0] + 1e-4 * t * slope_dir) {
                        accepted = true;
                        break;
                    }
                    t *= 0.5;
                }
                if (!accepted) {
                    converged = fabs(s[1]) + fabs(s[2]) < 1e-6 * fmax(1., fabs(s[0]));
                    break;
                }
                a += t * da;
                b += t * db;
    #pragma unroll
                for (int k = 0; k < 6; ++k) s[k] = trial[k];
                if (fabs(t * da) < tol * fmax(1., fmax(fabs(a), fabs(b))) &&
                    fabs(t * db) < tol * fmax(1., fmax(fabs(a), fabs(b)))) {
                    converged = true;
                    ++it;
                    break;
                }
            }
            double fin[6];
            long_terms(slab, valid, nk, a, b, const_w, fin);
            bool negative = false, all_zero = true;
            for (int p = lane; p < n; p += 32) {
                const double ll = sp.log_lambda[off + p];
                const double mc = interp_linear(m.mean_cont_x, m.mean_cont_y, m.num_mean_cont,
                                                ll - zp1) * sp.transmission_correction[off + p];
                const double line = b * (ll - ll_min) / (ll_max - ll_min) + a;
                const double c = line * mc;
                if (out.continuum) out.continuum[off + p] = c;
                negative |= c < 0;
                all_zero &= c == 0;
            }
            negative = __any_sync(0xffffffffu, negative);
            all_zero = __all_sync(0xffffffffu, all_zero);
            if (lane == 0) {
                int status = converged ? 0 : 1;
                if (negative) status = 2;
                if (all_zero) status = 3;
                out.zero_point[f] = status == 0 ? a : NAN;
                out.slope[f] = status == 0 ? b : NAN;
                out.chi2[f] = status == 0 ? fin[0] : NAN;
                out.ndata[f] = nd;
                out.status[f] = status;
                out.iterations[f] = it;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision fit (PG_FIT_MIXED): FP32 per-pixel terms, FP32 lane and
// warp sums, FP64 2x2 Newton solve. GB300 executes FP64 at 1/64 of the FP32
// rate, so the per-pixel work avoids FP64 except for the three differences
// whose operands are close (the rest-frame argument of the mean continuum,
// its offset from the interpolation node, and the offset from the forest's
// lower wavelength limit). The model tables are copied to shared memory in
// FP32 (plus the FP64 nodes of the mean continuum and per-interval slopes
// computed in FP64), so the interpolation searches use FP32 comparisons.
// Newton steps larger than 1e-3 of max(1, |a|, |b|) are damped by an Armijo
// line search on chi2; smaller steps, inside the region of quadratic
// convergence, are taken in full, because there the change of chi2 is below
// the resolution of FP32 sums. The iteration stops when the step is below
// max(tol, 1e-6) * max(1, |a|, |b|): the error left is about the square of
// the last step plus the FP32 rounding of the gradient (about 1e-8
// relative). The reported chi2 sums the FP32 terms with compensation; the
// continuum is (b x + a) mc in FP32, stored as FP64.
// ---------------------------------------------------------------------------
// One lane's pixels of the mixed fit, in the warp's shared-memory slab
// (slot k of lane l at k * 32 + l: conflict-free, and no lane reads another
// lane's entries). Unused and masked slots hold mc = 0, f = 0, q = 1,
// vl = fi = 0 and contribute exactly nothing.
struct FitSlab {
    float4 *a;  // mc, x, f, q
    float2 *b;  // vl, fi
};

constexpr size_t kFitSlabBytes = (size_t)kContK * 32 * (sizeof(float4) + sizeof(float2));

// chi2 (with want_val), gradient and Hessian in (a, b) of one lane's pixels,
// summed over the warp: s = {chi2, ga, gb, haa, hab, hbb}. The per-pixel
// algebra with h = dD/dC / 2, e = h / D:
//     dchi2/dC / 2   = e - r/D (1 + r h / D)
//     d2chi2/dC2 / 2 = 1/D + h' (1/D - (r/D)^2) + e (4 (r/D)(1 + r h/D) - 2 e)
// where h' = d2D/dC2 / 2 = vl + 6 fi C^2. Without want_val (the Newton
// iterations near the optimum) the reciprocal is the approximate one (two
// ulps) and chi2 itself is not formed.
__device__ __noinline__ void fit_terms(const FitSlab &px, int lane, int nk, float a, float b,
                                          bool const_w, bool want_val, float s[6]) {
    float val = 0.f, ga = 0.f, gb = 0.f, haa = 0.f, hab = 0.f, hbb = 0.f;
#pragma unroll 1
    for (int k = 0; k < nk; ++k) {
        const float4 pa = px.a[k * 32 + lane];
        const float2 pb = px.b[k * 32 + lane];
        const float c = pa.x * fmaf(b, pa.y, a);
        const float c2 = c * c;
        const float t1 = fmaf(pb.y, c2, pb.x);
        const float d = fmaf(t1, c2, pa.w);
        const float hd = c * fmaf(pb.y, c2, t1);                         // (dD/dC) / 2
        const float h2 = fmaf(4.f * pb.y, c2, fmaf(pb.y, c2, t1));       // vl + 6 fi C^2
        const float r = pa.z - c;
        const float id = want_val ? 1.f / d : __fdividef(1.f, d);
        const float rid = r * id;
        const float e = hd * id;
        const float w1 = fmaf(rid, hd, 1.f);
        const float g = fmaf(-rid, w1, e);
        const float hh = fmaf(h2, fmaf(-rid, rid, id), id) + e * fmaf(4.f * rid, w1, -2.f * e);
        const float gj = g * pa.x;
        ga += gj;
        gb = fmaf(gj, pa.y, gb);
        const float hj = hh * pa.x * pa.x;
        haa += hj;
        const float hjx = hj * pa.y;
        hab += hjx;
        hbb = fmaf(hjx, pa.y, hbb);
        if (want_val) val += fmaf(r, rid, const_w ? 0.f : logf(d));
    }
    // gradient and Hessian of chi2 (the factors 2 of the half-derivatives)
    s[0] = val;
    s[1] = 2.f * ga; s[2] = 2.f * gb;
    s[3] = 2.f * haa; s[4] = 2.f * hab; s[5] = 2.f * hbb;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int q = 0; q < 6; ++q) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    }
}

constexpr int kFitGroup = 8;  // forests per work item of the mixed fit

struct FitSlot {
    int64_t f, off;
    int n, nd, status, it, write;
    float lm_hi, lm_lo;     // Lmin = rest-frame start + log10(1 + z), two floats
    float ah, al, bh, bl;   // the start, then the result (two-float sums)
    float cs, ce;           // chi2 (compensated)
};

// Mixed-precision fit: FP32 per-pixel terms, (a, b) as two-float sums.
// Forests are handed out kFitGroup at a time from a work counter; the
// per-forest FP64 scalars (log10(1 + z), the start, the outputs) are
// computed by the group's lanes in parallel rather than by one lane per
// forest.
//
// cert_chi2 > 0 selects the certificate stop of the warm-started fit
// (pg_cont_fit_warm). Once a Newton step d = -H^-1 g is at most
// sqrt(cert_ab) * max(1, |a|, |b|) (Newton's convergence is quadratic, so the
// error after it is of order |d|^2), the step is taken and the iteration
// ends; the final pass, which evaluates chi2 at the new point anyway, also
// sums the gradient g' there and certifies the point: the remaining step
// H^-1 g' (with the last Hessian) at most cert_ab * max(1, |a|, |b|) and half
// the Newton decrement, g'.H^-1 g' / 2 (chi2's excess over the minimum of its
// quadratic model), at most cert_chi2 * max(|chi2|, ndata). There is no FP64
// finish; a forest not certified within max_iter iterations gets status 1
// (the caller re-fits it with the plain fit).
__global__ void __launch_bounds__(kContBlock, 4) cont_fit_mixed_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const double *__restrict__ start, const int32_t *__restrict__ index, int64_t count,
    int max_iter, double tol, const __grid_constant__ pg_cont_fit out, Scratch *scratch,
    float cert_chi2, float cert_ab) {
    extern __shared__ __align__(16) unsigned char smem[];
    const FitTables tab = load_fit_tables(m, smem + kFitSlabBytes * (kContBlock / 32));
    const int lane = threadIdx.x & 31;
    FitSlab px;
    px.a = reinterpret_cast<float4 *>(smem + kFitSlabBytes * (threadIdx.x >> 5));
    px.b = reinterpret_cast<float2 *>(px.a + kContK * 32);
    const bool const_w = m.use_constant_weight != 0;
    const float eff_tol = tol > 1e-6 ? (float)tol : 1e-6f;
    const bool evaluate_only = max_iter == 0 && start != nullptr;
    const bool certify = cert_chi2 > 0.f;
    const float inv_span = (float)(1.0 / (m.log_lambda_rest_max - m.log_lambda_rest_min));
    const int64_t num_groups = (count + kFitGroup - 1) / kFitGroup;
    // the group's per-forest scalars and results, in shared memory (not
    // registers) while the warp fits the forests one after the other
    __shared__ FitSlot s_slots[kContBlock / 32][kFitGroup];
    FitSlot *slots = s_slots[threadIdx.x >> 5];
    for (;;) {
        int64_t group = 0;
        if (lane == 0) group = atomicAdd(&scratch->work_counter, 1);
        group = __shfl_sync(0xffffffffu, group, 0);
        if (group >= num_groups) break;
        if (lane < kFitGroup) {
            FitSlot sl;
            sl.f = -1;
            sl.off = 0;
            sl.n = 0;
            sl.lm_hi = sl.lm_lo = sl.ah = sl.al = sl.bh = sl.bl = 0.f;
            sl.cs = NAN;
            sl.ce = 0.f;
            sl.nd = 0;
            sl.status = 1;
            sl.it = 0;
            sl.write = 0;
            if (group * kFitGroup + lane < count) {
                const int64_t w = group * kFitGroup + lane;
                sl.f = index ? (int64_t)index[w] : w;
                sl.off = sp.pix_offset[sl.f];
                sl.n = (int)(sp.pix_offset[sl.f + 1] - sl.off);
                const float2 lm = split_f64(m.log_lambda_rest_min + log10(1. + sp.z_qso[sl.f]));
                sl.lm_hi = lm.x;
                sl.lm_lo = lm.y;
                if (start) {
                    const float2 sa = split_f64(start[2 * sl.f]);
                    const float2 sb =
                        m.order == 0 ? make_float2(0.f, 0.f) : split_f64(start[2 * sl.f + 1]);
                    // renormalise (hi + lo) to a two-float sum
                    sl.ah = sa.x + sa.y;
                    sl.al = sa.y - (sl.ah - sa.x);
                    sl.bh = sb.x + sb.y;
                    sl.bl = sb.y - (sl.bh - sb.x);
                }
            }
            slots[lane] = sl;
        }
        __syncwarp();
        for (int j = 0; j < kFitGroup; ++j) {
            const int64_t f = slots[j].f;
            if (f < 0) break;
            const int64_t off = slots[j].off;
            const int n = slots[j].n;
            if (n > 32 * kContK) continue;  // a long forest: cont_fit_long_kernel
            if (lane == j) slots[j].write = 1;
            if (n <= 0) continue;           // empty: the defaults (status 1, NaN)
            const float lmh = slots[j].lm_hi;
            const float lml = slots[j].lm_lo;
            const int nk = (n + 31) >> 5;
            if (j + 1 < kFitGroup && slots[j + 1].f >= 0) {
                // the group's next forest into L2 while this one is fitted
                const int64_t noff = slots[j + 1].off;
                const int nn = slots[j + 1].n < 32 * kContK ? slots[j + 1].n : 32 * kContK;
                for (int p = lane; p < nn; p += 32) {
                    prefetch_l2(sp.log_lambda + noff + p);
                    prefetch_l2(sp.flux + noff + p);
                    prefetch_l2(sp.ivar + noff + p);
                    prefetch_l2(sp.transmission_correction + noff + p);
                }
            }
            unsigned valid = 0;
            float sfi = 0.f, si = 0.f;
#pragma unroll 2
            for (int k = 0; k < nk; ++k) {
                float4 pa = make_float4(0.f, 0.f, 0.f, 1.f);
                float2 pb = make_float2(0.f, 0.f);
                const int p = lane + 32 * k;
                if (p < n) {
                    const float iv = f64_to_f32(sp.ivar[off + p]);
                    const float fl = f64_to_f32(sp.flux[off + p]);
                    sfi = fmaf(fl, iv, sfi);
                    si += iv;
                    if (iv > 0.f) {
                        const float2 ll = split_f64(sp.log_lambda[off + p]);
                        const float u = (ll.x - lmh) + (ll.y - lml);  // L - Lmin
                        pa.y = u * inv_span;
                        pa.x = fit_mean_cont(tab, u) * f64_to_f32(sp.transmission_correction[off + p]);
                        pa.z = fl;
                        if (!const_w) {
                            float eta, var_lss, fudge;
                            fit_var_funcs(tab, ll.x + ll.y, eta, var_lss, fudge);
                            pa.w = __fdividef(eta, fmaxf(iv, 1.17549435e-38f));
                            pb.x = var_lss;
                            pb.y = fudge * iv;
                        }
                        valid |= 1u << k;
                    }
                }
                px.a[k * 32 + lane] = pa;
                px.b[k * 32 + lane] = pb;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sfi += __shfl_xor_sync(0xffffffffu, sfi, o);
                si += __shfl_xor_sync(0xffffffffu, si, o);
            }
            // starting point (utils.py:92): FP32 sums, only a start
            const float a0f = sfi / si;
            int nd = 0;
#pragma unroll 1
            for (int k = 0; k < nk; ++k) {
                if ((valid >> k) & 1u) {
                    const float4 pa = px.a[k * 32 + lane];
                    const float2 pb = px.b[k * 32 + lane];
                    const float c = a0f * pa.x;
                    const float c2 = c * c;
                    nd += fmaf(fmaf(pb.y, c2, pb.x), c2, pa.w) > 0.f ? 1 : 0;
                }
            }
            nd = __reduce_add_sync(0xffffffffu, nd);
            float ah = a0f, al = 0.f, bh = 0.f, bl = 0.f;
            if (start) {
                ah = slots[j].ah;
                al = slots[j].al;
                bh = slots[j].bh;
                bl = slots[j].bl;
            }
            float s[6];
            bool have_val = false;
            fit_terms(px, lane, nk, ah, bh, const_w, !evaluate_only, s);
            have_val = !evaluate_only;
            int it = 0;
            bool converged = evaluate_only;
            for (; it < max_iter; ++it) {
                // Newton step from the exact-product 2x2 solve
                float da, db;
                bool newton = true;  // d = -H^-1 g (not the gradient fallback)
                if (m.order == 0) {
                    newton = s[3] > 0.f;
                    da = newton ? -s[1] / s[3] : -s[1];
                    db = 0.f;
                } else {
                    const float det = diff_prod(s[3], s[5], s[4], s[4]);
                    da = db = 0.f;
                    if (det > 0.f && s[3] > 0.f) {
                        da = -diff_prod(s[5], s[1], s[4], s[2]) / det;
                        db = -diff_prod(s[3], s[2], s[4], s[1]) / det;
                    }
                    if ((da == 0.f && db == 0.f) || da * s[1] + db * s[2] >= 0.f) {
                        // singular Hessian or not a descent direction: gradient step
                        const float scale = fmaxf(fabsf(s[3]), fabsf(s[5]));
                        da = -s[1] / (scale > 0.f ? scale : 1.f);
                        db = -s[2] / (scale > 0.f ? scale : 1.f);
                        newton = false;
                    }
                }
                const float ref = fmaxf(1.f, fmaxf(fabsf(ah), fabsf(bh)));
                float t = 1.f;
                // a Newton step small enough that the point after it is within
                // cert_ab: take it; the final pass certifies the new point
                if (certify && newton && fabsf(da) <= sqrtf(cert_ab) * ref &&
                    fabsf(db) <= sqrtf(cert_ab) * ref) {
                    float hi = ah + da, bb = hi - ah;
                    al += (ah - (hi - bb)) + (da - bb);
                    ah = hi;
                    hi = bh + db;
                    bb = hi - bh;
                    bl += (bh - (hi - bb)) + (db - bb);
                    bh = hi;
                    converged = true;
                    ++it;
                    break;
                }
                float trial[6];
                if (fabsf(da) < 1e-3f * ref && fabsf(db) < 1e-3f * ref) {
                    fit_terms(px, lane, nk, ah + da, bh + db, const_w, false, trial);
                    have_val = false;
                } else {
                    if (!have_val) fit_terms(px, lane, nk, ah, bh, const_w, true, s);
                    const float slope_dir = da * s[1] + db * s[2];
                    bool accepted = false;
                    for (int ls = 0; ls < 40; ++ls) {
                        fit_terms(px, lane, nk, ah + t * da, bh + t * db, const_w, true, trial);
                        if (isfinite(trial[0]) && trial[0] <= s[0] + 1e-4f * t * slope_dir) {
                            accepted = true;
                            break;
                        }
                        t *= 0.5f;
                    }
                    if (!accepted) break;
                    have_val = true;
                }
                {
                    // (ah, al) += t da exactly to FP32-pair precision (TwoSum)
                    const float sa = t * da, sb = t * db;
                    float hi = ah + sa, bb = hi - ah;
                    al += (ah - (hi - bb)) + (sa - bb);
                    ah = hi;
                    hi = bh + sb;
                    bb = hi - bh;
                    bl += (bh - (hi - bb)) + (sb - bb);
                    bh = hi;
                }
#pragma unroll
                for (int k = 0; k < 6; ++k) s[k] = trial[k];
                const float ref2 = fmaxf(1.f, fmaxf(fabsf(ah), fabsf(bh)));
                if (!certify && fabsf(t * da) < eff_tol * ref2 && fabsf(t * db) < eff_tol * ref2) {
                    converged = true;
                    ++it;
                    break;
                }
            }
            // chi2 at the solution (compensated FP32 sums, lanes and warp),
            // the scale of the gradient's FP32 rounding (the per-pixel
            // roundings are independent, so it grows as the root of the sum
            // of squares of the per-pixel gradient terms), the gradient for
            // the certificate, and the continuum
            float cs = 0.f, ce = 0.f, ga_abs = 0.f, gb_abs = 0.f, ga_s = 0.f, gb_s = 0.f;
            bool negative = false, all_zero = true;
            const float af = ah, bf = bh;
#pragma unroll 1
            for (int k = 0; k < nk; ++k) {
                const int p = lane + 32 * k;
                if (p >= n) continue;
                float cont;
                if ((valid >> k) & 1u) {
                    const float4 pa = px.a[k * 32 + lane];
                    const float2 pb = px.b[k * 32 + lane];
                    const float c = pa.x * fmaf(bf, pa.y, af);
                    cont = c;
                    const float c2 = c * c;
                    const float t1 = fmaf(pb.y, c2, pb.x);
                    const float d = fmaf(t1, c2, pa.w);
                    const float r = pa.z - c;
                    const float id = 1.f / d;
                    const float rid = r * id;
                    const float dd = 2.f * c * fmaf(pb.y, c2, t1);
                    const float g = fabsf(2.f * rid) + rid * rid * fabsf(dd) + fabsf(dd * id);
                    const float jb = pa.y * pa.x;
                    ga_abs += (g * pa.x) * (g * pa.x);
                    gb_abs += (g * jb) * (g * jb);
                    if (certify) {
                        const float gs = fmaf(-rid, fmaf(rid, dd, 2.f), dd * id);
                        ga_s = fmaf(gs, pa.x, ga_s);
                        gb_s = fmaf(gs, jb, gb_s);
                    }
                    const float term = fmaf(r, rid, const_w ? 0.f : logf(d));
                    const float ns = cs + term;
                    const float bb = ns - cs;
                    ce += (cs - (ns - bb)) + (term - bb);
                    cs = ns;
                } else {
                    // masked pixel: the continuum only
                    const float2 ll = split_f64(sp.log_lambda[off + p]);
                    const float u = (ll.x - lmh) + (ll.y - lml);
                    const float mc = fit_mean_cont(tab, u) *
                                     f64_to_f32(sp.transmission_correction[off + p]);
                    cont = mc * fmaf(bf, u * inv_span, af);
                }
                if (out.continuum) out.continuum[off + p] = f32_to_f64(cont);
                negative |= cont < 0.f;
                all_zero &= cont == 0.f;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float os = __shfl_xor_sync(0xffffffffu, cs, o);
                const float oe = __shfl_xor_sync(0xffffffffu, ce, o);
                const float ns = cs + os;
                const float bb = ns - cs;
                ce += oe + ((cs - (ns - bb)) + (os - bb));
                cs = ns;
                ga_abs += __shfl_xor_sync(0xffffffffu, ga_abs, o);
                gb_abs += __shfl_xor_sync(0xffffffffu, gb_abs, o);
                if (certify) {
                    ga_s += __shfl_xor_sync(0xffffffffu, ga_s, o);
                    gb_s += __shfl_xor_sync(0xffffffffu, gb_s, o);
                }
            }
            negative = __any_sync(0xffffffffu, negative);
            all_zero = __all_sync(0xffffffffu, all_zero);
            const float ref = fmaxf(1.f, fmaxf(fabsf(ah), fabsf(bh)));
            if (certify) {
                // certificate at the accepted point, with the last Hessian
                bool cert = false;
                if (converged) {
                    float ra = 0.f, rb = 0.f;
                    bool ok_h;
                    if (m.order == 0) {
                        ok_h = s[3] > 0.f;
                        ra = ok_h ? -ga_s / s[3] : 0.f;
                    } else {
                        const float det = diff_prod(s[3], s[5], s[4], s[4]);
                        ok_h = det > 0.f && s[3] > 0.f;
                        if (ok_h) {
                            ra = -diff_prod(s[5], ga_s, s[4], gb_s) / det;
                            rb = -diff_prod(s[3], gb_s, s[4], ga_s) / det;
                        }
                    }
                    const float half_dec = -0.5f * (ra * ga_s + rb * gb_s);
                    cert = ok_h && fabsf(ra) <= cert_ab * ref && fabsf(rb) <= cert_ab * ref &&
                           half_dec <= cert_chi2 * fmaxf(fabsf(cs + ce), (float)nd);
                }
                converged = cert;
            }
            // estimate of the optimum's shift by that rounding, |H^-1| (8 u
            // rms(g)): large when the data barely separate a from b (a forest
            // covering a short stretch of the rest-frame window)
            bool refine = false;
            if (converged && !evaluate_only && !certify) {
                const float ua = 8.f * 5.96e-8f * sqrtf(ga_abs);
                const float ub = 8.f * 5.96e-8f * sqrtf(gb_abs);
                float ea, eb;
                if (m.order == 0) {
                    ea = s[3] > 0.f ? ua / s[3] : INFINITY;
                    eb = 0.f;
                } else {
                    const float det = diff_prod(s[3], s[5], s[4], s[4]);
                    ea = det > 0.f ? (fabsf(s[5]) * ua + fabsf(s[4]) * ub) / det : INFINITY;
                    eb = det > 0.f ? (fabsf(s[4]) * ua + fabsf(s[3]) * ub) / det : INFINITY;
                }
                refine = !(ea <= 2e-6f * ref && eb <= 2e-6f * ref);
            }
            if (lane == j) {
                int status = converged ? (refine ? 4 : 0) : 1;
                if (negative) status = 2;
                if (all_zero) status = 3;
                FitSlot &sl = slots[j];
                sl.status = status;
                sl.ah = ah; sl.al = al; sl.bh = bh; sl.bl = bl; sl.cs = cs; sl.ce = ce;
                sl.nd = nd;
                sl.it = it;
            }
        }
        __syncwarp();
        if (lane < kFitGroup && slots[lane].write) {
            const FitSlot sl = slots[lane];
            const bool keep = sl.status == 0 || sl.status == 4;
            out.zero_point[sl.f] = keep ? f32_to_f64(sl.ah) + f32_to_f64(sl.al) : NAN;
            out.slope[sl.f] = keep ? f32_to_f64(sl.bh) + f32_to_f64(sl.bl) : NAN;
            out.chi2[sl.f] = keep ? f32_to_f64(sl.cs) + f32_to_f64(sl.ce) : NAN;
            out.ndata[sl.f] = sl.nd;
            out.status[sl.f] = sl.status;
            out.iterations[sl.f] = sl.it;
        }
        __syncwarp();
    }
}

// forest weights of Dr16ExpectedFlux.compute_forest_weights
// (dr16_expected_flux.py:466-488)
__device__ __forceinline__ double forest_weight(const pg_cont_model &m, double ll, double iv,
                                                double cont) {
    if (!(iv > 0)) return 0.;
    const double var_pipe = 1. / iv / (cont * cont);
    double eta = 0., vlss = 1., fudge = 0.;
    if (!m.use_constant_weight) {
        eta = eval_ppoly(m.var_breaks, m.eta_coef, m.num_var_intervals, ll);
        vlss = eval_ppoly(m.var_breaks, m.var_lss_coef, m.num_var_intervals, ll);
        fudge = eval_ppoly(m.var_breaks, m.fudge_coef, m.num_var_intervals, ll);
    }
    return 1.0 / (eta * var_pipe + m.var_lss_mod * vlss + fudge / var_pipe);
}

// find_bins_log / find_bins_lin (delta_extraction/utils.py:139-186): the
// nearest node of an evenly spaced grid in log10(lambda) (grid0, step in
// log10 Angstrom) or in lambda (grid0, step in Angstrom; the value's lambda is
// 10**x). The int conversion truncates toward zero, as astype(int64) does.
__device__ __forceinline__ int64_t find_bin(double x, double grid0, double step, int lin) {
    if (lin) return (int64_t)((pow(10.0, x) - grid0) / step + 0.5);
    return (int64_t)((x - grid0) / step + 0.5);
}

// eta, var_lss and fudge at v in FP64 from the model's coefficient arrays:
// one search (searchsorted right, the end pieces extrapolated) and the three
// cubics as eval_ppoly evaluates them.
__device__ void var_funcs_f64(const pg_cont_model &m, double v, double &eta, double &vlss,
                              double &fudge) {
    const int mi = m.num_var_intervals;
    int lo = 0, hi = mi + 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (m.var_breaks[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    int i = lo - 1;
    i = i < 0 ? 0 : (i > mi - 1 ? mi - 1 : i);
    const double dx = v - m.var_breaks[i];
    const double *c = m.eta_coef;
    eta = ((c[i] * dx + c[mi + i]) * dx + c[2 * mi + i]) * dx + c[3 * mi + i];
    c = m.var_lss_coef;
    vlss = ((c[i] * dx + c[mi + i]) * dx + c[2 * mi + i]) * dx + c[3 * mi + i];
    c = m.fudge_coef;
    fudge = ((c[i] * dx + c[mi + i]) * dx + c[2 * mi + i]) * dx + c[3 * mi + i];
}

// ---- two-float (double-float) arithmetic -----------------------------------
// Values as unevaluated sums hi + lo of two floats (about 48 significant
// bits): the FP32 pipe stands in for the narrow FP64 pipe where FP32 alone
// would lose the reference's FP64 accuracy.
struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl dfl_fast(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ dfl dfl_of(double v) {
    const float2 p = split_f64(v);
    return dfl_fast(p.x, p.y);
}

__device__ __forceinline__ dfl dfl_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dfl dfl_add(dfl x, dfl y) {
    dfl s = dfl_two_sum(x.hi, y.hi);
    const dfl t = dfl_two_sum(x.lo, y.lo);
    s.lo += t.hi;
    s = dfl_fast(s.hi, s.lo);
    s.lo += t.lo;
    return dfl_fast(s.hi, s.lo);
}

__device__ __forceinline__ dfl dfl_mul(dfl x, dfl y) {
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return dfl_fast(p, e);
}

// x / y: a quotient estimate corrected once with the exact residual
__device__ __forceinline__ dfl dfl_div(dfl x, dfl y) {
    const float q1 = __fdividef(x.hi, y.hi);
    const float p = q1 * y.hi;
    const float pe = fmaf(q1, y.hi, -p);
    // r = x - q1 y, from the exact product p + pe (+ q1 y.lo)
    const dfl r = dfl_add(x, dfl{-p, -fmaf(q1, y.lo, pe)});
    const float q2 = __fdividef(r.hi, y.hi);
    return dfl_fast(q1, q2);
}

__device__ __forceinline__ double dfl_to_f64(dfl x) { return f32_to_f64(x.hi) + f32_to_f64(x.lo); }

// hi/lo histogram bin += x: FP32 atomic adds whose rounding error is
// recovered exactly from the value each one replaced (TwoSum against the
// returned old value) and added to the low word with the low part of x
__device__ __forceinline__ void hist_add(float *hi, float *lo, int bin, dfl x) {
    const float old = atomicAdd(&hi[bin], x.hi);
    const float s = old + x.hi;
    const float bb = s - old;
    const float err = (old - (s - bb)) + (x.hi - bb);
    atomicAdd(&lo[bin], err + x.lo);
}

// trunc(t) of a bin coordinate t evaluated in FP32 with absolute error
// below guard: certain when t is farther than guard from an integer
__device__ __forceinline__ bool bin_certain(float t, float guard, int &bin) {
    const float a = fabsf(t);
    const float fr = a - truncf(a);
    bin = __float2int_rz(t);  // toward zero, as astype(int64)
    return a < 1.0e6f && fr > guard && fr < 1.f - guard;
}

// ---- two-float finish of the mixed fit ------------------------------------
// The forests the mixed fit flagged (status 4: FP32 rounding could move their
// optimum by more than 2e-6 of max(1, |a|, |b|), a short stretch of the
// rest-frame window barely separating a from b) are finished here, in the
// same call, to FP64 accuracy without the FP64 pipe: every per-pixel input
// (x, the mean continuum, the variance functions) is formed in two-float
// arithmetic from the FP64 model, the gradient of chi2 is summed in
// two-float, and Newton steps from the mixed solution (the Hessian in FP32
// is enough for a correction step) run until the step is below 1e-11 of
// max(1, |a|, |b|). chi2 is re-evaluated with the logarithm in FP32 plus its
// first-order two-float correction.
constexpr int kRefineWarps = 4;
constexpr size_t kRefineSlabBytes = (size_t)kContK * 32 * 3 * sizeof(float4);

__host__ __device__ inline size_t refine_smem_bytes(int nmc, int m) {
    return (size_t)kRefineWarps * kRefineSlabBytes + (size_t)3 * nmc * 8 + (size_t)(m + 1) * 8 +
           (size_t)12 * m * 8 + 16;
}

// sign of x - y (two-float values)
__device__ __forceinline__ bool dfl_less(dfl x, dfl y) {
    return (x.hi - y.hi) + (x.lo - y.lo) < 0.f;
}

__device__ __forceinline__ dfl dfl_neg(dfl x) { return {-x.hi, -x.lo}; }

__device__ __forceinline__ dfl warp_sum_dfl(dfl v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const dfl w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = dfl_add(v, w);
    }
    return v;
}

__global__ void __launch_bounds__(32 * kRefineWarps) cont_fit_refine_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const int32_t *__restrict__ index, int64_t count, const __grid_constant__ pg_cont_fit out,
    Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int nmc = m.num_mean_cont;
    const int mi = m.use_constant_weight ? 0 : m.num_var_intervals;
    const bool const_w = mi == 0;
    float4 *slab = reinterpret_cast<float4 *>(smem + kRefineSlabBytes * (threadIdx.x >> 5));
    dfl *node = reinterpret_cast<dfl *>(smem + kRefineSlabBytes * kRefineWarps);  // off, y, slope
    dfl *brk = node + 3 * nmc;
    dfl *coef = brk + (mi + 1);  // [i][12]: eta, var_lss, fudge (c3 c2 c1 c0)
    const double rest_min = m.log_lambda_rest_min;
    for (int i = threadIdx.x; i < nmc; i += blockDim.x) {
        const double x = m.mean_cont_x[i], y = m.mean_cont_y[i];
        node[3 * i] = dfl_of(x - rest_min);
        node[3 * i + 1] = dfl_of(y);
        node[3 * i + 2] = dfl_of(i + 1 < nmc ? (m.mean_cont_y[i + 1] - y) / (m.mean_cont_x[i + 1] - x)
                                             : 0.);
    }
    for (int i = threadIdx.x; i <= mi; i += blockDim.x) brk[i] = dfl_of(m.var_breaks[i]);
    for (int i = threadIdx.x; i < mi; i += blockDim.x) {
        for (int k = 0; k < 4; ++k) {
            coef[12 * i + k] = dfl_of(m.eta_coef[k * mi + i]);
            coef[12 * i + 4 + k] = dfl_of(m.var_lss_coef[k * mi + i]);
            coef[12 * i + 8 + k] = dfl_of(m.fudge_coef[k * mi + i]);
        }
    }
    __syncthreads();
    const dfl inv_span = dfl_of(1.0 / (m.log_lambda_rest_max - m.log_lambda_rest_min));
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp_global * 32; base < count; base += nwarps * 32) {
        int64_t lane_f = -1;
        bool flagged = false;
        double lane_lmin = 0.;
        if (base + lane < count) {
            lane_f = index ? (int64_t)index[base + lane] : base + lane;
            flagged = out.status[lane_f] == 4;
            if (flagged) lane_lmin = rest_min + log10(1. + sp.z_qso[lane_f]);
        }
        unsigned todo = __ballot_sync(0xffffffffu, flagged);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const int64_t f = __shfl_sync(0xffffffffu, lane_f, src);
            const dfl lmin = dfl_of(__shfl_sync(0xffffffffu, lane_lmin, src));
            const int64_t off = sp.pix_offset[f];
            const int n = (int)(sp.pix_offset[f + 1] - off);
            const int nk = (n + 31) >> 5;
            // two-float pixel terms: slab[3 (k 32 + lane) + {0, 1, 2}] =
            // (mc, x), (f, q), (vl, fi), each as hi, lo
            unsigned valid = 0;
            for (int k = 0; k < nk; ++k) {
                const int p = lane + 32 * k;
                dfl mc = {0.f, 0.f}, x = {0.f, 0.f}, fl = {0.f, 0.f}, q = {1.f, 0.f};
                dfl vl = {0.f, 0.f}, fi = {0.f, 0.f};
                if (p < n) {
                    const dfl L = dfl_of(sp.log_lambda[off + p]);
                    const dfl u = dfl_add(L, dfl_neg(lmin));  // L - Lmin
                    x = dfl_mul(u, inv_span);
                    int lo = 0, hi = nmc;
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (dfl_less(node[3 * mid], u)) lo = mid + 1;
                        else hi = mid;
                    }
                    const int i = lo < 1 ? 0 : (lo > nmc - 1 ? nmc - 2 : lo - 1);
                    mc = dfl_add(node[3 * i + 1],
                                 dfl_mul(node[3 * i + 2], dfl_add(u, dfl_neg(node[3 * i]))));
                    mc = dfl_mul(mc, dfl_of(sp.transmission_correction[off + p]));
                    const dfl iv = dfl_of(sp.ivar[off + p]);
                    if (iv.hi > 0.f) {
                        fl = dfl_of(sp.flux[off + p]);
                        if (!const_w) {
                            int a = 0, b = mi + 1;
                            while (a < b) {
                                const int mid = (a + b) >> 1;
                                if (!dfl_less(L, brk[mid])) a = mid + 1;
                                else b = mid;
                            }
                            int j = a - 1;
                            j = j < 0 ? 0 : (j > mi - 1 ? mi - 1 : j);
                            const dfl dx = dfl_add(L, dfl_neg(brk[j]));
                            dfl v3[3];
#pragma unroll
                            for (int g = 0; g < 3; ++g) {
                                const dfl *c = coef + 12 * j + 4 * g;
                                dfl acc = c[0];
                                acc = dfl_add(dfl_mul(acc, dx), c[1]);
                                acc = dfl_add(dfl_mul(acc, dx), c[2]);
                                v3[g] = dfl_add(dfl_mul(acc, dx), c[3]);
                            }
                            q = dfl_div(v3[0], iv);
                            vl = v3[1];
                            fi = dfl_mul(v3[2], iv);
                        }
                        valid |= 1u << k;
                    }
                }
                float4 *e = slab + 3 * (k * 32 + lane);
                e[0] = make_float4(mc.hi, mc.lo, x.hi, x.lo);
                e[1] = make_float4(fl.hi, fl.lo, q.hi, q.lo);
                e[2] = make_float4(vl.hi, vl.lo, fi.hi, fi.lo);
            }
            dfl a = dfl_of(out.zero_point[f]);
            dfl b = m.order == 0 ? dfl{0.f, 0.f} : dfl_of(out.slope[f]);
            int it = 0;
            bool converged = false;
            float h3 = 0.f, h4 = 0.f, h5 = 0.f;
            for (; it < 10; ++it) {
                // gradient (two-float) and Hessian (FP32) at (a, b)
                dfl ga = {0.f, 0.f}, gb = {0.f, 0.f};
                float haa = 0.f, hab = 0.f, hbb = 0.f;
                for (int k = 0; k < nk; ++k) {
                    if (!((valid >> k) & 1u)) continue;
                    const float4 *e = slab + 3 * (k * 32 + lane);
                    const float4 e0 = e[0], e1 = e[1], e2 = e[2];
                    const dfl mc = {e0.x, e0.y}, x = {e0.z, e0.w}, fl = {e1.x, e1.y};
                    const dfl q = {e1.z, e1.w}, vl = {e2.x, e2.y}, fi = {e2.z, e2.w};
                    const dfl c = dfl_mul(mc, dfl_add(a, dfl_mul(b, x)));
                    const dfl c2 = dfl_mul(c, c);
                    const dfl fc2 = dfl_mul(fi, c2);
                    const dfl t1 = dfl_add(vl, fc2);
                    const dfl d = dfl_add(q, dfl_mul(t1, c2));
                    const dfl hd = dfl_mul(c, dfl_add(t1, fc2));
                    const dfl r = dfl_add(fl, dfl_neg(c));
                    const dfl id = dfl_div(dfl{1.f, 0.f}, d);
                    const dfl rid = dfl_mul(r, id);
                    const dfl e_ = dfl_mul(hd, id);
                    const dfl w1 = dfl_add(dfl{1.f, 0.f}, dfl_mul(rid, hd));
                    const dfl g = dfl_add(e_, dfl_neg(dfl_mul(rid, w1)));
                    const dfl gj = dfl_mul(g, mc);
                    ga = dfl_add(ga, gj);
                    gb = dfl_add(gb, dfl_mul(gj, x));
                    // Hessian from the leading parts
                    const float h2 = fmaf(5.f * fi.hi, c2.hi, t1.hi);
                    const float hh = fmaf(h2, fmaf(-rid.hi, rid.hi, id.hi), id.hi) +
                                     e_.hi * fmaf(4.f * rid.hi, w1.hi, -2.f * e_.hi);
                    const float hj = hh * mc.hi * mc.hi;
                    haa += hj;
                    hab = fmaf(hj, x.hi, hab);
                    hbb = fmaf(hj * x.hi, x.hi, hbb);
                }
                ga = warp_sum_dfl(ga);
                gb = warp_sum_dfl(gb);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    haa += __shfl_xor_sync(0xffffffffu, haa, o);
                    hab += __shfl_xor_sync(0xffffffffu, hab, o);
                    hbb += __shfl_xor_sync(0xffffffffu, hbb, o);
                }
                // half-derivatives: the factors 2 cancel in the Newton step
                h3 = 2.f * haa;
                h4 = 2.f * hab;
                h5 = 2.f * hbb;
                const float g1 = 2.f * (ga.hi + ga.lo), g2 = 2.f * (gb.hi + gb.lo);
                float da, db;
                if (m.order == 0) {
                    if (!(h3 > 0.f)) break;
                    da = -g1 / h3;
                    db = 0.f;
                } else {
                    const float det = diff_prod(h3, h5, h4, h4);
                    if (!(det > 0.f && h3 > 0.f)) break;
                    da = -diff_prod(h5, g1, h4, g2) / det;
                    db = -diff_prod(h3, g2, h4, g1) / det;
                }
                if (!isfinite(da) || !isfinite(db)) break;
                a = dfl_add(a, dfl{da, 0.f});
                b = dfl_add(b, dfl{db, 0.f});
                const float ref = fmaxf(1.f, fmaxf(fabsf(a.hi), fabsf(b.hi)));
                if (fabsf(da) <= 1e-11f * ref && fabsf(db) <= 1e-11f * ref) {
                    converged = true;
                    ++it;
                    break;
                }
            }
            // chi2 and the continuum at the solution
            dfl chi = {0.f, 0.f};
            bool negative = false, all_zero = true;
            for (int k = 0; k < nk; ++k) {
                const int p = lane + 32 * k;
                if (p >= n) continue;
                const float4 *e = slab + 3 * (k * 32 + lane);
                const float4 e0 = e[0];
                const dfl mc = {e0.x, e0.y}, x = {e0.z, e0.w};
                const dfl c = dfl_mul(mc, dfl_add(a, dfl_mul(b, x)));
                if ((valid >> k) & 1u) {
                    const float4 e1 = e[1], e2 = e[2];
                    const dfl fl = {e1.x, e1.y}, q = {e1.z, e1.w};
                    const dfl vl = {e2.x, e2.y}, fi = {e2.z, e2.w};
                    const dfl c2 = dfl_mul(c, c);
                    const dfl d = dfl_add(q, dfl_mul(dfl_add(vl, dfl_mul(fi, c2)), c2));
                    const dfl r = dfl_add(fl, dfl_neg(c));
                    const dfl term = dfl_div(dfl_mul(r, r), d);
                    chi = dfl_add(chi, term);
                    if (!const_w) chi = dfl_add(chi, dfl_fast(logf(d.hi), d.lo / d.hi));
                }
                if (out.continuum) out.continuum[off + p] = dfl_to_f64(c);
                negative |= c.hi < 0.f;
                all_zero &= c.hi == 0.f;
            }
            chi = warp_sum_dfl(chi);
            negative = __any_sync(0xffffffffu, negative);
            all_zero = __all_sync(0xffffffffu, all_zero);
            if (lane == 0) {
                int status = converged ? 0 : 1;
                if (negative) status = 2;
                if (all_zero) status = 3;
                const bool keep = status == 0;
                out.zero_point[f] = keep ? dfl_to_f64(a) : NAN;
                out.slope[f] = keep ? dfl_to_f64(b) : NAN;
                out.chi2[f] = keep ? dfl_to_f64(chi) : NAN;
                out.status[f] = status;
                out.iterations[f] += it;
                atomicAdd(&scratch->work_items, 1ull);
            }
        }
    }
}

// Histograms of one Dr16 iteration. Persistent blocks (one warp per forest,
// pixels across lanes, forests drawn kStackGroup at a time from the work
// counter) accumulate the rest-frame mean continuum, the observed-frame stack
// and the variance statistics in shared memory and add them to the global
// FP64 sums once at the end: 400k forests add to a few thousand bins.
//
// GB300's FP64 pipe is 1/64 of its FP32 pipe, so the per-pixel arithmetic is
// two-float: the FP64 inputs are split on the integer pipe, the weights,
// flux ratios and delta moments are formed with FP32 error-free
// transformations (relative error about 1e-13, against the 1e-16 of the
// reference's FP64), and the histograms are hi/lo pairs of FP32 words. Bin
// indices are evaluated in FP32 and used where they are certain (farther
// than a guard from a bin edge); the few pixels within the guard take the
// reference's FP64 formula. The variance functions are tabulated (FP64,
// stored as two floats) on the observed-frame grid and read for pixels on a
// grid node (all of them for forests rebinned to the grid); others evaluate
// them in FP64.
constexpr int kStackBlock = 512;
constexpr int kStackGroup = 8;

struct StackSlot {
    int64_t off;
    int n, skip;
    double zp1;
    float zr_hi, zr_lo;  // log10(1 + z) + rest grid start (log grid) or log10(1 + z) (linear)
};

__host__ __device__ inline size_t stack_smem_bytes(const pg_cont_stacks &st, bool table) {
    const size_t nvar = (size_t)st.var_lambda_bins * kVarBins;
    return (size_t)8 * (2 * st.rest_bins + 2 * st.obs_bins + 3 * nvar) + (size_t)8 * nvar +
           (table ? (size_t)32 * st.obs_bins : 0) + 64;
}

__global__ void __launch_bounds__(kStackBlock) cont_stacks_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const __grid_constant__ pg_cont_fit fit, const __grid_constant__ pg_cont_stacks st,
    Scratch *scratch, int use_table) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t seen[kStackBlock / 32][64];  // per-warp bitmap of var bins (<= 2048)
    __shared__ StackSlot s_slots[kStackBlock / 32][kStackGroup];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int nvar = st.var_lambda_bins * kVarBins;
    const int mi = m.use_constant_weight ? 0 : m.num_var_intervals;
    const int R = st.rest_bins, O = st.obs_bins;
    // layout: table (float4 x 2 per obs bin), then hi/lo FP32 histograms, then counts
    float4 *table = reinterpret_cast<float4 *>(smem_raw);
    float *hist = reinterpret_cast<float *>(smem_raw + (use_table ? (size_t)32 * O : 0));
    float *mc_num_h = hist, *mc_num_l = mc_num_h + R, *mc_w_h = mc_num_l + R, *mc_w_l = mc_w_h + R;
    float *s_num_h = mc_w_l + R, *s_num_l = s_num_h + O, *s_w_h = s_num_l + O, *s_w_l = s_w_h + O;
    float *v_mean_h = s_w_l + O, *v_mean_l = v_mean_h + nvar;
    float *v_d2_h = v_mean_l + nvar, *v_d2_l = v_d2_h + nvar;
    float *v_d4_h = v_d2_l + nvar, *v_d4_l = v_d4_h + nvar;
    uint32_t *v_np = reinterpret_cast<uint32_t *>(v_d4_l + nvar), *v_nq = v_np + nvar;
    const int nwords = 4 * R + 4 * O + 8 * nvar;
    for (int k = threadIdx.x; k < nwords; k += blockDim.x) hist[k] = 0.f;
    if (use_table) {
        // variance functions on the observed-frame grid nodes
        for (int j = threadIdx.x; j < O; j += blockDim.x) {
            const double g = st.obs_grid0 + j * st.obs_step;
            const double node = st.wave_lin ? log10(g) : g;
            double eta, vlss, fudge;
            var_funcs_f64(m, node, eta, vlss, fudge);
            const dfl n = dfl_of(node), e = dfl_of(eta), v = dfl_of(vlss), f = dfl_of(fudge);
            table[2 * j] = make_float4(n.hi, n.lo, e.hi, e.lo);
            table[2 * j + 1] = make_float4(v.hi, v.lo, f.hi, f.lo);
        }
    }
    __syncthreads();
    const bool do_mc = st.mean_cont_num != nullptr;
    const bool do_stack = st.stack_num != nullptr;
    const bool do_var = st.var_mean != nullptr && nvar <= 2048;
    const bool lin = st.wave_lin != 0;
    const double mod64 = m.var_lss_mod;
    const dfl mod = dfl_of(mod64);
    const dfl obs0 = dfl_of(lin ? st.obs_grid0 : st.obs_grid0);
    const dfl var0 = dfl_of(st.var_grid0);
    const float inv_obs = (float)(1.0 / st.obs_step), inv_rest = (float)(1.0 / st.rest_step);
    const float inv_var = (float)(1.0 / st.var_step);
    const float guard = lin ? 5e-3f : 1e-3f;
    constexpr float kLn10 = 2.302585093f;
    const int64_t num_groups = (sp.num + kStackGroup - 1) / kStackGroup;
    StackSlot *slots = s_slots[wib];
    for (;;) {
        int64_t group = 0;
        if (lane == 0) group = atomicAdd(&scratch->work_counter, 1);
        group = __shfl_sync(0xffffffffu, group, 0);
        if (group >= num_groups) break;
        if (lane < kStackGroup) {
            StackSlot sl;
            const int64_t f = group * kStackGroup + lane;
            sl.skip = 1;
            sl.off = 0;
            sl.n = 0;
            sl.zp1 = 0.;
            sl.zr_hi = sl.zr_lo = 0.f;
            if (f < sp.num && fit.status[f] == 0) {
                sl.skip = 0;
                sl.off = sp.pix_offset[f];
                sl.n = (int)(sp.pix_offset[f + 1] - sl.off);
                sl.zp1 = log10(1 + sp.z_qso[f]);
                const dfl zr = dfl_of(lin ? sl.zp1 : sl.zp1 + st.rest_grid0);
                sl.zr_hi = zr.hi;
                sl.zr_lo = zr.lo;
            }
            slots[lane] = sl;
        }
        __syncwarp();
        for (int jf = 0; jf < kStackGroup; ++jf) {
            if (slots[jf].skip) continue;
            const int64_t off = slots[jf].off;
            const int n = slots[jf].n;
            const double zp1 = slots[jf].zp1;
            const dfl zr = {slots[jf].zr_hi, slots[jf].zr_lo};
            if (do_var) {
                for (int k = lane; k < 64; k += 32) seen[wib][k] = 0u;
                __syncwarp();
            }
            for (int p = lane; p < n; p += 32) {
                const double ll = sp.log_lambda[off + p];
                const double iv64 = sp.ivar[off + p];
                const dfl L = dfl_of(ll), F = dfl_of(sp.flux[off + p]);
                const dfl C = dfl_of(fit.continuum[off + p]);
                const dfl IV = dfl_of(iv64);
                const bool has_iv = IV.hi > 0.f;
                // observed-frame bin (stack, variance-function table)
                int jobs = -1;
                if (do_stack || use_table) {
                    float t;
                    if (lin) {
                        const float lam = exp10f(L.hi) * fmaf(L.lo, kLn10, 1.f);
                        t = fmaf(lam - (float)st.obs_grid0, inv_obs, 0.5f);
                    } else {
                        t = fmaf((L.hi - obs0.hi) + (L.lo - obs0.lo), inv_obs, 0.5f);
                    }
                    if (!bin_certain(t, guard, jobs))
                        jobs = (int)find_bin(ll, st.obs_grid0, st.obs_step, st.wave_lin);
                }
                // X = ivar C^2 and var_pipe = 1 / X
                dfl X = {0.f, 0.f}, vp = {0.f, 0.f}, Q = {0.f, 0.f};
                if (has_iv) {
                    X = dfl_mul(IV, dfl_mul(C, C));
                    vp = dfl_div(dfl{1.f, 0.f}, X);
                    Q = dfl_div(F, C);
                }
                if (do_mc || do_stack) {
                    // compute_forest_weights (dr16_expected_flux.py:466-488)
                    dfl w = {0.f, 0.f};
                    if (has_iv) {
                        dfl eta = {0.f, 0.f}, vlss = {1.f, 0.f}, fudge = {0.f, 0.f};
                        if (mi > 0) {
                            bool done = false;
                            if (use_table && jobs >= 0 && jobs < O) {
                                const float4 t0 = table[2 * jobs];
                                if (fabsf((L.hi - t0.x) + (L.lo - t0.y)) <= 1e-12f) {
                                    const float4 t1 = table[2 * jobs + 1];
                                    eta = dfl{t0.z, t0.w};
                                    vlss = dfl{t1.x, t1.y};
                                    fudge = dfl{t1.z, t1.w};
                                    done = true;
                                }
                            }
                            if (!done) {
                                double e, v, f;
                                var_funcs_f64(m, ll, e, v, f);
                                eta = dfl_of(e);
                                vlss = dfl_of(v);
                                fudge = dfl_of(f);
                            }
                        }
                        const dfl den = dfl_add(dfl_add(dfl_mul(eta, vp), dfl_mul(mod, vlss)),
                                                dfl_mul(fudge, X));
                        w = dfl_div(dfl{1.f, 0.f}, den);
                    }
                    if (do_mc) {
                        // _compute_mean_cont: (f / (C + 1e-16)) * w binned in the rest frame
                        float t;
                        if (lin) {
                            const dfl x = dfl_add(L, dfl{-zr.hi, -zr.lo});
                            const float lam = exp10f(x.hi) * fmaf(x.lo, kLn10, 1.f);
                            t = fmaf(lam - (float)st.rest_grid0, inv_rest, 0.5f);
                        } else {
                            t = fmaf((L.hi - zr.hi) + (L.lo - zr.lo), inv_rest, 0.5f);
                        }
                        int bin;
                        if (!bin_certain(t, guard, bin))
                            bin = (int)find_bin(ll - zp1, st.rest_grid0, st.rest_step, st.wave_lin);
                        if (bin >= 0 && bin < R) {
                            if (has_iv) {
                                dfl ratio = Q;
                                if (!(fabsf(C.hi) > 1e-4f)) {
                                    // the 1e-16 offset matters: the reference's formula
                                    const double c64 = fit.continuum[off + p];
                                    ratio = dfl_of(sp.flux[off + p] / (c64 + 1e-16));
                                }
                                hist_add(mc_num_h, mc_num_l, bin, dfl_mul(ratio, w));
                                hist_add(mc_w_h, mc_w_l, bin, w);
                            }
                        } else {
                            report_error(scratch, PG_ERR_BIN_RANGE, bin);
                        }
                    }
                    if (do_stack) {
                        // compute_delta_stack: delta = f / C where ivar > 0
                        if (jobs >= 0 && jobs < O) {
                            if (has_iv) {
                                hist_add(s_num_h, s_num_l, jobs, dfl_mul(Q, w));
                                hist_add(s_w_h, s_w_l, jobs, w);
                            }
                        } else {
                            report_error(scratch, PG_ERR_BIN_RANGE, jobs);
                        }
                    }
                }
                if (do_var && has_iv) {
                    // LeastsSquaresVarStats.initialize_delta_arrays
                    // (least_squares_var_stats.py:134-184)
                    constexpr float kMin = (float)kVarPipeMin, kMax = (float)kVarPipeMax;
                    const float lv = log10f(vp.hi) + vp.lo / (vp.hi * kLn10);
                    bool in_range;
                    int vbin = 0;
                    const float tv = (lv - kMin) * (float)(kVarBins / (kVarPipeMax - kVarPipeMin));
                    if (fabsf(lv - kMin) > 1e-4f && fabsf(lv - kMax) > 1e-4f &&
                        bin_certain(tv, 1e-3f, vbin)) {
                        in_range = lv > kMin && lv < kMax;
                    } else {
                        const double c64 = fit.continuum[off + p];
                        const double lv64 = log10(1 / iv64 / (c64 * c64));
                        in_range = lv64 > kVarPipeMin && lv64 < kVarPipeMax;
                        vbin = (int)((lv64 - kVarPipeMin) / (kVarPipeMax - kVarPipeMin) * kVarBins);
                    }
                    if (in_range) {
                        float t;
                        if (lin) {
                            const float lam = exp10f(L.hi) * fmaf(L.lo, kLn10, 1.f);
                            t = fmaf(lam - (float)st.var_grid0, inv_var, 0.5f);
                        } else {
                            t = fmaf((L.hi - var0.hi) + (L.lo - var0.lo), inv_var, 0.5f);
                        }
                        int lbin;
                        if (!bin_certain(t, guard, lbin))
                            lbin = (int)find_bin(ll, st.var_grid0, st.var_step, st.wave_lin);
                        const int64_t bin = vbin + (int64_t)kVarBins * lbin;
                        if (lbin >= 0 && bin >= 0 && bin < nvar) {
                            const dfl delta = dfl_add(Q, dfl{-1.f, 0.f});
                            const dfl d2 = dfl_mul(delta, delta);
                            hist_add(v_mean_h, v_mean_l, (int)bin, delta);
                            hist_add(v_d2_h, v_d2_l, (int)bin, d2);
                            hist_add(v_d4_h, v_d4_l, (int)bin, dfl_mul(d2, d2));
                            atomicAdd(&v_np[bin], 1u);
                            atomicOr(&seen[wib][bin >> 5], 1u << (bin & 31));
                        } else {
                            report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bin);
                        }
                    }
                }
            }
            if (do_var) {
                __syncwarp();
                for (int k = lane; k < 64; k += 32) {
                    uint32_t bits = seen[wib][k];
                    while (bits) {
                        const int bit = __ffs(bits) - 1;
                        bits &= bits - 1;
                        atomicAdd(&v_nq[k * 32 + bit], 1u);
                    }
                }
                __syncwarp();
            }
        }
        __syncwarp();
    }
    __syncthreads();
    // one FP64 add per nonzero bin and block
    auto flush = [&](double *dst, const float *h, const float *l, int count) {
        if (!dst) return;
        for (int k = threadIdx.x; k < count; k += blockDim.x)
            if (h[k] != 0.f || l[k] != 0.f) atomicAdd(&dst[k], (double)h[k] + (double)l[k]);
    };
    auto flush_count = [&](double *dst, const uint32_t *c, int count) {
        if (!dst) return;
        for (int k = threadIdx.x; k < count; k += blockDim.x)
            if (c[k]) atomicAdd(&dst[k], (double)c[k]);
    };
    flush(st.mean_cont_num, mc_num_h, mc_num_l, R);
    flush(st.mean_cont_weight, mc_w_h, mc_w_l, R);
    flush(st.stack_num, s_num_h, s_num_l, O);
    flush(st.stack_weight, s_w_h, s_w_l, O);
    if (do_var) {
        flush(st.var_mean, v_mean_h, v_mean_l, nvar);
        flush(st.var_delta2, v_d2_h, v_d2_l, nvar);
        flush(st.var_delta4, v_d4_h, v_d4_l, nvar);
        flush_count(st.var_npix, v_np, nvar);
        flush_count(st.var_nqso, v_nq, nvar);
    }
}

__global__ void __launch_bounds__(kContBlock) cont_deltas_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    const __grid_constant__ pg_cont_fit fit, double *__restrict__ delta,
    double *__restrict__ weights) {
    const int lane = threadIdx.x & 31;
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t f = warp_global; f < sp.num; f += nwarps) {
        const int64_t off = sp.pix_offset[f];
        const int64_t n = sp.pix_offset[f + 1] - off;
        const bool ok = fit.status[f] == 0;
        for (int64_t p = lane; p < n; p += 32) {
            double w = 0., d = 0.;
            if (ok) {
                const double ll = sp.log_lambda[off + p];
                double expected = fit.continuum[off + p];
                if (m.stack_x) expected *= interp_nearest(m.stack_x, m.stack_y, m.num_stack, ll);
                w = forest_weight(m, ll, sp.ivar[off + p], expected);
                if (w > 0) d = sp.flux[off + p] / expected - 1;
            }
            delta[off + p] = d;
            weights[off + p] = w;
        }
    }
}

// Warm-start network inputs (see pg_mlp_features in include/picca_gb300.h),
// forest by forest with forest_feature_sums; log10(1 + z) by the lanes of a
// group of forests in parallel.
__global__ void __launch_bounds__(kContBlock) mlp_features_kernel(
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model m,
    __nv_bfloat16 *__restrict__ feat, int stride, double *__restrict__ a0_out, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float sums[kContBlock / 32][2][kFeatBins];
    __shared__ float s_lm[kContBlock / 32][kFitGroup][2];
    const FitTables tab = load_fit_tables(m, smem);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const float bins_per_span =
        (float)(kFeatBins / (m.log_lambda_rest_max - m.log_lambda_rest_min));
    const int64_t num_groups = (sp.num + kFitGroup - 1) / kFitGroup;
    for (;;) {
        int64_t group = 0;
        if (lane == 0) group = atomicAdd(&scratch->work_counter, 1);
        group = __shfl_sync(0xffffffffu, group, 0);
        if (group >= num_groups) break;
        if (lane < kFitGroup && group * kFitGroup + lane < sp.num) {
            const float2 lm = forest_lmin(sp, m, group * kFitGroup + lane);
            s_lm[wib][lane][0] = lm.x;
            s_lm[wib][lane][1] = lm.y;
        }
        __syncwarp();
        for (int j = 0; j < kFitGroup; ++j) {
            const int64_t f = group * kFitGroup + j;
            if (f >= sp.num) break;
            const FeatScalars fs = forest_feature_sums(sp, tab, f, s_lm[wib][j][0],
                                                       s_lm[wib][j][1], bins_per_span,
                                                       sums[wib], lane);
            __nv_bfloat16 *row = feat + f * (int64_t)stride;
            for (int k = lane; k < stride; k += 32)
                row[k] = __float2bfloat16(forest_feature(sums[wib], fs, k));
            if (lane == 0) a0_out[f] = f32_to_f64(fs.a0);
            __syncwarp();
        }
    }
}

unsigned blocks_for(int64_t num, int num_sms) {
    const int64_t warps = (num + 0) > 0 ? num : 1;
    int64_t blocks = (warps * 32 + kContBlock - 1) / kContBlock;
    const int64_t cap = (int64_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    return (unsigned)(blocks < 1 ? 1 : blocks);
}

}  // namespace

int launch_cont_fit(const pg_spectra &sp, const pg_cont_model &m, const double *start,
                    const int32_t *index, int64_t count, int max_iter, double tol, int mode,
                    const pg_cont_fit &out, Scratch *scratch, int num_sms, cudaStream_t stream,
                    float cert_chi2, float cert_ab) {
    if (count <= 0) return PG_OK;
    const unsigned blocks = blocks_for(count, num_sms);
    if (mode == PG_FIT_MIXED) {
        const size_t smem = kFitSlabBytes * (kContBlock / 32) +
                            fit_smem_bytes(m.num_mean_cont, m.num_var_intervals);
        if (smem > 200 * 1024) return PG_ERR_UNSUPPORTED;
        cudaError_t err = cudaFuncSetAttribute(
            cont_fit_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return check_cuda(err);
        // persistent blocks drawing groups of forests from the work counter
        int per_sm = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cont_fit_mixed_kernel,
                                                            kContBlock, smem);
        if (err != cudaSuccess) return check_cuda(err);
        const int64_t groups = (count + kFitGroup - 1) / kFitGroup;
        int64_t mixed_blocks = (groups + kContBlock / 32 - 1) / (kContBlock / 32);
        const int64_t resident = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
        if (mixed_blocks > resident) mixed_blocks = resident;
        cont_fit_mixed_kernel<<<(unsigned)mixed_blocks, kContBlock, smem, stream>>>(
            sp, m, start, index, count, max_iter, tol, out, scratch, cert_chi2, cert_ab);
    } else {
        cont_fit_kernel<double><<<blocks, kContBlock, 0, stream>>>(sp, m, start, index, count,
                                                                    max_iter, tol, out, scratch);
    }
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return check_cuda(err);
    // forests longer than the register kernels hold (the linear grid), in FP64
    const size_t long_smem = (size_t)kLongWarps * 6 * 32 * kLongK * sizeof(double);
    err = cudaFuncSetAttribute(cont_fit_long_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)long_smem);
    if (err != cudaSuccess) return check_cuda(err);
    // the long kernel has no certificate: under it the warm-started fit of a
    // long forest runs to convergence with the plain fit's iteration limit
    const int long_iter = cert_chi2 > 0.f && max_iter < 100 ? 100 : max_iter;
    int64_t long_blocks = (count + 32 * kLongWarps - 1) / (32 * kLongWarps);
    if (long_blocks > (int64_t)num_sms * 8) long_blocks = (int64_t)num_sms * 8;
    cont_fit_long_kernel<<<(unsigned)(long_blocks < 1 ? 1 : long_blocks), 32 * kLongWarps,
                           long_smem, stream>>>(sp, m, start, index, count, long_iter,
                                                cert_chi2 > 0.f ? 1e-10 : tol, out, scratch);
    err = cudaGetLastError();
    if (err != cudaSuccess) return check_cuda(err);
    if (mode == PG_FIT_MIXED && max_iter > 0 && !(cert_chi2 > 0.f)) {
        // the two-float finish of the forests flagged status 4, same stream
        const size_t rsmem = refine_smem_bytes(m.num_mean_cont, m.num_var_intervals);
        if (rsmem > 200 * 1024) return PG_ERR_UNSUPPORTED;
        err = cudaFuncSetAttribute(cont_fit_refine_kernel,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem);
        if (err != cudaSuccess) return check_cuda(err);
        // every SM filled: the flagged forests are scattered over the list
        int per_sm = 0;
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cont_fit_refine_kernel,
                                                            32 * kRefineWarps, rsmem);
        if (err != cudaSuccess) return check_cuda(err);
        int64_t rblocks = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
        const int64_t need = (count + 32 * kRefineWarps - 1) / (32 * kRefineWarps);
        if (rblocks > need) rblocks = need;
        cont_fit_refine_kernel<<<(unsigned)rblocks, 32 * kRefineWarps, rsmem, stream>>>(
            sp, m, index, count, out, scratch);
        err = cudaGetLastError();
    }
    return check_cuda(err);
}

int launch_cont_stacks(const pg_spectra &sp, const pg_cont_model &m, const pg_cont_fit &fit,
                       const pg_cont_stacks &st, Scratch *scratch, int num_sms,
                       cudaStream_t stream) {
    if (sp.num <= 0) return PG_OK;
    if (st.var_mean && st.var_lambda_bins * kVarBins > 2048) return PG_ERR_UNSUPPORTED;
    const bool want_table = !m.use_constant_weight && (st.mean_cont_num || st.stack_num);
    // the variance-function table when it fits beside the histograms
    int use_table = want_table && stack_smem_bytes(st, true) <= 200 * 1024 ? 1 : 0;
    const size_t smem = stack_smem_bytes(st, use_table != 0);
    if (smem > 200 * 1024) return PG_ERR_UNSUPPORTED;
    cudaError_t err = cudaFuncSetAttribute(cont_stacks_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cont_stacks_kernel, kStackBlock,
                                                        smem);
    if (err != cudaSuccess) return check_cuda(err);
    const int64_t groups = (sp.num + kStackGroup - 1) / kStackGroup;
    int64_t blocks = (groups + kStackBlock / 32 - 1) / (kStackBlock / 32);
    const int64_t resident = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
    if (blocks > resident) blocks = resident;
    cont_stacks_kernel<<<(unsigned)(blocks < 1 ? 1 : blocks), kStackBlock, smem, stream>>>(
        sp, m, fit, st, scratch, use_table);
    return check_cuda(cudaGetLastError());
}

int launch_mlp_features(const pg_spectra &sp, const pg_cont_model &m, uint16_t *features,
                        int stride, double *a0, Scratch *scratch, int num_sms, cudaStream_t stream) {
    if (sp.num <= 0) return PG_OK;
    const size_t smem = fit_smem_bytes(m.num_mean_cont, m.num_var_intervals);
    if (smem > 200 * 1024) return PG_ERR_UNSUPPORTED;
    cudaError_t err = cudaFuncSetAttribute(
        mlp_features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int per_sm = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mlp_features_kernel, kContBlock,
                                                        smem);
    if (err != cudaSuccess) return check_cuda(err);
    const int64_t groups = (sp.num + kFitGroup - 1) / kFitGroup;
    int64_t blocks = (groups + kContBlock / 32 - 1) / (kContBlock / 32);
    const int64_t resident = (int64_t)num_sms * (per_sm > 0 ? per_sm : 1);
    if (blocks > resident) blocks = resident;
    mlp_features_kernel<<<(unsigned)blocks, kContBlock, smem, stream>>>(
        sp, m, reinterpret_cast<__nv_bfloat16 *>(features), stride, a0, scratch);
    return check_cuda(cudaGetLastError());
}

int launch_cont_deltas(const pg_spectra &sp, const pg_cont_model &m, const pg_cont_fit &fit,
                       double *delta, double *weights, int num_sms, cudaStream_t stream) {
    if (sp.num <= 0) return PG_OK;
    cont_deltas_kernel<<<blocks_for(sp.num, num_sms), kContBlock, 0, stream>>>(sp, m, fit, delta,
                                                                               weights);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
