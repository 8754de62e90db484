// Fast metal distortion matrices: calc_fast_metal_dmat of
// picca_fast_metal_dmat.py (py/picca/bin/picca_fast_metal_dmat.py:30-251)
// and of picca_fast_metal_xdmat.py (py/picca/bin/picca_fast_metal_xdmat.py:
// 28-215).
//
// The reference forms every pair (i, j) of two pixel lists (the stacked
// deltas' wavelength grid against itself, or against the quasars' redshift
// histogram) as numpy arrays of n1 n2 elements and histograms them:
//  * r_par of the pair seen as the assumed absorbers ("output") against
//    r_par seen as the true absorbers ("input") on the r_par edges
//    (np.histogram2d, :152-155),
//  * the ratio of the pair's mean distances, output / input, on 4 (nt + 1)
//    equal-width bins spanning the ratio's range, with weight w / dist_in^2
//    where |r_par_in| < 20 Mpc/h (np.histogram, :173-177),
//  * w, w r_par_out and w (z1 + z2) / 2 on the r_par edges of r_par_out
//    (:220-231).
// Here a first kernel finds the ratio's range with order-preserving integer
// keys; the second rebuilds numpy's equal-width edges from it (linspace) and
// bins every pair with numpy's own index rules, so each pair lands in the
// bin the reference gives it. A thread takes pixel i of side 1 and a run of
// consecutive side-2 pixels, sums runs of pairs that share a bin in
// registers and adds each run to per-CTA shared-memory histograms, which
// the CTA adds to the output once.
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kFmBlock = 128;
constexpr int kFmChunk = 8;  // side-2 pixels per thread and pass

struct FmSide {
    const double *r_in, *r_out, *z_in, *w;
    int64_t num;
};

struct FmConst {
    double r_par_min, r_par_step;  // edge k = r_par_min + r_par_step * k
    double near_r_par;
    int32_t np, nr, signed_r_par;
    int32_t shared_2d;  // the np x np histogram lives in shared memory
};

__device__ __forceinline__ unsigned long long fm_max(unsigned long long a,
                                                     unsigned long long b) {
    return a > b ? a : b;
}

// Range of ratio = ((ro1 + ro2) / 2) / ((ri1 + ri2) / 2) over all pairs.
// The minimum is kept as the complement of its key so that both ends use
// atomicMax on a zeroed word.
__global__ void __launch_bounds__(kFmBlock)
    fm_range_kernel(FmSide s1, FmSide s2, Scratch *scratch) {
    unsigned long long lo = 0, hi = 0;
    for (int64_t i = blockIdx.x; i < s1.num; i += gridDim.x) {
        const double ri = s1.r_in[i], ro = s1.r_out[i];
        for (int64_t j = threadIdx.x; j < s2.num; j += kFmBlock) {
            const double din = (ri + s2.r_in[j]) / 2, dout = (ro + s2.r_out[j]) / 2;
            const unsigned long long key = order_key(dout / din);
            lo = fm_max(lo, ~key);
            hi = fm_max(hi, key);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        lo = fm_max(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fm_max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
    }
    if ((threadIdx.x & 31) == 0) {
        if (lo) atomicMax(&scratch->ratio_lo_inv_key, lo);
        if (hi) atomicMax(&scratch->ratio_hi_key, hi);
    }
}

// np.histogram's bin of x on ascending edges e[0..n]: [e_k, e_k+1) and the
// last bin closed; -1 outside [e_0, e_n].
__device__ __forceinline__ int fm_edge_bin(double x, const double *e, int n, double inv_step) {
    if (!(x >= e[0] && x <= e[n])) return -1;
    int b = (int)((x - e[0]) * inv_step);
    b = b < 0 ? 0 : (b > n - 1 ? n - 1 : b);
    while (b > 0 && x < e[b]) --b;
    while (b < n - 1 && x >= e[b + 1]) ++b;
    return b;
}

__global__ void __launch_bounds__(kFmBlock)
    fm_hist_kernel(FmConst c, FmSide s1, FmSide s2, pg_fast_metal_sums out,
                   const Scratch *scratch, int empty) {
    extern __shared__ double fm_smem[];
    const int np = c.np, nr = c.nr;
    double *h2 = c.shared_2d ? fm_smem : out.rp_dmat;  // [np][np]: output bin, input bin
    double *base = fm_smem + (c.shared_2d ? (size_t)np * np : 0);
    double *hr = base;                // [nr] ratio histogram
    double *h1w = hr + nr;            // [np] sums of w on the output r_par bins
    double *h1rp = h1w + np;          // w r_par_out
    double *h1z = h1rp + np;          // w (z1 + z2) / 2
    double *rp_edges = h1z + np;      // [np + 1]
    double *r_edges = rp_edges + np + 1;  // [nr + 1]
    const int tid = threadIdx.x;

    // the ratio's range (numpy's _get_outer_edges) and its edges (np.linspace)
    double first = 0., last = 1.;
    if (!empty) {
        first = order_value(~scratch->ratio_lo_inv_key);
        last = order_value(scratch->ratio_hi_key);
    }
    if (first == last) {
        first = first - 0.5;
        last = last + 0.5;
    }
    const double delta = last - first;
    const double step = delta / nr;
    const double denom = last - first;
    for (int k = tid; k <= nr; k += kFmBlock) {
        double y = (double)k;
        if (step == 0.) {
            y = y / nr;
            y = y * delta;
        } else {
            y = y * step;
        }
        r_edges[k] = k == nr ? last : y + first;
    }
    for (int k = tid; k <= np; k += kFmBlock) rp_edges[k] = c.r_par_min + c.r_par_step * k;
    const int local = (c.shared_2d ? np * np : 0) + nr + 3 * np;
    for (int k = tid; k < local; k += kFmBlock) fm_smem[k] = 0.;
    __syncthreads();
    if (blockIdx.x == 0)
        for (int k = tid; k <= nr; k += kFmBlock) out.ratio_edges[k] = r_edges[k];
    const double inv_rp_step = 1. / c.r_par_step;

    for (int64_t i = blockIdx.x; i < s1.num; i += gridDim.x) {
        const double ri1 = s1.r_in[i], ro1 = s1.r_out[i], zi1 = s1.z_in[i], w1 = s1.w[i];
        for (int64_t j0 = (int64_t)tid * kFmChunk; j0 < s2.num;
             j0 += (int64_t)kFmBlock * kFmChunk) {
            const int64_t j1 = j0 + kFmChunk < s2.num ? j0 + kFmChunk : s2.num;
            int run1 = -1, run2 = -1, runr = -1;
            double a_w = 0., a_rp = 0., a_z = 0., a_2 = 0., a_r = 0.;
            for (int64_t j = j0; j < j1; ++j) {
                const double ri2 = s2.r_in[j], ro2 = s2.r_out[j];
                double irp = ri1 - ri2, orp = ro1 - ro2;
                if (!c.signed_r_par) {
                    irp = fabs(irp);
                    orp = fabs(orp);
                }
                const double din = (ri1 + ri2) / 2, dout = (ro1 + ro2) / 2;
                const double w = w1 * s2.w[j];
                const int bo = fm_edge_bin(orp, rp_edges, np, inv_rp_step);
                if (bo >= 0) {
                    if (bo != run1) {
                        if (run1 >= 0) {
                            atomicAdd(&h1w[run1], a_w);
                            atomicAdd(&h1rp[run1], a_rp);
                            atomicAdd(&h1z[run1], a_z);
                        }
                        run1 = bo;
                        a_w = a_rp = a_z = 0.;
                    }
                    a_w += w;
                    a_rp += w * orp;
                    a_z += w * ((zi1 + s2.z_in[j]) / 2.);
                    const int bi = fm_edge_bin(irp, rp_edges, np, inv_rp_step);
                    if (bi >= 0) {
                        const int key = bo * np + bi;
                        if (key != run2) {
                            if (run2 >= 0) atomicAdd(&h2[run2], a_2);
                            run2 = key;
                            a_2 = 0.;
                        }
                        a_2 += w;
                    }
                }
                if (fabs(irp) < c.near_r_par) {
                    // numpy's equal-width rule: estimate, then fix by the edges
                    const double x = dout / din;
                    int k = (int)(((x - first) / denom) * (double)nr);
                    k = k < 0 ? 0 : (k > nr - 1 ? nr - 1 : k);
                    if (x < r_edges[k] && k > 0) --k;
                    if (k != nr - 1 && x >= r_edges[k + 1]) ++k;
                    if (k != runr) {
                        if (runr >= 0) atomicAdd(&hr[runr], a_r);
                        runr = k;
                        a_r = 0.;
                    }
                    a_r += w / (din * din);
                }
            }
            if (run1 >= 0) {
                atomicAdd(&h1w[run1], a_w);
                atomicAdd(&h1rp[run1], a_rp);
                atomicAdd(&h1z[run1], a_z);
            }
            if (run2 >= 0) atomicAdd(&h2[run2], a_2);
            if (runr >= 0) atomicAdd(&hr[runr], a_r);
        }
    }
    __syncthreads();
    if (c.shared_2d)
        for (int k = tid; k < np * np; k += kFmBlock)
            if (h2[k] != 0.) atomicAdd(&out.rp_dmat[k], h2[k]);
    for (int k = tid; k < nr; k += kFmBlock)
        if (hr[k] != 0.) atomicAdd(&out.ratio_weights[k], hr[k]);
    for (int k = tid; k < np; k += kFmBlock) {
        if (h1w[k] != 0.) atomicAdd(&out.out_weight[k], h1w[k]);
        if (h1rp[k] != 0.) atomicAdd(&out.out_weight_rp[k], h1rp[k]);
        if (h1z[k] != 0.) atomicAdd(&out.out_weight_z[k], h1z[k]);
    }
}

}  // namespace

int launch_fast_metal(const pg_fast_metal_params &p, const pg_fast_metal_side &a,
                      const pg_fast_metal_side &b, const pg_fast_metal_sums &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream) {
    const int np = p.num_bins_r_par, nr = p.num_ratio_bins;
    cudaError_t err;
    const size_t n2d = (size_t)np * np;
    err = cudaMemsetAsync(out.rp_dmat, 0, n2d * sizeof(double), stream);
    if (err == cudaSuccess)
        err = cudaMemsetAsync(out.ratio_weights, 0, (size_t)nr * sizeof(double), stream);
    double *sums1d[3] = {out.out_weight, out.out_weight_rp, out.out_weight_z};
    for (double *ptr : sums1d)
        if (err == cudaSuccess) err = cudaMemsetAsync(ptr, 0, (size_t)np * sizeof(double), stream);
    if (err != cudaSuccess) return check_cuda(err);

    FmSide s1{a.r_in, a.r_out, a.z_in, a.weight, a.num};
    FmSide s2{b.r_in, b.r_out, b.z_in, b.weight, b.num};
    const int empty = (a.num == 0 || b.num == 0);
    if (empty) s1.num = 0;

    FmConst c;
    c.r_par_min = p.r_par_min;
    c.r_par_step = (p.r_par_max - p.r_par_min) / np;
    c.near_r_par = p.near_r_par;
    c.np = np;
    c.nr = nr;
    c.signed_r_par = p.signed_r_par != 0;
    const size_t small = (size_t)nr + 3 * (size_t)np + (size_t)np + 1 + (size_t)nr + 1;
    constexpr size_t kSmemLimit = 200 * 1024;
    c.shared_2d = (n2d + small) * sizeof(double) <= kSmemLimit;
    const size_t smem = ((c.shared_2d ? n2d : 0) + small) * sizeof(double);
    if (smem > kSmemLimit) return PG_ERR_UNSUPPORTED;
    err = cudaFuncSetAttribute(fm_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kSmemLimit);
    if (err != cudaSuccess) return check_cuda(err);
    int occ = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fm_hist_kernel, kFmBlock, smem);
    if (err != cudaSuccess || occ < 1) return PG_ERR_CUDA;

    if (!empty) {
        const int64_t grid = std::min<int64_t>((int64_t)num_sms * 8, a.num);
        fm_range_kernel<<<(int)grid, kFmBlock, 0, stream>>>(s1, s2, scratch);
        if ((err = cudaGetLastError()) != cudaSuccess) return check_cuda(err);
    }
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms * occ, s1.num));
    fm_hist_kernel<<<(int)grid, kFmBlock, smem, stream>>>(c, s1, s2, out, scratch, empty);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
