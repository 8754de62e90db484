// Cross Wick terms T2-T4 by factorisation: xcf.compute_wickT1234_pairs
// (py/picca/xcf.py:1220-1351) without the O(K^2) sweep.
//
// For a forest with its quasars, the pairs of listed (pixel, quasar) pairs
// split into same quasar (T2), same pixel (T3) and the rest (T4), and
//   T2 + T4 [P, Q] = sum_{a in P, b in Q} X1'[i_a, i_b] zw_a zw_b = (U^T X1' U)[P, Q]
// with U[i, P] = sum of zw over the listed pairs of pixel i in bin P (X1' is
// the forest's weighted 1D correlation with a zero diagonal), and
//   T3 [P, Q] = sum_i c_i W[i, P] W[i, Q] - delta_PQ sum_{a in P} c_{i_a} w12_a^2
// with W[i, P] = sum of w12 = w1 w_q over the listed pairs of pixel i in bin
// P and c_i = zw1_i / w1_i. T2 itself is small (pairs of pixels seen from the
// same quasar: a contiguous pixel interval per quasar) and is summed
// directly; T4 = (U^T X1' U) - T2. The two products U^T (X1' U) and
// W^T (c W) run as FP64 GEMMs over the forest's nonempty bins, then every
// cell is added to its (bin, bin) place. Per forest this is
// O(n1^2 nz + n1 nz^2) instead of O(K^2) for K listed pairs.
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kXfBlock = 256;

struct XfConst {
    double r_par_min, r_par_max, r_trans_max, range;
    int32_t np, nt, nb, pad;
};

// Bin of a (pixel, quasar) pair or -1 (xcf.py:1282-1316, r_par signed).
__device__ __forceinline__ int xf_bin(const XfConst &c, double r1, double r2, double cc,
                                      double ss) {
    const double r_par = __dmul_rn(__dsub_rn(r1, r2), cc);
    const double r_trans = __dmul_rn(__dadd_rn(r1, r2), ss);
    if (!(r_par < c.r_par_max && r_trans < c.r_trans_max && r_par >= c.r_par_min)) return -1;
    const int bp = (int)__dmul_rn(__ddiv_rn(__dsub_rn(r_par, c.r_par_min), c.range), (double)c.np);
    const int bt = (int)__dmul_rn(__ddiv_rn(r_trans, c.r_trans_max), (double)c.nt);
    // a quotient that rounds up to 1 would index past the last bin (the
    // reference writes out of bounds there); such a pair is dropped
    if (bp >= c.np || bt >= c.nt) return -1;
    return bt + c.nt * bp;
}

struct XfItem {
    int f, nq, n1;
    int64_t o1;
    int32_t q0;
};

struct XfScratch {
    int32_t *used, *col, *bins, *lo, *hi, *nz;
    unsigned long long *listed;  // listed (pixel, quasar) pairs of the item
    double *qcos, *qsin, *qr, *qw, *qzw;
    double *U, *W, *Wc, *Y, *T24, *T3, *T2, *D;
};

__global__ void xf_quasars(XfItem it, pg_forest_set forests, pg_forest_set objs,
                           const double *zw_obj, const int32_t *obj_index,
                           const double *obj_angle, XfScratch s) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < it.nq; k += gridDim.x * blockDim.x) {
        const int g = obj_index[it.q0 + k];
        const int f = it.f;
        const double ang = obj_angle ? obj_angle[it.q0 + k]
                                     : angle_between(forests.x_cart[f], forests.y_cart[f],
                                                     forests.z_cart[f], forests.ra[f],
                                                     forests.dec[f], forests.cos_dec[f],
                                                     objs.x_cart[g], objs.y_cart[g],
                                                     objs.z_cart[g], objs.ra[g], objs.dec[g]);
        s.qcos[k] = cos(ang / 2);
        s.qsin[k] = sin(ang / 2);
        s.qr[k] = objs.obj_r_comov[g];
        s.qw[k] = objs.obj_weight[g];
        s.qzw[k] = zw_obj[g];
        s.lo[k] = it.n1;
        s.hi[k] = -1;
    }
}

// Mark the bins that hold listed pairs.
__global__ void xf_mark(XfConst c, XfItem it, pg_forest_set forests, XfScratch s) {
    const int64_t total = (int64_t)it.n1 * it.nq;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / it.n1), i = (int)(t - (int64_t)j * it.n1);
        const int b = xf_bin(c, forests.r_comov[it.o1 + i], s.qr[j], s.qcos[j], s.qsin[j]);
        if (b < 0) continue;
        s.used[b] = 1;
        atomicMin(&s.lo[j], i);
        atomicMax(&s.hi[j], i);
        atomicAdd(s.listed, 1ull);
    }
}

// Compact column of every used bin (one block).
__global__ void xf_scan(int nb, XfScratch s) {
    __shared__ int chunk_sum[1024];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (nb + nt - 1) / nt;
    const int b0 = tid * per, b1 = min(nb, b0 + per);
    int local = 0;
    for (int b = b0; b < b1; ++b) local += s.used[b];
    chunk_sum[tid] = local;
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int k = 0; k < nt; ++k) {
            const int v = chunk_sum[k];
            chunk_sum[k] = run;
            run += v;
        }
        *s.nz = run;
    }
    __syncthreads();
    int run = chunk_sum[tid];
    for (int b = b0; b < b1; ++b) {
        if (s.used[b]) {
            s.col[b] = run;
            s.bins[run] = b;
            ++run;
        } else {
            s.col[b] = -1;
        }
    }
}

// U, W, c W, the diagonal correction of T3, and WALL / NB / T1 (per listed
// pair, as xcf.py:1318-1323).
__global__ void xf_fill(XfConst c, XfItem it, pg_forest_set forests, const double *zw1, int nz,
                        XfScratch s, pg_wick_sums out) {
    const int64_t total = (int64_t)it.n1 * it.nq;
    const int nb = c.nb;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / it.n1), i = (int)(t - (int64_t)j * it.n1);
        const int b = xf_bin(c, forests.r_comov[it.o1 + i], s.qr[j], s.qcos[j], s.qsin[j]);
        if (b < 0) continue;
        const int col = s.col[b];
        const double w1 = forests.weights[it.o1 + i];
        const double w12 = __dmul_rn(w1, s.qw[j]);
        const double ci = __ddiv_rn(zw1[it.o1 + i], w1);
        const int64_t cell = (int64_t)i * nz + col;
        atomicAdd(&s.U[cell], s.qzw[j]);
        atomicAdd(&s.W[cell], w12);
        atomicAdd(&s.Wc[cell], __dmul_rn(ci, w12));
        atomicAdd(&s.D[col], __dmul_rn(ci, __dmul_rn(w12, w12)));
        atomicAdd(&out.weights_wick[b], w12);
        atomicAdd(reinterpret_cast<unsigned long long *>(&out.num_pairs_wick[b]), 1ull);
        atomicAdd(&out.t1[(int64_t)b * nb + b],
                  __dmul_rn(__ddiv_rn(__dmul_rn(w12, w12), w1), zw1[it.o1 + i]));
    }
}

// T2: pairs of pixels seen from the same quasar (one block per quasar).
__global__ void xf_t2(XfConst c, XfItem it, pg_forest_set forests, const double *x1, int nz,
                      XfScratch s) {
    for (int j = blockIdx.x; j < it.nq; j += gridDim.x) {
        const int lo = s.lo[j], hi = s.hi[j];
        if (hi < lo) continue;
        const int len = hi - lo + 1;
        const double z2 = __dmul_rn(s.qzw[j], s.qzw[j]);
        for (int t = threadIdx.x; t < len * len; t += blockDim.x) {
            const int i = lo + t / len, k = lo + t % len;
            if (i == k) continue;
            const int bi = xf_bin(c, forests.r_comov[it.o1 + i], s.qr[j], s.qcos[j], s.qsin[j]);
            const int bk = xf_bin(c, forests.r_comov[it.o1 + k], s.qr[j], s.qcos[j], s.qsin[j]);
            if (bi < 0 || bk < 0) continue;
            atomicAdd(&s.T2[(int64_t)s.col[bi] * nz + s.col[bk]],
                      __dmul_rn(x1[(int64_t)i * it.n1 + k], z2));
        }
    }
}

// C[m][n] = sum_k A[k][m] B[k][n] (row-major, FP64): 64 x 64 tiles, 256
// threads of 4 x 4 outputs, K in steps of 16 through shared memory.
constexpr int kGm = 64, kGn = 64, kGk = 16;

__global__ void __launch_bounds__(256)
    xf_gemm_tn(int m, int n, int k, const double *__restrict__ a, int64_t lda,
               const double *__restrict__ b, int64_t ldb, double *__restrict__ c, int64_t ldc) {
    __shared__ double as[kGk][kGm];
    __shared__ double bs[kGk][kGn];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * kGm, n0 = blockIdx.x * kGn;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < k; k0 += kGk) {
        for (int e = threadIdx.x; e < kGk * kGm; e += 256) {
            const int kk = e / kGm, mm = e % kGm;
            const int gk = k0 + kk, gm = m0 + mm, gn = n0 + mm;
            as[kk][mm] = (gk < k && gm < m) ? a[(int64_t)gk * lda + gm] : 0.;
            bs[kk][mm] = (gk < k && gn < n) ? b[(int64_t)gk * ldb + gn] : 0.;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGk; ++kk) {
            double av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                av[r] = as[kk][ty * 4 + r];
                bv[r] = bs[kk][tx * 4 + r];
            }
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[r][q] = fma(av[r], bv[q], acc[r][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int gm = m0 + ty * 4 + r;
        if (gm >= m) continue;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int gn = n0 + tx * 4 + q;
            if (gn < n) c[(int64_t)gm * ldc + gn] = acc[r][q];
        }
    }
}

// Add the forest's compact blocks to the (bin, bin) cells.
__global__ void xf_scatter(int nz, int nb, XfScratch s, pg_wick_sums out) {
    const int64_t total = (int64_t)nz * nz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int p = (int)(t / nz), q = (int)(t - (int64_t)p * nz);
        const int64_t cell = (int64_t)s.bins[p] * nb + s.bins[q];
        const double t2 = s.T2[t];
        out.t2[cell] += t2;
        out.t4[cell] += s.T24[t] - t2;
        out.t3[cell] += p == q ? s.T3[t] - s.D[p] : s.T3[t];
    }
}

XfScratch carve(char *work, int nb, int max_pixels, int max_quasars) {
    XfScratch s;
    auto take = [&](size_t bytes) {
        char *p = work;
        work += (bytes + 255) & ~(size_t)255;
        return p;
    };
    s.used = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * nb));
    s.col = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * nb));
    s.bins = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * nb));
    s.lo = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * max_quasars));
    s.hi = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * max_quasars));
    s.nz = reinterpret_cast<int32_t *>(take(sizeof(int32_t)));
    s.listed = reinterpret_cast<unsigned long long *>(take(sizeof(unsigned long long)));
    double **q[5] = {&s.qcos, &s.qsin, &s.qr, &s.qw, &s.qzw};
    for (double **p : q) *p = reinterpret_cast<double *>(take(sizeof(double) * max_quasars));
    double **mats[4] = {&s.U, &s.W, &s.Wc, &s.Y};
    for (double **p : mats)
        *p = reinterpret_cast<double *>(take(sizeof(double) * (size_t)max_pixels * nb));
    double **sq[3] = {&s.T24, &s.T3, &s.T2};
    for (double **p : sq) *p = reinterpret_cast<double *>(take(sizeof(double) * (size_t)nb * nb));
    s.D = reinterpret_cast<double *>(take(sizeof(double) * nb));
    return s;
}

}  // namespace

uint64_t xwick_factored_bytes(int nb, int max_pixels, int max_quasars) {
    auto r = [](uint64_t b) { return (b + 255) & ~(uint64_t)255; };
    return 3 * r(4ull * nb) + 2 * r(4ull * max_quasars) + r(4) + r(8) + 5 * r(8ull * max_quasars) +
           4 * r(8ull * max_pixels * nb) + 3 * r(8ull * nb * nb) + r(8ull * nb);
}

int run_xwick_factored(const pg_corr_params &p, const pg_forest_set &forests,
                       const pg_forest_set &objs, const double *zw1, const double *zw_obj,
                       const int64_t *xo_host, const double *xa, const int32_t *item_forest,
                       const int32_t *item_start, const int32_t *item_count,
                       const int32_t *obj_index, const double *obj_angle, int64_t num_items,
                       const int64_t *pix_offset_host, int max_pixels, int max_quasars,
                       char *work, const pg_wick_sums &out, Scratch *scratch, int num_sms,
                       cudaStream_t st) {
    XfConst c;
    c.r_par_min = p.r_par_min;
    c.r_par_max = p.r_par_max;
    c.r_trans_max = p.r_trans_max;
    c.range = p.r_par_max - p.r_par_min;
    c.np = p.num_bins_r_par;
    c.nt = p.num_bins_r_trans;
    c.nb = c.np * c.nt;
    c.pad = 0;
    XfScratch s = carve(work, c.nb, max_pixels, max_quasars);
    const int grid = num_sms * 4;
    unsigned long long pairs2 = 0, macs = 0, items_done = 0;
    for (int64_t q = 0; q < num_items; ++q) {
        XfItem it;
        it.f = item_forest[q];
        it.q0 = item_start[q];
        it.nq = item_count[q];
        it.o1 = pix_offset_host[it.f];
        it.n1 = (int)(pix_offset_host[it.f + 1] - it.o1);
        if (it.nq < 1 || it.n1 < 1) continue;
        if (it.nq > max_quasars || it.n1 > max_pixels) return PG_ERR_INVALID_ARGUMENT;
        cudaError_t err = cudaMemsetAsync(s.used, 0, sizeof(int32_t) * c.nb, st);
        if (err == cudaSuccess) err = cudaMemsetAsync(s.listed, 0, sizeof(unsigned long long), st);
        if (err != cudaSuccess) return check_cuda(err);
        xf_quasars<<<std::max(1, std::min(grid, (it.nq + kXfBlock - 1) / kXfBlock)), kXfBlock, 0,
                     st>>>(it, forests, objs, zw_obj, obj_index, obj_angle, s);
        xf_mark<<<grid, kXfBlock, 0, st>>>(c, it, forests, s);
        xf_scan<<<1, 1024, 0, st>>>(c.nb, s);
        int nz = 0;
        unsigned long long listed = 0;
        err = cudaMemcpyAsync(&nz, s.nz, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess)
            err = cudaMemcpyAsync(&listed, s.listed, sizeof(listed), cudaMemcpyDeviceToHost, st);
        if (err == cudaSuccess) err = cudaStreamSynchronize(st);
        if (err != cudaSuccess) return check_cuda(err);
        if (nz == 0) continue;
        pairs2 += listed * listed;
        macs += (unsigned long long)it.n1 * it.n1 * nz + 2ull * it.n1 * nz * nz;
        ++items_done;
        const size_t mat = sizeof(double) * (size_t)it.n1 * nz;
        double *zero[3] = {s.U, s.W, s.Wc};
        for (double *ptr : zero)
            if ((err = cudaMemsetAsync(ptr, 0, mat, st)) != cudaSuccess) return check_cuda(err);
        if ((err = cudaMemsetAsync(s.T2, 0, sizeof(double) * (size_t)nz * nz, st)) != cudaSuccess ||
            (err = cudaMemsetAsync(s.D, 0, sizeof(double) * nz, st)) != cudaSuccess)
            return check_cuda(err);
        xf_fill<<<grid, kXfBlock, 0, st>>>(c, it, forests, zw1, nz, s, out);
        const double *x1 = xa + xo_host[it.f];
        xf_t2<<<std::min(it.nq, grid * 2), kXfBlock, 0, st>>>(c, it, forests, x1, nz, s);
        // Y = X1'^T U (X1' symmetric), T24 = U^T Y, T3 = W^T (c W)
        const dim3 gy((nz + kGn - 1) / kGn, (it.n1 + kGm - 1) / kGm);
        xf_gemm_tn<<<gy, 256, 0, st>>>(it.n1, nz, it.n1, x1, it.n1, s.U, nz, s.Y, nz);
        const dim3 gt((nz + kGn - 1) / kGn, (nz + kGm - 1) / kGm);
        xf_gemm_tn<<<gt, 256, 0, st>>>(nz, nz, it.n1, s.U, nz, s.Y, nz, s.T24, nz);
        xf_gemm_tn<<<gt, 256, 0, st>>>(nz, nz, it.n1, s.W, nz, s.Wc, nz, s.T3, nz);
        xf_scatter<<<grid, kXfBlock, 0, st>>>(nz, c.nb, s, out);
        if ((err = cudaGetLastError()) != cudaSuccess) return check_cuda(err);
    }
    // run statistics for pg_plan_stats: work items, the (a, b) pairs the
    // sweep form would evaluate, and the GEMM multiply-adds
    cudaError_t err = cudaMemcpyAsync(&scratch->work_items, &items_done, sizeof(items_done),
                                      cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(&scratch->visited_pairs, &pairs2, sizeof(pairs2),
                              cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(&scratch->gemm_macs, &macs, sizeof(macs), cudaMemcpyHostToDevice,
                              st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    return check_cuda(err);
}

}  // namespace pg
