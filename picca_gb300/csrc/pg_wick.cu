// Wick covariance of the auto-correlation, terms T1-T3:
// cf.compute_wick_terms + cf.compute_wickT123_pairs (py/picca/cf.py:
// 1328-1495, :1498-1626), and of the delta x quasar cross-correlation,
// terms T1-T4: xcf.compute_wick_terms + xcf.compute_wickT1234_pairs
// (py/picca/xcf.py:838-1008, :1220-1351).
//
// For a forest pair the reference lists the pixel pairs inside the r_par /
// r_trans range with their bin, then visits every pair of listed pixel
// pairs (a, b): a shared pixel of forest 1 adds X2[j_a, j_b] w1 zw1 to T2, a
// shared pixel of forest 2 adds X1[i_a, i_b] w2 zw2 to T2, and otherwise
// X1[i_a, i_b] X2[j_a, j_b] goes to T3, in the cell (bin a, bin b) and its
// mirror. X is the weighted 1D correlation of a forest's own pixels,
// (w w^T) xi_1d(|dlog_lambda|) sqrt(v v^T). This is O(K^2) in the K listed
// pixel pairs of a forest pair.
//
// Two kernels:
//  * wick_xmat_kernel: X of each listed forest, once, into an arena (the
//    reference recomputes it for every pair). The diagonal is stored as 0:
//    no term uses it, and a zero there lets T3 run without branches. xi_1d
//    is scipy's nearest-neighbour rule (count of cell bounds below |dll|).
//  * wick_t123_kernel: one CTA per forest pair (persistent). It counts the
//    listed pixel pairs per bin in shared memory (with WALL, NB and the
//    diagonal T1), sorts them by bin into a per-CTA list (counting sort),
//    then every warp takes 32 pixel pairs a of one bin P and sweeps all b
//    in bin order: lanes read X1[i_b][i_a] and X2[j_b][j_a] (rows of the
//    symmetric matrices, so the 32 lanes touch one or two cache lines),
//    one FP64 FMA per (a, b) for T3 and predicated FMAs for the shared-pixel
//    T2 terms, and at each end of a bin Q the warp reduces and adds the
//    (P, Q) cell to the output with one atomic.
//  * xwick_kernel: the cross. A work item is one forest with its
//    neighbouring quasars (each with its own angle); the listed pairs are
//    (pixel, quasar). T2 (same quasar) and T4 (different quasars) are both
//    X1[i_a, i_b] zw_a zw_b: the sweep keeps the sum over all b and the
//    same-quasar part, T4 is their difference; T3 (same pixel) sums
//    w12_b and is scaled by w12_a / w1 zw1 at the flush.
// All arithmetic is FP64; the sums differ from the reference's only in
// summation order.
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kWkBlock = 512;   // auto: two CTAs per SM up to 2,500 bins
constexpr int kXwBlock = 1024;  // cross: one CTA per SM at 5,000 bins
constexpr int kXmBlock = 256;
constexpr int kWkBatch = 4;  // pixel pairs b whose loads are in flight together
// Listed pixel pair: i in bits 0-14, j in bits 15-30, bit 31 marks the last
// pair of its bin.
constexpr uint32_t kWkEnd = 0x80000000u;

__device__ __forceinline__ uint32_t wick_pack(int i, int j, bool last) {
    return (uint32_t)i | ((uint32_t)j << 15) | (last ? kWkEnd : 0u);
}
__device__ __forceinline__ int wick_i(uint32_t u) { return (int)(u & 0x7fffu); }
__device__ __forceinline__ int wick_j(uint32_t u) { return (int)((u >> 15) & 0xffffu); }

// Next 32-pair task of this CTA (a warp-wide counter in shared memory).
__device__ __forceinline__ int wick_next_task(int32_t *counter, int lane) {
    int t = 0;
    if (lane == 0) t = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, t, 0);
}

struct WickConst {
    double r_par_min, r_par_max, r_trans_max, range;
    int32_t np, nt, nb, x_correlation;
    int64_t cap;  // list entries per CTA
};

__global__ void __launch_bounds__(kXmBlock)
    wick_xmat_kernel(pg_forest_set s, const double *log_lambda, const double *variance,
                     const double *bounds, const double *values, int32_t num_values,
                     const int32_t *forests, int64_t num_forests, const int64_t *x_offsets,
                     double *arena) {
    extern __shared__ double xm_bounds[];
    for (int k = threadIdx.x; k < num_values - 1; k += kXmBlock) xm_bounds[k] = bounds[k];
    __syncthreads();
    for (int64_t q = blockIdx.x; q < num_forests; q += gridDim.x) {
        const int f = forests[q];
        const int64_t o = s.pix_offset[f];
        const int n = (int)(s.pix_offset[f + 1] - o);
        double *x = arena + x_offsets[f];
        for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += kXmBlock) {
            const int i = (int)(t / n), k = (int)(t - (int64_t)i * n);
            if (i == k) {
                x[t] = 0.;
                continue;
            }
            const double d = fabs(log_lambda[o + k] - log_lambda[o + i]);
            // searchsorted(bounds, d, 'left'): number of bounds below d
            int lo = 0, hi = num_values - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (xm_bounds[mid] < d)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            const double wi = s.weights[o + i], wk = s.weights[o + k];
            const double vi = variance[o + i], vk = variance[o + k];
            x[t] = ((wk * wi) * values[lo]) * sqrt(vk * vi);
        }
    }
}

// A work unit may be cut into slices run by different CTAs: each CTA lists
// the unit's pixel pairs itself (the order inside a bin differs from CTA to
// CTA), so a slice owns whole bins P (every slice-th nonempty bin) and
// sweeps all b for them.
struct WickSmem {
    int32_t *count;   // [nb] listed pixel pairs per bin, then the write cursor
    int32_t *start;   // [nb + 1] bin starts in the list
    int32_t *nonempty;  // [nb] bins with pixel pairs, ascending
    int32_t *own;     // [nb] nonempty bins of this slice
    int32_t *task_start;  // [nb + 1] first 32-pair task of each owned bin
    int32_t *npairs;  // [nb]
    double *wall, *t1;  // [nb]
    int32_t *scalars;  // num nonempty, num tasks, task counter
};

__device__ __forceinline__ WickSmem wick_smem(void *base, int nb) {
    WickSmem m;
    double *d = static_cast<double *>(base);
    m.wall = d;
    m.t1 = d + nb;
    int32_t *p = reinterpret_cast<int32_t *>(d + 2 * nb);
    m.count = p;
    m.start = p + nb;
    m.nonempty = m.start + nb + 1;
    m.own = m.nonempty + nb;
    m.task_start = m.own + nb;
    m.npairs = m.task_start + nb + 1;
    m.scalars = m.npairs + nb;
    return m;
}

// Bin of the pixel pair (i, j), or -1 outside the range (cf.py:1561-1594).
__device__ __forceinline__ int wick_bin(const WickConst &c, double r1, double r2, double cc,
                                        double ss) {
    double r_par = __dmul_rn(__dsub_rn(r1, r2), cc);
    if (!c.x_correlation) r_par = fabs(r_par);
    const double r_trans = __dmul_rn(__dadd_rn(r1, r2), ss);
    if (!(r_par < c.r_par_max && r_trans < c.r_trans_max && r_par >= c.r_par_min)) return -1;
    const int bp = (int)__dmul_rn(__ddiv_rn(__dsub_rn(r_par, c.r_par_min), c.range), (double)c.np);
    const int bt = (int)__dmul_rn(__ddiv_rn(r_trans, c.r_trans_max), (double)c.nt);
    // a quotient that rounds up to 1 would index past the last bin (the
    // reference writes out of bounds there); such a pair is dropped
    if (bp >= c.np || bt >= c.nt) return -1;
    return bt + c.nt * bp;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;
}

__global__ void __launch_bounds__(kWkBlock)
    wick_t123_kernel(WickConst c, pg_forest_set s1, pg_forest_set s2, const double *zw1,
                     const double *zw2, const int64_t *xo1, const double *xa1,
                     const int64_t *xo2, const double *xa2, const int32_t *pair_first,
                     const int32_t *pair_second, const double *pair_angle,
                     const int32_t *unit_slice, const int32_t *unit_slices, int64_t num_pairs,
                     uint32_t *work, pg_wick_sums out, Scratch *scratch) {
    extern __shared__ double wk_smem[];
    __shared__ int s_item;
    const int nb = c.nb, tid = threadIdx.x, lane = tid & 31;
    WickSmem m = wick_smem(wk_smem, nb);
    uint32_t *list = work + (int64_t)blockIdx.x * c.cap;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&scratch->work_counter, 1);
        for (int k = tid; k < nb; k += kWkBlock) {
            m.count[k] = 0;
            m.npairs[k] = 0;
            m.wall[k] = 0.;
            m.t1[k] = 0.;
        }
        __syncthreads();
        const int64_t q = s_item;
        if (q >= num_pairs) break;
        const int f = pair_first[q], g = pair_second[q];
        const int slice = unit_slice ? unit_slice[q] : 0, slices = unit_slices ? unit_slices[q] : 1;
        const double ang = pair_angle ? pair_angle[q]
                                      : angle_between(s1.x_cart[f], s1.y_cart[f], s1.z_cart[f],
                                                      s1.ra[f], s1.dec[f], s1.cos_dec[f],
                                                      s2.x_cart[g], s2.y_cart[g], s2.z_cart[g],
                                                      s2.ra[g], s2.dec[g]);
        const double cc = cos(ang / 2), ss = sin(ang / 2);
        const int64_t o1 = s1.pix_offset[f], o2 = s2.pix_offset[g];
        const int n1 = (int)(s1.pix_offset[f + 1] - o1), n2 = (int)(s2.pix_offset[g + 1] - o2);
        const int64_t grid = (int64_t)n1 * n2;
        if (grid > c.cap) {
            if (tid == 0) report_error(scratch, PG_ERR_INVALID_ARGUMENT, (int32_t)q);
            __syncthreads();
            continue;
        }
        if (tid == 0 && slice == 0) atomicAdd(&scratch->work_items, 1ull);
        // pass 1: counts, WALL, NB and T1 per bin
        for (int64_t t = tid; t < grid; t += kWkBlock) {
            const int j = (int)(t / n1), i = (int)(t - (int64_t)j * n1);
            const int b = wick_bin(c, s1.r_comov[o1 + i], s2.r_comov[o2 + j], cc, ss);
            if (b < 0) continue;
            const double w12 = __dmul_rn(s1.weights[o1 + i], s2.weights[o2 + j]);
            atomicAdd(&m.count[b], 1);
            atomicAdd(&m.npairs[b], 1);
            atomicAdd(&m.wall[b], w12);
            atomicAdd(&m.t1[b], __dmul_rn(w12, __dmul_rn(zw1[o1 + i], zw2[o2 + j])));
        }
        __syncthreads();
        if (tid == 0) {
            int run = 0, nz = 0, owned = 0, tasks = 0;
            for (int b = 0; b < nb; ++b) {
                const int n = m.count[b];
                m.start[b] = run;
                m.count[b] = run;  // write cursor
                if (n) {
                    if (nz % slices == slice) {
                        m.own[owned] = b;
                        m.task_start[owned] = tasks;
                        tasks += (n + 31) >> 5;
                        ++owned;
                    }
                    m.nonempty[nz] = b;
                    ++nz;
                }
                run += n;
            }
            m.start[nb] = run;
            m.task_start[owned] = tasks;
            m.scalars[3] = owned;
            m.scalars[0] = nz;
            m.scalars[1] = tasks;
            m.scalars[2] = 0;
            // (a, b) pairs of listed pixel pairs the sweep evaluates
            if (slice == 0)
                atomicAdd(&scratch->visited_pairs,
                          (unsigned long long)run * (unsigned long long)run);
        }
        __syncthreads();
        const int nz = m.scalars[0], num_tasks = m.scalars[1];
        // pass 2: list of (i, j) sorted by bin
        for (int64_t t = tid; t < grid; t += kWkBlock) {
            const int j = (int)(t / n1), i = (int)(t - (int64_t)j * n1);
            const int b = wick_bin(c, s1.r_comov[o1 + i], s2.r_comov[o2 + j], cc, ss);
            if (b < 0) continue;
            const int pos = atomicAdd(&m.count[b], 1);
            list[pos] = wick_pack(i, j, pos == m.start[b + 1] - 1);
        }
        for (int k = tid; k < nz && slice == 0; k += kWkBlock) {
            const int b = m.nonempty[k];
            atomicAdd(&out.weights_wick[b], m.wall[b]);
            atomicAdd(reinterpret_cast<unsigned long long *>(&out.num_pairs_wick[b]),
                      (unsigned long long)m.npairs[b]);
            atomicAdd(&out.t1[(int64_t)b * nb + b], m.t1[b]);
        }
        __syncthreads();
        const int num_listed = m.start[nb];
        const double *__restrict__ x1 = xa1 + xo1[f];
        const double *__restrict__ x2 = xa2 + xo2[g];
        for (;;) {
            const int task = wick_next_task(&m.scalars[2], lane);
            if (task >= num_tasks) break;
            // the nonempty bin holding this task
            int lo = 0, hi = m.scalars[3] - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (m.task_start[mid] <= task)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int bin_p = m.own[lo];
            const int a = m.start[bin_p] + ((task - m.task_start[lo]) << 5) + lane;
            const bool valid = a < m.start[bin_p + 1];
            const uint32_t ua = valid ? list[a] : 0u;
            const int ia = wick_i(ua), ja = wick_j(ua);
            const double c1a = valid ? __dmul_rn(s1.weights[o1 + ia], zw1[o1 + ia]) : 0.;
            const double c2a = valid ? __dmul_rn(s2.weights[o2 + ja], zw2[o2 + ja]) : 0.;
            double acc3 = 0., acc2 = 0.;
            bool have2 = false;  // warp-uniform: acc2 got terms since the last flush
            int kq = 0;
            for (int b0 = 0; b0 < num_listed; b0 += 32) {
                const int nbatch = min(32, num_listed - b0);
                const uint32_t mine = lane < nbatch ? list[b0 + lane] : 0u;
                // b of this batch that share a pixel with some lane: their T2
                // terms are added after the branch-free T3 sweep (a predicated
                // FP64 FMA would take the FP64 pipe for the whole warp)
                uint32_t pending = 0u;
                auto drain = [&]() {
                    if (pending) have2 = true;
                    while (pending) {
                        const int k = __ffs(pending) - 1;
                        pending &= pending - 1u;
                        const uint32_t u = __shfl_sync(0xffffffffu, mine, k);
                        const int ib = wick_i(u), jb = wick_j(u);
                        if (ia == ib) acc2 = fma(__ldg(x2 + (int64_t)jb * n2 + ja), c1a, acc2);
                        if (ja == jb) acc2 = fma(__ldg(x1 + (int64_t)ib * n1 + ia), c2a, acc2);
                    }
                };
                for (int k = 0; k < nbatch; k += kWkBatch) {
                    uint32_t ub[kWkBatch];
                    double v1[kWkBatch], v2[kWkBatch];
#pragma unroll
                    for (int r = 0; r < kWkBatch; ++r) {
                        ub[r] = __shfl_sync(0xffffffffu, mine, (k + r) & 31);
                        v1[r] = __ldg(x1 + (int64_t)wick_i(ub[r]) * n1 + ia);
                        v2[r] = __ldg(x2 + (int64_t)wick_j(ub[r]) * n2 + ja);
                    }
#pragma unroll
                    for (int r = 0; r < kWkBatch; ++r) {
                        if (k + r >= nbatch) break;
                        acc3 = fma(v1[r], v2[r], acc3);
                        const bool shared = ia == wick_i(ub[r]) || ja == wick_j(ub[r]);
                        if (__any_sync(0xffffffffu, shared)) pending |= 1u << (k + r);
                        if (ub[r] & kWkEnd) {
                            drain();
                            // the reduction's additions run on the FP64 pipe
                            // too: T2's only when this bin had shared pixels
                            const double r3 = warp_sum(valid ? acc3 : 0.);
                            const double r2 = have2 ? warp_sum(valid ? acc2 : 0.) : 0.;
                            if (lane == 0) {
                                const int64_t cell = (int64_t)bin_p * nb + m.nonempty[kq];
                                if (r3 != 0.) atomicAdd(&out.t3[cell], r3);
                                if (r2 != 0.) atomicAdd(&out.t2[cell], r2);
                            }
                            acc3 = acc2 = 0.;
                            have2 = false;
                            ++kq;
                        }
                    }
                }
                drain();
            }
        }
        __syncthreads();
    }
}

struct XWickConst {
    double r_par_min, r_par_max, r_trans_max, range;
    int32_t np, nt, nb, pad;
    int64_t cap, max_quasars;
};

// Bin of a (pixel, quasar) pair, or -1 (xcf.py:1282-1316, r_par signed).
__device__ __forceinline__ int xwick_bin(const XWickConst &c, double r1, double r2, double cc,
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

__global__ void __launch_bounds__(kXwBlock)
    xwick_kernel(XWickConst c, pg_forest_set forests, pg_forest_set objs, const double *zw1,
                 const double *zw_obj, const int64_t *xo, const double *xa,
                 const int32_t *item_forest, const int32_t *item_start,
                 const int32_t *item_count, const int32_t *obj_index, const double *obj_angle,
                 const int32_t *unit_slice, const int32_t *unit_slices, int64_t num_items,
                 char *work, int64_t cta_bytes, pg_wick_sums out, Scratch *scratch) {
    extern __shared__ double wk_smem[];
    __shared__ int s_item;
    const int nb = c.nb, tid = threadIdx.x, lane = tid & 31;
    WickSmem m = wick_smem(wk_smem, nb);
    char *base = work + (int64_t)blockIdx.x * cta_bytes;
    double *zql = reinterpret_cast<double *>(base);                  // [cap]
    double *q_cos = zql + c.cap, *q_sin = q_cos + c.max_quasars;       // [max_quasars]
    double *q_r = q_sin + c.max_quasars, *q_w = q_r + c.max_quasars, *q_zw = q_w + c.max_quasars;
    uint32_t *list = reinterpret_cast<uint32_t *>(q_zw + c.max_quasars);  // [cap]
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&scratch->work_counter, 1);
        for (int k = tid; k < nb; k += kXwBlock) {
            m.count[k] = 0;
            m.npairs[k] = 0;
            m.wall[k] = 0.;
            m.t1[k] = 0.;
        }
        __syncthreads();
        const int64_t q = s_item;
        if (q >= num_items) break;
        const int f = item_forest[q];
        const int32_t q0 = item_start[q], nq = item_count[q];
        const int slice = unit_slice ? unit_slice[q] : 0, slices = unit_slices ? unit_slices[q] : 1;
        const int64_t o1 = forests.pix_offset[f];
        const int n1 = (int)(forests.pix_offset[f + 1] - o1);
        const int64_t grid = (int64_t)n1 * nq;
        if (nq > c.max_quasars || grid > c.cap) {
            if (tid == 0) report_error(scratch, PG_ERR_INVALID_ARGUMENT, (int32_t)q);
            __syncthreads();
            continue;
        }
        if (tid == 0 && slice == 0) atomicAdd(&scratch->work_items, 1ull);
        for (int k = tid; k < nq; k += kXwBlock) {
            const int g = obj_index[q0 + k];
            const double ang =
                obj_angle ? obj_angle[q0 + k]
                          : angle_between(forests.x_cart[f], forests.y_cart[f], forests.z_cart[f],
                                          forests.ra[f], forests.dec[f], forests.cos_dec[f],
                                          objs.x_cart[g], objs.y_cart[g], objs.z_cart[g],
                                          objs.ra[g], objs.dec[g]);
            q_cos[k] = cos(ang / 2);
            q_sin[k] = sin(ang / 2);
            q_r[k] = objs.obj_r_comov[g];
            q_w[k] = objs.obj_weight[g];
            q_zw[k] = zw_obj[g];
        }
        __syncthreads();
        // pass 1: counts, WALL, NB and T1 = w12^2 / w1 zw1 per bin
        for (int64_t t = tid; t < grid; t += kXwBlock) {
            const int j = (int)(t / n1), i = (int)(t - (int64_t)j * n1);
            const int b = xwick_bin(c, forests.r_comov[o1 + i], q_r[j], q_cos[j], q_sin[j]);
            if (b < 0) continue;
            const double w1 = forests.weights[o1 + i];
            const double w12 = __dmul_rn(w1, q_w[j]);
            atomicAdd(&m.count[b], 1);
            atomicAdd(&m.npairs[b], 1);
            atomicAdd(&m.wall[b], w12);
            atomicAdd(&m.t1[b], __dmul_rn(__ddiv_rn(__dmul_rn(w12, w12), w1), zw1[o1 + i]));
        }
        __syncthreads();
        if (tid == 0) {
            int run = 0, nz = 0, owned = 0, tasks = 0;
            for (int b = 0; b < nb; ++b) {
                const int n = m.count[b];
                m.start[b] = run;
                m.count[b] = run;
                if (n) {
                    if (nz % slices == slice) {
                        m.own[owned] = b;
                        m.task_start[owned] = tasks;
                        tasks += (n + 31) >> 5;
                        ++owned;
                    }
                    m.nonempty[nz] = b;
                    ++nz;
                }
                run += n;
            }
            m.start[nb] = run;
            m.task_start[owned] = tasks;
            m.scalars[3] = owned;
            m.scalars[0] = nz;
            m.scalars[1] = tasks;
            m.scalars[2] = 0;
            // (a, b) pairs of listed pixel pairs the sweep evaluates
            if (slice == 0)
                atomicAdd(&scratch->visited_pairs,
                          (unsigned long long)run * (unsigned long long)run);
        }
        __syncthreads();
        const int nz = m.scalars[0], num_tasks = m.scalars[1];
        for (int64_t t = tid; t < grid; t += kXwBlock) {
            const int j = (int)(t / n1), i = (int)(t - (int64_t)j * n1);
            const int b = xwick_bin(c, forests.r_comov[o1 + i], q_r[j], q_cos[j], q_sin[j]);
            if (b < 0) continue;
            const int pos = atomicAdd(&m.count[b], 1);
            list[pos] = wick_pack(i, j, pos == m.start[b + 1] - 1);
            zql[pos] = q_zw[j];
        }
        for (int k = tid; k < nz && slice == 0; k += kXwBlock) {
            const int b = m.nonempty[k];
            atomicAdd(&out.weights_wick[b], m.wall[b]);
            atomicAdd(reinterpret_cast<unsigned long long *>(&out.num_pairs_wick[b]),
                      (unsigned long long)m.npairs[b]);
            atomicAdd(&out.t1[(int64_t)b * nb + b], m.t1[b]);
        }
        __syncthreads();
        const int num_listed = m.start[nb];
        const double *__restrict__ x1 = xa + xo[f];
        for (;;) {
            const int task = wick_next_task(&m.scalars[2], lane);
            if (task >= num_tasks) break;
            int lo = 0, hi = m.scalars[3] - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (m.task_start[mid] <= task)
                    lo = mid;
                else
                    hi = mid - 1;
            }
            const int bin_p = m.own[lo];
            const int a = m.start[bin_p] + ((task - m.task_start[lo]) << 5) + lane;
            const bool valid = a < m.start[bin_p + 1];
            const uint32_t ua = valid ? list[a] : 0u;
            const int ia = wick_i(ua), ja = wick_j(ua);
            const double w1a = forests.weights[o1 + ia];
            const double zwa = valid ? q_zw[ja] : 0.;
            // T3 scale: w12_a / w1 zw1 (xcf.py:1335-1341)
            const double c3a =
                valid ? __dmul_rn(__ddiv_rn(__dmul_rn(w1a, q_w[ja]), w1a), zw1[o1 + ia]) : 0.;
            double acc_all = 0., acc2 = 0., acc3 = 0.;
            int kq = 0;
            for (int b0 = 0; b0 < num_listed; b0 += 32) {
                const int nbatch = min(32, num_listed - b0);
                const uint32_t mine = lane < nbatch ? list[b0 + lane] : 0u;
                const double zmine = lane < nbatch ? zql[b0 + lane] : 0.;
                // b sharing the quasar (T2) or the pixel (T3) with some lane,
                // added after the branch-free sweep
                uint32_t pending = 0u;
                auto drain = [&]() {
                    while (pending) {
                        const int k = __ffs(pending) - 1;
                        pending &= pending - 1u;
                        const uint32_t u = __shfl_sync(0xffffffffu, mine, k);
                        const double z = __shfl_sync(0xffffffffu, zmine, k);
                        const int ib = wick_i(u), jb = wick_j(u);
                        if (ja == jb)
                            acc2 = fma(__ldg(x1 + (int64_t)ib * n1 + ia), z, acc2);
                        else if (ia == ib)
                            acc3 += __dmul_rn(forests.weights[o1 + ib], q_w[jb]);
                    }
                };
                for (int k = 0; k < nbatch; k += kWkBatch) {
                    uint32_t ub[kWkBatch];
                    double v1[kWkBatch], zb[kWkBatch];
#pragma unroll
                    for (int r = 0; r < kWkBatch; ++r) {
                        ub[r] = __shfl_sync(0xffffffffu, mine, (k + r) & 31);
                        zb[r] = __shfl_sync(0xffffffffu, zmine, (k + r) & 31);
                        v1[r] = __ldg(x1 + (int64_t)wick_i(ub[r]) * n1 + ia);
                    }
#pragma unroll
                    for (int r = 0; r < kWkBatch; ++r) {
                        if (k + r >= nbatch) break;
                        acc_all = fma(v1[r], zb[r], acc_all);
                        const bool shared = ja == wick_j(ub[r]) || ia == wick_i(ub[r]);
                        if (__any_sync(0xffffffffu, shared)) pending |= 1u << (k + r);
                        if (ub[r] & kWkEnd) {
                            drain();
                            const double r2 = warp_sum(valid ? zwa * acc2 : 0.);
                            const double r4 = warp_sum(valid ? zwa * (acc_all - acc2) : 0.);
                            const double r3 = warp_sum(valid ? c3a * acc3 : 0.);
                            if (lane == 0) {
                                const int64_t cell = (int64_t)bin_p * nb + m.nonempty[kq];
                                if (r2 != 0.) atomicAdd(&out.t2[cell], r2);
                                if (r3 != 0.) atomicAdd(&out.t3[cell], r3);
                                if (r4 != 0.) atomicAdd(&out.t4[cell], r4);
                            }
                            acc_all = acc2 = acc3 = 0.;
                            ++kq;
                        }
                    }
                }
                drain();
            }
        }
        __syncthreads();
    }
}

}  // namespace

int wick_xmat_smem(int num_values) { return (int)(sizeof(double) * std::max(1, num_values - 1)); }

int launch_wick_xmat(const pg_forest_set &s, const double *log_lambda, const double *variance,
                     const double *bounds, const double *values, int32_t num_values,
                     const int32_t *forests, int64_t num_forests, const int64_t *x_offsets,
                     double *arena, int num_sms, cudaStream_t stream) {
    if (num_forests == 0) return PG_OK;
    const int smem = wick_xmat_smem(num_values);
    cudaError_t err = cudaFuncSetAttribute(
        wick_xmat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (err != cudaSuccess) return check_cuda(err);
    const int64_t grid = std::min<int64_t>((int64_t)num_sms * 8, num_forests);
    wick_xmat_kernel<<<(int)grid, kXmBlock, smem, stream>>>(s, log_lambda, variance, bounds,
                                                            values, num_values, forests,
                                                            num_forests, x_offsets, arena);
    return check_cuda(cudaGetLastError());
}

size_t wick_t123_smem(int nb) {
    return (size_t)2 * nb * sizeof(double) + ((size_t)6 * nb + 2 + 4) * sizeof(int32_t);
}

int wick_t123_grid(int nb, int num_sms, int *grid) {
    const size_t smem = wick_t123_smem(nb);
    cudaError_t err = cudaFuncSetAttribute(
        wick_t123_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int occ = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, wick_t123_kernel, kWkBlock, smem);
    if (err != cudaSuccess || occ < 1) return PG_ERR_CUDA;
    *grid = num_sms * occ;
    return PG_OK;
}

int launch_wick_t123(const pg_corr_params &p, const pg_forest_set &s1, const pg_forest_set &s2,
                     const double *zw1, const double *zw2, const int64_t *xo1,
                     const double *xa1, const int64_t *xo2, const double *xa2,
                     const int32_t *pair_first, const int32_t *pair_second,
                     const double *pair_angle, const int32_t *unit_slice,
                     const int32_t *unit_slices, int64_t num_pairs, uint32_t *work,
                     int64_t cap, int grid, const pg_wick_sums &out, Scratch *scratch,
                     cudaStream_t stream) {
    if (num_pairs == 0) return PG_OK;
    WickConst c;
    c.r_par_min = p.r_par_min;
    c.r_par_max = p.r_par_max;
    c.r_trans_max = p.r_trans_max;
    c.range = p.r_par_max - p.r_par_min;
    c.np = p.num_bins_r_par;
    c.nt = p.num_bins_r_trans;
    c.nb = c.np * c.nt;
    c.x_correlation = p.x_correlation;
    c.cap = cap;
    const size_t smem = wick_t123_smem(c.nb);
    const int64_t blocks = std::min<int64_t>(grid, num_pairs);
    wick_t123_kernel<<<(int)blocks, kWkBlock, smem, stream>>>(
        c, s1, s2, zw1, zw2, xo1, xa1, xo2, xa2, pair_first, pair_second, pair_angle, unit_slice,
        unit_slices, num_pairs, work, out, scratch);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg

namespace pg {

int64_t xwick_cta_bytes(int64_t cap, int64_t max_quasars) {
    const int64_t bytes = cap * (int64_t)sizeof(double) + 5 * max_quasars * (int64_t)sizeof(double) +
                          cap * (int64_t)sizeof(uint32_t);
    return (bytes + 255) & ~(int64_t)255;
}

int xwick_grid(int nb, int num_sms, int *grid) {
    const size_t smem = wick_t123_smem(nb);
    cudaError_t err = cudaFuncSetAttribute(
        xwick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    int occ = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, xwick_kernel, kXwBlock, smem);
    if (err != cudaSuccess || occ < 1) return PG_ERR_CUDA;
    *grid = num_sms * occ;
    return PG_OK;
}

int launch_xwick(const pg_corr_params &p, const pg_forest_set &forests, const pg_forest_set &objs,
                 const double *zw1, const double *zw_obj, const int64_t *xo, const double *xa,
                 const int32_t *item_forest, const int32_t *item_start, const int32_t *item_count,
                 const int32_t *obj_index, const double *obj_angle, const int32_t *unit_slice,
                 const int32_t *unit_slices, int64_t num_items, char *work, int64_t cap,
                 int64_t max_quasars, int grid, const pg_wick_sums &out, Scratch *scratch,
                 cudaStream_t stream) {
    if (num_items == 0) return PG_OK;
    XWickConst c;
    c.r_par_min = p.r_par_min;
    c.r_par_max = p.r_par_max;
    c.r_trans_max = p.r_trans_max;
    c.range = p.r_par_max - p.r_par_min;
    c.np = p.num_bins_r_par;
    c.nt = p.num_bins_r_trans;
    c.nb = c.np * c.nt;
    c.pad = 0;
    c.cap = cap;
    c.max_quasars = max_quasars;
    const size_t smem = wick_t123_smem(c.nb);
    const int64_t blocks = std::min<int64_t>(grid, num_items);
    xwick_kernel<<<(int)blocks, kXwBlock, smem, stream>>>(
        c, forests, objs, zw1, zw_obj, xo, xa, item_forest, item_start, item_count, obj_index,
        obj_angle, unit_slice, unit_slices, num_items, work, xwick_cta_bytes(cap, max_quasars),
        out, scratch);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
