// Plain all-FP64 pair accumulation (the "plain GPU drop-in" form).
//
// Persistent kernel: each CTA pops a work item (one forest of set 1 with all
// of its neighbours) from a global counter, accumulates every pixel pair in
// FP64 with exactly the decisions and operation order of
// cf.compute_xi_forest_pairs_fast (py/picca/cf.py:250-387) or
// xcf.compute_xi_forest_pairs_fast (py/picca/xcf.py:223-322), into a
// per-CTA shared-memory histogram (FP64 sums, int32 counts), and adds the
// histogram to the FP64 row of the forest's healpix when the item is done.
// When the histogram does not fit in shared memory the kernel adds straight
// into the global rows.
//
// cf mapping: warps take neighbour forests round-robin; within a forest pair
// lanes own pixels j of forest 2 and loop over the pixels i of forest 1.
// xcf mapping: lanes own quasars, looping over the forest's pixels.
#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kBlock64 = 512;

struct Hist64 {
    double *we, *xi, *rp, *rt, *z;
    int32_t *nb;       // shared-memory counts (nullptr: use nb64)
    int64_t *nb64;     // global counts
};

__device__ __forceinline__ void add_pair(const Hist64 &h, int64_t bin, double dw12, double w12,
                                         double r_par, double r_trans, double z) {
    atomicAdd(&h.xi[bin], dw12);
    atomicAdd(&h.we[bin], w12);
    atomicAdd(&h.rp[bin], __dmul_rn(r_par, w12));
    atomicAdd(&h.rt[bin], __dmul_rn(r_trans, w12));
    atomicAdd(&h.z[bin], __dmul_rn(z, w12));
    if (h.nb) atomicAdd(&h.nb[bin], 1);
    else atomicAdd((unsigned long long *)&h.nb64[bin], 1ull);
}

// Shared histogram layout: 5 * nbins doubles then nbins int32.
__device__ __forceinline__ Hist64 smem_hist(unsigned char *smem, int nbins) {
    double *d = reinterpret_cast<double *>(smem);
    Hist64 h;
    h.we = d;
    h.xi = d + nbins;
    h.rp = d + 2 * (size_t)nbins;
    h.rt = d + 3 * (size_t)nbins;
    h.z = d + 4 * (size_t)nbins;
    h.nb = reinterpret_cast<int32_t *>(d + 5 * (size_t)nbins);
    h.nb64 = nullptr;
    return h;
}

__device__ __forceinline__ Hist64 row_hist(const pg_xi_rows &out, int32_t row, int nbins) {
    const size_t o = (size_t)row * nbins;
    Hist64 h;
    h.we = out.weights + o;
    h.xi = out.xi + o;
    h.rp = out.r_par + o;
    h.rt = out.r_trans + o;
    h.z = out.z + o;
    h.nb = nullptr;
    h.nb64 = out.num_pairs + o;
    return h;
}

__device__ __forceinline__ void flush_hist(const Hist64 &s, const pg_xi_rows &out, int32_t row,
                                           int nbins) {
    const size_t o = (size_t)row * nbins;
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        const int32_t nb = s.nb[b];
        if (nb != 0) {
            atomicAdd(&out.weights[o + b], s.we[b]);
            atomicAdd(&out.xi[o + b], s.xi[b]);
            atomicAdd(&out.r_par[o + b], s.rp[b]);
            atomicAdd(&out.r_trans[o + b], s.rt[b]);
            atomicAdd(&out.z[o + b], s.z[b]);
            atomicAdd((unsigned long long *)&out.num_pairs[o + b], (unsigned long long)nb);
            s.we[b] = 0.; s.xi[b] = 0.; s.rp[b] = 0.; s.rt[b] = 0.; s.z[b] = 0.;
            s.nb[b] = 0;
        }
    }
}

__device__ __forceinline__ void zero_hist(const Hist64 &s, int nbins) {
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        s.we[b] = 0.; s.xi[b] = 0.; s.rp[b] = 0.; s.rt[b] = 0.; s.z[b] = 0.;
        s.nb[b] = 0;
    }
}

__device__ __forceinline__ int next_item(Scratch *scratch, int *slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(&scratch->work_counter, 1);
    __syncthreads();
    return *slot;
}

template <bool SMEM>
__global__ void __launch_bounds__(kBlock64) cf_xi_fp64_kernel(
    Binning b, pg_forest_set s1, pg_forest_set s2, const int64_t *__restrict__ nbr_offsets,
    const int32_t *__restrict__ nbr_index, const double *__restrict__ nbr_angle,
    const int32_t *__restrict__ work_order,
    int64_t num_work, pg_xi_rows out, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    Hist64 sh{};
    if (SMEM) {
        sh = smem_hist(smem, b.nbins);
        zero_hist(sh, b.nbins);
    }
    for (;;) {
        const int item = next_item(scratch, &item_slot);
        if (item >= num_work) break;
        const int64_t f1 = work_order ? work_order[item] : item;
        const int32_t row = s1.row[f1];
        const Hist64 h = SMEM ? sh : row_hist(out, row, b.nbins);
        const int64_t a0 = s1.pix_offset[f1], n1 = s1.pix_offset[f1 + 1] - a0;
        const double x1 = s1.x_cart[f1], y1 = s1.y_cart[f1], zc1 = s1.z_cart[f1];
        const double ra1 = s1.ra[f1], dec1 = s1.dec[f1], cd1 = s1.cos_dec[f1];
        const double zq1 = s1.z_qso[f1];
        const int64_t k0 = nbr_offsets[f1], k1 = nbr_offsets[f1 + 1];
        for (int64_t k = k0 + warp; k < k1; k += nwarps) {
            const int64_t g = nbr_index[k];
            const double ang = nbr_angle ? nbr_angle[k]
                                         : angle_between(x1, y1, zc1, ra1, dec1, cd1, s2.x_cart[g],
                                                         s2.y_cart[g], s2.z_cart[g], s2.ra[g],
                                                         s2.dec[g]);
            const double c = cos(ang / 2), s = sin(ang / 2);
            bool shp = false;
            if (b.remove_shp) {
                const int64_t p1 = s1.plate[f1], p2 = s2.plate[g];
                const int64_t fb1 = s1.fiberid[f1], fb2 = s2.fiberid[g];
                shp = (p1 == p2) && ((fb1 <= 500 && fb2 <= 500) || (fb1 > 500 && fb2 > 500));
            }
            const bool zerr_pair = b.zerr_on && (ang < b.zerr_ang);
            const double zq2 = s2.z_qso[g];
            const int64_t b0 = s2.pix_offset[g], n2 = s2.pix_offset[g + 1] - b0;
            for (int64_t jb = 0; jb < n2; jb += 32) {
                const int64_t j = jb + lane;
                const bool jvalid = j < n2;
                double z2 = 0, r2 = 0, m2 = 0, w2 = 0, dw2 = 0;
                if (jvalid) {
                    z2 = s2.z[b0 + j];
                    r2 = s2.r_comov[b0 + j];
                    m2 = s2.dist_m[b0 + j];
                    w2 = s2.weights[b0 + j];
                    dw2 = __dmul_rn(s2.delta[b0 + j], w2);
                }
                bool jok = jvalid && (w2 != 0);
                if (jok && zerr_pair && zerr_veto(z2, zq1, b.zerr_kms)) jok = false;
                for (int64_t i = 0; i < n1; ++i) {
                    const double w1 = s1.weights[a0 + i];
                    if (w1 == 0) continue;
                    const double z1 = s1.z[a0 + i];
                    if (zerr_pair && zerr_veto(z1, zq2, b.zerr_kms)) continue;
                    if (!jok) continue;
                    double r_par, r_trans, z;
                    const int64_t bin = cf_pair_bin(b, z1, s1.r_comov[a0 + i], s1.dist_m[a0 + i],
                                                    z2, r2, m2, ang, c, s, shp, r_par, r_trans, z);
                    if (bin < 0) continue;
                    if (bin >= b.nbins) {
                        report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bin);
                        continue;
                    }
                    const double dw1 = __dmul_rn(s1.delta[a0 + i], w1);
                    add_pair(h, bin, __dmul_rn(dw1, dw2), __dmul_rn(w1, w2), r_par, r_trans, z);
                }
            }
        }
        if (SMEM) {
            __syncthreads();
            flush_hist(sh, out, row, b.nbins);
        }
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
}

template <bool SMEM>
__global__ void __launch_bounds__(kBlock64) xcf_xi_fp64_kernel(
    Binning b, pg_forest_set fs, pg_forest_set objs, const int64_t *__restrict__ nbr_offsets,
    const int32_t *__restrict__ nbr_index, const double *__restrict__ nbr_angle,
    const int32_t *__restrict__ work_order,
    int64_t num_work, pg_xi_rows out, Scratch *scratch) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int item_slot;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    Hist64 sh{};
    if (SMEM) {
        sh = smem_hist(smem, b.nbins);
        zero_hist(sh, b.nbins);
    }
    for (;;) {
        const int item = next_item(scratch, &item_slot);
        if (item >= num_work) break;
        const int64_t f = work_order ? work_order[item] : item;
        const int32_t row = fs.row[f];
        const Hist64 h = SMEM ? sh : row_hist(out, row, b.nbins);
        const int64_t a0 = fs.pix_offset[f], n1 = fs.pix_offset[f + 1] - a0;
        const double x1 = fs.x_cart[f], y1 = fs.y_cart[f], zc1 = fs.z_cart[f];
        const double ra1 = fs.ra[f], dec1 = fs.dec[f], cd1 = fs.cos_dec[f];
        const int64_t k0 = nbr_offsets[f], k1 = nbr_offsets[f + 1];
        // each warp takes 32 quasars at a time
        for (int64_t kb = k0 + (int64_t)warp * 32; kb < k1; kb += (int64_t)nwarps * 32) {
            const int64_t k = kb + lane;
            const bool valid = k < k1;
            double zq = 0, rq = 0, mq = 0, wq = 0, ang = 0, c = 0, s = 0;
            if (valid) {
                const int64_t g = nbr_index[k];
                ang = nbr_angle ? nbr_angle[k]
                                : angle_between(x1, y1, zc1, ra1, dec1, cd1, objs.x_cart[g],
                                                objs.y_cart[g], objs.z_cart[g], objs.ra[g],
                                                objs.dec[g]);
                c = cos(ang / 2);
                s = sin(ang / 2);
                zq = objs.z_qso[g];
                rq = objs.obj_r_comov[g];
                mq = objs.obj_dist_m[g];
                wq = objs.obj_weight[g];
            }
            const bool qok = valid && (wq != 0);
            for (int64_t i = 0; i < n1; ++i) {
                const double w1 = fs.weights[a0 + i];
                if (w1 == 0 || !qok) continue;
                double r_par, r_trans, z;
                const int64_t bin = xcf_pair_bin(b, fs.z[a0 + i], fs.r_comov[a0 + i],
                                                 fs.dist_m[a0 + i], zq, rq, mq, ang, c, s, r_par,
                                                 r_trans, z);
                if (bin < 0) continue;
                if (bin >= b.nbins) {
                    report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bin);
                    continue;
                }
                // delta1[i] * weights1[i] * weights2[j], left to right
                const double dw = __dmul_rn(__dmul_rn(fs.delta[a0 + i], w1), wq);
                add_pair(h, bin, dw, __dmul_rn(w1, wq), r_par, r_trans, z);
            }
        }
        if (SMEM) {
            __syncthreads();
            flush_hist(sh, out, row, b.nbins);
        }
        if (threadIdx.x == 0) atomicAdd(&scratch->work_items, 1ull);
    }
}

template <typename K>
int launch_persistent(K kernel, size_t smem, int num_sms, int64_t num_work, cudaStream_t stream,
                      int *grid_out) {
    if (smem > 48 * 1024) {
        cudaError_t err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
        if (err != cudaSuccess) return check_cuda(err);
    }
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock64, smem);
    if (err != cudaSuccess) return check_cuda(err);
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    if (grid > num_work) grid = num_work;
    if (grid < 1) grid = 1;
    *grid_out = (int)grid;
    return PG_OK;
}

size_t hist64_bytes(int nbins) { return (size_t)nbins * (5 * sizeof(double) + sizeof(int32_t)); }

}  // namespace

int launch_cf_xi_fp64(const Binning &b, const pg_forest_set &s1, const pg_forest_set &s2,
                      const int64_t *nbr_offsets, const int32_t *nbr_index, const double *nbr_angle,
                      const int32_t *work_order, int64_t num_work, const pg_xi_rows &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream) {
    if (num_work <= 0) return PG_OK;
    const size_t smem = hist64_bytes(b.nbins);
    int grid = 0, rc;
    if (smem <= 220 * 1024) {
        rc = launch_persistent(cf_xi_fp64_kernel<true>, smem, num_sms, num_work, stream, &grid);
        if (rc) return rc;
        cf_xi_fp64_kernel<true><<<grid, kBlock64, smem, stream>>>(
            b, s1, s2, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out, scratch);
    } else {
        rc = launch_persistent(cf_xi_fp64_kernel<false>, 0, num_sms, num_work, stream, &grid);
        if (rc) return rc;
        cf_xi_fp64_kernel<false><<<grid, kBlock64, 0, stream>>>(
            b, s1, s2, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out, scratch);
    }
    return check_cuda(cudaGetLastError());
}

int launch_xcf_xi_fp64(const Binning &b, const pg_forest_set &forests, const pg_forest_set &objs,
                       const int64_t *nbr_offsets, const int32_t *nbr_index, const double *nbr_angle,
                       const int32_t *work_order, int64_t num_work, const pg_xi_rows &out,
                       Scratch *scratch, int num_sms, cudaStream_t stream) {
    if (num_work <= 0) return PG_OK;
    const size_t smem = hist64_bytes(b.nbins);
    int grid = 0, rc;
    if (smem <= 220 * 1024) {
        rc = launch_persistent(xcf_xi_fp64_kernel<true>, smem, num_sms, num_work, stream, &grid);
        if (rc) return rc;
        xcf_xi_fp64_kernel<true><<<grid, kBlock64, smem, stream>>>(
            b, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out, scratch);
    } else {
        rc = launch_persistent(xcf_xi_fp64_kernel<false>, 0, num_sms, num_work, stream, &grid);
        if (rc) return rc;
        xcf_xi_fp64_kernel<false><<<grid, kBlock64, 0, stream>>>(
            b, forests, objs, nbr_offsets, nbr_index, nbr_angle, work_order, num_work, out, scratch);
    }
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
