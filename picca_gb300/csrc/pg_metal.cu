// Metal distortion matrices: cf.compute_metal_dmat (py/picca/cf.py:890-1218)
// and, with the quasars as one-pixel forests, xcf.compute_metal_dmat
// (py/picca/xcf.py:677-800).
//
// For every kept forest pair the reference bins all pixel pairs twice: with
// the tracer's distances (data bin, r_par / r_trans of the delta files) and
// with the distances the two pixels would have if they were absorbers abs1 /
// abs2 (model bin), and adds w1 w2 to the data-bin weights and
// w1 w2 zevol to the (data bin, model bin) cell and the model bin's
// effective r_par / r_trans / z / weight (numpy bincounts). Pixels whose
// absorber redshift is not below the quasar redshift are dropped; the caller
// encodes that as a zero weight in the absorber arrays. Here a CTA runs one
// kept forest pair per work item, a thread per pixel of forest 1 walks the
// pixels of forest 2, sums runs of pairs that share (data bin, model bin) in
// registers and adds each run with global atomics. All arithmetic is FP64 in
// the reference's expressions; the bin quotients are estimated with
// reciprocals and formed exactly next to a bin edge.
#include <algorithm>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kMdBlock = 256;

struct MetalConst {
    Binning b;
    int32_t nmp, nmt, nm;
    double inv_range, inv_rtmax;
    double inv_zevol_den;  // 1 / (1 + z_ref)^(alpha1 + alpha2 - 2)
    int32_t xcf;           // delta x quasar rules (py/picca/xcf.py:735-770)
};

__device__ __forceinline__ double md_floor(double est, double num, double den, int32_t n) {
    const double y = __dmul_rn(est, (double)n);
    const double f = floor(y);
    if (__dsub_rn(y, f) > 1e-9 && __dsub_rn(__dadd_rn(f, 1.), y) > 1e-9) return f;
    return floor(__dmul_rn(num / den, (double)n));
}

__global__ void __launch_bounds__(kMdBlock)
    metal_dmat_kernel(MetalConst c, pg_forest_set s1, pg_forest_set s2, pg_metal_pixels a1,
                      pg_metal_pixels a2, const int32_t *pair_first,
                      const int32_t *pair_second, const double *pair_angle, int64_t num_pairs,
                      pg_dmat_sums out, Scratch *scratch) {
    __shared__ int s_item;
    const int tid = threadIdx.x;
    const int nm = c.nm;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&scratch->work_counter, 1);
        __syncthreads();
        const int64_t q = s_item;
        __syncthreads();
        if (q >= num_pairs) break;
        const int f = pair_first[q], g = pair_second[q];
        const double ang = pair_angle ? pair_angle[q]
                                      : angle_between(s1.x_cart[f], s1.y_cart[f], s1.z_cart[f],
                                                      s1.ra[f], s1.dec[f], s1.cos_dec[f],
                                                      s2.x_cart[g], s2.y_cart[g], s2.z_cart[g],
                                                      s2.ra[g], s2.dec[g]);
        const double cc = cos(ang / 2), ss = sin(ang / 2);
        bool shp = false;
        if (c.b.remove_shp && s1.plate[f] == s2.plate[g]) {
            const int64_t fa = s1.fiberid[f], fb = s2.fiberid[g];
            shp = (fa <= 500 && fb <= 500) || (fa > 500 && fb > 500);
        }
        const int64_t o1 = s1.pix_offset[f], o2 = s2.pix_offset[g];
        const int n1 = (int)(s1.pix_offset[f + 1] - o1), n2 = (int)(s2.pix_offset[g + 1] - o2);
        if (tid == 0) atomicAdd(&scratch->work_items, 1ull);
        for (int i = tid; i < n1; i += kMdBlock) {
            const double w1 = a1.weights[o1 + i];
            if (w1 == 0.) continue;
            const double r1 = s1.r_comov[o1 + i], m1 = s1.dist_m[o1 + i];
            const double ra1 = a1.r_comov[o1 + i], ma1 = a1.dist_m[o1 + i];
            const double za1 = a1.z[o1 + i], zf1 = a1.zfac[o1 + i];
            // runs of equal data bin (weights) and of equal (data, model) bin
            int32_t run_b = -1;
            double k_w = 0.;
            int64_t run = -1;
            int32_t run_m = 0;
            double k_wz = 0., k_rp = 0., k_rt = 0., k_z = 0.;
            auto flush = [&]() {
                atomicAdd(&out.dmat[run], k_wz);
                atomicAdd(&out.r_par_eff[run_m], k_rp);
                atomicAdd(&out.r_trans_eff[run_m], k_rt);
                atomicAdd(&out.z_eff[run_m], k_z);
                atomicAdd(&out.weight_eff[run_m], k_wz);
            };
            for (int j = 0; j < n2; ++j) {
                const double w2 = a2.weights[o2 + j];
                if (w2 == 0.) continue;
                // data bin with the tracer's distances (cf.py:995-1021)
                double rp = __dmul_rn(__dsub_rn(r1, s2.r_comov[o2 + j]), cc);
                if (!c.b.x_correlation) rp = fabs(rp);
                const double rt = __dmul_rn(__dadd_rn(m1, s2.dist_m[o2 + j]), ss);
                if (shp && fabs(rp) < c.b.half_plate_cut) continue;  // weight set to 0
                // the cross tests the distances (strict), the auto its bin indices
                if (c.xcf && !(rp > c.b.r_par_min && rp < c.b.r_par_max &&
                               rt < c.b.r_trans_max))
                    continue;
                const double xp = __dsub_rn(rp, c.b.r_par_min);
                const double bp = md_floor(__dmul_rn(xp, c.inv_range), xp, c.b.r_par_range,
                                           c.b.np);
                const double bt = md_floor(__dmul_rn(rt, c.inv_rtmax), rt, c.b.r_trans_max,
                                           c.b.nt);
                if (!(bp < c.b.np && bt < c.b.nt && bp >= 0.)) {
                    if (c.xcf) report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)bp);
                    continue;
                }
                const double w12 = __dmul_rn(w1, w2);
                const int32_t b = (int32_t)bt + c.b.nt * (int32_t)bp;
                if (b != run_b) {
                    if (run_b >= 0) atomicAdd(&out.weights_dmat[run_b], k_w);
                    run_b = b;
                    k_w = 0.;
                }
                k_w += w12;
                // model bin with the absorbers' distances (cf.py:1023-1086)
                double rpa = __dmul_rn(__dsub_rn(ra1, a2.r_comov[o2 + j]), cc);
                if (!c.b.x_correlation) rpa = fabs(rpa);
                const double rta = __dmul_rn(__dadd_rn(ma1, a2.dist_m[o2 + j]), ss);
                if (c.xcf && !(rpa > c.b.r_par_min && rpa < c.b.r_par_max &&
                               rta < c.b.r_trans_max))
                    continue;
                const double xm = __dsub_rn(rpa, c.b.r_par_min);
                const double mp = md_floor(__dmul_rn(xm, c.inv_range), xm, c.b.r_par_range,
                                           c.nmp);
                const double mt = md_floor(__dmul_rn(rta, c.inv_rtmax), rta, c.b.r_trans_max,
                                           c.nmt);
                if (!(mp < c.nmp && mt < c.nmt && mp >= 0.)) {
                    if (c.xcf) report_error(scratch, PG_ERR_BIN_RANGE, (int32_t)mp);
                    continue;
                }
                const int32_t mb = (int32_t)mt + c.nmt * (int32_t)mp;
                const int64_t key = (int64_t)b * nm + mb;
                if (key != run) {
                    if (run >= 0) flush();
                    run = key;
                    run_m = mb;
                    k_wz = k_rp = k_rt = k_z = 0.;
                }
                const double zevol =
                    __dmul_rn(__dmul_rn(zf1, a2.zfac[o2 + j]), c.inv_zevol_den);
                const double wz = __dmul_rn(w12, zevol);
                k_wz += wz;
                k_rp += __dmul_rn(rpa, wz);
                k_rt += __dmul_rn(rta, wz);
                k_z += __dmul_rn(__dadd_rn(za1, a2.z[o2 + j]) / 2, wz);
            }
            if (run_b >= 0) atomicAdd(&out.weights_dmat[run_b], k_w);
            if (run >= 0) flush();
        }
    }
}

}  // namespace

int launch_metal_dmat(const pg_corr_params &p, const pg_dmat_params &d, double zevol_den,
                      const pg_forest_set &s1, const pg_forest_set &s2,
                      const pg_metal_pixels &a1, const pg_metal_pixels &a2,
                      const int32_t *pair_first, const int32_t *pair_second,
                      const double *pair_angle, int64_t num_pairs, const pg_dmat_sums &out,
                      Scratch *scratch, int num_sms, cudaStream_t stream, bool xcf) {
    if (num_pairs == 0) return PG_OK;
    MetalConst c;
    c.b = make_binning(p);
    c.nmp = d.num_model_bins_r_par;
    c.nmt = d.num_model_bins_r_trans;
    c.nm = c.nmp * c.nmt;
    c.inv_range = 1. / c.b.r_par_range;
    c.inv_rtmax = 1. / c.b.r_trans_max;
    c.inv_zevol_den = 1. / zevol_den;
    c.xcf = xcf;
    if (xcf) {  // r_par is signed and the cross has no half-plate veto
        c.b.x_correlation = 1;
        c.b.remove_shp = 0;
    }
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, metal_dmat_kernel, kMdBlock, 0) !=
            cudaSuccess ||
        occ < 1)
        return PG_ERR_CUDA;
    const int64_t grid = std::min<int64_t>((int64_t)num_sms * occ, num_pairs);
    metal_dmat_kernel<<<(int)grid, kMdBlock, 0, stream>>>(c, s1, s2, a1, a2, pair_first,
                                                          pair_second, pair_angle, num_pairs,
                                                          out, scratch);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
