// C-ABI entry points of libpicca_gb300 (declared in include/picca_gb300.h).
#include <vector>
#include <stdlib.h>

#include <algorithm>

#include "pg_internal.cuh"

struct pg_plan {
    int device;
    int num_sms;
    void *scratch;      // pg::Scratch followed by the precision-form constants
    cudaStream_t last_stream;
    pg_tuning tuning;   // launch shapes of the precision-form pair kernels (0: default)
};

namespace pg {

int check_cuda(cudaError_t err) {
    if (err == cudaSuccess) return PG_OK;
    if (err == cudaErrorMemoryAllocation) return PG_ERR_NO_MEMORY;
    if (err == cudaErrorNoDevice || err == cudaErrorInsufficientDriver) return PG_ERR_NO_DEVICE;
    return PG_ERR_CUDA;
}

namespace {

size_t scratch_bytes() { return ((sizeof(Scratch) + 255) & ~(size_t)255) + fast_const_bytes(); }

Scratch *scratch_of(pg_plan *plan) { return static_cast<Scratch *>(plan->scratch); }

void *fast_const_of(pg_plan *plan) {
    return static_cast<char *>(plan->scratch) + ((sizeof(Scratch) + 255) & ~(size_t)255);
}

bool finite_positive(double v) { return isfinite(v) && v > 0; }

int validate_params(const pg_corr_params *p) {
    if (!p) return PG_ERR_INVALID_ARGUMENT;
    if (p->num_bins_r_par <= 0 || p->num_bins_r_trans <= 0) return PG_ERR_INVALID_ARGUMENT;
    if ((int64_t)p->num_bins_r_par * p->num_bins_r_trans > (1 << 24)) return PG_ERR_INVALID_ARGUMENT;
    if (!isfinite(p->r_par_min) || !isfinite(p->r_par_max) || !(p->r_par_max > p->r_par_min))
        return PG_ERR_INVALID_ARGUMENT;
    if (!finite_positive(p->r_trans_max)) return PG_ERR_INVALID_ARGUMENT;
    if (!(p->ang_max > 0)) return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

int validate_set(const pg_forest_set *s, bool needs_pixels, bool needs_objects) {
    if (!s || s->num < 0 || s->num > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (s->num == 0) return PG_OK;
    if (!s->ra || !s->dec || !s->x_cart || !s->y_cart || !s->z_cart || !s->cos_dec ||
        !s->z_qso || !s->thingid)
        return PG_ERR_INVALID_ARGUMENT;
    if (needs_pixels) {
        if (!s->pix_offset || !s->z || !s->r_comov || !s->dist_m || !s->weights || !s->delta ||
            !s->row || s->num_rows <= 0 || s->max_pixels <= 0 || s->num_pixels < 0)
            return PG_ERR_INVALID_ARGUMENT;
    }
    if (needs_objects) {
        if (!s->obj_r_comov || !s->obj_dist_m || !s->obj_weight) return PG_ERR_INVALID_ARGUMENT;
    }
    return PG_OK;
}

int validate_rows(const pg_xi_rows *out) {
    if (!out || !out->weights || !out->xi || !out->r_par || !out->r_trans || !out->z ||
        !out->num_pairs)
        return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

int reset_scratch(pg_plan *plan, cudaStream_t stream) {
    return check_cuda(cudaMemsetAsync(plan->scratch, 0, sizeof(Scratch), stream));
}

int select_device(pg_plan *plan) {
    int current = -1;
    cudaError_t err = cudaGetDevice(&current);
    if (err != cudaSuccess) return check_cuda(err);
    if (current != plan->device) return PG_ERR_INVALID_ARGUMENT;  // plan bound to another device
    return PG_OK;
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" {

const char *pg_strerror(int status) {
    switch (status) {
        case PG_OK: return "ok";
        case PG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PG_ERR_CUDA: return "CUDA runtime error";
        case PG_ERR_TIMEOUT: return "device wait timed out";
        case PG_ERR_BIN_RANGE: return "bin index outside the histogram";
        case PG_ERR_NO_MEMORY: return "out of device memory";
        case PG_ERR_UNSUPPORTED: return "unsupported configuration (forest or histogram too large)";
        case PG_ERR_NO_DEVICE: return "no usable CUDA device";
        default: return "unknown status";
    }
}

int pg_version(void) { return 10000; }

int pg_plan_create(pg_plan **plan) {
    if (!plan) return PG_ERR_INVALID_ARGUMENT;
    *plan = nullptr;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return check_cuda(err);
    int sms = 0;
    err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess) return check_cuda(err);
    pg_plan *p = static_cast<pg_plan *>(calloc(1, sizeof(pg_plan)));
    if (!p) return PG_ERR_NO_MEMORY;
    p->device = device;
    p->num_sms = sms;
    err = cudaMalloc(&p->scratch, scratch_bytes());
    if (err != cudaSuccess) {
        free(p);
        return check_cuda(err);
    }
    err = cudaMemset(p->scratch, 0, scratch_bytes());
    if (err != cudaSuccess) {
        cudaFree(p->scratch);
        free(p);
        return check_cuda(err);
    }
    *plan = p;
    return PG_OK;
}

int pg_plan_destroy(pg_plan *plan) {
    if (!plan) return PG_OK;
    int rc = check_cuda(cudaFree(plan->scratch));
    free(plan);
    return rc;
}

int pg_plan_set_tuning(pg_plan *plan, const pg_tuning *tuning) {
    if (!plan || !tuning) return PG_ERR_INVALID_ARGUMENT;
    if (tuning->cf_warps < 0 || tuning->cf_warps > 32 || tuning->cf_blocks_per_sm < 0 ||
        tuning->xcf_warps < 0 || tuning->xcf_warps > 32 || tuning->xcf_blocks_per_sm < 0)
        return PG_ERR_INVALID_ARGUMENT;
    plan->tuning = *tuning;
    return PG_OK;
}

int pg_plan_get_tuning(pg_plan *plan, pg_tuning *tuning) {
    if (!plan || !tuning) return PG_ERR_INVALID_ARGUMENT;
    *tuning = plan->tuning;
    return PG_OK;
}

int pg_plan_stats(pg_plan *plan, pg_run_stats *stats) {
    if (!plan || !stats) return PG_ERR_INVALID_ARGUMENT;
    int rc = check_cuda(cudaStreamSynchronize(plan->last_stream));
    if (rc) return rc;
    Scratch host;
    rc = check_cuda(cudaMemcpy(&host, plan->scratch, sizeof(Scratch), cudaMemcpyDeviceToHost));
    if (rc) return rc;
    stats->status = host.status;
    stats->error_detail = host.error_detail;
    stats->rechecked_pairs = (int64_t)host.rechecked_pairs;
    stats->recheck_overflows = (int64_t)host.recheck_overflows;
    stats->work_items = (int64_t)host.work_items;
    stats->visited_pairs = (int64_t)host.visited_pairs;
    stats->gemm_macs = (int64_t)host.gemm_macs;
    return PG_OK;
}

int pg_cf_neighbours(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
                     const pg_forest_set *s2, int64_t *counts, const int64_t *offsets,
                     int32_t *index, void *stream) {
    if (!plan) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(s1, false, false))) return rc;
    if (s2 && (rc = validate_set(s2, false, false))) return rc;
    if (offsets == nullptr && counts == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if (offsets != nullptr && index == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_cf_neighbours(*params, *s1, s2 ? *s2 : *s1, s2 == nullptr, nullptr, counts,
                                offsets, index, st);
}

int pg_xcf_neighbours(pg_plan *plan, const pg_corr_params *params,
                      const pg_forest_set *forests, const pg_forest_set *objs,
                      int64_t *counts, const int64_t *offsets, int32_t *index, void *stream) {
    if (!plan || !forests || !objs) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(forests, false, false))) return rc;
    if ((rc = validate_set(objs, false, objs->num > 0))) return rc;
    if (forests->num > 0 && (!forests->r_first || !forests->r_last)) return PG_ERR_INVALID_ARGUMENT;
    if (offsets == nullptr && counts == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if (offsets != nullptr && index == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_xcf_neighbours(*params, *forests, *objs, nullptr, counts, offsets, index, st);
}

static int validate_groups(const pg_nbr_groups *g) {
    if (!g || g->num_groups1 < 0 || g->num_groups2 < 0 || g->num_blocks < 0)
        return PG_ERR_INVALID_ARGUMENT;
    if (g->num_blocks > 0 &&
        (!g->start2 || !g->cand_offsets || !g->cand_groups || !g->block_group ||
         !g->block_first || !g->block_end))
        return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

int pg_cf_neighbours_grouped(pg_plan *plan, const pg_corr_params *params,
                             const pg_forest_set *s1, const pg_forest_set *s2,
                             const pg_nbr_groups *groups, int64_t *counts,
                             const int64_t *offsets, int32_t *index, void *stream) {
    if (!plan) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(s1, false, false))) return rc;
    if (s2 && (rc = validate_set(s2, false, false))) return rc;
    if ((rc = validate_groups(groups))) return rc;
    if (offsets == nullptr && counts == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if (offsets != nullptr && index == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_cf_neighbours(*params, *s1, s2 ? *s2 : *s1, s2 == nullptr, groups, counts,
                                offsets, index, st);
}

int pg_xcf_neighbours_grouped(pg_plan *plan, const pg_corr_params *params,
                              const pg_forest_set *forests, const pg_forest_set *objs,
                              const pg_nbr_groups *groups, int64_t *counts,
                              const int64_t *offsets, int32_t *index, void *stream) {
    if (!plan || !forests || !objs) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(forests, false, false))) return rc;
    if ((rc = validate_set(objs, false, objs->num > 0))) return rc;
    if (forests->num > 0 && (!forests->r_first || !forests->r_last)) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = validate_groups(groups))) return rc;
    if (offsets == nullptr && counts == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if (offsets != nullptr && index == nullptr) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_xcf_neighbours(*params, *forests, *objs, groups, counts, offsets, index, st);
}

int pg_cf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
             const pg_forest_set *s2, const int64_t *nbr_offsets, const int32_t *nbr_index,
             const double *nbr_angle, const int32_t *work_order, int64_t num_work,
             int32_t mode, const pg_xi_rows *out, void *stream) {
    if (!plan) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(s1, true, false))) return rc;
    if (s2 && (rc = validate_set(s2, true, false))) return rc;
    if ((rc = validate_rows(out))) return rc;
    if (num_work < 0 || num_work > s1->num || num_work > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (num_work > 0 && (!nbr_offsets || !nbr_index)) return PG_ERR_INVALID_ARGUMENT;
    if (mode != PG_MODE_FP64 && mode != PG_MODE_FP32_GUARD) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    const Binning b = make_binning(*params);
    const pg_forest_set &other = s2 ? *s2 : *s1;
    // the precision form covers the (r_par, r_trans) geometry with every cut
    // and the r-mu binning without the z-pair, zerr and half-plate cuts
    const bool rmu_cuts = b.rmu && (b.remove_shp || b.zmin_on || b.zmax_on || b.zerr_on);
    const bool fast = mode == PG_MODE_FP32_GUARD && !rmu_cuts && !b.ang_corr &&
                      s1->max_pixels <= 65535;
    if (fast)
        return launch_cf_xi_fast(b, params->ang_max, *s1, other, nbr_offsets, nbr_index,
                                 nbr_angle, work_order, num_work, *out, scratch_of(plan),
                                 fast_const_of(plan), plan->num_sms, st,
                                 LaunchTuning{plan->tuning.cf_warps, plan->tuning.cf_blocks_per_sm});
    return launch_cf_xi_fp64(b, *s1, other, nbr_offsets, nbr_index, nbr_angle, work_order,
                             num_work, *out,
                             scratch_of(plan), plan->num_sms, st);
}

int pg_xcf_xi(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *forests,
              const pg_forest_set *objs, const int64_t *nbr_offsets, const int32_t *nbr_index,
              const double *nbr_angle, const int32_t *work_order, int64_t num_work,
              int32_t mode, const pg_xi_rows *out, void *stream) {
    if (!plan || !forests || !objs) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_params(params);
    if (rc) return rc;
    if ((rc = validate_set(forests, true, false))) return rc;
    if ((rc = validate_set(objs, false, objs->num > 0))) return rc;
    if ((rc = validate_rows(out))) return rc;
    if (num_work < 0 || num_work > forests->num || num_work > INT32_MAX)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_work > 0 && (!nbr_offsets || !nbr_index)) return PG_ERR_INVALID_ARGUMENT;
    if (mode != PG_MODE_FP64 && mode != PG_MODE_FP32_GUARD) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    const Binning b = make_binning(*params);
    const bool fast = mode == PG_MODE_FP32_GUARD && !b.rmu && !b.ang_corr &&
                      forests->max_pixels <= 65535;
    if (fast)
        return launch_xcf_xi_fast(
            b, params->ang_max, *forests, *objs, nbr_offsets, nbr_index, nbr_angle, work_order,
            num_work, *out, scratch_of(plan), fast_const_of(plan), plan->num_sms, st,
            LaunchTuning{plan->tuning.xcf_warps, plan->tuning.xcf_blocks_per_sm});
    return launch_xcf_xi_fp64(b, *forests, *objs, nbr_offsets, nbr_index, nbr_angle, work_order,
                              num_work,
                              *out, scratch_of(plan), plan->num_sms, st);
}

static int validate_dmat(const pg_corr_params *params, const pg_dmat_params *dparams) {
    int rc = validate_params(params);
    if (rc) return rc;
    if (!dparams || dparams->num_model_bins_r_par <= 0 || dparams->num_model_bins_r_trans <= 0)
        return PG_ERR_INVALID_ARGUMENT;
    if (params->ang_correlation) return PG_ERR_UNSUPPORTED;
    return PG_OK;
}

int pg_cf_dmat_work_bytes(pg_plan *plan, const pg_corr_params *params,
                          const pg_dmat_params *dparams, int32_t max_pixels1,
                          int32_t max_pixels2, int64_t max_ctas, uint64_t *bytes) {
    if (!plan || !bytes) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_dmat(params, dparams);
    if (rc) return rc;
    if ((rc = select_device(plan))) return rc;
    DmatConstHost h;
    if ((rc = dmat_config(*params, *dparams, max_pixels1, max_pixels2, plan->num_sms, h, false)))
        return rc;
    if (max_ctas < 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t ctas = max_ctas > 0 ? std::min<int64_t>(max_ctas, h.max_grid) : h.max_grid;
    *bytes = (uint64_t)ctas * (uint64_t)h.cta_doubles * sizeof(double);
    return PG_OK;
}

int pg_cf_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
               const pg_forest_set *s1, const pg_forest_set *s2, const double *log_lambda1,
               const double *log_lambda2, const int32_t *order1, const int32_t *order2,
               const int32_t *pair_first, const int32_t *pair_second, const double *pair_angle,
               int64_t num_pairs, void *work, uint64_t work_bytes, const pg_dmat_sums *out,
               void *stream) {
    if (!plan || !s1 || !out) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_dmat(params, dparams);
    if (rc) return rc;
    if ((rc = validate_set(s1, true, false))) return rc;
    if (s2 && (rc = validate_set(s2, true, false))) return rc;
    if (!out->weights_dmat || !out->dmat || !out->r_par_eff || !out->r_trans_eff ||
        !out->z_eff || !out->weight_eff)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_pairs < 0 || num_pairs > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (num_pairs > 0 && (!pair_first || !pair_second || !log_lambda1 || !order1 || !work))
        return PG_ERR_INVALID_ARGUMENT;
    if (s2 && num_pairs > 0 && (!log_lambda2 || !order2)) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    const pg_forest_set &other = s2 ? *s2 : *s1;
    DmatConstHost h;
    if ((rc = dmat_config(*params, *dparams, s1->max_pixels, other.max_pixels, plan->num_sms, h,
                          false)))
        return rc;
    const uint64_t per_cta = (uint64_t)h.cta_doubles * sizeof(double);
    const uint64_t fit = work_bytes / per_cta;
    const int grid = (int)std::min<uint64_t>((uint64_t)h.max_grid, fit);
    if (num_pairs > 0 && grid < 1) return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(work) % 16) return PG_ERR_INVALID_ARGUMENT;
    return launch_cf_dmat(*params, *dparams, h, *s1, other, log_lambda1,
                          s2 ? log_lambda2 : log_lambda1, order1, s2 ? order2 : order1,
                          pair_first, pair_second, pair_angle, num_pairs,
                          static_cast<double *>(work), grid, *out, scratch_of(plan), st);
}

static int validate_spectra(const pg_spectra *sp) {
    if (!sp || sp->num < 0 || sp->num_pixels < 0) return PG_ERR_INVALID_ARGUMENT;
    if (sp->num == 0) return PG_OK;
    if (!sp->pix_offset || !sp->log_lambda || !sp->flux || !sp->ivar ||
        !sp->transmission_correction || !sp->z_qso)
        return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

static int validate_model(const pg_cont_model *m) {
    if (!m || m->num_mean_cont < 2 || !m->mean_cont_x || !m->mean_cont_y)
        return PG_ERR_INVALID_ARGUMENT;
    if (!m->use_constant_weight &&
        (m->num_var_intervals < 1 || !m->var_breaks || !m->eta_coef || !m->var_lss_coef ||
         !m->fudge_coef))
        return PG_ERR_INVALID_ARGUMENT;
    if (m->stack_x && (m->num_stack < 1 || !m->stack_y)) return PG_ERR_INVALID_ARGUMENT;
    if (!(m->log_lambda_rest_max > m->log_lambda_rest_min)) return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

static int validate_fit(const pg_cont_fit *f, bool need_continuum) {
    if (!f || !f->zero_point || !f->slope || !f->chi2 || !f->ndata || !f->status ||
        !f->iterations)
        return PG_ERR_INVALID_ARGUMENT;
    if (need_continuum && !f->continuum) return PG_ERR_INVALID_ARGUMENT;
    return PG_OK;
}

int pg_cont_fit_batch(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                const double *start, int32_t max_iter, double tol, int32_t mode,
                const pg_cont_fit *out, void *stream) {
    if (!spectra) return PG_ERR_INVALID_ARGUMENT;
    return pg_cont_fit_select(plan, spectra, model, start, nullptr, spectra->num, max_iter, tol,
                              mode, out, stream);
}

int pg_cont_fit_select(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                       const double *start, const int32_t *forest_index, int64_t num_index,
                       int32_t max_iter, double tol, int32_t mode, const pg_cont_fit *out,
                       void *stream) {
    if (!plan) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model)) ||
        (rc = validate_fit(out, false)))
        return rc;
    if (max_iter < 0 || (max_iter == 0 && !start) || !(tol > 0) ||
        (mode != PG_FIT_FP64 && mode != PG_FIT_MIXED))
        return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    if (num_index < 0 || (forest_index == nullptr && num_index != spectra->num) ||
        num_index > INT32_MAX)
        return PG_ERR_INVALID_ARGUMENT;
    return launch_cont_fit(*spectra, *model, start, forest_index, num_index, max_iter, tol, mode,
                           *out, scratch_of(plan), plan->num_sms, st);
}

int pg_cont_fit_warm(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                     const double *start, const int32_t *forest_index, int64_t num_index,
                     int32_t max_iter, double chi2_tol, double ab_tol, const pg_cont_fit *out,
                     void *stream) {
    if (!plan || !start) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model)) ||
        (rc = validate_fit(out, false)))
        return rc;
    if (max_iter < 1 || !(chi2_tol > 0) || !(ab_tol > 0) || !(ab_tol < 1))
        return PG_ERR_INVALID_ARGUMENT;
    if (num_index < 0 || (forest_index == nullptr && num_index != spectra->num) ||
        num_index > INT32_MAX)
        return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_cont_fit(*spectra, *model, start, forest_index, num_index, max_iter, 1e-10,
                           PG_FIT_MIXED, *out, scratch_of(plan), plan->num_sms, st,
                           (float)chi2_tol, (float)ab_tol);
}

int pg_cont_stacks_accumulate(pg_plan *plan, const pg_spectra *spectra,
                              const pg_cont_model *model, const pg_cont_fit *fit,
                              const pg_cont_stacks *stacks, void *stream) {
    if (!plan || !stacks) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model)) ||
        (rc = validate_fit(fit, true)))
        return rc;
    if (stacks->mean_cont_num && (!stacks->mean_cont_weight || stacks->rest_bins < 1 ||
                                  !(stacks->rest_step > 0)))
        return PG_ERR_INVALID_ARGUMENT;
    if (stacks->var_mean && (!stacks->var_delta2 || !stacks->var_delta4 || !stacks->var_npix ||
                             !stacks->var_nqso || stacks->var_lambda_bins < 1 ||
                             !(stacks->var_step > 0)))
        return PG_ERR_INVALID_ARGUMENT;
    if (stacks->stack_num && (!stacks->stack_weight || stacks->obs_bins < 1 ||
                              !(stacks->obs_step > 0)))
        return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_cont_stacks(*spectra, *model, *fit, *stacks, scratch_of(plan), plan->num_sms,
                              st);
}

int pg_cont_deltas(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                   const pg_cont_fit *fit, double *delta, double *weights, void *stream) {
    if (!plan || !delta || !weights) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model)) ||
        (rc = validate_fit(fit, true)))
        return rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_cont_deltas(*spectra, *model, *fit, delta, weights, plan->num_sms, st);
}

int64_t pg_mlp_packed_elems(void) { return mlp_packed_elems(); }

int pg_mlp_pack(const uint16_t *params16, uint16_t *packed, void *stream) {
    if (!params16 || !packed) return PG_ERR_INVALID_ARGUMENT;
    return launch_mlp_pack(params16, packed, static_cast<cudaStream_t>(stream));
}

int pg_mlp_forward(pg_plan *plan, const uint16_t *packed, const float *params, const uint16_t *x,
                   int64_t m, int32_t stride, float *y, void *stream) {
    if (!plan || !packed || !params || !y || m < 0 || (m > 0 && !x)) return PG_ERR_INVALID_ARGUMENT;
    // rows are read as 16-byte vectors: 80 padded features, 16-byte aligned
    if (stride < 80 || stride % 8 != 0 || (reinterpret_cast<uintptr_t>(x) & 15u) ||
        (reinterpret_cast<uintptr_t>(packed) & 15u))
        return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_mlp_forward_tc(packed, params, x, m, stride, y, scratch_of(plan), plan->num_sms,
                                 st);
}

int pg_mlp_warm_start(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                      const uint16_t *packed, const float *params, float *y, double *a0,
                      void *stream) {
    if (!plan || !packed || !params || !y || !a0) return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(packed) & 15u) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model))) return rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_mlp_warm_start_tc(*spectra, *model, packed, params, y, a0, scratch_of(plan),
                                    plan->num_sms, st);
}

int pg_mlp_features(pg_plan *plan, const pg_spectra *spectra, const pg_cont_model *model,
                    uint16_t *features, int32_t feat_stride, double *a0, void *stream) {
    if (!plan || !features || !a0 || feat_stride < 66) return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = validate_spectra(spectra)) || (rc = validate_model(model))) return rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_mlp_features(*spectra, *model, features, feat_stride, a0, scratch_of(plan),
                               plan->num_sms, st);
}

int pg_xcf_dmat_work_bytes(pg_plan *plan, const pg_corr_params *params,
                           const pg_dmat_params *dparams, int32_t max_pixels, int64_t max_ctas,
                           uint64_t *bytes) {
    if (!plan || !bytes) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_dmat(params, dparams);
    if (rc) return rc;
    if ((rc = select_device(plan))) return rc;
    DmatConstHost h;
    if ((rc = dmat_config(*params, *dparams, max_pixels, 0, plan->num_sms, h, true))) return rc;
    if (max_ctas < 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t ctas = max_ctas > 0 ? std::min<int64_t>(max_ctas, h.max_grid) : h.max_grid;
    *bytes = (uint64_t)ctas * (uint64_t)h.cta_doubles * sizeof(double);
    return PG_OK;
}

int pg_xcf_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                const pg_forest_set *forests, const pg_forest_set *objs, const double *log_lambda,
                const int32_t *order, const int32_t *item_forest, const int32_t *item_start,
                const int32_t *item_count, const int32_t *obj_index, const double *obj_angle,
                int64_t num_items, void *work, uint64_t work_bytes, const pg_dmat_sums *out,
                void *stream) {
    if (!plan || !forests || !objs || !out) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_dmat(params, dparams);
    if (rc) return rc;
    if ((rc = validate_set(forests, true, false))) return rc;
    if ((rc = validate_set(objs, false, objs->num > 0))) return rc;
    if (!out->weights_dmat || !out->dmat || !out->r_par_eff || !out->r_trans_eff ||
        !out->z_eff || !out->weight_eff)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_items < 0 || num_items > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (num_items > 0 && (!item_forest || !item_start || !item_count || !obj_index ||
                          !log_lambda || !order || !work))
        return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    DmatConstHost h;
    if ((rc = dmat_config(*params, *dparams, forests->max_pixels, 0, plan->num_sms, h, true)))
        return rc;
    const uint64_t per_cta = (uint64_t)h.cta_doubles * sizeof(double);
    const int grid = (int)std::min<uint64_t>((uint64_t)h.max_grid, work_bytes / per_cta);
    if (num_items > 0 && grid < 1) return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(work) % 16) return PG_ERR_INVALID_ARGUMENT;
    return launch_xcf_dmat(*params, *dparams, h, *forests, *objs, log_lambda, order, item_forest,
                           item_start, item_count, obj_index, obj_angle, num_items,
                           static_cast<double *>(work), grid, *out, scratch_of(plan), st);
}

static int metal_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                      double zevol_den, const pg_forest_set *s1, const pg_forest_set *s2,
                      const pg_metal_pixels *a1, const pg_metal_pixels *a2,
                      const int32_t *pair_first, const int32_t *pair_second,
                      const double *pair_angle, int64_t num_pairs, const pg_dmat_sums *out,
                      void *stream, int cross) {
    if (!plan || !s1 || !a1 || !a2 || !out) return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_dmat(params, dparams);
    if (rc) return rc;
    if ((rc = validate_set(s1, true, false))) return rc;
    if (s2 && (rc = validate_set(s2, true, false))) return rc;
    if (!out->weights_dmat || !out->dmat || !out->r_par_eff || !out->r_trans_eff ||
        !out->z_eff || !out->weight_eff)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_pairs < 0 || num_pairs > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (!(zevol_den > 0) || !isfinite(zevol_den)) return PG_ERR_INVALID_ARGUMENT;
    const pg_metal_pixels *sides[2] = {a1, a2};
    for (const pg_metal_pixels *a : sides)
        if (num_pairs > 0 && (!a->r_comov || !a->dist_m || !a->z || !a->zfac || !a->weights))
            return PG_ERR_INVALID_ARGUMENT;
    if (num_pairs > 0 && (!pair_first || !pair_second)) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_metal_dmat(*params, *dparams, zevol_den, *s1, s2 ? *s2 : *s1, *a1, *a2,
                             pair_first, pair_second, pair_angle, num_pairs, *out,
                             scratch_of(plan), plan->num_sms, st, cross != 0);
}

int pg_cf_metal_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                     double zevol_den, const pg_forest_set *s1, const pg_forest_set *s2,
                     const pg_metal_pixels *a1, const pg_metal_pixels *a2,
                     const int32_t *pair_first, const int32_t *pair_second,
                     const double *pair_angle, int64_t num_pairs, const pg_dmat_sums *out,
                     void *stream) {
    return metal_dmat(plan, params, dparams, zevol_den, s1, s2, a1, a2, pair_first, pair_second,
                      pair_angle, num_pairs, out, stream, 0);
}

int pg_xcf_metal_dmat(pg_plan *plan, const pg_corr_params *params, const pg_dmat_params *dparams,
                      double zevol_den, const pg_forest_set *forests,
                      const pg_forest_set *quasar_pixels, const pg_metal_pixels *a1,
                      const pg_metal_pixels *a2, const int32_t *pair_first,
                      const int32_t *pair_second, const double *pair_angle, int64_t num_pairs,
                      const pg_dmat_sums *out, void *stream) {
    if (!quasar_pixels) return PG_ERR_INVALID_ARGUMENT;
    return metal_dmat(plan, params, dparams, zevol_den, forests, quasar_pixels, a1, a2,
                      pair_first, pair_second, pair_angle, num_pairs, out, stream, 1);
}

int pg_wick_xi_matrices(pg_plan *plan, const pg_forest_set *set, const double *log_lambda,
                        const double *variance, const double *xi_bounds,
                        const double *xi_values, int32_t num_xi, const int32_t *forests,
                        int64_t num_forests, const int64_t *x_offsets, double *arena,
                        void *stream) {
    if (!plan || !set || num_forests < 0 || num_xi < 1 || num_xi > 28000)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_forests > 0 && (!log_lambda || !variance || !xi_values || !forests ||
                            !x_offsets || !arena || (num_xi > 1 && !xi_bounds)))
        return PG_ERR_INVALID_ARGUMENT;
    int rc = validate_set(set, true, false);
    if (rc) return rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    return launch_wick_xmat(*set, log_lambda, variance, xi_bounds, xi_values, num_xi, forests,
                            num_forests, x_offsets, arena, plan->num_sms, st);
}

static int wick_bins(const pg_corr_params *params, int *nb) {
    if (!params || params->num_bins_r_par < 1 || params->num_bins_r_trans < 1 ||
        !(params->r_par_max > params->r_par_min) || !(params->r_trans_max > 0))
        return PG_ERR_INVALID_ARGUMENT;
    const int64_t n = (int64_t)params->num_bins_r_par * params->num_bins_r_trans;
    if (n > 6000) return PG_ERR_UNSUPPORTED;
    *nb = (int)n;
    return PG_OK;
}

int pg_cf_wick_work_bytes(pg_plan *plan, const pg_corr_params *params, int32_t max_pixels1,
                          int32_t max_pixels2, int64_t max_ctas, uint64_t *bytes) {
    if (!plan || !bytes || max_pixels1 < 1 || max_pixels2 < 1 || max_pixels1 > 32767 ||
        max_pixels2 > 32767)
        return PG_ERR_INVALID_ARGUMENT;
    int nb = 0, grid = 0;
    int rc = wick_bins(params, &nb);
    if (rc) return rc;
    if ((rc = select_device(plan))) return rc;
    if ((rc = wick_t123_grid(nb, plan->num_sms, &grid))) return rc;
    if (max_ctas > 0) grid = (int)std::min<int64_t>(grid, max_ctas);
    *bytes = (uint64_t)grid * (uint64_t)max_pixels1 * (uint64_t)max_pixels2 * sizeof(uint32_t);
    return PG_OK;
}

int pg_cf_wick(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *s1,
               const pg_forest_set *s2, const double *zw1, const double *zw2,
               const int64_t *x_offsets1, const double *arena1, const int64_t *x_offsets2,
               const double *arena2, const int32_t *pair_first, const int32_t *pair_second,
               const double *pair_angle, const int32_t *unit_slice, const int32_t *unit_slices,
               int64_t num_pairs, void *work, uint64_t work_bytes, const pg_wick_sums *out,
               void *stream) {
    if (!plan || !s1 || !out) return PG_ERR_INVALID_ARGUMENT;
    int nb = 0, rc = wick_bins(params, &nb);
    if (rc) return rc;
    const pg_forest_set *t = s2 ? s2 : s1;
    if ((rc = validate_set(s1, true, false)) || (rc = validate_set(t, true, false))) return rc;
    if (num_pairs < 0 || num_pairs > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (s1->max_pixels < 1 || t->max_pixels < 1 || s1->max_pixels > 32767 ||
        t->max_pixels > 32767)
        return PG_ERR_INVALID_ARGUMENT;
    if ((unit_slice == nullptr) != (unit_slices == nullptr)) return PG_ERR_INVALID_ARGUMENT;
    if (!out->weights_wick || !out->num_pairs_wick || !out->t1 || !out->t2 || !out->t3)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_pairs > 0 && (!zw1 || !zw2 || !x_offsets1 || !arena1 || !x_offsets2 || !arena2 ||
                          !pair_first || !pair_second || !work))
        return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(work) % 16) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    int grid = 0;
    if ((rc = wick_t123_grid(nb, plan->num_sms, &grid))) return rc;
    const int64_t cap = (int64_t)s1->max_pixels * t->max_pixels;
    grid = (int)std::min<uint64_t>((uint64_t)grid, work_bytes / ((uint64_t)cap * 4));
    if (num_pairs > 0 && grid < 1) return PG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_wick_t123(*params, *s1, *t, zw1, zw2, x_offsets1, arena1, x_offsets2, arena2,
                            pair_first, pair_second, pair_angle, unit_slice, unit_slices, num_pairs,
                            static_cast<uint32_t *>(work), cap, grid, *out, scratch_of(plan), st);
}


int pg_xcf_wick_work_bytes(pg_plan *plan, const pg_corr_params *params, int32_t max_pixels,
                           int32_t max_quasars, int64_t max_ctas, uint64_t *bytes) {
    if (!plan || !bytes || max_pixels < 1 || max_quasars < 1 || max_pixels > 32767 ||
        max_quasars > 65535)
        return PG_ERR_INVALID_ARGUMENT;
    int nb = 0, grid = 0;
    int rc = wick_bins(params, &nb);
    if (rc) return rc;
    if ((rc = select_device(plan))) return rc;
    if ((rc = xwick_grid(nb, plan->num_sms, &grid))) return rc;
    if (max_ctas > 0) grid = (int)std::min<int64_t>(grid, max_ctas);
    *bytes = (uint64_t)grid *
             (uint64_t)xwick_cta_bytes((int64_t)max_pixels * max_quasars, max_quasars);
    return PG_OK;
}

int pg_xcf_wick(pg_plan *plan, const pg_corr_params *params, const pg_forest_set *forests,
                const pg_forest_set *objs, const double *zw1, const double *zw_obj,
                const int64_t *x_offsets, const double *arena, const int32_t *item_forest,
                const int32_t *item_start, const int32_t *item_count, const int32_t *obj_index,
                const double *obj_angle, const int32_t *unit_slice, const int32_t *unit_slices,
                int64_t num_items, int32_t max_quasars, void *work, uint64_t work_bytes,
                const pg_wick_sums *out, void *stream) {
    if (!plan || !forests || !objs || !out) return PG_ERR_INVALID_ARGUMENT;
    int nb = 0, rc = wick_bins(params, &nb);
    if (rc) return rc;
    if ((rc = validate_set(forests, true, false)) || (rc = validate_set(objs, false, true)))
        return rc;
    if (num_items < 0 || num_items > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (forests->max_pixels < 1 || forests->max_pixels > 32767 || max_quasars < 1 ||
        max_quasars > 65535)
        return PG_ERR_INVALID_ARGUMENT;
    if ((unit_slice == nullptr) != (unit_slices == nullptr)) return PG_ERR_INVALID_ARGUMENT;
    if (!out->weights_wick || !out->num_pairs_wick || !out->t1 || !out->t2 || !out->t3 ||
        !out->t4)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_items > 0 && (!zw1 || !zw_obj || !x_offsets || !arena || !item_forest ||
                          !item_start || !item_count || !obj_index || !work))
        return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(work) % 16) return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    int grid = 0;
    if ((rc = xwick_grid(nb, plan->num_sms, &grid))) return rc;
    const int64_t cap = (int64_t)forests->max_pixels * max_quasars;
    const uint64_t per_cta = (uint64_t)xwick_cta_bytes(cap, max_quasars);
    grid = (int)std::min<uint64_t>((uint64_t)grid, work_bytes / per_cta);
    if (num_items > 0 && grid < 1) return PG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_xwick(*params, *forests, *objs, zw1, zw_obj, x_offsets, arena, item_forest,
                        item_start, item_count, obj_index, obj_angle, unit_slice, unit_slices,
                        num_items, static_cast<char *>(work), cap, max_quasars, grid, *out,
                        scratch_of(plan), st);
}


int pg_read_delta_file(const uint8_t *bytes, int64_t size, double z_min_qso, double z_max_qso,
                       pg_delta_arrays *out) {
    if (!bytes || size < 0 || !out) return PG_ERR_INVALID_ARGUMENT;
    if (out->los_id && (!out->plate || !out->mjd || !out->fiberid || !out->ra || !out->dec ||
                        !out->z_qso || !out->pix_offset || !out->wave || !out->delta ||
                        !out->weights || !out->cont))
        return PG_ERR_INVALID_ARGUMENT;
    return read_delta_file(bytes, size, z_min_qso, z_max_qso, out);
}

int pg_project_deltas(int64_t num_los, const int64_t *pix_offset, const double *log_lambda,
                      const double *weights, double *delta, const int32_t *order,
                      int32_t threads) {
    if (num_los < 0) return PG_ERR_INVALID_ARGUMENT;
    if (num_los > 0 && (!pix_offset || !log_lambda || !weights || !delta || !order))
        return PG_ERR_INVALID_ARGUMENT;
    for (int64_t f = 0; f < num_los; ++f)
        if ((order[f] != 0 && order[f] != 1) || pix_offset[f + 1] < pix_offset[f])
            return PG_ERR_INVALID_ARGUMENT;
    return project_deltas(num_los, pix_offset, log_lambda, weights, delta, order, threads);
}

int pg_xcf_wick_factored_work_bytes(pg_plan *plan, const pg_corr_params *params,
                                    int32_t max_pixels, int32_t max_quasars, uint64_t *bytes) {
    if (!plan || !bytes || max_pixels < 1 || max_quasars < 1) return PG_ERR_INVALID_ARGUMENT;
    int nb = 0;
    int rc = wick_bins(params, &nb);
    if (rc) return rc;
    *bytes = xwick_factored_bytes(nb, max_pixels, max_quasars);
    return PG_OK;
}

int pg_xcf_wick_factored(pg_plan *plan, const pg_corr_params *params,
                         const pg_forest_set *forests, const pg_forest_set *objs,
                         const double *zw1, const double *zw_obj, const int64_t *x_offsets,
                         const double *arena, const int32_t *item_forest,
                         const int32_t *item_start, const int32_t *item_count,
                         const int32_t *obj_index, const double *obj_angle, int64_t num_items,
                         int32_t max_quasars, void *work, uint64_t work_bytes,
                         const pg_wick_sums *out, void *stream) {
    if (!plan || !forests || !objs || !out) return PG_ERR_INVALID_ARGUMENT;
    int nb = 0, rc = wick_bins(params, &nb);
    if (rc) return rc;
    if ((rc = validate_set(forests, true, false)) || (rc = validate_set(objs, false, true)))
        return rc;
    if (num_items < 0 || max_quasars < 1 || forests->max_pixels < 1)
        return PG_ERR_INVALID_ARGUMENT;
    if (!out->weights_wick || !out->num_pairs_wick || !out->t1 || !out->t2 || !out->t3 ||
        !out->t4)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_items == 0) return PG_OK;
    if (!zw1 || !zw_obj || !x_offsets || !arena || !item_forest || !item_start || !item_count ||
        !obj_index || !work)
        return PG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(work) % 256) return PG_ERR_INVALID_ARGUMENT;
    if (work_bytes < xwick_factored_bytes(nb, forests->max_pixels, max_quasars))
        return PG_ERR_INVALID_ARGUMENT;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    // the host loop needs the items, the forests' pixel offsets and the arena offsets
    std::vector<int32_t> hf(num_items), hs(num_items), hc(num_items);
    std::vector<int64_t> po(forests->num + 1), xo(forests->num);
    cudaError_t err = cudaMemcpyAsync(hf.data(), item_forest, 4 * num_items,
                                      cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(hs.data(), item_start, 4 * num_items, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(hc.data(), item_count, 4 * num_items, cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(po.data(), forests->pix_offset, 8 * po.size(),
                              cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(xo.data(), x_offsets, 8 * xo.size(), cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (err != cudaSuccess) return check_cuda(err);
    if ((rc = reset_scratch(plan, st))) return rc;
    for (int64_t q = 0; q < num_items; ++q)
        if (hf[q] < 0 || hf[q] >= forests->num || hc[q] > max_quasars || hc[q] < 0 ||
            po[hf[q] + 1] - po[hf[q]] > forests->max_pixels)
            return PG_ERR_INVALID_ARGUMENT;
    return run_xwick_factored(*params, *forests, *objs, zw1, zw_obj, xo.data(), arena, hf.data(),
                              hs.data(), hc.data(), obj_index, obj_angle, num_items, po.data(),
                              forests->max_pixels, max_quasars, static_cast<char *>(work), *out,
                              scratch_of(plan), plan->num_sms, st);
}

int pg_fast_metal_dmat(pg_plan *plan, const pg_fast_metal_params *params,
                       const pg_fast_metal_side *s1, const pg_fast_metal_side *s2,
                       const pg_fast_metal_sums *out, void *stream) {
    if (!plan || !params || !s1 || !s2 || !out) return PG_ERR_INVALID_ARGUMENT;
    const int np = params->num_bins_r_par, nr = params->num_ratio_bins;
    if (np < 1 || nr < 1 || np > 4096 || nr > 65536) return PG_ERR_INVALID_ARGUMENT;
    if (!(params->r_par_max > params->r_par_min) || !isfinite(params->r_par_min) ||
        !isfinite(params->r_par_max) || !(params->near_r_par >= 0))
        return PG_ERR_INVALID_ARGUMENT;
    const pg_fast_metal_side *sides[2] = {s1, s2};
    for (const pg_fast_metal_side *s : sides) {
        if (s->num < 0 || s->num > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
        if (s->num > 0 && (!s->r_in || !s->r_out || !s->z_in || !s->weight))
            return PG_ERR_INVALID_ARGUMENT;
    }
    if (!out->rp_dmat || !out->ratio_weights || !out->ratio_edges || !out->out_weight ||
        !out->out_weight_rp || !out->out_weight_z)
        return PG_ERR_INVALID_ARGUMENT;
    int rc;
    if ((rc = select_device(plan))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    plan->last_stream = st;
    if ((rc = reset_scratch(plan, st))) return rc;
    return launch_fast_metal(*params, *s1, *s2, *out, scratch_of(plan), plan->num_sms, st);
}

}  // extern "C"

