// C-ABI entry points of libpicca_gb300 (declared in include/picca_gb300.h).
#include <stdlib.h>

#include "pg_internal.cuh"

struct pg_plan {
    int device;
    int num_sms;
    void *scratch;      // pg::Scratch followed by the precision-form constants
    cudaStream_t last_stream;
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
    return launch_cf_neighbours(*params, *s1, s2 ? *s2 : *s1, s2 == nullptr, counts, offsets,
                                index, st);
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
    return launch_xcf_neighbours(*params, *forests, *objs, counts, offsets, index, st);
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
    // the precision form covers the standard (r_par, r_trans) geometry
    const bool fast = mode == PG_MODE_FP32_GUARD && !b.rmu && !b.ang_corr &&
                      s1->max_pixels <= 65535;
    if (fast)
        return launch_cf_xi_fast(b, params->ang_max, *s1, other, nbr_offsets, nbr_index,
                                 nbr_angle, work_order, num_work, *out, scratch_of(plan),
                                 fast_const_of(plan), plan->num_sms, st);
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
        return launch_xcf_xi_fast(b, params->ang_max, *forests, *objs, nbr_offsets, nbr_index,
                                  nbr_angle, work_order, num_work, *out, scratch_of(plan),
                                  fast_const_of(plan), plan->num_sms, st);
    return launch_xcf_xi_fp64(b, *forests, *objs, nbr_offsets, nbr_index, nbr_angle, work_order,
                              num_work,
                              *out, scratch_of(plan), plan->num_sms, st);
}

}  // extern "C"
