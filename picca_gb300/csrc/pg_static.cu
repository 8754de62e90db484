// pg_cf_xi_static: the pair accumulation of pg_cf_xi for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc at all: code running while another
// framework owns the device allocator (a memory pool that forbids side
// allocations), hosts that pre-size every buffer at start-up and treat a
// later allocation as a failure, or callers on a device whose memory is fully
// reserved. pg_cf_xi needs a pg_plan, and creating a plan allocates the
// kernels' scratch with cudaMalloc. This entry point uses instead a
// file-scope device array holding the same scratch (work-queue head, status
// word, counters and the precision-form constants), so the only device memory
// it touches is that array and the caller's inputs and outputs.
//
// Properties of the array, which callers must keep in mind:
//  - its size is fixed at build time (PG_STATIC_SCRATCH_BYTES); every GPU
//    that loads the library holds it until the process exits;
//  - all calls on a device share it and it keeps the last call's contents:
//    each call clears the part that must start at zero, so calls that
//    overlap on the GPU (different streams, or a call issued before the
//    previous one finished) race on it and give wrong results. Calls on one
//    stream are safe: this function synchronises the stream before it
//    returns;
//  - its device address is looked up once per device by the first call made
//    with that device current (cudaGetSymbolAddress).
// The call is synchronous (stream synchronise, then a blocking copy of the
// status word), so it cannot be issued inside a CUDA graph capture.
#include <mutex>

#include "pg_internal.cuh"

namespace pg {
namespace {

static __device__ __align__(256) unsigned char g_static_scratch[PG_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 128;

struct StaticSlot {
    bool ready;
    void *ptr;
    int num_sms;
};

std::mutex g_static_mutex;
StaticSlot g_static_slots[kMaxDevices];

size_t scratch_head_bytes() { return (sizeof(Scratch) + 255) & ~(size_t)255; }

// Once per device, with that device current: the device address of the
// array and the SM count.
int static_setup(int device, StaticSlot *out) {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (device < 0 || device >= kMaxDevices) return PG_ERR_UNSUPPORTED;
    StaticSlot &slot = g_static_slots[device];
    if (!slot.ready) {
        void *ptr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (err != cudaSuccess) return check_cuda(err);
        int sms = 0;
        err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (err != cudaSuccess) return check_cuda(err);
        slot.ptr = ptr;
        slot.num_sms = sms;
        slot.ready = true;
    }
    *out = slot;
    return PG_OK;
}

bool set_ok(const pg_forest_set *s) {
    if (!s || s->num < 0 || s->num > INT32_MAX) return false;
    if (s->num == 0) return true;
    return s->ra && s->dec && s->x_cart && s->y_cart && s->z_cart && s->cos_dec && s->z_qso &&
           s->thingid && s->pix_offset && s->z && s->r_comov && s->dist_m && s->weights &&
           s->delta && s->row && s->num_rows > 0 && s->max_pixels > 0 && s->num_pixels >= 0;
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" int pg_cf_xi_static(const pg_corr_params *params, const pg_forest_set *s1,
                               const pg_forest_set *s2, const int64_t *nbr_offsets,
                               const int32_t *nbr_index, const double *nbr_angle,
                               const int32_t *work_order, int64_t num_work, int32_t mode,
                               const pg_xi_rows *out, void *stream) {
    if (!params || params->num_bins_r_par <= 0 || params->num_bins_r_trans <= 0 ||
        (int64_t)params->num_bins_r_par * params->num_bins_r_trans > (1 << 24) ||
        !isfinite(params->r_par_min) || !isfinite(params->r_par_max) ||
        !(params->r_par_max > params->r_par_min) || !isfinite(params->r_trans_max) ||
        !(params->r_trans_max > 0) || !(params->ang_max > 0))
        return PG_ERR_INVALID_ARGUMENT;
    if (!set_ok(s1) || (s2 && !set_ok(s2))) return PG_ERR_INVALID_ARGUMENT;
    if (!out || !out->weights || !out->xi || !out->r_par || !out->r_trans || !out->z ||
        !out->num_pairs)
        return PG_ERR_INVALID_ARGUMENT;
    if (num_work < 0 || num_work > s1->num || num_work > INT32_MAX) return PG_ERR_INVALID_ARGUMENT;
    if (num_work > 0 && (!nbr_offsets || !nbr_index)) return PG_ERR_INVALID_ARGUMENT;
    if (mode != PG_MODE_FP64 && mode != PG_MODE_FP32_GUARD) return PG_ERR_INVALID_ARGUMENT;
    // the scratch this call needs must fit in the array
    const size_t need = scratch_head_bytes() + fast_const_bytes();
    if (need > (size_t)PG_STATIC_SCRATCH_BYTES) return PG_ERR_UNSUPPORTED;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return check_cuda(err);
    StaticSlot slot;
    int rc = static_setup(device, &slot);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Scratch *scratch = static_cast<Scratch *>(slot.ptr);
    void *fast_const = static_cast<char *>(slot.ptr) + scratch_head_bytes();
    // clear the queue head, status word and counters left by the last call
    if ((rc = check_cuda(cudaMemsetAsync(scratch, 0, sizeof(Scratch), st)))) return rc;
    const Binning b = make_binning(*params);
    const pg_forest_set &other = s2 ? *s2 : *s1;
    const bool fast = mode == PG_MODE_FP32_GUARD && !b.rmu && !b.ang_corr &&
                      s1->max_pixels <= 65535;
    if (fast)
        rc = launch_cf_xi_fast(b, params->ang_max, *s1, other, nbr_offsets, nbr_index, nbr_angle,
                               work_order, num_work, *out, scratch, fast_const, slot.num_sms, st);
    else
        rc = launch_cf_xi_fp64(b, *s1, other, nbr_offsets, nbr_index, nbr_angle, work_order,
                               num_work, *out, scratch, slot.num_sms, st);
    if (rc) return rc;
    // wait for the kernel and report its device-side status
    if ((rc = check_cuda(cudaStreamSynchronize(st)))) return rc;
    int32_t status = 0;
    if ((rc = check_cuda(cudaMemcpy(&status, &scratch->status, sizeof(status),
                                    cudaMemcpyDeviceToHost))))
        return rc;
    return status;
}
