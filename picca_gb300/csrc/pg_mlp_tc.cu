// Learned warm start: the inference forward pass of the 66-256-256-256-2
// network as one fused Blackwell kernel (no counterpart in the reference;
// see include/picca_gb300.h).
//
// A persistent CTA (16 warps) takes 128 forests at a time through all four
// layers without leaving the SM: the feature tile and each hidden activation
// live in shared memory as the A operand of tcgen05.mma (BF16 x BF16 -> FP32,
// M = 128, N = 256, K = 16 per instruction, issued by one thread), the
// accumulator lives in tensor memory (256 columns), and the epilogue (bias,
// GELU, BF16 rounding) reads it back with tcgen05.ld and writes the next
// layer's A operand in place. The weights are pre-packed once into the exact
// shared-memory image of the B operand (pg_mlp_pack) and copied in per layer
// with asynchronous copies issued as soon as the previous MMAs completed, so
// that they overlap the epilogue.
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices, row
// group g and K chunk c at byte (g * KC + c) * 128 with KC = K / 8 chunks, so
// the descriptor's leading-dimension offset (between the two K-adjacent core
// matrices of one instruction) is 128 bytes and its stride offset (between
// 8-row groups) is KC * 128 bytes; instruction s of a layer starts 256 * s
// bytes in.
#include <cuda_bf16.h>

#include "pg_cont_common.cuh"
#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kTcThreads = 512;  // 16 warps: four per TMEM lane quarter
constexpr int kTcRows = 128;     // forests per tile (the MMA's M)
constexpr int kHidden = 256;
constexpr int kIn = 66, kInPad = 80;  // features, padded to a multiple of 16
constexpr int kOut = 2, kOutPad = 16;
constexpr int kTmemCols = 256;
constexpr size_t kTcABytes = (size_t)kTcRows * kHidden * 2;     // 64 KB
constexpr size_t kTcWBytes = (size_t)kHidden * kHidden * 2;     // 128 KB

// packed operand images, in bf16 elements
constexpr int64_t kPackW1 = (int64_t)kHidden * kInPad;
constexpr int64_t kPackW2 = (int64_t)kHidden * kHidden;
constexpr int64_t kPackW4 = (int64_t)kOutPad * kHidden;
constexpr int64_t kPackTotal = kPackW1 + 2 * kPackW2 + kPackW4;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading and stride byte offsets
// (16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 and M >> 4
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::
                     "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void proxy_fence() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16-byte global -> shared copy through the asynchronous copy path;
// src_bytes = 0 fills the 16 bytes with zeros (nothing is read)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem_dst)),
                 "l"(gsrc), "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// bounded wait on an mbarrier phase; false when the bound ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int i = 0; i < (1 << 20); ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tc_gelu(float x) {
    return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}

// byte offset of (row, K chunk) in an operand image with kc chunks per row group
__device__ __forceinline__ uint32_t img_off(int row, int chunk, int kc) {
    return (uint32_t)(((row >> 3) * kc + chunk) * 128 + (row & 7) * 16);
}

// B operand images of the four layers from the BF16 parameters (per layer
// W [fan_in][fan_out] row-major, then the bias): element (n, k) of layer l's
// image sits at ((n / 8) KC + k / 8) 64 + (n % 8) 8 + k % 8, zero outside
// the layer's (fan_out, fan_in).
__global__ void mlp_pack_kernel(const __nv_bfloat16 *__restrict__ params,
                                __nv_bfloat16 *__restrict__ packed) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kPackTotal) return;
    int64_t base, w_off;
    int kpad, kin, nout;
    if (e < kPackW1) {
        base = 0; w_off = 0; kpad = kInPad; kin = kIn; nout = kHidden;
    } else if (e < kPackW1 + kPackW2) {
        base = kPackW1; w_off = (int64_t)kIn * kHidden + kHidden; kpad = kHidden; kin = kHidden;
        nout = kHidden;
    } else if (e < kPackW1 + 2 * kPackW2) {
        base = kPackW1 + kPackW2;
        w_off = (int64_t)kIn * kHidden + kHidden + (int64_t)kHidden * kHidden + kHidden;
        kpad = kHidden; kin = kHidden; nout = kHidden;
    } else {
        base = kPackW1 + 2 * kPackW2;
        w_off = (int64_t)kIn * kHidden + kHidden + 2 * ((int64_t)kHidden * kHidden + kHidden);
        kpad = kHidden; kin = kHidden; nout = kOut;
    }
    const int64_t r = e - base;
    const int kc = kpad / 8;
    const int g = (int)(r / (kc * 64)), rem = (int)(r % (kc * 64));
    const int c = rem / 64, rr = (rem % 64) / 8, kk = rem % 8;
    const int nn = g * 8 + rr, k = c * 8 + kk;
    packed[e] = (nn < nout && k < kin) ? params[w_off + (int64_t)k * nout + nn]
                                       : __float2bfloat16(0.f);
}

// FEAT = false: the features are read from x [m, stride]. FEAT = true (the
// warm start in one kernel): each warp forms the features of 8 of the tile's
// forests from the spectra (forest_feature_sums, the model tables in shared
// memory after the operand buffers) straight into the A operand, and writes
// their a0; m = sp.num.
template <bool FEAT>
__global__ void __launch_bounds__(kTcThreads, 1) mlp_forward_tc_kernel(
    const __nv_bfloat16 *__restrict__ x, int64_t m, int stride, const uint4 *__restrict__ packed,
    const float *__restrict__ params, float *__restrict__ y, Scratch *scratch,
    const __grid_constant__ pg_spectra sp, const __grid_constant__ pg_cont_model model,
    double *__restrict__ a0_out) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *A = smem;
    unsigned char *W = smem + kTcABytes;
    __shared__ float s_feat_sums[FEAT ? kTcThreads / 32 : 1][2][kFeatBins];
    __shared__ float s_lm[FEAT ? kTcThreads / 32 : 1][8][2];
    FitTables tab{};
    if (FEAT) tab = load_fit_tables(model, smem + kTcABytes + kTcWBytes);
    __shared__ float s_bias[3 * kHidden + kOutPad];
    __shared__ __align__(8) uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // biases (FP32 parameters, after each layer's weights)
    const int64_t ob1 = (int64_t)kIn * kHidden;
    const int64_t ob2 = ob1 + kHidden + (int64_t)kHidden * kHidden;
    const int64_t ob3 = ob2 + kHidden + (int64_t)kHidden * kHidden;
    const int64_t ob4 = ob3 + kHidden + (int64_t)kHidden * kOut;
    for (int i = tid; i < kHidden; i += kTcThreads) {
        s_bias[i] = params[ob1 + i];
        s_bias[kHidden + i] = params[ob2 + i];
        s_bias[2 * kHidden + i] = params[ob3 + i];
    }
    if (tid < kOutPad) s_bias[3 * kHidden + tid] = tid < kOut ? params[ob4 + tid] : 0.f;
    const uint32_t mbar = smem_u32(&s_mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s_tmem)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t a_addr = smem_u32(A), w_addr = smem_u32(W);
    const int quarter = warp & 3;  // this warp's TMEM lanes: 32 quarter .. + 31
    const int part = warp >> 2;    // this warp's quarter of the 256 columns
    const int row = quarter * 32 + lane;
    const uint32_t t_lane = tmem + ((uint32_t)(quarter * 32) << 16);
    uint32_t parity = 0;
    bool ok = true;
    const int64_t ntiles = (m + kTcRows - 1) / kTcRows;
    // operand copies go through the asynchronous copy path, so that the
    // copy for the next MMA overlaps the epilogue of the current one
    auto copy_w = [&](int layer) {
        const int64_t woff = layer == 0 ? 0 : kPackW1 + (int64_t)(layer - 1) * kPackW2;
        const int64_t welems = layer == 0 ? kPackW1 : (layer == 3 ? kPackW4 : kPackW2);
        const uint4 *src = packed + woff / 8;
        for (int64_t e = tid; e < welems / 8; e += kTcThreads)
            cp_async16(reinterpret_cast<uint4 *>(W) + e, src + e, 16u);
    };
    auto copy_x = [&](int64_t row0) {
        if (!FEAT) {
            // features -> A (K = 80: 10 chunks per row), rows past m zero
            for (int e = tid; e < kTcRows * (kInPad / 8); e += kTcThreads) {
                const int r = e / (kInPad / 8), c = e % (kInPad / 8);
                const bool in = row0 + r < m;
                cp_async16(A + img_off(r, c, kInPad / 8),
                           in ? x + (row0 + r) * stride + 8 * c : x, in ? 16u : 0u);
            }
            return;
        }
        // the warp's 8 forests of the tile, features formed in place
        const float bins_per_span =
            (float)(kFeatBins / (model.log_lambda_rest_max - model.log_lambda_rest_min));
        const int r0 = warp * 8;
        if (lane < 8 && row0 + r0 + lane < m) {
            const float2 lm = forest_lmin(sp, model, row0 + r0 + lane);
            s_lm[warp][lane][0] = lm.x;
            s_lm[warp][lane][1] = lm.y;
        }
        __syncwarp();
        for (int j = 0; j < 8; ++j) {
            const int r = r0 + j;
            const int64_t f = row0 + r;
            FeatScalars fs{0.f, 0.f, 0.f};
            if (f < m) {
                fs = forest_feature_sums(sp, tab, f, s_lm[warp][j][0], s_lm[warp][j][1],
                                         bins_per_span, s_feat_sums[warp], lane);
                if (lane == 0) a0_out[f] = f32_to_f64(fs.a0);
            }
            if (lane < kInPad / 8) {
                uint32_t w[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k = 8 * lane + 2 * i;
                    const float lo = f < m ? forest_feature(s_feat_sums[warp], fs, k) : 0.f;
                    const float hi = f < m ? forest_feature(s_feat_sums[warp], fs, k + 1) : 0.f;
                    w[i] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(lo)) |
                           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(hi)) << 16);
                }
                *reinterpret_cast<uint4 *>(A + img_off(r, lane, kInPad / 8)) =
                    make_uint4(w[0], w[1], w[2], w[3]);
            }
            __syncwarp();
        }
    };
    if ((int64_t)blockIdx.x < ntiles) {
        copy_x((int64_t)blockIdx.x * kTcRows);
        copy_w(0);
    }
    cp_async_wait_all();
    proxy_fence();
    tc_fence_before();
    __syncthreads();
    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t row0 = tile * kTcRows;
        for (int layer = 0; layer < 4; ++layer) {
            const int kc = layer == 0 ? kInPad / 8 : kHidden / 8;
            const int n = layer == 3 ? kOutPad : kHidden;
            if (tid == 0) {
                tc_fence_after();
                const uint32_t idesc = tc_idesc(kTcRows, n);
                const uint32_t sbo = (uint32_t)kc * 128u;
                for (int st = 0; st < kc / 2; ++st)
                    tc_mma(tmem, tc_desc(a_addr + 256u * st, 128u, sbo),
                           tc_desc(w_addr + 256u * st, 128u, sbo), idesc, st > 0 ? 1u : 0u);
                tc_commit(mbar);
            }
            ok = __syncthreads_and(mbar_wait(mbar, parity)) != 0;
            parity ^= 1u;
            tc_fence_after();
            if (!ok) break;
            // both operands are free once the MMAs completed: start the copies
            // of the next layer's weights (or of the next tile's features and
            // first weights) under the epilogue
            if (layer < 3) {
                copy_w(layer + 1);
            } else if (tile + gridDim.x < ntiles) {
                copy_w(0);
                copy_x((tile + gridDim.x) * kTcRows);
            }
            if (layer < 3) {
                // bias + GELU, rounded to BF16 into A: the next layer's input
                const float *bias = s_bias + layer * kHidden;
#pragma unroll 1
                for (int j = 0; j < 2; ++j) {
                    const int col0 = part * 64 + 32 * j;
                    float v[32];
                    tmem_ld32(t_lane + (uint32_t)col0, v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t w[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int c0 = 8 * q + 2 * i;
                            const __nv_bfloat16 lo = __float2bfloat16(tc_gelu(v[c0] + bias[col0 + c0]));
                            const __nv_bfloat16 hi =
                                __float2bfloat16(tc_gelu(v[c0 + 1] + bias[col0 + c0 + 1]));
                            w[i] = (uint32_t)__bfloat16_as_ushort(lo) |
                                   ((uint32_t)__bfloat16_as_ushort(hi) << 16);
                        }
                        *reinterpret_cast<uint4 *>(A + img_off(row, col0 / 8 + q, kHidden / 8)) =
                            make_uint4(w[0], w[1], w[2], w[3]);
                    }
                }
            } else if (part == 0) {
                float v[32];
                tmem_ld32(t_lane, v);
                if (row0 + row < m) {
                    y[(row0 + row) * kOut] = v[0] + s_bias[3 * kHidden];
                    y[(row0 + row) * kOut + 1] = v[1] + s_bias[3 * kHidden + 1];
                }
            }
            // copies landed, TMEM reads and A writes done before the next MMA
            cp_async_wait_all();
            proxy_fence();
            tc_fence_before();
            __syncthreads();
        }
    }
    cp_async_wait_all();
    if (!ok && tid == 0) report_error(scratch, PG_ERR_TIMEOUT, 0);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(kTmemCols)
                     : "memory");
    }
}

}  // namespace

int64_t mlp_packed_elems() { return kPackTotal; }

int launch_mlp_pack(const uint16_t *params16, uint16_t *packed, cudaStream_t stream) {
    const int threads = 256;
    const unsigned blocks = (unsigned)((kPackTotal + threads - 1) / threads);
    mlp_pack_kernel<<<blocks, threads, 0, stream>>>(
        reinterpret_cast<const __nv_bfloat16 *>(params16), reinterpret_cast<__nv_bfloat16 *>(packed));
    return check_cuda(cudaGetLastError());
}

int launch_mlp_forward_tc(const uint16_t *packed, const float *params, const uint16_t *x, int64_t m,
                          int stride, float *y, Scratch *scratch, int num_sms,
                          cudaStream_t stream) {
    if (m <= 0) return PG_OK;
    const size_t smem = kTcABytes + kTcWBytes;
    cudaError_t err = cudaFuncSetAttribute(
        mlp_forward_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    const int64_t ntiles = (m + kTcRows - 1) / kTcRows;
    const unsigned blocks = (unsigned)(ntiles < num_sms ? ntiles : num_sms);
    pg_spectra no_sp{};
    pg_cont_model no_model{};
    mlp_forward_tc_kernel<false><<<blocks, kTcThreads, smem, stream>>>(
        reinterpret_cast<const __nv_bfloat16 *>(x), m, stride,
        reinterpret_cast<const uint4 *>(packed), params, y, scratch, no_sp, no_model, nullptr);
    return check_cuda(cudaGetLastError());
}

int launch_mlp_warm_start_tc(const pg_spectra &sp, const pg_cont_model &model,
                             const uint16_t *packed, const float *params, float *y, double *a0,
                             Scratch *scratch, int num_sms, cudaStream_t stream) {
    if (sp.num <= 0) return PG_OK;
    const size_t smem =
        kTcABytes + kTcWBytes + fit_smem_bytes(model.num_mean_cont, model.num_var_intervals);
    if (smem > 220 * 1024) return PG_ERR_UNSUPPORTED;
    cudaError_t err = cudaFuncSetAttribute(
        mlp_forward_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return check_cuda(err);
    const int64_t ntiles = (sp.num + kTcRows - 1) / kTcRows;
    const unsigned blocks = (unsigned)(ntiles < num_sms ? ntiles : num_sms);
    mlp_forward_tc_kernel<true><<<blocks, kTcThreads, smem, stream>>>(
        nullptr, sp.num, 0, reinterpret_cast<const uint4 *>(packed), params, y, scratch, sp, model,
        a0);
    return check_cuda(cudaGetLastError());
}

}  // namespace pg
