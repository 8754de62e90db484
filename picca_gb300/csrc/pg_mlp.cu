// Learned warm start for the continuum fit: kernels of a small MLP
// (BF16 tensor-core GEMM with FP32 accumulation and fused epilogues, column
// sums for bias gradients, the MSE-loss gradient and Adam). The reference
// has no counterpart; see include/picca_gb300.h.
//
// GEMM: C[M,N] = A[M,K] B[K,N] with arbitrary element strides for A and B
// (so X W, dZ W^T and X^T dZ all use one kernel). CTA tile 64 x 64 x 32,
// four warps in a 2 x 2 arrangement, each warp 32 x 32 built from
// mma.sync m16n8k16 BF16 -> FP32 tiles. Operands are staged through shared
// memory with bounds checks (zero fill), so M, N and K need no padding.
#include <cuda_bf16.h>

#include "pg_internal.cuh"

namespace pg {
namespace {

constexpr int kBM = 64, kBN = 64, kBK = 32;
constexpr int kGemmThreads = 128;
constexpr int kPadA = 8, kPadB = 8;

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    uint32_t l = (uint32_t)__bfloat16_as_ushort(lo);
    uint32_t h = (uint32_t)__bfloat16_as_ushort(hi);
    return l | (h << 16);
}

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float gelu(float x) {
    return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

struct GemmArgs {
    const __nv_bfloat16 *a;
    int64_t sam, sak;
    const __nv_bfloat16 *b;
    int64_t sbk, sbn;
    int m, n, k;
    const float *bias;         // [n] or nullptr
    int epilogue;              // PG_MLP_EPI_* flags
    const float *zin;          // pre-activations for the GELU backward, [m, ldz]
    float *zout;               // pre-activations written by the forward, [m, ldz]
    int64_t ldz;
    __nv_bfloat16 *c;          // bf16 output [m, ldc] or nullptr
    float *cf;                 // fp32 output [m, ldc] or nullptr
    int64_t ldc;
    float beta;                // fp32 output: cf = acc + beta * cf
};

__global__ void __launch_bounds__(kGemmThreads) gemm_bf16_kernel(const GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[kBM][kBK + kPadA];
    __shared__ __align__(16) __nv_bfloat16 Bs[kBK][kBN + kPadB];
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int group = lane >> 2, tig = lane & 3;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = 0; k0 < g.k; k0 += kBK) {
        for (int e = tid; e < kBM * kBK; e += kGemmThreads) {
            const int mm = e / kBK, kk = e % kBK;
            const int gm = m0 + mm, gk = k0 + kk;
            As[mm][kk] = (gm < g.m && gk < g.k) ? g.a[gm * g.sam + gk * g.sak] : zero;
        }
        for (int e = tid; e < kBK * kBN; e += kGemmThreads) {
            const int kk = e / kBN, nn = e % kBN;
            const int gk = k0 + kk, gn = n0 + nn;
            Bs[kk][nn] = (gk < g.k && gn < g.n) ? g.b[gk * g.sbk + gn * g.sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < kBK; ks += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm * 32 + i * 16 + group;
                const int c = ks + tig * 2;
                af[i][0] = pack_bf16(As[r][c], As[r][c + 1]);
                af[i][1] = pack_bf16(As[r + 8][c], As[r + 8][c + 1]);
                af[i][2] = pack_bf16(As[r][c + 8], As[r][c + 9]);
                af[i][3] = pack_bf16(As[r + 8][c + 8], As[r + 8][c + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int nn = wn * 32 + j * 8 + group;
                const int kk = ks + tig * 2;
                bfr[j][0] = pack_bf16(Bs[kk][nn], Bs[kk + 1][nn]);
                bfr[j][1] = pack_bf16(Bs[kk + 8][nn], Bs[kk + 9][nn]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bfr[j]);
        }
        __syncthreads();
    }
    // epilogue
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int gm = m0 + wm * 32 + i * 16 + group + ((r >> 1) << 3);
                const int gn = n0 + wn * 32 + j * 8 + tig * 2 + (r & 1);
                if (gm >= g.m || gn >= g.n) continue;
                float v = acc[i][j][r];
                if (g.bias) v += g.bias[gn];
                if (g.zout) g.zout[gm * g.ldz + gn] = v;
                if (g.epilogue & PG_MLP_EPI_GELU) v = gelu(v);
                if (g.epilogue & PG_MLP_EPI_GELU_GRAD) v *= gelu_grad(g.zin[gm * g.ldz + gn]);
                if (g.c) g.c[gm * g.ldc + gn] = __float2bfloat16(v);
                if (g.cf) {
                    const int64_t o = gm * g.ldc + gn;
                    g.cf[o] = g.beta != 0.f ? v + g.beta * g.cf[o] : v;
                }
            }
        }
    }
}

// column sums of a bf16 [m, ldx] matrix (bias gradients)
__global__ void colsum_kernel(const __nv_bfloat16 *__restrict__ x, int m, int n, int64_t ldx,
                              float *__restrict__ out) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= n) return;
    float s = 0.f;
    for (int r = 0; r < m; ++r) s += __bfloat162float(x[r * ldx + col]);
    out[col] = s;
}

// dY = 2 (Y - T) / m (MSE over m rows), written as bf16; loss partial sums
__global__ void mse_grad_kernel(const float *__restrict__ y, const float *__restrict__ t, int m,
                                int n, __nv_bfloat16 *__restrict__ dy, float *__restrict__ loss) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < (int64_t)m * n) {
        const float d = y[i] - t[i];
        dy[i] = __float2bfloat16(2.f * d / (float)m);
        l = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l / (float)m);
}

__global__ void adam_kernel(float *__restrict__ p, const float *__restrict__ grad,
                            float *__restrict__ m1, float *__restrict__ m2,
                            __nv_bfloat16 *__restrict__ p16, int64_t n, float lr, float beta1,
                            float beta2, float eps, float bc1, float bc2, float weight_decay) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i] + weight_decay * p[i];
    const float a = beta1 * m1[i] + (1.f - beta1) * g;
    const float b = beta2 * m2[i] + (1.f - beta2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float mh = a / bc1, vh = b / bc2;
    const float np = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = np;
    if (p16) p16[i] = __float2bfloat16(np);
}

__global__ void to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y,
                               int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16(x[i]);
}

}  // namespace
}  // namespace pg

using namespace pg;

extern "C" {

int pg_mlp_gemm(const uint16_t *a, int64_t sam, int64_t sak, const uint16_t *b, int64_t sbk,
                int64_t sbn, int32_t m, int32_t n, int32_t k, const float *bias, int32_t epilogue,
                const float *zin, float *zout, int64_t ldz, uint16_t *c, float *cf, int64_t ldc,
                float beta, void *stream) {
    if (!a || !b || m < 0 || n < 0 || k < 0 || (!c && !cf)) return PG_ERR_INVALID_ARGUMENT;
    if ((epilogue & PG_MLP_EPI_GELU_GRAD) && !zin) return PG_ERR_INVALID_ARGUMENT;
    if ((zin || zout) && ldz < n) return PG_ERR_INVALID_ARGUMENT;
    if (ldc < n) return PG_ERR_INVALID_ARGUMENT;
    if (m == 0 || n == 0) return PG_OK;
    GemmArgs g;
    g.a = reinterpret_cast<const __nv_bfloat16 *>(a);
    g.sam = sam; g.sak = sak;
    g.b = reinterpret_cast<const __nv_bfloat16 *>(b);
    g.sbk = sbk; g.sbn = sbn;
    g.m = m; g.n = n; g.k = k;
    g.bias = bias; g.epilogue = epilogue; g.zin = zin; g.zout = zout; g.ldz = ldz;
    g.c = reinterpret_cast<__nv_bfloat16 *>(c); g.cf = cf; g.ldc = ldc; g.beta = beta;
    const dim3 grid((unsigned)((n + kBN - 1) / kBN), (unsigned)((m + kBM - 1) / kBM));
    gemm_bf16_kernel<<<grid, kGemmThreads, 0, static_cast<cudaStream_t>(stream)>>>(g);
    return check_cuda(cudaGetLastError());
}

int pg_mlp_colsum(const uint16_t *x, int32_t m, int32_t n, int64_t ldx, float *out,
                  void *stream) {
    if (!x || !out || m < 0 || n < 0 || ldx < n) return PG_ERR_INVALID_ARGUMENT;
    if (n == 0) return PG_OK;
    colsum_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        reinterpret_cast<const __nv_bfloat16 *>(x), m, n, ldx, out);
    return check_cuda(cudaGetLastError());
}

int pg_mlp_mse_grad(const float *y, const float *t, int32_t m, int32_t n, uint16_t *dy,
                    float *loss, void *stream) {
    if (!y || !t || !dy || m <= 0 || n <= 0) return PG_ERR_INVALID_ARGUMENT;
    const int64_t total = (int64_t)m * n;
    mse_grad_kernel<<<(unsigned)((total + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        y, t, m, n, reinterpret_cast<__nv_bfloat16 *>(dy), loss);
    return check_cuda(cudaGetLastError());
}

int pg_mlp_adam(float *params, const float *grads, float *m1, float *m2, uint16_t *params_bf16,
                int64_t n, float lr, float beta1, float beta2, float eps, int32_t step,
                float weight_decay, void *stream) {
    if (!params || !grads || !m1 || !m2 || n < 0 || step < 1) return PG_ERR_INVALID_ARGUMENT;
    if (n == 0) return PG_OK;
    const float bc1 = 1.f - powf(beta1, (float)step);
    const float bc2 = 1.f - powf(beta2, (float)step);
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grads, m1, m2, reinterpret_cast<__nv_bfloat16 *>(params_bf16), n, lr, beta1, beta2,
        eps, bc1, bc2, weight_decay);
    return check_cuda(cudaGetLastError());
}

int pg_mlp_to_bf16(const float *x, uint16_t *y, int64_t n, void *stream) {
    if (!x || !y || n < 0) return PG_ERR_INVALID_ARGUMENT;
    if (n == 0) return PG_OK;
    to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        x, reinterpret_cast<__nv_bfloat16 *>(y), n);
    return check_cuda(cudaGetLastError());
}

}  // extern "C"
