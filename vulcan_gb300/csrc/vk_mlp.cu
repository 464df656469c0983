// BF16 MLP kernels for the learned warm start (forward, backward, Adam).
//
// The network proposes a near-steady log mixing-ratio profile per layer; it
// has no counterpart in the reference.  Weights and activations are BF16,
// accumulation FP32 (tensor-core mma.sync m16n8k16), master weights and
// optimiser state FP32.  All buffers are device pointers owned by the caller.
//
//   forward layer   Z = X W + b,  H = silu(Z) (or Z)          X [B,K], W [K,N]
//   backward layer  dZ = dH o silu'(Z);  dW = X^T dZ;  db = sum_rows dZ;
//                   dX = dZ W^T
//   Adam            m, v, w (FP32) and the BF16 copy of w
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "vk_internal.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 32;      // CTA tile; 4 warps of 32x32
constexpr int PADA = 8, PADB = 8;

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

enum Epi { EPI_FWD = 0, EPI_F32 = 1 };

// C[M,N] = sum_k A(m,k) B(k,n); A(m,k) = A[m*sam + k*sak], B(k,n) = B[k*sbk + n*sbn].
// EPI_FWD: Z = C + bias (FP32, optional), H = bf16(silu?(Z)) (optional).
// EPI_F32: Cf[m*N + n] = C (+ Cf if accumulate).
template <int EPI>
__global__ void __launch_bounds__(128)
k_gemm_bf16(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, long long sam, long long sak,
            const __nv_bfloat16 *__restrict__ B, long long sbk, long long sbn,
            const float *__restrict__ bias, float *__restrict__ Z, __nv_bfloat16 *__restrict__ H,
            int act, float *__restrict__ Cf, int accumulate) {
    __shared__ __nv_bfloat16 As[BM][BK + PADA];
    __shared__ __nv_bfloat16 Bs[BK][BN + PADB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int e = tid; e < BM * BK; e += 128) {
            const int r = e / BK, c = e - r * BK;
            const int gm = m0 + r, gk = k0 + c;
            As[r][c] = (gm < M && gk < K) ? A[gm * sam + gk * sak] : zero;
        }
        for (int e = tid; e < BK * BN; e += 128) {
            const int r = e / BN, c = e - r * BN;
            const int gk = k0 + r, gn = n0 + c;
            Bs[r][c] = (gk < K && gn < N) ? B[gk * sbk + gn * sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + 16 * i + g;
                af[i][0] = pack_bf16(As[r][kk + 2 * t], As[r][kk + 2 * t + 1]);
                af[i][1] = pack_bf16(As[r + 8][kk + 2 * t], As[r + 8][kk + 2 * t + 1]);
                af[i][2] = pack_bf16(As[r][kk + 2 * t + 8], As[r][kk + 2 * t + 9]);
                af[i][3] = pack_bf16(As[r + 8][kk + 2 * t + 8], As[r + 8][kk + 2 * t + 9]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + 8 * j + g;
                bf[j][0] = pack_bf16(Bs[kk + 2 * t][c], Bs[kk + 2 * t + 1][c]);
                bf[j][1] = pack_bf16(Bs[kk + 2 * t + 8][c], Bs[kk + 2 * t + 9][c]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int m = m0 + wm + 16 * i + g + (q >= 2 ? 8 : 0);
                const int n = n0 + wn + 8 * j + 2 * t + (q & 1);
                if (m >= M || n >= N) continue;
                const float v = acc[i][j][q];
                if (EPI == EPI_FWD) {
                    const float z = v + (bias ? bias[n] : 0.0f);
                    if (Z) Z[(long long)m * N + n] = z;
                    if (H) H[(long long)m * N + n] = __float2bfloat16(act ? silu(z) : z);
                } else {
                    const long long o = (long long)m * N + n;
                    Cf[o] = accumulate ? Cf[o] + v : v;
                }
            }
}

// dZ = dH o silu'(Z) (or dH) -> BF16; db[n] += column sums handled by k_colsum.
__global__ void k_act_bwd(long long total, const float *__restrict__ dH, const float *__restrict__ Z,
                          int act, __nv_bfloat16 *__restrict__ dZ) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const float d = act ? dH[i] * dsilu(Z[i]) : dH[i];
    dZ[i] = __float2bfloat16(d);
}

// db[n] = sum_m dZ[m, n] (deterministic: one thread per column, fixed order)
__global__ void k_colsum(int M, int N, const __nv_bfloat16 *__restrict__ dZ, float *__restrict__ db) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) s += __bfloat162float(dZ[(long long)m * N + n]);
    db[n] = s;
}

__global__ void k_adam(long long n, float *__restrict__ w, __nv_bfloat16 *__restrict__ wb,
                       const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

int mlp_fail(const char *msg) {
    vk::set_global_error(msg);
    return VK_EINVAL;
}

int launch_check(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        vk::set_global_error(std::string(what) + ": " + cudaGetErrorString(e));
        return VK_ECUDA;
    }
    return VK_OK;
}

}  // namespace

extern "C" int vk_mlp_forward(int B, int K, int N, const void *X, const void *W, const float *bias,
                              float *Z, void *H, int silu_act, void *stream) {
    if (B <= 0 || K <= 0 || N <= 0 || !X || !W) return mlp_fail("vk_mlp_forward: bad arguments");
    if (!Z && !H) return mlp_fail("vk_mlp_forward: no output");
    dim3 grid((N + BN - 1) / BN, (B + BM - 1) / BM);
    k_gemm_bf16<EPI_FWD><<<grid, 128, 0, (cudaStream_t)stream>>>(
        B, N, K, (const __nv_bfloat16 *)X, K, 1, (const __nv_bfloat16 *)W, N, 1, bias, Z,
        (__nv_bfloat16 *)H, silu_act, nullptr, 0);
    return launch_check("vk_mlp_forward");
}

extern "C" int vk_mlp_backward(int B, int K, int N, const void *X, const void *W, const float *Z,
                               const float *dH, int silu_act, void *dZ_scratch, float *dW,
                               float *db, float *dX, void *stream) {
    if (B <= 0 || K <= 0 || N <= 0 || !X || !W || !Z || !dH || !dZ_scratch)
        return mlp_fail("vk_mlp_backward: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    const long long total = (long long)B * N;
    __nv_bfloat16 *dZ = (__nv_bfloat16 *)dZ_scratch;
    k_act_bwd<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(total, dH, Z, silu_act, dZ);
    if (dW) {   // dW[K,N] = X^T dZ : A(m=k, kk=b) = X[b*K + k], B(kk=b, n) = dZ[b*N + n]
        dim3 grid((N + BN - 1) / BN, (K + BM - 1) / BM);
        k_gemm_bf16<EPI_F32><<<grid, 128, 0, s>>>(K, N, B, (const __nv_bfloat16 *)X, 1, K, dZ, N, 1,
                                                  nullptr, nullptr, nullptr, 0, dW, 0);
    }
    if (db) k_colsum<<<(N + 127) / 128, 128, 0, s>>>(B, N, dZ, db);
    if (dX) {   // dX[B,K] = dZ W^T : A(m=b, kk=n) = dZ[b*N + n], B(kk=n, col=k) = W[k*N + n]
        dim3 grid((K + BN - 1) / BN, (B + BM - 1) / BM);
        k_gemm_bf16<EPI_F32><<<grid, 128, 0, s>>>(B, K, N, dZ, N, 1, (const __nv_bfloat16 *)W, 1, N,
                                                  nullptr, nullptr, nullptr, 0, dX, 0);
    }
    return launch_check("vk_mlp_backward");
}

extern "C" int vk_mlp_adam(long long n, float *w, void *w_bf16, const float *g, float *m, float *v,
                           float lr, float beta1, float beta2, float eps, int step, void *stream) {
    if (n <= 0 || !w || !g || !m || !v || step < 1) return mlp_fail("vk_mlp_adam: bad arguments");
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        n, w, (__nv_bfloat16 *)w_bf16, g, m, v, lr, beta1, beta2, eps, c1, c2);
    return launch_check("vk_mlp_adam");
}
