// Block-Thomas factorisations with register-resident Gauss-Jordan inversion.
//
//   k_lu_reg64  FP64: D'_j = c0 I + (-J_j) - diag(dA_j) - diag(dC_j) G_{j-1} diag(dB_{j-1}),
//               G_j = D'_j^-1 stored (natural order) + forward sweep of the first
//               right-hand side  z_j = G_j (f_j + dC_j o z_{j-1}).
//   k_lu_reg32  FP32 on the power-of-two row/column-scaled blocks (see vk_mixed.cu):
//               G~_j = (R_j D'_j S_j)^-1 stored in FP32 with the scales.
// One CTA per column; each CTA walks its layers in order.  Block sizes up to
// 160 species are covered by four register tilings (vk_gjreg.cuh).
#include <cuda_runtime.h>
#include <math.h>

#include "vk_gjreg.cuh"
#include "vk_internal.cuh"

namespace vk {

namespace {

__device__ __forceinline__ double pow2_scale_r(double m) {
    if (!(m > 0.0) || !isfinite(m)) return 1.0;
    int e;
    frexp(m, &e);
    return ldexp(1.0, -e);
}

template <int TY>
__device__ __forceinline__ void tile_coords(int &ty, int &tx) {
    ty = threadIdx.x % TY;
    tx = threadIdx.x / TY;
}

}  // namespace

template <int TY, int RA, int RB>
__global__ void __launch_bounds__(16 * TY, TY == 16 ? 2 : 1)
k_lu_reg64(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
           const double *__restrict__ dB, const double *__restrict__ dC,
           const double *__restrict__ dt, const double *__restrict__ rhs,
           double *__restrict__ G, double *__restrict__ z, int *__restrict__ status) {
    extern __shared__ double smd[];
    const int n = net.ni, nn = n * n;
    const int c = blockIdx.x;
    if (b.active && !b.active[c]) return;
    const int l0 = b.col_off[c], nz = b.col_off[c + 1] - l0;
    double *Gs = smd;                  // [n*n] natural-order inverse of the previous layer
    double *rowv = Gs + nn;
    double *colv = rowv + n;
    double *zp = colv + n;
    double *bb = zp + n;
    double *zr = bb + n;
    int *perm = reinterpret_cast<int *>(zr + n);
    int *kinv = perm + n;
    int *used = kinv + n;
    __shared__ int s_piv, s_sing;
    __shared__ double s_pval;
    GJShared<double> sh{rowv, colv, perm, kinv, used, &s_piv, &s_pval, &s_sing};
    int ty, tx;
    tile_coords<TY>(ty, tx);
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    if (tid == 0) s_sing = 0;
    const double c0 = 1.0 / (R_ROS * dt[c]);
    for (int j = 0; j < nz; ++j) {
        const size_t l = (size_t)l0 + j;
        const double *jl = jv + l * net.nnz;
        const double *cj = dC + l * n;
        const double *aj = dA + l * n;
        const double *bm = j > 0 ? dB + (l - 1) * n : dB;
        double M[RA][RB];
#pragma unroll
        for (int a = 0; a < RA; ++a) {
            const int r = ty + TY * a;
#pragma unroll
            for (int q = 0; q < RB; ++q) {
                const int cc = tx + 16 * q;
                double v = 0.0;
                if (r < n && cc < n) {
                    if (j > 0) v = -cj[r] * Gs[r * n + cc] * bm[cc];
                    if (r == cc) v += c0 - aj[r];
                    const int e = net.jmap[r * n + cc];
                    if (e >= 0) v += jl[e];
                }
                M[a][q] = v;
            }
        }
        for (int t = tid; t < n; t += nth) {
            bb[t] = rhs[l * n + t] + (j > 0 ? cj[t] * zp[t] : 0.0);
            used[t] = 0;
        }
        __syncthreads();
        gj_invert_reg<double, TY, RA, RB>(M, n, ty, tx, sh);
        gj_store_natural<double, TY, RA, RB>(M, n, ty, tx, sh, Gs);
        double *Gl = G + l * nn;
        for (int e = tid; e < nn; e += nth) Gl[e] = Gs[e];
        for (int r = warp; r < n; r += nwarp) {
            double s = 0.0;
            for (int q = lane; q < n; q += 32) s += Gs[r * n + q] * bb[q];
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) zr[r] = s;
        }
        __syncthreads();
        for (int t = tid; t < n; t += nth) {
            zp[t] = zr[t];
            z[l * n + t] = zr[t];
        }
        __syncthreads();
    }
    if (tid == 0 && s_sing) status[c] = s_sing == 2 ? VK_ENAN : VK_ESINGULAR;
}

template <int TY, int RA, int RB>
__global__ void __launch_bounds__(16 * TY, TY == 16 ? 3 : 1)
k_lu_reg32(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
           const double *__restrict__ dB, const double *__restrict__ dC,
           const double *__restrict__ dt, float *__restrict__ G32, double *__restrict__ rsc,
           double *__restrict__ csc, int *__restrict__ status) {
    extern __shared__ double smd[];
    const int n = net.ni, nn = n * n;
    const int c = blockIdx.x;
    if (b.active && !b.active[c]) return;
    const int l0 = b.col_off[c], nz = b.col_off[c + 1] - l0;
    double *rs = smd;
    double *cs = rs + n;
    double *rs_prev = cs + n;
    double *cs_prev = rs_prev + n;
    float *Gs = reinterpret_cast<float *>(cs_prev + n);     // [n*n]
    float *rowv = Gs + nn;
    float *colv = rowv + n;
    float *alpha = colv + n;
    float *beta = alpha + n;
    int *perm = reinterpret_cast<int *>(beta + n);
    int *kinv = perm + n;
    int *used = kinv + n;
    int *cexp = used + n;
    __shared__ int s_piv, s_sing;
    __shared__ float s_pval;
    GJShared<float> sh{rowv, colv, perm, kinv, used, &s_piv, &s_pval, &s_sing};
    int ty, tx;
    tile_coords<TY>(ty, tx);
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    if (tid == 0) s_sing = 0;
    const double c0 = 1.0 / (R_ROS * dt[c]);
    for (int j = 0; j < nz; ++j) {
        const size_t l = (size_t)l0 + j;
        const double *jl = jv + l * net.nnz;
        const double *aj = dA + l * n;
        // row scales: row maxima of the FP64 diagonal block D_j
        for (int r = warp; r < n; r += nwarp) {
            double m = 0.0;
            for (int e = net.jrowptr[r] + lane; e < net.jrowptr[r + 1]; e += 32) {
                double v = jl[e];
                if (net.jcol[e] == r) v += c0 - aj[r];
                m = fmax(m, fabs(v));
            }
            for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) rs[r] = pow2_scale_r(fmax(m, fabs(c0 - aj[r])));
        }
        for (int t = tid; t < n; t += nth) { cexp[t] = -100000; used[t] = 0; }
        __syncthreads();
        // column scales: column maxima of R_j D_j (exponents)
        for (int e = tid; e < net.nnz + n; e += nth) {
            int r, q;
            double v;
            if (e < net.nnz) {
                r = net.jrow[e]; q = net.jcol[e];
                v = jl[e] + (r == q ? c0 - aj[r] : 0.0);
            } else {
                r = q = e - net.nnz;
                v = c0 - aj[r];
            }
            v = fabs(v * rs[r]);
            if (v > 0.0 && isfinite(v)) {
                int ex;
                frexp(v, &ex);
                atomicMax(&cexp[q], ex);
            }
        }
        __syncthreads();
        for (int t = tid; t < n; t += nth) {
            cs[t] = cexp[t] > -100000 ? ldexp(1.0, -cexp[t]) : 1.0;
            if (j > 0) {
                alpha[t] = (float)(rs[t] * dC[l * n + t] * cs_prev[t]);
                beta[t] = (float)(rs_prev[t] * dB[(l - 1) * n + t] * cs[t]);
            }
        }
        __syncthreads();
        float M[RA][RB];
#pragma unroll
        for (int a = 0; a < RA; ++a) {
            const int r = ty + TY * a;
#pragma unroll
            for (int q = 0; q < RB; ++q) {
                const int cc = tx + 16 * q;
                float v = 0.0f;
                if (r < n && cc < n) {
                    if (j > 0) v = -alpha[r] * Gs[r * n + cc] * beta[cc];
                    double d = (r == cc) ? c0 - aj[r] : 0.0;
                    const int e = net.jmap[r * n + cc];
                    if (e >= 0) d += jl[e];
                    if (d != 0.0) v += (float)(rs[r] * d * cs[cc]);
                }
                M[a][q] = v;
            }
        }
        __syncthreads();
        gj_invert_reg<float, TY, RA, RB>(M, n, ty, tx, sh);
        gj_store_natural<float, TY, RA, RB>(M, n, ty, tx, sh, Gs);
        float *Gl = G32 + l * nn;
        for (int e = tid; e < nn; e += nth) Gl[e] = Gs[e];
        for (int t = tid; t < n; t += nth) {
            rsc[l * n + t] = rs[t];
            csc[l * n + t] = cs[t];
            rs_prev[t] = rs[t];
            cs_prev[t] = cs[t];
        }
        __syncthreads();
    }
    if (tid == 0 && s_sing) status[c] = s_sing == 2 ? VK_ENAN : VK_ESINGULAR;
}

// ---------------------------------------------------------------------------
static size_t smem64(int n) { return (size_t)(n * n + 5 * n) * sizeof(double) + 3 * n * sizeof(int) + 16; }
static size_t smem32(int n) {
    return (size_t)4 * n * sizeof(double) + (size_t)(n * n + 4 * n) * sizeof(float) + 4 * n * sizeof(int) + 16;
}

#define VK_LU_TILINGS(X) X(16, 3, 3) X(16, 5, 5) X(16, 7, 7) X(32, 5, 10)

static int tiling_of(int n) {
    if (n <= 48) return 0;
    if (n <= 80) return 1;
    if (n <= 112) return 2;
    return 3;
}

cudaError_t init_lureg_kernels(int n) {
    cudaError_t e = cudaSuccess;
    size_t s64 = smem64(n), s32 = smem32(n);
#define SETATTR(TY, RA, RB)                                                                      \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lu_reg64<TY, RA, RB>,                       \
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s64); \
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_lu_reg32<TY, RA, RB>,                       \
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s32);
    VK_LU_TILINGS(SETATTR)
#undef SETATTR
    return e;
}

void launch_lu_reg64(const DevNet &net, const DevBatch &b, const Work &w, const double *rhs,
                     double *z, cudaStream_t s) {
    const int n = net.ni;
    size_t sm = smem64(n);
    switch (tiling_of(n)) {
    case 0: k_lu_reg64<16, 3, 3><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, w.G, z, w.status); break;
    case 1: k_lu_reg64<16, 5, 5><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, w.G, z, w.status); break;
    case 2: k_lu_reg64<16, 7, 7><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, w.G, z, w.status); break;
    default: k_lu_reg64<32, 5, 10><<<b.ncols, 512, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, w.G, z, w.status); break;
    }
}

void launch_lu_reg32(const DevNet &net, const DevBatch &b, const Work &w, cudaStream_t s) {
    const int n = net.ni;
    size_t sm = smem32(n);
    switch (tiling_of(n)) {
    case 0: k_lu_reg32<16, 3, 3><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, w.G32, w.rs, w.cs, w.status); break;
    case 1: k_lu_reg32<16, 5, 5><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, w.G32, w.rs, w.cs, w.status); break;
    case 2: k_lu_reg32<16, 7, 7><<<b.ncols, 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, w.G32, w.rs, w.cs, w.status); break;
    default: k_lu_reg32<32, 5, 10><<<b.ncols, 512, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, w.G32, w.rs, w.cs, w.status); break;
    }
}

}  // namespace vk
