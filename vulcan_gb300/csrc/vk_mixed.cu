// Mixed-precision block-tridiagonal solve: FP32 factorisation on scaled
// blocks, FP64 residual and iterative refinement.
//
// The system is the Ros2 LHS  A = c0 I - J_chem - J_diff  (op.py:1973-2042):
// dense diagonal blocks D_j = c0 I + (-J_j) - diag(dA_j) and diagonal couplings
// L_j = -diag(dC_j) (to layer j-1), U_j = -diag(dB_j) (to layer j+1).
//
// k_lu_f32 (one CTA per column) factorises the scaled system R A S, with
// per-layer power-of-two row scales R_j (row maxima of D_j) and column scales
// S_j (column maxima of R_j D_j), so the scaling itself is exact.  Each
// Schur-complemented scaled block  D~'_j = R_j D_j S_j - L~_j G~_{j-1} U~_{j-1}
// is inverted in place in shared memory by FP32 Gauss-Jordan with partial
// pivoting; G~_j is stored in FP32 (half the bytes of the FP64 path).
//
// k_refine (one CTA per column) solves A x = b: x = 0, r = b; repeat
// { d = S M~^-1 R r  (FP32 forward/back sweeps with G~);  x += d (FP64);
//   r = b - A x  (FP64, matrix-free from the sparse -J and dA/dB/dC) }
// until max |d| / (|x| + |yscale| + 1e-10 n_0) <= tol or max sweeps; a
// column that does not converge is flagged for the FP64 path.
#include <cuda_runtime.h>
#include <math.h>

#include "vk_internal.cuh"

namespace vk {

__device__ __forceinline__ double pow2_scale(double m) {
    // 2^-e with m = f 2^e, f in [0.5, 1): scaled value in [0.5, 1)
    if (!(m > 0.0) || !isfinite(m)) return 1.0;
    int e;
    frexp(m, &e);
    return ldexp(1.0, -e);
}

// In-place FP32 Gauss-Jordan inversion (partial pivoting, lowest row on ties).
__device__ void gj_invert_f32(float *A, int n, float *colk, float *rowk, int *perm,
                              int *s_piv, float *s_pval, int *s_sing) {
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nn = n * n;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            float best = -1.0f;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                float a = fabsf(A[i * n + k]);
                if (a > best) { best = a; bi = i; }
            }
            for (int o = 16; o; o >>= 1) {
                float ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) {
                if (best < 0.0f || bi >= n || isinf(best)) { *s_sing = 2; bi = k; }
                else if (!(best > 0.0f)) { if (*s_sing == 0) *s_sing = 1; bi = k; }
                *s_piv = bi;
                *s_pval = A[bi * n + k];
                perm[k] = bi;
            }
        }
        __syncthreads();
        const int p = *s_piv;
        const float pval = *s_pval;
        const float pinv = 1.0f / pval;
        for (int t = tid; t < n; t += nth) {
            float ak = A[k * n + t], ap = A[p * n + t];
            rowk[t] = (t == k) ? pinv : ap * pinv;
            if (p != k) A[p * n + t] = ak;
            colk[t] = (t == k) ? pval : ((t == p) ? A[k * n + k] : A[t * n + k]);
        }
        __syncthreads();
        for (int e = tid; e < nn; e += nth) {
            int i = e / n, jj = e - i * n;
            if (i == k) A[e] = rowk[jj];
            else A[e] = (jj == k ? 0.0f : A[e]) - colk[i] * rowk[jj];
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
        int p = perm[k];
        if (p != k) {
            for (int t = tid; t < n; t += nth) {
                float a = A[t * n + k];
                A[t * n + k] = A[t * n + p];
                A[t * n + p] = a;
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(256)
k_lu_f32(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
         const double *__restrict__ dB, const double *__restrict__ dC,
         const double *__restrict__ dt, float *__restrict__ G32, double *__restrict__ rsc,
         double *__restrict__ csc, int *__restrict__ status) {
    extern __shared__ float smf[];
    const int n = net.ni, nn = n * n;
    const int c = blockIdx.x;
    if (b.active && !b.active[c]) return;
    const int l0 = b.col_off[c], nz = b.col_off[c + 1] - l0;
    float *A = smf;                                  // [n*n]
    float *colk = A + nn;
    float *rowk = colk + n;
    float *alpha = rowk + n;
    float *beta = alpha + n;
    int *perm = reinterpret_cast<int *>(beta + n);
    int *cexp = perm + n;
    double *rs = reinterpret_cast<double *>(cexp + n + (n & 1));   // 8-byte aligned
    double *cs = rs + n;
    double *rs_prev = cs + n;
    double *cs_prev = rs_prev + n;
    __shared__ int s_piv, s_sing;
    __shared__ float s_pval;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    if (tid == 0) s_sing = 0;
    const double c0 = 1.0 / (R_ROS * dt[c]);
    for (int j = 0; j < nz; ++j) {
        const size_t l = (size_t)l0 + j;
        const double *jl = jv + l * net.nnz;
        const double *aj = dA + l * n;
        // row scales from the FP64 diagonal block D_j (warp per row, CSR by row)
        for (int r = warp; r < n; r += nwarp) {
            double m = 0.0;
            for (int e = net.jrowptr[r] + lane; e < net.jrowptr[r + 1]; e += 32) {
                double v = jl[e];
                if (net.jcol[e] == r) v += c0 - aj[r];
                m = fmax(m, fabs(v));
            }
            for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) {
                m = fmax(m, fabs(c0 - aj[r]));
                rs[r] = pow2_scale(m);
            }
        }
        for (int t = tid; t < n; t += nth) cexp[t] = -100000;
        __syncthreads();
        // column scales from R_j D_j (exponent max per column)
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
        // scaled Schur complement in FP32 (A holds G~_{j-1})
        for (int e = tid; e < nn; e += nth) {
            int r = e / n, q = e - r * n;
            float v = j > 0 ? -alpha[r] * A[e] * beta[q] : 0.0f;
            if (r == q) v += (float)(rs[r] * (c0 - aj[r]) * cs[r]);
            A[e] = v;
        }
        __syncthreads();
        for (int e = tid; e < net.nnz; e += nth) {
            int r = net.jrow[e], q = net.jcol[e];
            A[r * n + q] += (float)(rs[r] * jl[e] * cs[q]);
        }
        __syncthreads();
        gj_invert_f32(A, n, colk, rowk, perm, &s_piv, &s_pval, &s_sing);
        float *Gl = G32 + l * nn;
        for (int e = tid; e < nn; e += nth) Gl[e] = A[e];
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

// Iterative refinement of A x = b with the FP32 factors (one CTA per column).
// yscale (may be NULL) widens the convergence floor: k1/k2 enter sol next to y.
__global__ void __launch_bounds__(256)
k_refine(DevNet net, DevBatch b, const float *__restrict__ G32, const double *__restrict__ rsc,
         const double *__restrict__ csc, const double *__restrict__ jv,
         const double *__restrict__ dA, const double *__restrict__ dB,
         const double *__restrict__ dC, const double *__restrict__ dt,
         const double *__restrict__ rhs, double *__restrict__ x, double *__restrict__ res,
         float *__restrict__ zf, const double *__restrict__ yscale, double *__restrict__ yk2,
         const double *__restrict__ y, int max_sweeps, double tol, int *__restrict__ fallback,
         int *__restrict__ sweeps_out) {
    extern __shared__ float smr[];
    const int n = net.ni, nn = n * n;
    const int c = blockIdx.x;
    if (b.active && !b.active[c]) return;
    const int l0 = b.col_off[c], nz = b.col_off[c + 1] - l0;
    float *vin = smr;               // [n]
    float *vout = vin + n;          // [n]
    __shared__ double red[8];
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    const double c0 = 1.0 / (R_ROS * dt[c]);
    const size_t base = (size_t)l0 * n;
    for (int e = tid; e < nz * n; e += nth) {
        x[base + e] = 0.0;
        res[base + e] = rhs[base + e];
    }
    __syncthreads();
    int sweep = 0, converged = 0;
    for (; sweep < max_sweeps && !converged; ++sweep) {
        // forward: z~_j = G~_j (R_j r_j + R_j dC_j S_{j-1} z~_{j-1})
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            for (int t = tid; t < n; t += nth) {
                double v = rsc[l * n + t] * res[l * n + t];
                if (j > 0) v += rsc[l * n + t] * dC[l * n + t] * csc[(l - 1) * n + t] * (double)vout[t];
                vin[t] = (float)v;
            }
            __syncthreads();
            const float *Gl = G32 + l * nn;
            for (int r = warp; r < n; r += nwarp) {
                float s = 0.0f;
                for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * vin[q];
                for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == 0) { zf[l * n + r] = s; vout[r] = s; }
            }
            __syncthreads();
        }
        // back: x~_j = z~_j + G~_j (R_j dB_j S_{j+1} x~_{j+1}); x += S_j x~_j
        double dmax = 0.0;
        for (int j = nz - 1; j >= 0; --j) {
            const size_t l = (size_t)l0 + j;
            if (j < nz - 1) {
                const float *Gl = G32 + l * nn;
                for (int r = warp; r < n; r += nwarp) {
                    float s = 0.0f;
                    for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * vin[q];
                    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                    if (lane == 0) vout[r] = zf[l * n + r] + s;
                }
            } else {
                for (int t = tid; t < n; t += nth) vout[t] = zf[l * n + t];
            }
            __syncthreads();
            for (int t = tid; t < n; t += nth) {
                const size_t e = l * n + t;
                double d = csc[e] * (double)vout[t];
                double xn = x[e] + d;
                x[e] = xn;
                double sc = fabs(xn) + (yscale ? fabs(yscale[e]) : 0.0)
                            + 1e-10 * b.atm[l * VK_ATM_NF + VK_ATM_N0];
                if (isfinite(d)) dmax = fmax(dmax, fabs(d) / sc);
                else dmax = INFINITY;
                if (j > 0) vin[t] = (float)(rsc[(l - 1) * n + t] * dB[(l - 1) * n + t] * csc[e] * (double)vout[t]);
            }
            __syncthreads();
        }
        for (int o = 16; o; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        if (lane == 0) red[warp] = dmax;
        __syncthreads();
        double m = red[0];
        for (int w = 1; w < nwarp; ++w) m = fmax(m, red[w]);
        __syncthreads();
        converged = (m <= tol);
        if (converged) break;
        // residual r = b - A x  (FP64, matrix-free)
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            const double *jl = jv + l * net.nnz;
            for (int s = tid; s < n; s += nth) {
                const size_t e = l * n + s;
                double ax = (c0 - dA[e]) * x[e];
                for (int k = net.jrowptr[s]; k < net.jrowptr[s + 1]; ++k) ax += jl[k] * x[l * n + net.jcol[k]];
                if (j > 0) ax -= dC[e] * x[e - n];
                if (j < nz - 1) ax -= dB[e] * x[e + n];
                res[e] = rhs[e] - ax;
            }
        }
        __syncthreads();
    }
    if (tid == 0) {
        if (!converged) fallback[c] = 1;
        if (sweeps_out) atomicMax(sweeps_out, sweep + (converged ? 1 : 0));
    }
    if (yk2) {
        for (int e = tid; e < nz * n; e += nth) yk2[base + e] = y[base + e] + x[base + e] / R_ROS;
    }
}

size_t lu_f32_smem(int n) {
    return (size_t)(n * n + 4 * n) * sizeof(float) + (size_t)(2 * n + 2) * sizeof(int)
           + (size_t)(4 * n) * sizeof(double) + 16;
}

cudaError_t init_mixed_kernels(int n) {
    cudaError_t e = cudaFuncSetAttribute(k_lu_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)lu_f32_smem(n));
    return e;
}

void launch_lu_f32(const DevNet &net, const DevBatch &b, const Work &w, cudaStream_t s) {
    k_lu_f32<<<b.ncols, 256, lu_f32_smem(net.ni), s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt,
                                                       w.G32, w.rs, w.cs, w.status);
}

void launch_refine(const DevNet &net, const DevBatch &b, const Work &w, const double *rhs,
                   double *x, const double *yscale, double *yk2, int max_sweeps, double tol,
                   cudaStream_t s) {
    k_refine<<<b.ncols, 256, 2 * net.ni * sizeof(float), s>>>(
        net, b, w.G32, w.rs, w.cs, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, x, w.r, w.zf, yscale, yk2,
        w.y, max_sweeps, tol, w.fallback, w.sweeps);
}

}  // namespace vk
