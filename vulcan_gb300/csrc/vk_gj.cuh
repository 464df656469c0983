// In-place Gauss-Jordan inversion of an n x n FP64 block in shared memory
// with partial pivoting (largest |a| in the pivot column, lowest row on
// ties), used by the block-Thomas factorisations.  All threads of the block
// must call it.  *s_sing becomes 1 for a zero pivot column, 2 when no finite
// pivot candidate exists (NaN state); the first cause seen is kept (a zero
// pivot makes every later candidate non-finite).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace vk {

__device__ __forceinline__ void gj_invert_f64(double *A, int n, double *colk, double *rowk, int *perm,
                              int *s_piv, double *s_pval, int *s_sing) {
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nn = n * n;
    // rank-1 update mapping: thread t owns column t % n of rows t / n + R q
    // (R = nth / n row groups); needs nth >= n, else a flat loop
    const int R = nth / n;
    const int my_col = R ? tid % n : 0, my_row0 = R ? tid / n : 0;
    const bool mapped = R > 0 && tid < R * n;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            double best = -1.0;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                double a = fabs(A[i * n + k]);
                if (a > best) { best = a; bi = i; }
            }
            for (int o = 16; o; o >>= 1) {
                double ob = __shfl_xor_sync(0xffffffffu, best, o);
                int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (lane == 0) {
                // no finite candidate -> NaN state (2); all zero -> singular (1)
                if (best < 0.0 || bi >= n) { if (*s_sing == 0) *s_sing = 2; bi = k; }
                else if (!(best > 0.0)) { if (*s_sing == 0) *s_sing = 1; bi = k; }
                *s_piv = bi;
                *s_pval = A[bi * n + k];
                perm[k] = bi;
            }
        }
        __syncthreads();
        const int p = *s_piv;
        const double pval = *s_pval;
        const double pinv = 1.0 / pval;
        for (int t = tid; t < n; t += nth) {
            double ak = A[k * n + t], ap = A[p * n + t];
            rowk[t] = (t == k) ? pinv : ap * pinv;
            if (p != k) A[p * n + t] = ak;
            colk[t] = (t == k) ? pval : ((t == p) ? A[k * n + k] : A[t * n + k]);
        }
        __syncthreads();
        if (R > 0) {
            if (mapped) {
                const double rj = rowk[my_col];
                const bool is_k = my_col == k;
                for (int i = my_row0; i < n; i += R) {
                    double *a = A + i * n + my_col;
                    if (i == k) *a = rj;
                    else *a = (is_k ? 0.0 : *a) - colk[i] * rj;
                }
            }
        } else {
            for (int e = tid; e < nn; e += nth) {
                int i = e / n, jj = e - i * n;
                if (i == k) A[e] = rowk[jj];
                else A[e] = (jj == k ? 0.0 : A[e]) - colk[i] * rowk[jj];
            }
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
        int p = perm[k];
        if (p != k) {
            for (int t = tid; t < n; t += nth) {
                double a = A[t * n + k];
                A[t * n + k] = A[t * n + p];
                A[t * n + p] = a;
            }
            __syncthreads();
        }
    }
}

}  // namespace vk
