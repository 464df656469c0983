// In-place Gauss-Jordan inversion of an n x n FP64 block in shared memory
// with partial pivoting (largest |a| in the pivot column, lowest row on
// ties), used by the block-Thomas factorisations.  All threads of the block
// must call it.  *s_sing becomes 1 for a zero pivot column, 2 when no finite
// pivot candidate exists (NaN state).
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
                if (best < 0.0 || bi >= n) { *s_sing = 2; bi = k; }
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

namespace vk {

// Warp 0: largest |v[i]| over lo <= i < n (lowest i on ties), with the
// singular / NaN classification of gj_invert_f64.  Returns the row to lane 0
// and records the pivot value and perm entry.
__device__ __forceinline__ void gj_pick_pivot(const double *v, int vstride, int lo, int n, int lane,
                                              int k, int *perm, int *s_piv, double *s_pval,
                                              int *s_sing) {
    double best = -1.0;
    int bi = n;
    for (int i = lo + lane; i < n; i += 32) {
        double a = fabs(v[i * vstride]);
        if (a > best) { best = a; bi = i; }
    }
    for (int o = 16; o; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) {
        if (best < 0.0 || bi >= n) { *s_sing = 2; bi = k; }
        else if (!(best > 0.0)) { if (*s_sing == 0) *s_sing = 1; bi = k; }
        *s_piv = bi;
        *s_pval = v[bi * vstride];
        perm[k] = bi;
    }
}

// Gauss-Jordan inversion two pivots per pass over the block: pivot k is chosen
// and its row/column formed as in gj_invert_f64; the column k+1 *after* that
// update is formed on its own (n FMAs) to choose pivot k+1; then one pass
// applies both rank-1 updates to every element.  Each element goes through the
// same two FMAs in the same order as with one pivot per pass, so the result is
// bit-identical to gj_invert_f64; shared-memory passes and barriers halve.
// Scratch: colk, rowk, colk2, rowk2, c2, tmp (n doubles each).
__device__ __forceinline__ void gj_invert_f64_x2(double *A, int n, double *colk, double *rowk,
                                                 double *colk2, double *rowk2, double *c2,
                                                 double *tmp, int *perm, int *s_piv,
                                                 double *s_pval, int *s_sing) {
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int R = nth / n;                     // row groups of the column mapping (nth >= n)
    const int my_col = tid % n, my_row0 = tid / n;
    const bool mapped = tid < R * n;
    int k = 0;
    for (; k + 1 < n; k += 2) {
        // ---- pivot k on column k
        if (warp == 0) gj_pick_pivot(A + k, n, k, n, lane, k, perm, s_piv, s_pval, s_sing);
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
        // ---- column k+1 after the pivot-k update; pivot k+1 on it
        const double rk1 = rowk[k + 1];
        for (int i = tid; i < n; i += nth)
            c2[i] = (i == k) ? rk1 : A[i * n + k + 1] - colk[i] * rk1;
        __syncthreads();
        if (warp == 0) gj_pick_pivot(c2, 1, k + 1, n, lane, k + 1, perm, s_piv, s_pval, s_sing);
        __syncthreads();
        const int p2 = *s_piv;
        const double pval2 = *s_pval;
        const double pinv2 = 1.0 / pval2;
        for (int t = tid; t < n; t += nth) {
            // row p2 after the pivot-k update becomes the new row k+1
            const double r2 = (t == k ? 0.0 : A[p2 * n + t]) - colk[p2] * rowk[t];
            rowk2[t] = (t == k + 1) ? pinv2 : r2 * pinv2;
            tmp[t] = A[(k + 1) * n + t];          // old row k+1 moves to row p2
            colk2[t] = (t == k + 1) ? pval2 : ((t == p2) ? c2[k + 1] : c2[t]);
        }
        __syncthreads();
        if (mapped) {
            const int j = my_col;
            const double rj = rowk[j], r2j = rowk2[j];
            const bool is_k = j == k, is_k1 = j == k + 1;
            for (int i = my_row0; i < n; i += R) {
                double *a = A + i * n + j;
                double v;
                if (i == k + 1) {
                    v = r2j;
                } else if (i == k) {
                    v = (is_k1 ? 0.0 : rj) - colk2[k] * r2j;
                } else {
                    const bool from1 = (i == p2) && (p2 != k + 1);
                    const double src = from1 ? tmp[j] : *a;
                    const double ck = from1 ? colk[k + 1] : colk[i];
                    const double a1 = (is_k ? 0.0 : src) - ck * rj;
                    v = (is_k1 ? 0.0 : a1) - colk2[i] * r2j;
                }
                *a = v;
            }
        }
        __syncthreads();
    }
    if (k < n) {                               // odd n: the last pivot alone
        if (warp == 0) gj_pick_pivot(A + k, n, k, n, lane, k, perm, s_piv, s_pval, s_sing);
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
        if (mapped) {
            const int j = my_col;
            const double rj = rowk[j];
            for (int i = my_row0; i < n; i += R) {
                double *a = A + i * n + j;
                *a = (i == k) ? rj : (j == k ? 0.0 : *a) - colk[i] * rj;
            }
        }
        __syncthreads();
    }
    for (int kk = n - 1; kk >= 0; --kk) {
        int q = perm[kk];
        if (q != kk) {
            for (int t = tid; t < n; t += nth) {
                double a = A[t * n + kk];
                A[t * n + kk] = A[t * n + q];
                A[t * n + q] = a;
            }
            __syncthreads();
        }
    }
}

}  // namespace vk
