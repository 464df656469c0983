// FP64 block helpers of the block-Thomas factorisations: in-place
// Gauss-Jordan inversion with partial pivoting, and the matrix-vector product
// with a block held in shared memory.
//
// FP64 arithmetic is the scarce resource on this chip: a warp-wide FP64
// instruction holds a sub-partition's FP64 unit for tens of cycles, whatever
// its kind.  So the only FP64 instructions here are the useful ones -- the
// rank-1 updates' FMAs, the pivot row's scaling, one division per pivot and
// the products' FMAs.  The pivot search compares the IEEE bit patterns of |a|
// as integers (for non-negative doubles the integer order is the value order),
// the reciprocal is computed once per pivot by one thread and shared, and the
// update runs over the block's elements as one flat range so every lane of
// every warp has an element.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace vk {

// In-place inversion of the n x n block A (shared memory, row-major) with
// partial pivoting: the largest |a| in the pivot column, the lowest row on
// ties; NaN entries are never chosen.  All threads of the block must call it.
// *s_sing becomes 1 for a zero pivot column, 2 when no finite pivot candidate
// exists (NaN state); the first cause seen is kept (a zero pivot makes every
// later candidate non-finite).  colk, rowk: n doubles each; perm: n ints.
__device__ __forceinline__ void gj_invert_f64(double *A, int n, double *colk, double *rowk, int *perm,
                                              int *s_sing) {
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nn = n * n;
    // flat element e = tid + nth*s as (row, column), advanced incrementally
    const int di = nth / n, dq = nth - di * n;
    const int i0 = tid / n, q0 = tid - i0 * n;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            long long best = -1;
            int bi = n;
            for (int i = k + lane; i < n; i += 32) {
                const long long a = __double_as_longlong(A[i * n + k]) & 0x7fffffffffffffffll;
                if (a <= 0x7ff0000000000000ll && a > best) { best = a; bi = i; }
            }
            for (int o = 16; o; o >>= 1) {
                const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            int flag = 0;                 // the same in every lane after the butterfly
            if (best < 0 || bi >= n) { flag = 2; bi = k; }
            else if (best == 0) { flag = 1; bi = k; }
            const int p = bi;
            double pval = 0.0, pinv = 0.0;
            if (lane == 0) {
                if (flag && *s_sing == 0) *s_sing = flag;
                pval = A[p * n + k];
                pinv = 1.0 / pval;
                perm[k] = p;
            }
            pval = __shfl_sync(0xffffffffu, pval, 0);
            pinv = __shfl_sync(0xffffffffu, pinv, 0);
            // pivot row (scaled) and pivot column of the current block; rows
            // k and p swap (row k's new values come from rowk in the update)
            for (int t = lane; t < n; t += 32) {
                const double ak = A[k * n + t], ap = A[p * n + t];
                rowk[t] = (t == k) ? pinv : ap * pinv;
                colk[t] = (t == k) ? pval : ((t == p) ? A[k * n + k] : A[t * n + k]);
                if (p != k) A[p * n + t] = ak;
            }
        }
        __syncthreads();
        int i = i0, q = q0;
        for (int e = tid; e < nn; e += nth) {
            const double r = rowk[q];
            const double a = (q == k) ? 0.0 : A[e];
            const double u = __fma_rn(-colk[i], r, a);
            A[e] = (i == k) ? r : u;
            q += dq;
            i += di;
            if (q >= n) { q -= n; ++i; }
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

// Look-ahead Gauss-Jordan: the same inversion, pivots and arithmetic as
// gj_invert_f64 (bit for bit), with the matrix in two shared-memory buffers.
// While warps 1.. apply step k's rank-1 update from A (cur) into the other
// buffer (row swap folded into the read), warp 0 computes the updated pivot
// column k+1 and pivot row of step k+1 itself from the same inputs, searches
// the pivot and prepares step k+1's scaled row and column -- so the pivot
// search, the reciprocal and the row scaling of step k+1 overlap step k's
// FMAs and a step costs one block barrier.  rowk, colk: [2][n] (step
// parity); perm: n ints.  Returns the buffer holding the inverse.
__device__ __forceinline__ double *gj_invert_f64_la(double *A, double *B, int n, double *colk,
                                                    double *rowk, int *perm, int *s_piv,
                                                    int *s_sing) {
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nn = n * n;
    // warp 0: pivot of column k (rows >= k) of the matrix whose column k is
    // given per row by colv(i); returns p, writes rowk/colk of step k
    auto prepare = [&](int k, int par, auto colv, auto rowv) {
        long long best = -1;
        int bi = n;
        for (int i = k + lane; i < n; i += 32) {
            const long long a = __double_as_longlong(colv(i)) & 0x7fffffffffffffffll;
            if (a <= 0x7ff0000000000000ll && a > best) { best = a; bi = i; }
        }
        for (int o = 16; o; o >>= 1) {
            const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        int flag = 0;
        if (best < 0 || bi >= n) { flag = 2; bi = k; }
        else if (best == 0) { flag = 1; bi = k; }
        const int p = bi;
        double pval = 0.0, pinv = 0.0;
        if (lane == 0) {
            if (flag && *s_sing == 0) *s_sing = flag;
            pval = colv(p);
            pinv = 1.0 / pval;
            perm[k] = p;
            s_piv[par] = p;
        }
        pval = __shfl_sync(0xffffffffu, pval, 0);
        pinv = __shfl_sync(0xffffffffu, pinv, 0);
        double *rk = rowk + par * n, *ck = colk + par * n;
        for (int t = lane; t < n; t += 32) {
            rk[t] = (t == k) ? pinv : rowv(p, t) * pinv;
            ck[t] = (t == k) ? pval : ((t == p) ? colv(k) : colv(t));
        }
    };
    // prologue: step 0's pivot from the matrix itself
    if (warp == 0)
        prepare(0, 0, [&](int i) { return A[i * n]; }, [&](int r, int q) { return A[r * n + q]; });
    __syncthreads();
    double *cur = A, *nxt = B;
    const int nb = nth - 32;                       // threads of the bulk update
    const int di = nb / n, dq = nb - di * n;
    const int tb = tid - 32;
    const int i0 = tb >= 0 ? tb / n : 0, q0 = tb >= 0 ? tb - i0 * n : 0;
    for (int k = 0; k < n; ++k) {
        const int par = k & 1;
        const int p = s_piv[par];
        const double *rk = rowk + par * n, *ck = colk + par * n;
        // updated entry (i, q) of step k, rows k and p exchanged
        auto upd = [&](int i, int q) {
            const double r = rk[q];
            if (i == k) return r;
            const int src = (i == p) ? k : i;
            const double a = (q == k) ? 0.0 : cur[src * n + q];
            return __fma_rn(-ck[i], r, a);
        };
        if (warp == 0) {
            if (k + 1 < n)
                prepare(k + 1, par ^ 1, [&](int i) { return upd(i, k + 1); },
                        [&](int r, int q) { return upd(r, q); });
        } else {
            int i = i0, q = q0;
            for (int e = tb; e < nn; e += nb) {
                const double r = rk[q];
                const int src = (i == p) ? k : i;
                const double a = (q == k) ? 0.0 : cur[src * n + q];
                const double u = __fma_rn(-ck[i], r, a);
                nxt[e] = (i == k) ? r : u;
                q += dq;
                i += di;
                if (q >= n) { q -= n; ++i; }
            }
        }
        __syncthreads();
        double *t = cur; cur = nxt; nxt = t;
    }
    for (int k = n - 1; k >= 0; --k) {
        int p = perm[k];
        if (p != k) {
            for (int t = tid; t < n; t += nth) {
                double a = cur[t * n + k];
                cur[t * n + k] = cur[t * n + p];
                cur[t * n + p] = a;
            }
            __syncthreads();
        }
    }
    return cur;
}

// out[r] = sum_q M[r*n + q] x[q] (+ add[r] when add is not NULL) for the n x n
// block M in shared memory.  Thread (r, g) sums the g-th of P = blockDim / n
// contiguous chunks of row r (lanes of a warp take consecutive rows: stride
// n doubles, conflict-free for odd n); the chunks are then added in order.
// part: P*n doubles of shared scratch.  All threads call it; it ends with a
// block barrier (out is readable by every thread afterwards).
__device__ __forceinline__ void matvec_f64(const double *M, int n, const double *x, double *part,
                                           double *out, const double *add) {
    const int tid = threadIdx.x, nth = blockDim.x;
    const int P = nth >= n ? (nth / n < 8 ? nth / n : 8) : 1;
    const int chunk = (n + P - 1) / P;
    for (int t = tid; t < P * n; t += nth) {
        const int g = t / n, r = t - g * n;
        const int q0 = g * chunk, q1 = q0 + chunk < n ? q0 + chunk : n;
        const double *row = M + r * n;
        double s = 0.0;
        for (int q = q0; q < q1; ++q) s = __fma_rn(row[q], x[q], s);
        part[g * n + r] = s;
    }
    __syncthreads();
    for (int r = tid; r < n; r += nth) {
        double s = part[r];
        for (int g = 1; g < P; ++g) s += part[g * n + r];
        out[r] = add ? add[r] + s : s;
    }
    __syncthreads();
}

}  // namespace vk
