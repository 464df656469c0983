// Register-resident Gauss-Jordan inversion of one n x n block per CTA.
//
// Thread layout: 16 column groups x TY row groups (TY = blockDim/16),
// tid = tx * TY + ty.  Thread (ty, tx) owns rows r = ty + TY*a (a < RA) and
// columns c = tx + 16*b (b < RB) and keeps those elements in registers for the
// whole inversion.  Pivoting is implicit (no row exchanges): step k picks, among
// rows not yet used, the row p with the largest |A[p][k]| (lowest p on ties) --
// the same pivot sequence as partial pivoting with row swaps -- and eliminates
// column k from every other row.  The TY owners of a column are consecutive
// lanes, so the pivot search is one shuffle reduction.  On return the
// registers hold the inverse with permuted labels:
//     inverse[kinv[r]][perm[c]] = M[r][c],
// perm[k] = pivot row of step k, kinv = its inverse (both in shared memory).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace vk {

template <typename T>
struct GJShared {
    T *rowv;       // [n] pivot row (scaled)
    T *colv;       // [n] pivot column (before elimination)
    int *perm;     // [n] pivot row of step k
    int *kinv;     // [n] step at which row r was the pivot
    int *used;     // [n] row already pivot
    int *s_piv;
    T *s_pval;
    int *s_sing;   // 1 zero pivot column, 2 no finite candidate
};

template <typename T>
__device__ __forceinline__ T gj_abs(T v) { return v < T(0) ? -v : v; }

// Registers (permuted inverse) -> shared memory in natural order.
template <typename T, int TY, int RA, int RB>
__device__ __forceinline__ void gj_store_natural(const T (&M)[RA][RB], int n, int ty, int tx,
                                                 const GJShared<T> &sh, T *G) {
#pragma unroll
    for (int a = 0; a < RA; ++a) {
        const int r = ty + TY * a;
        if (r >= n) continue;
        const int row = sh.kinv[r];
#pragma unroll
        for (int b = 0; b < RB; ++b) {
            const int c = tx + 16 * b;
            if (c < n) G[row * n + sh.perm[c]] = M[a][b];
        }
    }
    __syncthreads();
}

}  // namespace vk

namespace vk {

// Column kb / row pa of the register tile for a CTA-uniform runtime index:
// a switch on the index (one uniform branch) instead of a select per element.
#define VK_TILE_CASE(B, BODY) \
    case B:                   \
        if constexpr (B < LIM) { BODY(B); } \
        break;
#define VK_TILE_SWITCH(IDX, BODY)                                                     \
    switch (IDX) {                                                                    \
        VK_TILE_CASE(0, BODY) VK_TILE_CASE(1, BODY) VK_TILE_CASE(2, BODY)             \
        VK_TILE_CASE(3, BODY) VK_TILE_CASE(4, BODY) VK_TILE_CASE(5, BODY)             \
        VK_TILE_CASE(6, BODY) VK_TILE_CASE(7, BODY) VK_TILE_CASE(8, BODY)             \
        VK_TILE_CASE(9, BODY)                                                         \
    default: break;                                                                   \
    }

template <typename T, int RA, int RB>
__device__ __forceinline__ void tile_get_col(const T (&M)[RA][RB], int kb, T (&out)[RA]) {
    constexpr int LIM = RB;
    static_assert(RB <= 10, "tile switch covers 10 columns");
#define VK_BODY(B) _Pragma("unroll") for (int a = 0; a < RA; ++a) out[a] = M[a][B]
    VK_TILE_SWITCH(kb, VK_BODY)
#undef VK_BODY
}

template <typename T, int RA, int RB>
__device__ __forceinline__ void tile_set_col(T (&M)[RA][RB], int kb, const T (&v)[RA]) {
    constexpr int LIM = RB;
#define VK_BODY(B) _Pragma("unroll") for (int a = 0; a < RA; ++a) M[a][B] = v[a]
    VK_TILE_SWITCH(kb, VK_BODY)
#undef VK_BODY
}

template <typename T, int RA, int RB>
__device__ __forceinline__ void tile_get_row(const T (&M)[RA][RB], int pa, T (&out)[RB]) {
    constexpr int LIM = RA;
    static_assert(RA <= 10, "tile switch covers 10 rows");
#define VK_BODY(A) _Pragma("unroll") for (int b = 0; b < RB; ++b) out[b] = M[A][b]
    VK_TILE_SWITCH(pa, VK_BODY)
#undef VK_BODY
}

// Gauss-Jordan on the register tile with one block barrier per pivot step.
// The pivot row reaches the threads of each column group by warp shuffles
// (every thread finds row p of its own columns at lane p % TY of its group);
// only the pivot column goes through shared memory, in two buffers by parity
// of k (colv2[2n]), written together with the search of the next pivot right
// after each update -- so the next step needs one barrier.  s_piv2 holds two
// pivot slots (parity of k).
template <typename T, int TY, int RA, int RB>
__device__ __forceinline__ void gj_invert_reg1(T (&M)[RA][RB], int n, int ty, int tx,
                                               const GJShared<T> &sh, T *colv2, int *s_piv2) {
    int rr[RA], cc[RB];
#pragma unroll
    for (int a = 0; a < RA; ++a) rr[a] = ty + TY * a;
#pragma unroll
    for (int b = 0; b < RB; ++b) cc[b] = tx + 16 * b;
    const unsigned gmask = TY == 32 ? 0xffffffffu : (0xffffu << (threadIdx.x & 16));
    // pivot search of column k among this thread's unused rows, reduced over
    // the column group; lane ty == 0 records it (all owners know bi after)
    auto search = [&](int k) {
        const int kb = k >> 4;
        T colk[RA];
        tile_get_col(M, kb, colk);
        T best = T(-1);
        int bi = n;
#pragma unroll
        for (int a = 0; a < RA; ++a) {
            if (rr[a] < n && !sh.used[rr[a]]) {
                T v = gj_abs(colk[a]);
                if (v > best) { best = v; bi = rr[a]; }
            }
        }
#pragma unroll
        for (int o = TY >> 1; o; o >>= 1) {
            T ob = __shfl_xor_sync(gmask, best, o, TY);
            int oi = __shfl_xor_sync(gmask, bi, o, TY);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (ty == 0) {
            if (bi >= n || !(best >= T(0)) || isinf((double)best)) {
                *sh.s_sing = 2;
                for (int r = 0; r < n; ++r)
                    if (!sh.used[r]) { bi = r; break; }
            } else if (!(best > T(0))) {
                if (*sh.s_sing == 0) *sh.s_sing = 1;
            }
            s_piv2[k & 1] = bi;
            sh.perm[k] = bi;
            sh.kinv[bi] = k;
            sh.used[bi] = 1;
        }
        // the column (before elimination) for every row
        T *cv = colv2 + (k & 1) * n;
#pragma unroll
        for (int a = 0; a < RA; ++a)
            if (rr[a] < n) cv[rr[a]] = colk[a];
    };
    if (tx == 0) search(0);
    for (int k = 0; k < n; ++k) {
        __syncthreads();
        const int kx = k & 15, kb = k >> 4;
        const int p = s_piv2[k & 1];
        const T *cv = colv2 + (k & 1) * n;
        const T pinv = T(1) / cv[p];
        // pivot row of this thread's columns from its column group (lane p % TY)
        const int pa = p / TY, pl = p - pa * TY;
        T rp[RB];
        tile_get_row(M, pa, rp);
#pragma unroll
        for (int b = 0; b < RB; ++b) {
            // every lane runs this: full mask, segments of TY lanes
            const T v = __shfl_sync(0xffffffffu, rp[b], pl, TY);
            rp[b] = cc[b] < n ? v * pinv : T(0);
        }
        T fr[RA];
#pragma unroll
        for (int a = 0; a < RA; ++a) {
            fr[a] = rr[a] < n ? cv[rr[a]] : T(0);
            if (rr[a] == p) {
#pragma unroll
                for (int b = 0; b < RB; ++b) M[a][b] = rp[b];
            } else {
#pragma unroll
                for (int b = 0; b < RB; ++b) M[a][b] -= fr[a] * rp[b];
            }
        }
        if (tx == kx) {
            T pc[RA];
#pragma unroll
            for (int a = 0; a < RA; ++a) pc[a] = rr[a] == p ? pinv : -fr[a] * pinv;
            tile_set_col(M, kb, pc);
        }
        // next pivot: its column owners search their updated registers now
        if (k + 1 < n && tx == ((k + 1) & 15)) search(k + 1);
    }
    __syncthreads();
}

}  // namespace vk
