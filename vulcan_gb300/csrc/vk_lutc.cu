// FP32 block-Thomas factorisation on the tensor cores (mixed path, blocks of
// up to 128 species): k_lu_tc replaces k_lu32's register Gauss-Jordan with a
// blocked Gauss-Jordan whose trailing updates run as tcgen05 MMAs.
//
// Per column (work queue, one column at a time per CTA of 4 warps), per layer j:
//   A  the scaled block D~_j (R_j D_j S_j, written by k_prep32 zero-padded to
//      NP x NP, NP = ni rounded up to 16) arrives by a 2-D TMA tensor copy; the
//      Schur complement D~'_j = D~_j - diag(alpha) G~_{j-1} diag(beta) is formed
//      row by row (thread r <-> row r <-> TMEM lane r) and stored into TMEM,
//      which holds the block as an FP32 accumulator for the whole inversion;
//   B  Gauss-Jordan in panels of 16 pivot columns with implicit pivoting (rows
//      are never exchanged; step k takes the unused row with the largest |a|,
//      lowest row on ties):
//        B1 the panel's 16 columns leave TMEM (tcgen05.ld) for shared memory;
//        B2 one warp eliminates the 16 pivots on the panel alone (3-4 rows per
//           lane in registers, warp reductions, no block barrier per pivot);
//           the panel's eliminations form E = I + X S^T, S selecting the pivot
//           rows, X = (final panel) - S;
//        B3 the pivot rows of the block before the update, R = S^T A, leave
//           TMEM into shared memory (zero in the panel's columns), the final
//           panel goes back into TMEM;
//        B4 A <- A + X R on the tensor cores: X and R split into TF32 high and
//           low parts, D += Xh Rh + Xh Rl + Xl Rh (FP32 accumulate in TMEM),
//           K = 16 as two k-steps of 8;
//   C  the inverse (permuted labels: inverse[kinv[r]][perm[c]] = A[r][c]) is
//      stored in natural order into shared memory, kept for layer j+1's Schur
//      complement and written to G32 by a bulk copy.
// Split TF32 keeps FP32's accuracy for the refinement: a numpy emulation of
// this factorisation needs the same refinement sweeps as FP32 Gauss-Jordan.
//
// Every wait (TMA, MMA completion) is bounded; on a timeout the CTA records
// VK_ETIMEOUT for its column, waits (bounded) for its own copies and MMAs in
// flight, frees its TMEM and leaves.
//
// Reference: the banded LU of the Ros2 LHS, op.py:2913-2929 (solve_banded on
// the matrix store_bandM builds, op.py:2833-2858).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <math.h>

#include "vk_internal.cuh"
#include "vk_tc.cuh"
#include "vk_tma.cuh"

namespace vk {

namespace {

constexpr int kTmemCols = 128;          // D: NP <= 128 columns
constexpr int kPW = 16;                 // panel width (pivots per MMA update)
constexpr int kLdGroup = 1;             // TMEM loads of 16 columns per wait (1: no spills at 3 CTAs/SM)

struct TcSmem {
    // byte offsets into the dynamic shared memory (base 128-byte aligned)
    int dbuf, gs, ahi, alo, bhi, blo, pex, alpha, beta, perm, kinv, xch, bars, tslot, total;
};

__host__ __device__ inline int round_up(int x, int a) { return (x + a - 1) / a * a; }

__host__ __device__ inline TcSmem tc_layout(int n) {
    const int NP = round_up(n, 16);
    TcSmem s;
    int o = 0;
    s.dbuf = o;  o += round_up(NP * NP * 4, 128);
    s.gs = o;    o += round_up(block_stride32(n) * 4, 128);
    s.ahi = o;   o += 128 * kPW * 4;
    s.alo = o;   o += 128 * kPW * 4;
    s.bhi = o;   o += round_up(NP * kPW * 4, 128);
    s.blo = o;   o += round_up(NP * kPW * 4, 128);
    s.pex = o;   o += round_up(NP * (kPW + 1) * 4, 16);
    s.alpha = o; o += round_up(NP * 4, 16);
    s.beta = o;  o += round_up(NP * 4, 16);
    s.perm = o;  o += round_up(NP * 4, 16);
    s.kinv = o;  o += round_up(NP * 4, 16);
    s.xch = o;   o += round_up((2 * 4 * 20 + 4) * 4, 16);   // cooperative panel: [2][4 warps][20] + 4
    s.bars = o;  o += 4 * 8;
    s.tslot = o; o += 16;
    s.total = o + 128;                   // slack for aligning the base
    return s;
}

// operand offset (floats) of element (row i, k) in the K-major core-matrix layout
__device__ __forceinline__ int op_off(int i, int k) {
    return ((i >> 3) * 4 + (k >> 2)) * 32 + (i & 7) * 4 + (k & 3);
}

// Pivot of the panel warp's current column (slot 0 of every row it holds):
// the unused row with the largest |a|, lowest row on ties, found by one warp
// reduction of a key that is |a| with its 7 low mantissa bits replaced by
// 127 - row (so values equal to 2^-16 relative also go to the lowest row --
// any such choice is a valid partial pivot).  NaN rows never pivot.  Returns
// -1 (stat 2) when no finite candidate is left; stat 1 for a zero column.
template <int RA>
__device__ __forceinline__ int panel_pivot(const float (&col)[RA], unsigned umask, int lane,
                                           int &stat) {
    unsigned key = 0;
#pragma unroll
    for (int a = 0; a < RA; ++a) {
        const float v = fabsf(col[a]);
        const unsigned k = (__float_as_uint(v) & ~127u) | (unsigned)(127 - (lane + 32 * a));
        if (!((umask >> a) & 1u) && v == v) key = max(key, k | 0x80000000u);
    }
    const unsigned m = __reduce_max_sync(0xffffffffu, key);
    if (m == 0u || (m & 0x7fffffffu) >= 0x7f800000u) { stat = 2; return -1; }
    if (((m & 0x7fffff80u) == 0u) && stat == 0) stat = 1;
    return 127 - (int)(m & 127u);
}

// Gauss-Jordan on the panel alone, by one warp: P[a][q] holds row lane + 32a,
// panel column q.  The panel rotates one column to the left per pivot step
// (the consumed column moves to slot 15, where its inverse entries are
// stored), so the pivot column is always slot 0 and the loop body is the same
// code for every step; after kPW steps (padding steps rotate only) the slots
// are back in panel order.  Records perm / kinv in shared memory.
template <int RA>
__device__ __forceinline__ void panel_eliminate(float (&P)[RA][kPW], unsigned &umask, int lane,
                                                int k0, int w, int *perm, int *kinv, int &stat) {
    int myp = 0;
#pragma unroll 1
    for (int t = 0; t < kPW; ++t) {
        if (t >= w) {                     // past the last pivot: rotate only
#pragma unroll
            for (int a = 0; a < RA; ++a) {
                const float c0 = P[a][0];
#pragma unroll
                for (int q = 0; q < kPW - 1; ++q) P[a][q] = P[a][q + 1];
                P[a][kPW - 1] = c0;
            }
            continue;
        }
        float col[RA];
#pragma unroll
        for (int a = 0; a < RA; ++a) col[a] = P[a][0];
        int p = panel_pivot<RA>(col, umask, lane, stat);
        if (p < 0) {                      // no finite candidate: lowest unused row
            unsigned lowest = 0xffffffffu;
#pragma unroll
            for (int a = RA - 1; a >= 0; --a)
                if (!((umask >> a) & 1u)) lowest = (unsigned)(lane + 32 * a);
            p = (int)__reduce_min_sync(0xffffffffu, lowest);
        }
        if ((unsigned)p >= 32u * RA) p = 0;          // (cannot happen: a row is always left)
        const int pl = p & 31, pa = p >> 5;          // warp-uniform
        // pivot row from its lane (uniform switch on the row slot)
        float rs[kPW];
        switch (pa) {
#define VK_BCAST(A)                                                           \
        case A:                                                               \
            if constexpr (A < RA) {                                           \
                _Pragma("unroll") for (int q = 0; q < kPW; ++q)               \
                    rs[q] = __shfl_sync(0xffffffffu, P[A][q], pl);            \
            }                                                                 \
            break;
        VK_BCAST(0) VK_BCAST(1) VK_BCAST(2) VK_BCAST(3)
#undef VK_BCAST
        default: break;
        }
        float pinv;                                   // 1/pivot (FP32 factors: refined in FP64)
        asm("rcp.approx.f32 %0, %1;" : "=f"(pinv) : "f"(rs[0]));
#pragma unroll
        for (int q = 1; q < kPW; ++q) rs[q] *= pinv;
        // eliminate column 0 from every row, shifting left by one; the pivot
        // row itself becomes the scaled row with 1/pivot in the consumed slot
#pragma unroll
        for (int a = 0; a < RA; ++a) {
            const bool isp = lane + 32 * a == p;
            const float f = P[a][0];
#pragma unroll
            for (int q = 0; q < kPW - 1; ++q) {
                const float e = fmaf(-f, rs[q + 1], P[a][q + 1]);
                P[a][q] = isp ? rs[q + 1] : e;
            }
            P[a][kPW - 1] = isp ? pinv : -f * pinv;
            if (isp) umask |= 1u << a;
        }
        if (lane == t) myp = p;                      // lane t records step t
    }
    __syncwarp();
    if (lane < w) {
        perm[k0 + lane] = myp;
        kinv[myp] = k0 + lane;
    }
    __syncwarp();
}

// Gauss-Jordan on the panel by all four warps together: thread r holds row r
// of the panel (P, 16 columns) in registers.  Step t pivots on slot t (no
// rotation; the same values as panel_eliminate): every warp finds its
// best candidate with one reduction of the packed |a|-and-row key, its
// winning lane publishes its row and key in a per-step-parity slot, one block
// barrier, and every thread takes the largest of the four keys and the
// winner's row from shared memory.  The slots alternate by step parity, so a
// step needs no second barrier (a warp writes slot t+2 only after every warp
// has passed barrier t+1, that is after it has read slot t).  The rare steps
// without a finite candidate (NaN / inf state) take two more barriers to find
// the lowest unused row and fetch it.  All threads call it with the same w.
__device__ __forceinline__ void panel_eliminate_coop(float (&P)[kPW], bool &used, int r, int lane,
                                                     int warp, int k0, int w, int *perm, int *kinv,
                                                     float *xch, int &stat) {
#pragma unroll
    for (int t = 0; t < kPW; ++t) {
        if (t >= w) break;                        // uniform
        const float v = fabsf(P[t]);
        const unsigned key = (!used && v == v)
            ? ((__float_as_uint(v) & ~127u) | (unsigned)(127 - (r & 127)) | 0x80000000u) : 0u;
        const unsigned m = __reduce_max_sync(0xffffffffu, key);
        float *slot = xch + ((t & 1) * 4 + warp) * 20;
        if (m != 0u && key == m) {
#pragma unroll
            for (int q = 0; q < kPW; ++q) slot[q] = P[q];
        }
        if (lane == 0) reinterpret_cast<unsigned *>(slot)[16] = m;
        __syncthreads();
        const float *sl = xch + (t & 1) * 4 * 20;
        unsigned M = 0;
        int ws = 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const unsigned ku = reinterpret_cast<const unsigned *>(sl + u * 20)[16];
            if (ku > M) { M = ku; ws = u; }
        }
        int p;
        const float *prow;
        if (M == 0u || (M & 0x7fffffffu) >= 0x7f800000u) {
            // no finite candidate: the lowest unused row, fetched from its owner
            stat = 2;
            const unsigned lw = __reduce_min_sync(0xffffffffu, used ? 0xffffffffu : (unsigned)r);
            unsigned *mn = reinterpret_cast<unsigned *>(xch + 8 * 20);    // the spare words
            if (lane == 0) mn[warp] = lw;
            __syncthreads();
            unsigned lo = 0xffffffffu;
#pragma unroll
            for (int u = 0; u < 4; ++u) lo = min(lo, mn[u]);
            p = lo == 0xffffffffu ? 0 : (int)lo;
            float *fs = xch + (t & 1) * 4 * 20;      // the step's slot 0 is free again
            __syncthreads();
            if (r == p) {
#pragma unroll
                for (int q = 0; q < kPW; ++q) fs[q] = P[q];
            }
            __syncthreads();
            prow = fs;
        } else {
            if (((M & 0x7fffff80u) == 0u) && stat == 0) stat = 1;
            p = 127 - (int)(M & 127u);
            prow = sl + ws * 20;
        }
        float rs[kPW];
#pragma unroll
        for (int q = 0; q < kPW; ++q) rs[q] = prow[q];
        float pinv;
        asm("rcp.approx.f32 %0, %1;" : "=f"(pinv) : "f"(rs[t]));
#pragma unroll
        for (int q = 0; q < kPW; ++q) if (q != t) rs[q] *= pinv;
        const bool isp = r == p;
        const float f = P[t];
#pragma unroll
        for (int q = 0; q < kPW; ++q) {
            if (q == t) continue;
            const float e = fmaf(-f, rs[q], P[q]);
            P[q] = isp ? rs[q] : e;
        }
        P[t] = isp ? pinv : -f * pinv;
        if (isp) {
            used = true;
            perm[k0 + t] = p;
            kinv[p] = k0 + t;
        }
    }
}

template <int RA, bool COOP>
__global__ void __launch_bounds__(128, 3)
k_lu_tc(DevNet net, DevBatch b, const __grid_constant__ CUtensorMap tmap_d,
        const double *__restrict__ dB, const double *__restrict__ dC,
        const double *__restrict__ rsc, const double *__restrict__ csc,
        float *__restrict__ G32, int *__restrict__ status) {
    extern __shared__ unsigned char smraw[];
    unsigned char *smb = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smraw) + 127) & ~uintptr_t(127));
    const int n = net.ni, NP = round_up(n, 16), NNP = block_stride32(n);
    const TcSmem L = tc_layout(n);
    float *Dbuf = reinterpret_cast<float *>(smb + L.dbuf);   // [NP][NP] TMA tile
    float *Gs = reinterpret_cast<float *>(smb + L.gs);       // [n][n] (+pad) natural inverse
    float *Ahi = reinterpret_cast<float *>(smb + L.ahi);     // X, 128 x 16 operand
    float *Alo = reinterpret_cast<float *>(smb + L.alo);
    float *Bhi = reinterpret_cast<float *>(smb + L.bhi);     // R^T, NP x 16 operand
    float *Blo = reinterpret_cast<float *>(smb + L.blo);
    float *Pex = reinterpret_cast<float *>(smb + L.pex);     // [NP][17] panel exchange
    float *alpha = reinterpret_cast<float *>(smb + L.alpha); // [NP] Schur row factors
    float *beta = reinterpret_cast<float *>(smb + L.beta);   // [NP] Schur column factors
    int *perm = reinterpret_cast<int *>(smb + L.perm);       // [NP] pivot row of step k
    int *kinv = reinterpret_cast<int *>(smb + L.kinv);       // [NP] step of pivot row r
    float *xch = reinterpret_cast<float *>(smb + L.xch);     // cooperative panel exchange
    uint64_t *bars = reinterpret_cast<uint64_t *>(smb + L.bars);   // [0] TMA, [1] MMA
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smb + L.tslot);
    __shared__ int s_col, s_stat, s_pw;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // The panel warp (B2) runs alone while the others wait, and three CTAs
    // share an SM: give each CTA's panel warp its own sub-partition (warp
    // slot modulo 4) rather than warp 0 everywhere, which would put the three
    // panel chains on one issue port.  The CTA's index on the SM is read from
    // the hardware warp slot of its first warp (consecutive slots per CTA);
    // any value is correct, only the placement changes.
    if (tid == 0) {
        unsigned ws;
        asm volatile("mov.u32 %0, %%warpid;" : "=r"(ws));
        s_pw = (int)((ws >> 2) & 3u);
    }
    const int r = tid;                                       // row = TMEM lane
    const bool row_warp = warp * 32 < NP;                    // warp-uniform
    const uint32_t tbytes = (uint32_t)NP * NP * 4;
    const uint32_t idesc = idesc_tf32(128, NP);

    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
        asm volatile("prefetch.tensormap [%0];" ::"l"(&tmap_d) : "memory");
    }
    if (warp == 0) tmem_alloc(tslot, kTmemCols);
    // operands: rows beyond the block (A) stay zero for good
    for (int e = tid; e < 128 * kPW; e += 128) { Ahi[e] = 0.f; Alo[e] = 0.f; }
    for (int e = tid; e < NP * kPW; e += 128) { Bhi[e] = 0.f; Blo[e] = 0.f; }
    for (int e = n * n + tid; e < NNP; e += 128) Gs[e] = 0.f;
    fence_async_smem();                  // the zero rows are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int pw = s_pw;                 // panel warp of this CTA
    const uint32_t tlane = tmem + ((uint32_t)(warp * 32) << 16);   // this warp's lanes, column 0

    int u_tma = 0, u_mma = 0;          // completed phases of bars[0] / bars[1]
    bool failed = false;
    for (int c; !failed && (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        if (tid == 0) {
            s_stat = 0;
            tma_load_2d(Dbuf, &tmap_d, 0, l0 * NP, tbytes, &bars[0]);
        }
        for (int j = 0; j < nz && !failed; ++j) {
            const size_t l = (size_t)l0 + j;
            // ---- A: Schur complement into TMEM ----
            const bool ok = mbar_wait(&bars[0], u_tma & 1);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) { status[c] = VK_ETIMEOUT; mbar_wait(&bars[0], u_tma & 1); }
                failed = true;
                break;
            }
            ++u_tma;
            if (tid < NP) kinv[tid] = 1 << 30;          // no row is a pivot yet
            if (row_warp) {
                const bool live = r < n && j > 0;
                const float ar = live ? alpha[r] : 0.f;
#pragma unroll 1
                for (int q = 0; q < NP; q += 16) {
                    float v[16];
#pragma unroll
                    for (int t = 0; t < 16; t += 4) {
                        float4 d4 = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (r < NP) d4 = *reinterpret_cast<const float4 *>(Dbuf + r * NP + q + t);
                        v[t] = d4.x; v[t + 1] = d4.y; v[t + 2] = d4.z; v[t + 3] = d4.w;
                    }
#pragma unroll
                    for (int t = 0; t < 16; ++t) {
                        const int cc = q + t;
                        if (r >= n || cc >= n) v[t] = 0.f;
                        else if (live) v[t] -= ar * Gs[r * n + cc] * beta[cc];
                    }
                    tmem_st16(tlane + q, v);
                }
                tmem_wait_st();
            }
            tc_fence_before();
            __syncthreads();                 // Dbuf read by all; TMEM written
            tc_fence_after();
            if (tid == 0 && j + 1 < nz) tma_load_2d(Dbuf, &tmap_d, 0, (int)(l + 1) * NP, tbytes, &bars[0]);
            // Schur factors of layer j+1 (computed now, used after C)
            float a_nx = 0.f, b_nx = 0.f;
            if (tid < n && j + 1 < nz) {
                a_nx = (float)(rsc[(l + 1) * n + tid] * dC[(l + 1) * n + tid] * csc[l * n + tid]);
                b_nx = (float)(rsc[l * n + tid] * dB[l * n + tid] * csc[(l + 1) * n + tid]);
            }
            // ---- B: panels ----
            for (int k0 = 0; k0 < n && !failed; k0 += kPW) {
                const int w = n - k0 < kPW ? n - k0 : kPW;
                float Pc[kPW];                     // cooperative panel: this thread's row
                if constexpr (COOP) {
                    // B1+B2: every thread loads its row of the panel and the four
                    // warps eliminate the panel's pivots together
                    if (row_warp) tmem_ld16(tlane + k0, Pc);
                    else {
#pragma unroll
                        for (int t = 0; t < kPW; ++t) Pc[t] = 0.f;
                    }
                    bool used = r >= n || kinv[r] < k0;   // padding or pivot of an earlier panel
                    int stat = s_stat;
                    __syncthreads();                      // s_stat read by all before it changes
                    panel_eliminate_coop(Pc, used, r, lane, warp, k0, w, perm, kinv, xch, stat);
                    if (tid == 0) s_stat = stat;
                    __syncthreads();                      // perm / kinv of the panel visible
                    // X = panel - S (hi / lo TF32) -> A operand, this thread's row
                    if (r < n) {
                        const int kr = kinv[r] - k0;
#pragma unroll
                        for (int t = 0; t < kPW; t += 4) {
                            float xh[4], xl[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                float x = (t + e < w) ? Pc[t + e] - ((kr == t + e) ? 1.f : 0.f) : 0.f;
                                xh[e] = to_tf32(x);
                                xl[e] = to_tf32(x - xh[e]);
                            }
                            *reinterpret_cast<float4 *>(Ahi + op_off(r, t)) = make_float4(xh[0], xh[1], xh[2], xh[3]);
                            *reinterpret_cast<float4 *>(Alo + op_off(r, t)) = make_float4(xl[0], xl[1], xl[2], xl[3]);
                        }
                    }
                    fence_async_smem();
                } else {
                // B1: panel columns TMEM -> Pex
                if (row_warp) {
                    float v[16];
                    tmem_ld16(tlane + k0, v);
                    if (r < NP) {
#pragma unroll
                        for (int t = 0; t < 16; ++t) Pex[r * (kPW + 1) + t] = v[t];
                    }
                }
                __syncthreads();
                // B2: one warp eliminates the panel's pivots
                if (warp == pw) {
                    float P[RA][kPW];
                    unsigned umask = 0;
#pragma unroll
                    for (int a = 0; a < RA; ++a) {
                        const int rr = lane + 32 * a;
                        const bool in = rr < n;
                        if (!in || kinv[rr] < k0) umask |= 1u << a;   // padding or pivot of an earlier panel
#pragma unroll
                        for (int t = 0; t < kPW; ++t) P[a][t] = in ? Pex[rr * (kPW + 1) + t] : 0.f;
                    }
                    int stat = s_stat;
                    panel_eliminate<RA>(P, umask, lane, k0, w, perm, kinv, stat);
                    if (lane == 0) s_stat = stat;
                    // final panel -> Pex; X = panel - S (hi / lo TF32) -> A operand
#pragma unroll
                    for (int a = 0; a < RA; ++a) {
                        const int rr = lane + 32 * a;
                        if (rr >= n) continue;
                        const int kr = kinv[rr] - k0;           // this row's pivot slot in the panel
#pragma unroll
                        for (int t = 0; t < kPW; ++t) Pex[rr * (kPW + 1) + t] = P[a][t];
#pragma unroll
                        for (int t = 0; t < kPW; t += 4) {
                            float xh[4], xl[4];
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                float x = (t + e < w) ? P[a][t + e] - ((kr == t + e) ? 1.f : 0.f) : 0.f;
                                xh[e] = to_tf32(x);
                                xl[e] = to_tf32(x - xh[e]);
                            }
                            *reinterpret_cast<float4 *>(Ahi + op_off(rr, t)) = make_float4(xh[0], xh[1], xh[2], xh[3]);
                            *reinterpret_cast<float4 *>(Alo + op_off(rr, t)) = make_float4(xl[0], xl[1], xl[2], xl[3]);
                        }
                    }
                    fence_async_smem();
                }
                }                                          // !COOP
                __syncthreads();
                // B3: pivot rows (pre-update) -> B operand; final panel -> TMEM
                if (row_warp) {
                    const int kr = (r < n) ? kinv[r] - k0 : -1;
                    const bool piv = kr >= 0 && kr < w;
#pragma unroll 1
                    for (int g0 = 0; g0 < NP; g0 += 16 * kLdGroup) {
                        float v[kLdGroup][16];           // kLdGroup chunks per wait
#pragma unroll
                        for (int ch = 0; ch < kLdGroup; ++ch)
                            if (g0 + ch * 16 < NP) tmem_ld16_nowait(tlane + g0 + ch * 16, v[ch]);
                        tmem_wait_ld();
#pragma unroll
                        for (int ch = 0; ch < kLdGroup; ++ch) {
                            tmem_reg_dep(v[ch]);
                            if (piv && g0 + ch * 16 < NP) {
#pragma unroll
                                for (int t = 0; t < 16; ++t) {
                                    const int cc = g0 + ch * 16 + t;
                                    const float x = (cc >= k0 && cc < k0 + kPW) || cc >= n ? 0.f : v[ch][t];
                                    const float xh = to_tf32(x);
                                    Bhi[op_off(cc, kr)] = xh;
                                    Blo[op_off(cc, kr)] = to_tf32(x - xh);
                                }
                            }
                        }
                    }
                    float pv[16];
#pragma unroll
                    for (int t = 0; t < 16; ++t)
                        pv[t] = r < n ? (COOP ? Pc[t] : Pex[r * (kPW + 1) + t]) : 0.f;
                    tmem_st16(tlane + k0, pv);
                    tmem_wait_st();
                    fence_async_smem();
                }
                // a narrow last panel: the unused k-rows of B must be zero
                if (w < kPW) {
                    for (int e = tid; e < NP * (kPW - w); e += 128) {
                        const int cc = e / (kPW - w), t = w + e % (kPW - w);
                        Bhi[op_off(cc, t)] = 0.f;
                        Blo[op_off(cc, t)] = 0.f;
                    }
                    fence_async_smem();
                }
                tc_fence_before();
                __syncthreads();
                // B4: A += X R on the tensor cores
                if (tid == 0) {
                    tc_fence_after();
                    const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo);
                    const uint32_t bh = smem_u32(Bhi), bl = smem_u32(Blo);
                    const int ksteps = w > 8 ? 2 : 1;
                    for (int s = 0; s < ksteps; ++s) {
                        const uint32_t ko = 256u * s;
                        mma_tf32(tmem, smem_desc(ah + ko, 128, 512), smem_desc(bh + ko, 128, 512), idesc);
                        mma_tf32(tmem, smem_desc(ah + ko, 128, 512), smem_desc(bl + ko, 128, 512), idesc);
                        mma_tf32(tmem, smem_desc(al + ko, 128, 512), smem_desc(bh + ko, 128, 512), idesc);
                    }
                    mma_commit(&bars[1]);
                }
                const bool mok = mbar_wait(&bars[1], u_mma & 1);
                if (__syncthreads_or(!mok)) {
                    if (tid == 0) { status[c] = VK_ETIMEOUT; mbar_wait(&bars[1], u_mma & 1); }
                    failed = true;
                    break;
                }
                ++u_mma;
                tc_fence_after();
            }
            if (failed) break;
            // ---- C: natural-order inverse -> Gs -> G32 ----
            if (tid == 0) bulk_wait_read();        // the previous layer's store has read Gs
            __syncthreads();
            if (row_warp) {
                const int row = r < n ? kinv[r] : 0;
#pragma unroll 1
                for (int g0 = 0; g0 < NP; g0 += 16 * kLdGroup) {
                    float v[kLdGroup][16];
#pragma unroll
                    for (int ch = 0; ch < kLdGroup; ++ch)
                        if (g0 + ch * 16 < NP) tmem_ld16_nowait(tlane + g0 + ch * 16, v[ch]);
                    tmem_wait_ld();
#pragma unroll
                    for (int ch = 0; ch < kLdGroup; ++ch) {
                        tmem_reg_dep(v[ch]);
                        if (r < n) {
#pragma unroll
                            for (int t = 0; t < 16; ++t) {
                                const int cc = g0 + ch * 16 + t;
                                if (cc < n) Gs[row * n + perm[cc]] = v[ch][t];
                            }
                        }
                    }
                }
            }
            if (tid < n && j + 1 < nz) { alpha[tid] = a_nx; beta[tid] = b_nx; }
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) bulk_store(G32 + l * NNP, Gs, (uint32_t)NNP * 4);
        }
        if (failed) break;
        if (tid == 0 && s_stat) status[c] = s_stat == 2 ? VK_ENAN : VK_ESINGULAR;
    }
    if (tid == 0) bulk_wait_all();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

// ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

static cudaError_t get_encode() {
    if (g_encode) return cudaSuccess;
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess) return e;
    if (q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return cudaSuccess;
}

bool lu_tc_supported(int n) { return n >= 1 && n <= 128; }

size_t lu_tc_block_floats(int n) { int NP = round_up(n, 16); return (size_t)NP * NP; }

// Tensor map over the padded scaled blocks: [max_layers * NP rows][NP floats].
cudaError_t lu_tc_make_map(CUtensorMap *map, const float *D32, int n, int max_layers) {
    cudaError_t e = get_encode();
    if (e != cudaSuccess) return e;
    const int NP = round_up(n, 16);
    cuuint64_t dims[2] = {(cuuint64_t)NP, (cuuint64_t)max_layers * NP};
    cuuint64_t strides[1] = {(cuuint64_t)NP * 4};
    cuuint32_t box[2] = {(cuuint32_t)NP, (cuuint32_t)NP};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)D32, dims, strides, box,
                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

size_t lu_tc_smem(int n) { return (size_t)tc_layout(n).total; }

cudaError_t init_lu_tc(int n) {
    if (!lu_tc_supported(n)) return cudaSuccess;
    const int sm = (int)lu_tc_smem(n);
    cudaError_t e = raise_smem_limit(k_lu_tc<3, false>, sm);
    if (e == cudaSuccess)
        e = raise_smem_limit(k_lu_tc<4, false>, sm);
    if (e == cudaSuccess)
        e = raise_smem_limit(k_lu_tc<3, true>, sm);
    if (e == cudaSuccess)
        e = raise_smem_limit(k_lu_tc<4, true>, sm);
    return e;
}

void launch_lu_tc(const DevNet &net, const DevBatch &b, const Work &w, const CUtensorMap &map,
                  bool coop, cudaStream_t s) {
    const int n = net.ni, NP = round_up(n, 16);
    const size_t sm = lu_tc_smem(n);
    const int grid = column_grid(b, VK_TUNE_LU32, 3);
#define LAUNCH_TC(RA, CO) k_lu_tc<RA, CO><<<grid, 128, sm, s>>>(net, b, map, w.dB, w.dC, w.rs, w.cs, w.G32, w.status)
    if (NP <= 96) { if (coop) LAUNCH_TC(3, true); else LAUNCH_TC(3, false); }
    else          { if (coop) LAUNCH_TC(4, true); else LAUNCH_TC(4, false); }
#undef LAUNCH_TC
}

}  // namespace vk
