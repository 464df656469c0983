// FP32 block-Thomas factorisation with register-resident Gauss-Jordan inversion
// on the power-of-two row/column-scaled blocks (the mixed path, vk_mixed.cu):
//   k_prep32  per layer: scales R_j, S_j and the dense scaled block R_j D_j S_j;
//   k_lu32    per column: G~_j = (R_j D'_j S_j)^-1 stored in FP32, with
//             D'_j = D_j - diag(dC_j) G_{j-1} diag(dB_{j-1}).
// Columns come from the work queue (longest first); each CTA walks a column's
// layers in order.  Block sizes up to 160 species are covered by four
// register tilings (vk_gjreg.cuh).
#include <cuda.h>
#include <cuda_runtime.h>
#include <math.h>

#include "vk_gjreg.cuh"
#include "vk_internal.cuh"
#include "vk_tma.cuh"

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

// Biased IEEE exponent field of a double.
__device__ __forceinline__ int bexp64(double v) {
    return (int)((__double_as_longlong(v) >> 52) & 0x7ff);
}
// |v| as integer bits with NaN mapped to 0 (fmax ignores NaN operands).
__device__ __forceinline__ long long absbits_nonan(double v) {
    const long long a = __double_as_longlong(v) & 0x7fffffffffffffffll;
    return a > 0x7ff0000000000000ll ? 0ll : a;
}
// v x 2^k by the exponent field when the result stays normal (exact, as the
// FP64 product with a power of two is); returns false otherwise.
__device__ __forceinline__ bool scale_pow2(double v, int k, double &out) {
    const int E = bexp64(v);
    if (E < 1 || E > 2046 || E + k < 1 || E + k > 2046) return false;
    const long long bits = __double_as_longlong(v);
    out = __longlong_as_double((bits & ~(0x7ffll << 52)) | ((long long)(E + k) << 52));
    return true;
}
constexpr int kNoExp = -100000;        // "this row's scale has no exponent form"

// The FP64 expressions for values outside the normal range, as calls so the
// compiler branches around them instead of evaluating them for every element
// and selecting (they are FP64-pipe work).
__device__ __noinline__ int frexp_of_scaled(double v, double rs) {
    const double a = fabs(v * rs);
    if (!(a > 0.0) || !isfinite(a)) return kNoExp;
    int ex;
    frexp(a, &ex);
    return ex;
}
__device__ __noinline__ float scaled_f32(double rs, double v, double cs) {
    return (float)(rs * v * cs);
}

// Per-layer preparation for the FP32 factorisation (fully parallel over
// layers): power-of-two row scales (row maxima of D_j) and column scales
// (column maxima of R_j D_j), and the dense scaled block R_j D_j S_j rounded
// once to FP32, written with a 16-byte-aligned stride for TMA: rows of ld
// floats, bstride floats per layer (ld = n for k_lu32's packed blocks; ld =
// NP, the size rounded up to 16, for k_lu_tc's zero-padded NP x NP tiles).
// The scales are exact powers of two, so maxima, exponents and the scaled
// values are taken from the IEEE exponent fields with integer operations --
// the FP64 pipe (about 1/60 of the FP32 rate on this chip) only adds the
// diagonal and converts to FP32; values outside the normal range take the
// FP64 expressions, which give the same results.
__global__ void __launch_bounds__(256, 6)
k_prep32(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
         const double *__restrict__ dt, float *__restrict__ D32, double *__restrict__ rsc,
         double *__restrict__ csc, int ld, int bstride) {
    extern __shared__ double sp[];
    const int n = net.ni, nn = n * n, nnz = net.nnz;
    __shared__ double s_c0;
    // the CTAs stride over the layers (inactive columns' layers cost a test
    // each); every layer ends with a block barrier
    for (int l = blockIdx.x; l < b.L; l += gridDim.x) {
    const int c = b.lay_col[l];
    if (c < 0 || (b.active && !b.active[c])) continue;
    double *jls = sp;                       // [nnz]
    double *rs = jls + nnz;                 // [n]
    double *cs = rs + n;                    // [n]
    double *dg = cs + n;                    // [n] c0 - dA
    double *dd = dg + n;                    // [n] diagonal of D: -J_rr + c0 - dA_r
    float *dense = reinterpret_cast<float *>(dd + n);   // [nn]
    int *cexp = reinterpret_cast<int *>(dense + nn);    // [n]
    int *rexp = cexp + n;                   // [n] log2 rs (kNoExp: use rs)
    int *cxp = rexp + n;                    // [n] log2 cs
    const int tid = threadIdx.x, nth = blockDim.x;
    if (tid == 0) s_c0 = 1.0 / (R_ROS * dt[c]);     // one FP64 division per layer
    const double *jl = jv + (size_t)l * nnz;
    for (int e = tid; e < nnz; e += nth) jls[e] = jl[e];
    for (int e = tid; e < nn; e += nth) dense[e] = 0.0f;
    for (int t = tid; t < n; t += nth) cexp[t] = kNoExp;
    __syncthreads();
    for (int r = tid; r < n; r += nth) {
        dg[r] = s_c0 - dA[(size_t)l * n + r];
        const int e = net.jmap[r * n + r];
        dd[r] = e >= 0 ? jls[e] + dg[r] : dg[r];
    }
    __syncthreads();
    // row scales: 2^-e with |max| in [2^(e-1), 2^e)  (frexp / ldexp)
    for (int r = tid; r < n; r += nth) {
        long long m = absbits_nonan(dg[r]);
        for (int e = net.jrowptr[r]; e < net.jrowptr[r + 1]; ++e)
            m = max(m, absbits_nonan(net.jcol[e] == r ? dd[r] : jls[e]));
        const int E = (int)(m >> 52);
        if (m == 0 || E == 2047) {              // no positive finite maximum
            rs[r] = 1.0;
            rexp[r] = 0;
        } else if (E >= 1 && E <= 2044) {
            rexp[r] = 1022 - E;
            rs[r] = __longlong_as_double((long long)(1023 + 1022 - E) << 52);
        } else {                                // subnormal or huge maximum
            const double md = __longlong_as_double(m);
            int ex;
            frexp(md, &ex);
            rs[r] = ldexp(1.0, -ex);
            rexp[r] = kNoExp;
        }
    }
    __syncthreads();
    // column exponents of R_j D_j
    for (int e = tid; e < nnz + n; e += nth) {
        int r, q;
        double v;
        if (e < nnz) {
            r = net.jrow[e]; q = net.jcol[e];
            v = r == q ? dd[r] : jls[e];
        } else {
            r = q = e - nnz;
            v = dg[r];
        }
        if ((__double_as_longlong(v) & 0x7fffffffffffffffll) == 0) continue;    // v * rs = 0
        const int E = bexp64(v), k = rexp[r];
        if (k != kNoExp && E >= 1 && E <= 2046 && E + k >= 1 && E + k <= 2046) {
            atomicMax(&cexp[q], E + k - 1022);
        } else {
            const int ex = frexp_of_scaled(v, rs[r]);
            if (ex != kNoExp) atomicMax(&cexp[q], ex);
        }
    }
    __syncthreads();
    for (int t = tid; t < n; t += nth) {
        cs[t] = cexp[t] > kNoExp ? ldexp(1.0, -cexp[t]) : 1.0;
        cxp[t] = cexp[t] > kNoExp ? -cexp[t] : 0;
    }
    __syncthreads();
    // dense scaled block: (rs v) cs rounded once to FP32
    for (int e = tid; e < nnz + n; e += nth) {
        int r, q;
        double v;
        if (e < nnz) {
            r = net.jrow[e]; q = net.jcol[e];
            v = r == q ? dd[r] : jls[e];
        } else {
            r = q = e - nnz;
            if (net.jmap[r * n + r] >= 0) continue;     // the diagonal came with the Jacobian
            v = dg[r];
        }
        const int k = rexp[r];
        const long long vb = __double_as_longlong(v);
        double t1, t2;
        if ((vb & 0x7fffffffffffffffll) == 0)             // +-0 stays +-0
            dense[r * n + q] = __int_as_float((int)((unsigned long long)vb >> 32) & (int)0x80000000);
        else if (k != kNoExp && scale_pow2(v, k, t1) && scale_pow2(t1, cxp[q], t2))
            dense[r * n + q] = __double2float_rn(t2);
        else
            dense[r * n + q] = scaled_f32(rs[r], v, cs[q]);
    }
    __syncthreads();
    float *Dl = D32 + (size_t)l * bstride;
    if (ld == n) {
        for (int e = tid; e < nn; e += nth) Dl[e] = dense[e];
    } else {
        for (int e = tid; e < ld * ld; e += nth) {
            const int r = e / ld, q = e - r * ld;
            Dl[e] = (r < n && q < n) ? dense[r * n + q] : 0.0f;
        }
    }
    for (int t = tid; t < n; t += nth) {
        rsc[(size_t)l * n + t] = rs[t];
        csc[(size_t)l * n + t] = cs[t];
    }
    __syncthreads();
    }
}


// FP32 block-Thomas factorisation of the scaled system, one column at a time
// per CTA (columns from the work queue).
// The dense scaled block of layer j+1 streams into shared memory by TMA while
// layer j is inverted (register-resident Gauss-Jordan).
template <int TY, int RA, int RB>
__global__ void __launch_bounds__(16 * TY, TY == 16 && RA <= 5 ? 3 : 1)
k_lu32(DevNet net, DevBatch b, const float *__restrict__ D32, const double *__restrict__ dB,
       const double *__restrict__ dC, const double *__restrict__ rsc,
       const double *__restrict__ csc, float *__restrict__ G32, int *__restrict__ status,
       int nbuf) {
    extern __shared__ __align__(16) unsigned char smb[];
    const int n = net.ni, nn = n * n, NNP = block_stride32(n);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smb);             // [2]
    float *Dbuf = reinterpret_cast<float *>(smb + 16);             // [nbuf][NNP]
    float *Gs = Dbuf + nbuf * NNP;                                 // [nn]
    float *rowv = Gs + nn;
    float *colv = rowv + n;
    float *alpha = colv + n;
    float *beta = alpha + n;
    int *perm = reinterpret_cast<int *>(beta + n);
    int *kinv = perm + n;
    int *used = kinv + n;
    __shared__ int s_piv, s_sing, s_col, s_piv2[2];
    __shared__ float s_pval;
    GJShared<float> sh{rowv, colv, perm, kinv, used, &s_piv, &s_pval, &s_sing};
    float *colv2 = rowv;                                           // [2][n] (rowv, colv)
    int ty, tx;
    tile_coords<TY>(ty, tx);
    const int tid = threadIdx.x, nth = blockDim.x;
    const uint32_t bytes = (uint32_t)NNP * sizeof(float);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    // u counts the blocks this CTA has consumed over all its columns: block u
    // sits in buffer u&1 (use u>>1 of that barrier) with two buffers, in
    // buffer 0 (use u of barrier 0) with one
    int u = 0;
    auto buf_of = [&](int uu) { return nbuf == 2 ? (uu & 1) : 0; };
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        if (tid == 0) {
            s_sing = 0;
            tma_load_1d(Dbuf + buf_of(u) * NNP, D32 + (size_t)l0 * NNP, bytes, &bar[buf_of(u)]);
        }
        // per-thread copies of this layer's scales (threads t < n own species t)
        double rs_cur = 0, cs_cur = 0, dB_cur = 0;
        if (tid < n) {
            rs_cur = rsc[(size_t)l0 * n + tid];
            cs_cur = csc[(size_t)l0 * n + tid];
            dB_cur = dB[(size_t)l0 * n + tid];
        }
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            // prefetch the scales of the next layer into registers
            double rs_nx = 0, cs_nx = 0, dC_nx = 0, dB_nx = 0;
            if (tid < n && j + 1 < nz) {
                rs_nx = rsc[(l + 1) * n + tid];
                cs_nx = csc[(l + 1) * n + tid];
                dC_nx = dC[(l + 1) * n + tid];
                dB_nx = dB[(l + 1) * n + tid];
            }
            const int bsel = buf_of(u);
            const uint32_t par = nbuf == 2 ? (u >> 1) & 1 : u & 1;
            const bool ok = mbar_wait(&bar[bsel], par);
            if (__syncthreads_or(!ok)) {
                // the copy waited for is the only one in flight: let it land
                if (tid == 0) {
                    status[c] = VK_ETIMEOUT;
                    mbar_wait(&bar[bsel], par);
                }
                return;
            }
            ++u;
            if (nbuf == 2 && tid == 0 && j + 1 < nz)
                tma_load_1d(Dbuf + (bsel ^ 1) * NNP, D32 + (l + 1) * NNP, bytes, &bar[bsel ^ 1]);
            const float *Dj = Dbuf + bsel * NNP;
            float M[RA][RB];
#pragma unroll
            for (int a = 0; a < RA; ++a) {
                const int r = ty + TY * a;
#pragma unroll
                for (int q = 0; q < RB; ++q) {
                    const int cc = tx + 16 * q;
                    float v = 0.0f;
                    if (r < n && cc < n) {
                        v = Dj[r * n + cc];
                        if (j > 0) v -= alpha[r] * Gs[r * n + cc] * beta[cc];
                    }
                    M[a][q] = v;
                }
            }
            for (int t = tid; t < n; t += nth) used[t] = 0;
            __syncthreads();
            // one buffer: block j is in registers now, so the copy of block j+1
            // overwrites it while the inversion runs
            if (nbuf == 1 && tid == 0 && j + 1 < nz)
                tma_load_1d(Dbuf, D32 + (l + 1) * NNP, bytes, &bar[0]);
            gj_invert_reg1<float, TY, RA, RB>(M, n, ty, tx, sh, colv2, s_piv2);
            gj_store_natural<float, TY, RA, RB>(M, n, ty, tx, sh, Gs);
            float *Gl = G32 + l * NNP;
            for (int e = tid; e < nn; e += nth) Gl[e] = Gs[e];
            if (tid < n && j + 1 < nz) {
                alpha[tid] = (float)(rs_nx * dC_nx * cs_cur);
                beta[tid] = (float)(rs_cur * dB_cur * cs_nx);
                rs_cur = rs_nx;
                cs_cur = cs_nx;
                dB_cur = dB_nx;
            }
            __syncthreads();
        }
        if (tid == 0 && s_sing) status[c] = s_sing == 2 ? VK_ENAN : VK_ESINGULAR;
    }
}

// ---------------------------------------------------------------------------
static size_t smem32(int n, int nbuf) {
    return 16 + (size_t)nbuf * block_stride32(n) * sizeof(float) + (size_t)(n * n + 4 * n) * sizeof(float)
           + 3 * n * sizeof(int) + 16;
}
static int g_smem_optin = 0;         // opt-in shared memory per block of this device
// double-buffered block stream where it fits, else one buffer (ni above ~120)
static int lu32_nbuf(int n) { return smem32(n, 2) <= (size_t)g_smem_optin ? 2 : 1; }
static size_t smem_prep(const DevNet &net) {
    const int n = net.ni;
    return (size_t)(net.nnz + 4 * n) * sizeof(double) + (size_t)n * n * sizeof(float) + 3 * n * sizeof(int) + 16;
}

#define VK_LU_TILINGS(X) X(16, 3, 3) X(16, 5, 5) X(16, 7, 7) X(32, 5, 10)

// largest block each tiling covers (rows = TY * RA, columns = 16 * RB); tiling
// VK_LU_TC is the tensor-core factorisation (vk_lutc.cu), up to 128 species
static const int kTilingCap[4] = {48, 80, 112, 160};
int lu32_tiling_cap(int t) {
    if (t == VK_LU_TC || t == VK_LU_TC_COOP) return 128;
    return t >= 0 && t < 4 ? kTilingCap[t] : 0;
}

static int tiling_of(int n) {
    if (n <= 48) return 0;
    if (n <= 80) return 1;
    if (n <= 112) return 2;
    return 3;
}

// Resident CTAs per SM of k_prep32 for this network's shared memory.
int prep_blocks_per_sm(const DevNet &net) {
    int a = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_prep32, 256, smem_prep(net)) != cudaSuccess) a = 0;
    return a;
}

cudaError_t init_lureg_kernels(const DevNet &net) {
    const int n = net.ni;
    cudaError_t e = raise_smem_limit(k_prep32, (int)smem_prep(net));
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    size_t s32 = smem32(n, lu32_nbuf(n));
#define SETATTR(TY, RA, RB)                                                                      \
    if (e == cudaSuccess) e = raise_smem_limit(k_lu32<TY, RA, RB>, (int)s32);
    VK_LU_TILINGS(SETATTR)
#undef SETATTR
    return e;
}

void launch_lu_reg32(const DevNet &net, const DevBatch &b, const Work &w, cudaStream_t s) {
    const int n = net.ni;
    // vk_set_launch may pick a larger tiling than the smallest covering ni;
    // every tiling zero-pads the rows and columns beyond ni
    // default (-1): the tensor-core factorisation where it covers ni, with the
    // four warps sharing each panel
    int t = b.lu32_tiling == -1 ? (lu_tc_supported(n) ? VK_LU_TC_COOP : tiling_of(n))
          : (b.lu32_tiling >= tiling_of(n) ? b.lu32_tiling : tiling_of(n));
    const bool tc = t == VK_LU_TC || t == VK_LU_TC_COOP;
    if (tc && !w.tmap_d32) t = tiling_of(n);              // no tile map: CUDA-core kernel
    if (tc && w.tmap_d32) {
        const int NP = (n + 15) / 16 * 16;
        k_prep32<<<layer_grid(b, b.grid_prep), 256, smem_prep(net), s>>>(
            net, b, w.jv, w.dA, w.dt, w.D32, w.rs, w.cs, NP, NP * NP);
        cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
        launch_lu_tc(net, b, w, *static_cast<const CUtensorMap *>(w.tmap_d32), t == VK_LU_TC_COOP, s);
        return;
    }
    k_prep32<<<layer_grid(b, b.grid_prep), 256, smem_prep(net), s>>>(
        net, b, w.jv, w.dA, w.dt, w.D32, w.rs, w.cs, n, block_stride32(n));
    const int nb = lu32_nbuf(n);
    size_t sm = smem32(n, nb);
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    switch (t) {
    case 0: k_lu32<16, 3, 3><<<column_grid(b, VK_TUNE_LU32, 3), 256, sm, s>>>(net, b, w.D32, w.dB, w.dC, w.rs, w.cs, w.G32, w.status, nb); break;
    case 1: k_lu32<16, 5, 5><<<column_grid(b, VK_TUNE_LU32, 3), 256, sm, s>>>(net, b, w.D32, w.dB, w.dC, w.rs, w.cs, w.G32, w.status, nb); break;
    case 2: k_lu32<16, 7, 7><<<column_grid(b, VK_TUNE_LU32, 3), 256, sm, s>>>(net, b, w.D32, w.dB, w.dC, w.rs, w.cs, w.G32, w.status, nb); break;
    default: k_lu32<32, 5, 10><<<column_grid(b, VK_TUNE_LU32, 1), 512, sm, s>>>(net, b, w.D32, w.dB, w.dC, w.rs, w.cs, w.G32, w.status, nb); break;
    }
}

}  // namespace vk
