// Device kernels of the Ros2 kinetics-diffusion step (FP64 path).
//
//   k_rates      (a) rate/source: net rate of every reaction pair of one layer
//                    and the production/loss gather dy/dt, plus the transport
//                    operator; with JAC also (b): the sparse per-layer
//                    chemistry Jacobian and the diffusion coefficients that form
//                    the block-tridiagonal LHS.
//   k_lu_fwd_f64 (c) block-Thomas factorisation of c0 I - J along a column with
//                    in-place Gauss-Jordan inversion (partial pivoting) of each
//                    Schur-complemented diagonal block, fused with the forward
//                    sweep of the first right-hand side.
//   k_back_f64       back substitution -> k1, fused yk2 = y + k1/r.
//   k_solve_f64      forward + back sweeps for the second right-hand side.
//   k_stage      (d) sol, truncation error delta (masked, column max), ymix.
//
// Reference semantics: chem_funs.chemdf / neg_symjac (generated by
// make_chem_funs.py:113-430, 686-717), op.ODESolver.diffdf / diffdf_no_mol
// (op.py:1438-1597), lhs_jac_tot / lhs_jac_no_mol (op.py:1973-2042,
// 2122-2166), Ros2.solver (op.py:2860-3007).
#include <cuda_runtime.h>
#include <math.h>

#include "vk_internal.cuh"
#include "vk_geo.cuh"
#include "vk_gj.cuh"
#include "vk_tma.cuh"

namespace vk {

__device__ __forceinline__ double ipow(double x, int e) {
    double r = x;
    for (int i = 1; i < e; ++i) r = __dmul_rn(r, x);
    return r;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Value of one side of pair p in the generated lambda order k*t1*t2*...
__device__ __forceinline__ double side_rate(double kk, const PairDesc *pd, int side,
                                            const double *yl, double M) {
    double v = kk;
    const int nt = __ldg(&pd->nt[side]);
    for (int t = 0; t < nt; ++t) {
        const int s = __ldg(&pd->tsp[side][t]);
        const double f = s < 0 ? M : yl[s];
        const int e = __ldg(&pd->tnu[side][t]);
        v = __dmul_rn(v, e == 1 ? f : ipow(f, e));
    }
    return v;
}

// ---------------------------------------------------------------------------
// (a)+(b) rate / source / Jacobian kernel: a CTA per layer at a time.  The FP64 pipe
// bounds it, so every gathered term is one FP64 instruction (the gather form
// of vk_network.cpp) and the loops a warp runs have similar lengths (pairs,
// species, half terms and Jacobian entries in decreasing order of length).
template <bool JAC>
__global__ void __launch_bounds__(128, 8)
k_rates(DevNet net, DevBatch b, const double *__restrict__ y, double *__restrict__ f,
        double *__restrict__ jv, double *__restrict__ dA, double *__restrict__ dB,
        double *__restrict__ dC, const double *__restrict__ k1, const double *__restrict__ dt,
        const double *__restrict__ geo, int flags, int chem_only) {
    extern __shared__ double sm[];
    const int ni = net.ni;
    // the CTAs stride over the layers, so layers of inactive columns cost a
    // test each rather than a CTA launch (an attempt in which few columns
    // still run launches few CTAs' worth of work); every layer ends with a
    // block barrier before the next one's shared-memory writes
    for (int l = blockIdx.x; l < b.L; l += gridDim.x) {
    const int c = b.lay_col[l];
    if (c < 0 || (b.active && !b.active[c])) continue;   // gap layer of a slot, or inactive
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    const int j = l - l0;
    double *yl = sm;                       // [ni + 1] layer j, then M (factor index ni)
    double *ym = yl + ni + 1;              // [ni] layer j-1
    double *yp = ym + ni;                  // [ni] layer j+1
    double *sums = yp + ni;                // [8] column sums, ysum ratios, 2/(r dt)
    double *v = sums + 8;                  // [max(npair + nxm, nh)]
    const int tid = threadIdx.x, nth = blockDim.x;
    const double *al = b.atm + (size_t)l * VK_ATM_NF;
    const double M = al[VK_ATM_M];
    for (int t = tid; t < 3 * ni; t += nth) {
        const int w = t / ni, s = t - w * ni, jj = j - 1 + w;
        const double val = (jj >= 0 && jj < nz) ? y[(size_t)(l0 + jj) * ni + s] : 0.0;
        (w == 0 ? ym : (w == 1 ? yl : yp))[s] = val;
    }
    if (tid == 0) yl[ni] = M;
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const bool has_up = j + 1 < nz, has_dn = j > 0;
    if (warp == 0) {
        // layer sums and the state-dependent ysum ratios of the transport
        // operator, once per layer (FP64 divisions are costly on this chip)
        double s3[3];
        const double *yw[3] = {ym, yl, yp};
#pragma unroll
        for (int w = 0; w < 3; ++w) {
            double s = 0;
            for (int i = lane; i < ni; i += 32) s += yw[w][i];
            s3[w] = warp_sum(s);
        }
        if (lane == 0) {
            const double ysm = s3[0], ys0 = s3[1], ysp = s3[2];
            sums[0] = has_up ? (ysp + ys0) / (2. * ys0) : 0.0;
            sums[1] = has_dn ? (ys0 + ysm) / (2. * ys0) : 0.0;
            sums[2] = has_up ? (ysp + ys0) / (2. * ysp) : 0.0;
            sums[3] = has_dn ? (ys0 + ysm) / (2. * ysm) : 0.0;
            sums[4] = k1 ? 2. / (R_ROS * dt[c]) : 0.0;
        }
    }
    const double *kl = b.k + (size_t)l * net.nr;
    // net rate of each pair (written-order products: bit-identical to chemdf)
    for (int i = tid; i < net.npair; i += nth) {
        const int p = net.porder[i];
        const PairDesc *pd = net.pairs + p;
        const double2 kk = reinterpret_cast<const double2 *>(kl)[p];
        v[p] = side_rate(kk.x, pd, 0, yl, M) - side_rate(kk.y, pd, 1, yl, M);
    }
    __syncthreads();
    if (net.nxm > 0) {                     // products by coefficients that are not powers of two
        for (int m = tid; m < net.nxm; m += nth)
            v[net.npair + m] = __dmul_rn(net.xmul_fac[m], v[net.xmul_pair[m]]);
        __syncthreads();
    }
    // ysum ratios of the transport operator (state dependent part)
    const double qU0 = sums[0], qD0 = sums[1], qUp = sums[2], qDm = sums[3];
    const double hinv = sums[4];
    const double *gl = geo + (size_t)l * GEO_NF * ni;
    const double *spf = b.spf + (size_t)c * VK_SP_NF * ni;
    // production - loss gather (generated chemdf order, one fma per term) +
    // transport; species in decreasing order of term count
    for (int si = tid; si < ni; si += nth) {
        const int s = net.src_order[si];
        double acc = 0.0;
        for (int e = net.src_ptr[s]; e < net.src_ptr[s + 1]; ++e)
            acc = __fma_rn(net.src_c[e], v[net.src_slot[e]], acc);
        const double gU = gl[s], gD = gl[ni + s];
        double cA = -gU * qU0 - gD * qD0 + gl[2 * ni + s];
        double cB = has_up ? gU * qUp + gl[3 * ni + s] : 0.0;
        double cC = has_dn ? gD * qDm + gl[4 * ni + s] : 0.0;
        double out = acc;
        if (!chem_only) {
            double dif = cA * yl[s];
            if (has_up) dif += cB * yp[s];
            if (has_dn) dif += cC * ym[s];
            if ((flags & VK_F_TOPFLUX) && j == nz - 1)
                dif += spf[VK_SP_TOPFLUX * ni + s] / b.atm[(size_t)(l - 1) * VK_ATM_NF + VK_ATM_DZI];
            if ((flags & VK_F_BOTFLUX) && j == 0)
                dif += (spf[VK_SP_BOTFLUX * ni + s] - yl[s] * spf[VK_SP_BOTVDEP * ni + s]) / al[VK_ATM_DZI];
            out = acc + dif;
            if (k1) out = out - hinv * k1[(size_t)l * ni + s];
        }
        f[(size_t)l * ni + s] = out;
        if (JAC) {
            if ((flags & VK_F_BOTFLUX) && j == 0) cA -= spf[VK_SP_BOTVDEP * ni + s] / al[VK_ATM_DZI];
            dA[(size_t)l * ni + s] = cA;
            dB[(size_t)l * ni + s] = cB;
            dC[(size_t)l * ni + s] = cC;
        }
    }
    if (JAC) {
        __syncthreads();
        // derivative half terms: k_side x product of the side's remaining factors
        for (int h = tid; h < net.nh; h += nth) {
            double d = kl[net.hk[h]];
            for (int t = net.hptr[h]; t < net.hptr[h + 1]; ++t) d = __dmul_rn(d, yl[net.hfac[t]]);
            v[h] = d;
        }
        __syncthreads();
        double *jl = jv + (size_t)l * net.nnz;
        for (int ei = tid; ei < net.nnz; ei += nth) {
            const int e = net.jorder[ei];
            double acc = 0.0;
            for (int t = net.hjptr[e]; t < net.hjptr[e + 1]; ++t)
                acc = __fma_rn(net.hjcoef[t], v[net.hjterm[t]], acc);
            jl[e] = -acc;                      // entries of -J (neg_symjac)
        }
    }
    __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// (c) block-Thomas factorisation + forward sweep, FP64, one column at a time
// per CTA (work queue).  The diagonal block
//   D'_j = c0 I - J_j - diag(dA_j) - diag(dC_j) G_{j-1} diag(dB_{j-1})
// is built and inverted in shared memory by Gauss-Jordan elimination with
// partial pivoting (largest |a|, lowest row on ties).  FP64 throughput bounds
// it (about 1/60 of the FP32 rate on this chip), so the inversion issues no
// FP64 instruction beyond the useful ones (vk_gj.cuh); with LA the block has
// two buffers and each pivot's search and scaling overlap the previous
// pivot's update (blocks up to 117 species; the in-place inversion above).
// The inverses are stored with the padded stride block_stride64(n).
template <bool LA>
__global__ void __launch_bounds__(256)
k_lu_fwd_f64(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
             const double *__restrict__ dB, const double *__restrict__ dC,
             const double *__restrict__ dt, const double *__restrict__ rhs,
             double *__restrict__ G, double *__restrict__ z, int *__restrict__ status) {
    extern __shared__ double sm[];
    const int n = net.ni, nn = n * n, gst = block_stride64(n);
    const int tid = threadIdx.x, nth = blockDim.x;
    double *A = sm;                                  // [nn]
    double *B = A + nn;                              // [nn] (LA: second buffer)
    double *colk = LA ? B + nn : A + nn;             // [2n] (LA) / [n]
    double *rowk = colk + (LA ? 2 * n : n);
    double *zp = rowk + (LA ? 2 * n : n);
    double *bb = zp + n;
    double *part = bb + n;                           // [max(nth, n)]
    int *perm = reinterpret_cast<int *>(part + (nth > n ? nth : n));
    __shared__ int s_sing, s_col, s_piv[2];
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        if (tid == 0) s_sing = 0;
        const double c0 = 1.0 / (R_ROS * dt[c]);
        double *Ac = A;                              // holds G_{j-1}, then D'_j
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            const double *cj = dC + l * n;
            const double *bm = j > 0 ? dB + (l - 1) * n : dB;
            const double *aj = dA + l * n;
            for (int e = tid; e < nn; e += nth) {
                int r = e / n, q = e - r * n;
                double v = j > 0 ? -cj[r] * Ac[e] * bm[q] : 0.0;
                if (r == q) v += c0 - aj[r];
                Ac[e] = v;
            }
            for (int t = tid; t < n; t += nth)
                bb[t] = rhs[l * n + t] + (j > 0 ? cj[t] * zp[t] : 0.0);
            __syncthreads();
            const double *jl = jv + l * net.nnz;
            for (int e = tid; e < net.nnz; e += nth) Ac[net.jpos[e]] += jl[e];
            __syncthreads();
            if (LA) Ac = gj_invert_f64_la(Ac, Ac == A ? B : A, n, colk, rowk, perm, s_piv, &s_sing);
            else gj_invert_f64(Ac, n, colk, rowk, perm, &s_sing);
            double *Gl = G + l * gst;
            for (int e = tid; e < nn; e += nth) Gl[e] = Ac[e];
            matvec_f64(Ac, n, bb, part, zp, nullptr);     // z_j = G_j bb (ends with a barrier)
            for (int t = tid; t < n; t += nth) z[l * n + t] = zp[t];
        }
        if (tid == 0 && s_sing) status[c] = s_sing == 2 ? VK_ENAN : VK_ESINGULAR;
    }
}

// Shared memory of the FP64 sweeps: two mbarriers, nbuf blocks of the padded
// stride, two vectors and the product's partial sums.  Two buffers (the next
// block's copy overlaps this block's product) when they fit in a CTA's 227 KB,
// else one (ni >~ 115).
static __host__ __device__ inline size_t sweep64_smem(int n, int nth, int nbuf) {
    return 16 + (size_t)(nbuf * block_stride64(n) + 2 * n + (nth > n ? nth : n)) * sizeof(double);
}
static inline int sweep64_nbuf(int n) { return sweep64_smem(n, 256, 2) <= 232448 ? 2 : 1; }

// Copy k of a CTA's block stream lands in buffer k % nbuf and completes
// phase (k / nbuf) & 1 of that buffer's mbarrier.
__device__ __forceinline__ bool wait_copy(uint64_t *bar, unsigned k, int nbuf) {
    return nbuf == 2 ? mbar_wait(&bar[k & 1], (k >> 1) & 1) : mbar_wait(&bar[0], k & 1);
}

// After a bulk copy that never landed: wait (bounded) for the copies still in
// flight, visits [v, last), so none lands in a CTA that has left; the caller
// then records VK_ETIMEOUT and leaves.
__device__ __forceinline__ void drain_copies(uint64_t *bar, unsigned cnt, int v, int last, int nbuf) {
    for (int u = v; u < last; ++u) wait_copy(bar, cnt + (unsigned)u, nbuf);
}

// x_j = z_j + G_j (dB_j o x_{j+1}); optional yk2 = y + x / r.  The inverses
// G_{nz-2} .. G_0 stream into shared memory by bulk copies in sweep order,
// double-buffered (nbuf = 2): the next block's copy runs during this block's
// product.
__global__ void __launch_bounds__(256)
k_back_f64(DevNet net, DevBatch b, const double *__restrict__ G, const double *__restrict__ dB,
           const double *__restrict__ z, double *__restrict__ x, const double *__restrict__ y,
           double *__restrict__ yk2, int *__restrict__ status, int nbuf) {
    extern __shared__ __align__(16) unsigned char smb[];
    const int n = net.ni, gst = block_stride64(n);
    const int tid = threadIdx.x, nth = blockDim.x;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smb);      // [2]
    double *Gbuf = reinterpret_cast<double *>(smb + 16);    // [nbuf][gst]
    double *xs = Gbuf + nbuf * gst;                         // [n] dB_j o x_{j+1}
    double *xn = xs + n;                                    // [n]
    double *part = xn + n;                                  // [max(nth, n)]
    __shared__ int s_col;
    const uint32_t bytes = (uint32_t)gst * sizeof(double);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    unsigned cnt = 0;              // copies this CTA consumed before the current column
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        const int nvis = nz - 1;                            // G_{nz-2} .. G_0
        auto issue = [&](int v) {                           // thread 0
            const unsigned k = cnt + (unsigned)v, bi = k % (unsigned)nbuf;
            tma_load_1d(Gbuf + bi * gst, G + ((size_t)l0 + nz - 2 - v) * gst, bytes, &bar[bi]);
        };
        if (tid == 0)
            for (int v = 0; v < nbuf && v < nvis; ++v) issue(v);
        {
            const size_t l = (size_t)l0 + nz - 1;           // top layer: x = z
            for (int t = tid; t < n; t += nth) {
                const double xv = z[l * n + t];
                x[l * n + t] = xv;
                if (yk2) yk2[l * n + t] = y[l * n + t] + xv / R_ROS;
                if (nz > 1) xs[t] = dB[(l - 1) * n + t] * xv;
            }
        }
        __syncthreads();
        int v = 0, timed_out = 0;
        for (; v < nvis; ++v) {
            const int j = nz - 2 - v;
            const size_t l = (size_t)l0 + j;
            const unsigned k = cnt + (unsigned)v;
            const bool ok = wait_copy(bar, k, nbuf);
            if (__syncthreads_or(!ok)) { timed_out = 1; break; }
            matvec_f64(Gbuf + (k % (unsigned)nbuf) * gst, n, xs, part, xn, z + l * n);
            if (tid == 0 && v + nbuf < nvis) issue(v + nbuf);   // the buffer just read is free
            for (int t = tid; t < n; t += nth) {
                const double xv = xn[t];
                x[l * n + t] = xv;
                if (yk2) yk2[l * n + t] = y[l * n + t] + xv / R_ROS;
                if (j > 0) xs[t] = dB[(l - 1) * n + t] * xv;
            }
            __syncthreads();
        }
        if (timed_out) {
            drain_copies(bar, cnt, v, nvis < v + nbuf ? nvis : v + nbuf, nbuf);
            if (tid == 0) status[c] = VK_ETIMEOUT;
            return;
        }
        cnt += (unsigned)nvis;
    }
}

// Forward + back sweep with the stored inverses for a new right-hand side.
// The blocks stream in visit order: G_0 .. G_{nz-1} (forward), G_{nz-2} .. G_0
// (back), bulk copies as in k_back_f64.
__global__ void __launch_bounds__(256)
k_solve_f64(DevNet net, DevBatch b, const double *__restrict__ G, const double *__restrict__ dB,
            const double *__restrict__ dC, const double *__restrict__ rhs,
            double *__restrict__ zbuf, double *__restrict__ x, int *__restrict__ status, int nbuf) {
    extern __shared__ __align__(16) unsigned char smb[];
    const int n = net.ni, gst = block_stride64(n);
    const int tid = threadIdx.x, nth = blockDim.x;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smb);      // [2]
    double *Gbuf = reinterpret_cast<double *>(smb + 16);    // [nbuf][gst]
    double *vin = Gbuf + nbuf * gst;                        // [n]
    double *vout = vin + n;                                 // [n]
    double *part = vout + n;                                // [max(nth, n)]
    __shared__ int s_col;
    const uint32_t bytes = (uint32_t)gst * sizeof(double);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    unsigned cnt = 0;
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        const int nvis = 2 * nz - 1;
        auto layer_of = [&](int v) { return v < nz ? v : 2 * nz - 2 - v; };
        auto issue = [&](int v) {                           // thread 0
            const unsigned k = cnt + (unsigned)v, bi = k % (unsigned)nbuf;
            tma_load_1d(Gbuf + bi * gst, G + ((size_t)l0 + layer_of(v)) * gst, bytes, &bar[bi]);
        };
        if (tid == 0)
            for (int v = 0; v < nbuf && v < nvis; ++v) issue(v);
        int v = 0, timed_out = 0;
        for (; v < nvis; ++v) {
            const bool fwd = v < nz;
            const int j = layer_of(v);
            const size_t l = (size_t)l0 + j;
            if (fwd) {
                for (int t = tid; t < n; t += nth)
                    vin[t] = rhs[l * n + t] + (j > 0 ? dC[l * n + t] * vout[t] : 0.0);
            }
            const unsigned k = cnt + (unsigned)v;
            const bool ok = wait_copy(bar, k, nbuf);
            if (__syncthreads_or(!ok)) { timed_out = 1; break; }
            const double *Gs = Gbuf + (k % (unsigned)nbuf) * gst;
            matvec_f64(Gs, n, vin, part, vout, fwd ? nullptr : zbuf + l * n);
            if (tid == 0 && v + nbuf < nvis) issue(v + nbuf);
            for (int t = tid; t < n; t += nth) {
                const double xv = vout[t];
                if (fwd) zbuf[l * n + t] = xv;
                if (!fwd || j == nz - 1) {                  // back sweep (starts at the top: x = z)
                    x[l * n + t] = xv;
                    if (j > 0) vin[t] = dB[(l - 1) * n + t] * xv;
                }
            }
            __syncthreads();
        }
        if (timed_out) {
            drain_copies(bar, cnt, v, nvis < v + nbuf ? nvis : v + nbuf, nbuf);
            if (tid == 0) status[c] = VK_ETIMEOUT;
            return;
        }
        cnt += (unsigned)nvis;
    }
}

// (d) stage: sol, masked relative truncation error (column max), ymix.
__global__ void __launch_bounds__(256)
k_stage(DevNet net, DevBatch b, const double *__restrict__ y, const double *__restrict__ ymix,
        const double *__restrict__ k1, const double *__restrict__ k2,
        const double *__restrict__ yk2, double *__restrict__ sol, double *__restrict__ ymix_out,
        double *__restrict__ delta, int *__restrict__ status, int flags, double mtol, double atol) {
    __shared__ double wmax[8];
    const int n = net.ni;
    const int c = blockIdx.x;
    if (b.active && !b.active[c]) return;
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarp = blockDim.x >> 5;
    const double c1 = 3. / (2. * R_ROS), c2 = 1 / (2. * R_ROS);
    // the column's largest d / sol, kept as a fraction (num, den) compared by
    // cross-multiplication and divided once per thread (an FP64 division is a
    // long FP64-pipe sequence on this chip)
    double dnum = 0.0, dden = 1.0;
    int bad = 0;
    for (int j = warp; j < nz; j += nwarp) {
        const size_t l = (size_t)l0 + j;
        double s = 0.0;
        for (int i = lane; i < n; i += 32) {
            const size_t e = l * n + i;
            double sv = __dadd_rn(__dadd_rn(y[e], __dmul_rn(c1, k1[e])), __dmul_rn(c2, k2[e]));
            sol[e] = sv;
            bad |= !isfinite(sv);
            s += sv;
            double d = fabs(sv - yk2[e]);
            if (ymix[e] < mtol) d = 0.0;
            if (sv < atol) d = 0.0;
            if ((flags & VK_F_BOTFLUX) && j == 0) d = 0.0;
            if (sv > 0.0 && d * dden > dnum * sv) { dnum = d; dden = sv; }
        }
        s = warp_sum(s);
        for (int i = lane; i < n; i += 32) ymix_out[l * n + i] = sol[l * n + i] / s;
    }
    double dmax = dnum / dden;
    for (int o = 16; o; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if (lane == 0) wmax[warp] = dmax;
    bad = __syncthreads_or(bad);
    if (tid == 0) {
        if (bad && status[c] == 0) status[c] = VK_ENAN;
        double m = 0.0;
        for (int w = 0; w < nwarp; ++w) m = fmax(m, wmax[w]);
        delta[c] = m;
    }
}

// Transport geometry of every (layer, species) of the active columns.
__global__ void __launch_bounds__(256)
k_geometry(DevNet net, DevBatch b, double *__restrict__ geo, int flags) {
    const int ni = net.ni;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)b.L * ni) return;
    const int l = (int)(e / ni), i = (int)(e - (long long)l * ni);
    const int c = b.lay_col[l];
    if (c < 0 || (b.active && !b.active[c])) return;
    const GeoCol cv = make_geocol(b.atm, b.Dzz, b.spf, b.col_off, b.col_end, c, ni);
    double out[GEO_NF];
    geo_coef(cv, l - cv.l0, i, flags, out);
    double *gl = geo + (size_t)l * GEO_NF * ni;
    for (int k = 0; k < GEO_NF; ++k) gl[k * ni + i] = out[k];
}

void launch_geometry(const DevNet &net, const DevBatch &b, double *geo, int flags, cudaStream_t s) {
    long long n = (long long)b.L * net.ni;
    k_geometry<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(net, b, geo, flags);
}

// ---------------------------------------------------------------------------
static size_t rates_smem(const DevNet &net);
// block(s), colk, rowk, zp, bb, the product's partial sums (doubles) + perm
// (ints); the look-ahead variant keeps two blocks and two colk/rowk
static size_t lu_fwd_smem(int n, bool la) {
    const int nb = la ? 2 : 1;
    return (size_t)(nb * n * n + (2 * nb + 2) * n + (256 > n ? 256 : n)) * sizeof(double) +
           (size_t)n * sizeof(int);
}
static inline bool lu_fwd_la(int n) { return lu_fwd_smem(n, true) <= 232448; }

// Opt the kernels into the dynamic shared memory this network needs; called
// once per handle, outside any stream capture.
cudaError_t init_kernels(const DevNet &net) {
    size_t sr = rates_smem(net);
    const int n = net.ni;
    size_t sl = lu_fwd_smem(n, lu_fwd_la(n));
    cudaError_t e;
    if ((e = raise_smem_limit(k_rates<true>, (int)sr))) return e;
    if ((e = raise_smem_limit(k_rates<false>, (int)sr))) return e;
    if ((e = lu_fwd_la(n) ? raise_smem_limit(k_lu_fwd_f64<true>, (int)sl)
                          : raise_smem_limit(k_lu_fwd_f64<false>, (int)sl)))
        return e;
    const int ssw = (int)sweep64_smem(n, 256, sweep64_nbuf(n));
    if ((e = raise_smem_limit(k_back_f64, ssw))) return e;
    if ((e = raise_smem_limit(k_solve_f64, ssw))) return e;
    return cudaSuccess;
}

static size_t rates_smem(const DevNet &net) {
    const int m = net.npair + net.nxm > net.nh ? net.npair + net.nxm : net.nh;
    return (size_t)(3 * net.ni + 1 + 8 + m) * sizeof(double);
}

void launch_rates(const DevNet &net, const DevBatch &b, const double *y, double *f,
                  double *jv, double *dA, double *dB, double *dC, const double *k1,
                  const double *dt, const double *geo, int flags, bool with_jac, cudaStream_t s) {
    size_t sm = rates_smem(net);
    const int grid = layer_grid(b, b.grid_rates);
    if (with_jac)
        k_rates<true><<<grid, 128, sm, s>>>(net, b, y, f, jv, dA, dB, dC, k1, dt, geo, flags, 0);
    else
        k_rates<false><<<grid, 128, sm, s>>>(net, b, y, f, jv, dA, dB, dC, k1, dt, geo, flags, 0);
}

// Resident CTAs per SM of k_rates (the larger of its two forms' register
// footprints sets it) for this network's shared memory.
int rates_blocks_per_sm(const DevNet &net) {
    const size_t sm = rates_smem(net);
    int a = 0, c = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_rates<true>, 128, sm) != cudaSuccess) a = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_rates<false>, 128, sm) != cudaSuccess) c = 0;
    return a < c ? a : c;
}

void launch_chem_only(const DevNet &net, const DevBatch &b, const double *y, double *f,
                      const double *geo, cudaStream_t s) {
    size_t sm = rates_smem(net);
    k_rates<false><<<layer_grid(b, b.grid_rates), 128, sm, s>>>(net, b, y, f, nullptr, nullptr, nullptr, nullptr,
                                        nullptr, nullptr, geo, 0, 1);
}

void launch_lu_fwd_f64(const DevNet &net, const DevBatch &b, const Work &w,
                       const double *rhs, double *z, int flags, cudaStream_t s) {
    (void)flags;
    const int n = net.ni;
    const bool la = lu_fwd_la(n);
    size_t sm = lu_fwd_smem(n, la);
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    if (la)
        k_lu_fwd_f64<true><<<column_grid(b, VK_TUNE_LU64, 2), 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt,
                                                                          rhs, w.G, z, w.status);
    else
        k_lu_fwd_f64<false><<<column_grid(b, VK_TUNE_LU64, 2), 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt,
                                                                           rhs, w.G, z, w.status);
}

void launch_back_f64(const DevNet &net, const DevBatch &b, const double *G, const double *dB,
                     const double *z, double *x, const double *y, double *yk2, int *status,
                     cudaStream_t s) {
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    const int nbuf = sweep64_nbuf(net.ni);
    k_back_f64<<<column_grid(b, VK_TUNE_SWEEP64, 2), 256, sweep64_smem(net.ni, 256, nbuf), s>>>(
        net, b, G, dB, z, x, y, yk2, status, nbuf);
}

void launch_solve_f64(const DevNet &net, const DevBatch &b, const double *G, const double *dB,
                      const double *dC, const double *rhs, double *zbuf, double *x, int *status,
                      cudaStream_t s) {
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    const int nbuf = sweep64_nbuf(net.ni);
    k_solve_f64<<<column_grid(b, VK_TUNE_SWEEP64, 2), 256, sweep64_smem(net.ni, 256, nbuf), s>>>(
        net, b, G, dB, dC, rhs, zbuf, x, status, nbuf);
}

void launch_stage(const DevNet &net, const DevBatch &b, const Work &w, int flags, double mtol,
                  double atol, cudaStream_t s) {
    k_stage<<<b.ncols, 256, 0, s>>>(net, b, w.y, w.ymix, w.k1, w.k2, w.yk2, w.sol, w.ymix_out,
                                    w.delta, w.status, flags, mtol, atol);
}

}  // namespace vk
