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

// acc + c*v for a coefficient code (+1, -1: signed add without a multiply;
// 0: multiply by the tabulated coefficient).  Bit-identical to the
// reference's "acc -1*v" / "acc +2*v" terms.
__device__ __forceinline__ double add_coef(double acc, int code, double nu, double v) {
    if (code == 1) return __dadd_rn(acc, v);
    if (code == -1) return __dadd_rn(acc, __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ull));
    return __dadd_rn(acc, __dmul_rn(nu, v));
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

// d/dy_q of kM * prod y_s^e over merged factors (kM = k M^m); pos = index of q.
__device__ __forceinline__ double side_deriv(double kM, const int16_t *sp, const uint8_t *nu,
                                             int n, int pos, const double *yl) {
    double v = kM;
    for (int t = 0; t < n; ++t) {
        const double yv = yl[__ldg(sp + t)];
        const int e = __ldg(nu + t);
        if (t == pos) {
            if (e == 2) v *= yv + yv;
            else if (e > 2) v *= (double)e * ipow(yv, e - 1);
        } else {
            v *= ipow(yv, e);
        }
    }
    return v;
}

__device__ __forceinline__ double mpow(double M, int m) {
    return m == 0 ? 1.0 : (m == 1 ? M : (m == 2 ? M * M : M * M * M));
}

// ---------------------------------------------------------------------------
// (a)+(b) rate / source / Jacobian kernel: one CTA per layer.
template <bool JAC>
__global__ void __launch_bounds__(128)
k_rates(DevNet net, DevBatch b, const double *__restrict__ y, double *__restrict__ f,
        double *__restrict__ jv, double *__restrict__ dA, double *__restrict__ dB,
        double *__restrict__ dC, const double *__restrict__ k1, const double *__restrict__ dt,
        const double *__restrict__ geo, int flags, int chem_only) {
    extern __shared__ double sm[];
    const int ni = net.ni;
    const int l = blockIdx.x;
    const int c = b.lay_col[l];
    if (c < 0 || (b.active && !b.active[c])) return;     // gap layer of a slot, or inactive
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    const int j = l - l0;
    double *ys = sm;                       // [3][ni] layers j-1, j, j+1
    double *sums = ys + 3 * ni;            // [8] column sums, ysum ratios, 2/(r dt)
    double *v = sums + 8;                  // [max(npair, nw)]
    double *kM = v + (net.npair > net.nw ? net.npair : net.nw);   // [2*npair] (JAC only)
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int t = tid; t < 3 * ni; t += nth) {
        int jj = j - 1 + t / ni;
        ys[t] = (jj >= 0 && jj < nz) ? y[(size_t)(l0 + jj) * ni + (t % ni)] : 0.0;
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const bool has_up = j + 1 < nz, has_dn = j > 0;
    if (warp == 0) {
        // layer sums and the state-dependent ysum ratios of the transport
        // operator, once per layer (FP64 divisions are costly on this chip)
        double s3[3];
#pragma unroll
        for (int w = 0; w < 3; ++w) {
            double s = 0;
            for (int i = lane; i < ni; i += 32) s += ys[w * ni + i];
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
    const double *yl = ys + ni;
    const double *al = b.atm + (size_t)l * VK_ATM_NF;
    const double M = al[VK_ATM_M];
    const double *kl = b.k + (size_t)l * net.nr;
    // net rate of each pair
    for (int p = tid; p < net.npair; p += nth) {
        const PairDesc *pd = net.pairs + p;
        const double2 kk = reinterpret_cast<const double2 *>(kl)[p];
        v[p] = side_rate(kk.x, pd, 0, yl, M) - side_rate(kk.y, pd, 1, yl, M);
        if (JAC) {
            kM[2 * p] = kk.x * mpow(M, __ldg(&pd->fm));
            kM[2 * p + 1] = kk.y * mpow(M, __ldg(&pd->rm));
        }
    }
    __syncthreads();
    // ysum ratios of the transport operator (state dependent part)
    const double qU0 = sums[0], qD0 = sums[1], qUp = sums[2], qDm = sums[3];
    const double hinv = sums[4];
    const double *gl = geo + (size_t)l * GEO_NF * ni;
    const double *spf = b.spf + (size_t)c * VK_SP_NF * ni;
    // production - loss gather (generated chemdf order) + transport; species
    // in decreasing order of term count so a warp's lanes end together
    for (int si = tid; si < ni; si += nth) {
        const int s = net.src_order[si];
        double acc = 0.0;
        for (int e = net.src_ptr[s]; e < net.src_ptr[s + 1]; ++e) {
            const int2 t = net.src[e];
            acc = add_coef(acc, t.y, t.y ? 0.0 : net.src_nu[e], v[t.x]);
        }
        const double gU = gl[s], gD = gl[ni + s];
        double cA = -gU * qU0 - gD * qD0 + gl[2 * ni + s];
        double cB = has_up ? gU * qUp + gl[3 * ni + s] : 0.0;
        double cC = has_dn ? gD * qDm + gl[4 * ni + s] : 0.0;
        double out = acc;
        if (!chem_only) {
            double dif = cA * yl[s];
            if (has_up) dif += cB * ys[2 * ni + s];
            if (has_dn) dif += cC * ys[s];
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
    if (!JAC) return;
    __syncthreads();
    // derivative terms d v_p / d y_q
    for (int t = tid; t < net.nw; t += nth) {
        const WDesc wd = net.w[t];
        const PairDesc *pd = net.pairs + wd.pair;
        double d = 0.0;
        if (wd.fpos >= 0) d = side_deriv(kM[2 * wd.pair], pd->fsp, pd->fnu, __ldg(&pd->nf), wd.fpos, yl);
        if (wd.rpos >= 0) d -= side_deriv(kM[2 * wd.pair + 1], pd->rsp, pd->rnu, __ldg(&pd->nr), wd.rpos, yl);
        v[t] = d;
    }
    __syncthreads();
    double *jl = jv + (size_t)l * net.nnz;
    for (int ei = tid; ei < net.nnz; ei += nth) {
        const int e = net.jorder[ei];
        double acc = 0.0;
        for (int t = net.jptr[e]; t < net.jptr[e + 1]; ++t) {
            const int2 jt = net.jterm[t];
            acc = jt.y == 1 ? acc + v[jt.x]
                : (jt.y == -1 ? acc - v[jt.x] : fma(net.jterm_nu[t], v[jt.x], acc));
        }
        jl[e] = -acc;                      // entries of -J (neg_symjac)
    }
}

// ---------------------------------------------------------------------------
// (c) block-Thomas factorisation + forward sweep, FP64, one column at a time
// per CTA (work queue).  The diagonal block
//   D'_j = c0 I - J_j - diag(dA_j) - diag(dC_j) G_{j-1} diag(dB_{j-1})
// is built and inverted in place in shared memory by Gauss-Jordan elimination
// with partial pivoting (largest |a|, lowest row on ties).  (A variant with the
// block in registers, as the FP32 path has, measured 92.9 ms against 76.4 ms
// per attempt at 512 columns: FP64 throughput, not barriers, bounds this one.)
__global__ void __launch_bounds__(256)
k_lu_fwd_f64(DevNet net, DevBatch b, const double *__restrict__ jv, const double *__restrict__ dA,
             const double *__restrict__ dB, const double *__restrict__ dC,
             const double *__restrict__ dt, const double *__restrict__ rhs,
             double *__restrict__ G, double *__restrict__ z, int *__restrict__ status) {
    extern __shared__ double sm[];
    const int n = net.ni, nn = n * n;
    double *A = sm;
    double *colk = A + nn;
    double *rowk = colk + n;
    double *zp = rowk + n;
    double *bb = zp + n;
    int *perm = reinterpret_cast<int *>(bb + n);
    __shared__ int s_piv, s_sing, s_col;
    __shared__ double s_pval;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        if (tid == 0) s_sing = 0;
        const double c0 = 1.0 / (R_ROS * dt[c]);
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            const double *cj = dC + l * n;
            const double *bm = j > 0 ? dB + (l - 1) * n : dB;
            const double *aj = dA + l * n;
            for (int e = tid; e < nn; e += nth) {
                int r = e / n, q = e - r * n;
                double v = j > 0 ? -cj[r] * A[e] * bm[q] : 0.0;
                if (r == q) v += c0 - aj[r];
                A[e] = v;
            }
            for (int t = tid; t < n; t += nth)
                bb[t] = rhs[l * n + t] + (j > 0 ? cj[t] * zp[t] : 0.0);
            __syncthreads();
            const double *jl = jv + l * net.nnz;
            for (int e = tid; e < net.nnz; e += nth) A[net.jpos[e]] += jl[e];
            __syncthreads();
            gj_invert_f64(A, n, colk, rowk, perm, &s_piv, &s_pval, &s_sing);
            double *Gl = G + l * nn;
            for (int e = tid; e < nn; e += nth) Gl[e] = A[e];
            for (int r = warp; r < n; r += nwarp) {
                double s = 0.0;
                for (int q = lane; q < n; q += 32) s += A[r * n + q] * bb[q];
                s = warp_sum(s);
                if (lane == 0) rowk[r] = s;
            }
            __syncthreads();
            for (int t = tid; t < n; t += nth) {
                zp[t] = rowk[t];
                z[l * n + t] = rowk[t];
            }
            __syncthreads();
        }
        if (tid == 0 && s_sing) status[c] = s_sing == 2 ? VK_ENAN : VK_ESINGULAR;
    }
}

// x_j = z_j + G_j (dB_j o x_{j+1}); optional yk2 = y + x / r.
__global__ void __launch_bounds__(256)
k_back_f64(DevNet net, DevBatch b, const double *__restrict__ G, const double *__restrict__ dB,
           const double *__restrict__ z, double *__restrict__ x, const double *__restrict__ y,
           double *__restrict__ yk2) {
    extern __shared__ double sm[];
    const int n = net.ni, nn = n * n;
    double *xs = sm;          // x_{j+1} * dB_j
    double *xn = sm + n;
    __shared__ int s_col;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        for (int j = nz - 1; j >= 0; --j) {
            const size_t l = (size_t)l0 + j;
            if (j == nz - 1) {
                for (int t = tid; t < n; t += nth) xn[t] = z[l * n + t];
            } else {
                const double *Gl = G + l * nn;
                for (int r = warp; r < n; r += nwarp) {
                    double s = 0.0;
                    for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * xs[q];
                    s = warp_sum(s);
                    if (lane == 0) xn[r] = z[l * n + r] + s;
                }
            }
            __syncthreads();
            for (int t = tid; t < n; t += nth) {
                double xv = xn[t];
                x[l * n + t] = xv;
                if (yk2) yk2[l * n + t] = y[l * n + t] + xv / R_ROS;
                if (j > 0) xs[t] = dB[(l - 1) * n + t] * xv;
            }
            __syncthreads();
        }
    }
}

// Forward + back sweep with stored inverses for a new right-hand side.
__global__ void __launch_bounds__(256)
k_solve_f64(DevNet net, DevBatch b, const double *__restrict__ G, const double *__restrict__ dB,
            const double *__restrict__ dC, const double *__restrict__ rhs,
            double *__restrict__ zbuf, double *__restrict__ x) {
    extern __shared__ double sm[];
    const int n = net.ni, nn = n * n;
    double *vin = sm;
    double *vout = sm + n;
    __shared__ int s_col;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        for (int j = 0; j < nz; ++j) {
            const size_t l = (size_t)l0 + j;
            for (int t = tid; t < n; t += nth)
                vin[t] = rhs[l * n + t] + (j > 0 ? dC[l * n + t] * vout[t] : 0.0);
            __syncthreads();
            const double *Gl = G + l * nn;
            for (int r = warp; r < n; r += nwarp) {
                double s = 0.0;
                for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * vin[q];
                s = warp_sum(s);
                if (lane == 0) { vout[r] = s; zbuf[l * n + r] = s; }
            }
            __syncthreads();
        }
        for (int j = nz - 1; j >= 0; --j) {
            const size_t l = (size_t)l0 + j;
            if (j < nz - 1) {
                const double *Gl = G + l * nn;
                for (int r = warp; r < n; r += nwarp) {
                    double s = 0.0;
                    for (int q = lane; q < n; q += 32) s += Gl[r * n + q] * vin[q];
                    s = warp_sum(s);
                    if (lane == 0) vout[r] = zbuf[l * n + r] + s;
                }
            } else {
                for (int t = tid; t < n; t += nth) vout[t] = zbuf[l * n + t];
            }
            __syncthreads();
            for (int t = tid; t < n; t += nth) {
                x[l * n + t] = vout[t];
                if (j > 0) vin[t] = dB[(l - 1) * n + t] * vout[t];
            }
            __syncthreads();
        }
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
    double dmax = 0.0;
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
            if (sv > 0.0) dmax = fmax(dmax, d / sv);
        }
        s = warp_sum(s);
        for (int i = lane; i < n; i += 32) ymix_out[l * n + i] = sol[l * n + i] / s;
    }
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
// block, colk, rowk, zp, bb (doubles) + perm (ints)
static size_t lu_fwd_smem(int n) { return (size_t)(n * n + 4 * n) * sizeof(double) + (size_t)n * sizeof(int); }

// Opt the kernels into the dynamic shared memory this network needs; called
// once per handle, outside any stream capture.
cudaError_t init_kernels(const DevNet &net) {
    size_t sr = rates_smem(net);
    const int n = net.ni;
    size_t sl = lu_fwd_smem(n);
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_rates<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sr))) return e;
    if ((e = cudaFuncSetAttribute(k_rates<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sr))) return e;
    if ((e = cudaFuncSetAttribute(k_lu_fwd_f64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sl))) return e;
    return cudaSuccess;
}

static size_t rates_smem(const DevNet &net) {
    int m = net.npair > net.nw ? net.npair : net.nw;
    return (size_t)(3 * net.ni + 8 + m + 2 * net.npair) * sizeof(double);
}

void launch_rates(const DevNet &net, const DevBatch &b, const double *y, double *f,
                  double *jv, double *dA, double *dB, double *dC, const double *k1,
                  const double *dt, const double *geo, int flags, bool with_jac, cudaStream_t s) {
    size_t sm = rates_smem(net);
    if (with_jac)
        k_rates<true><<<b.L, 128, sm, s>>>(net, b, y, f, jv, dA, dB, dC, k1, dt, geo, flags, 0);
    else
        k_rates<false><<<b.L, 128, sm, s>>>(net, b, y, f, jv, dA, dB, dC, k1, dt, geo, flags, 0);
}

void launch_chem_only(const DevNet &net, const DevBatch &b, const double *y, double *f,
                      const double *geo, cudaStream_t s) {
    size_t sm = rates_smem(net);
    k_rates<false><<<b.L, 128, sm, s>>>(net, b, y, f, nullptr, nullptr, nullptr, nullptr,
                                        nullptr, nullptr, geo, 0, 1);
}

void launch_lu_fwd_f64(const DevNet &net, const DevBatch &b, const Work &w,
                       const double *rhs, double *z, int flags, cudaStream_t s) {
    (void)flags;
    const int n = net.ni;
    size_t sm = lu_fwd_smem(n);
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    k_lu_fwd_f64<<<column_grid(b, VK_TUNE_LU64, 2), 256, sm, s>>>(net, b, w.jv, w.dA, w.dB, w.dC, w.dt, rhs, w.G, z,
                                                    w.status);
}

void launch_back_f64(const DevNet &net, const DevBatch &b, const double *G, const double *dB,
                     const double *z, double *x, const double *y, double *yk2, cudaStream_t s) {
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    k_back_f64<<<column_grid(b, VK_TUNE_SWEEP64, 2), 256, 2 * net.ni * sizeof(double), s>>>(net, b, G, dB, z, x, y, yk2);
}

void launch_solve_f64(const DevNet &net, const DevBatch &b, const double *G, const double *dB,
                      const double *dC, const double *rhs, double *zbuf, double *x,
                      cudaStream_t s) {
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    k_solve_f64<<<column_grid(b, VK_TUNE_SWEEP64, 2), 256, 2 * net.ni * sizeof(double), s>>>(net, b, G, dB, dC, rhs, zbuf, x);
}

void launch_stage(const DevNet &net, const DevBatch &b, const Work &w, int flags, double mtol,
                  double atol, cudaStream_t s) {
    k_stage<<<b.ncols, 256, 0, s>>>(net, b, w.y, w.ymix, w.k1, w.k2, w.yk2, w.sol, w.ymix_out,
                                    w.delta, w.status, flags, mtol, atol);
}

}  // namespace vk
