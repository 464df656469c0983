// Mixed-precision block-tridiagonal solve: FP32 factorisation on scaled
// blocks, FP64 residual and iterative refinement.
//
// The system is the Ros2 LHS  A = c0 I - J_chem - J_diff  (op.py:1973-2042):
// dense diagonal blocks D_j = c0 I + (-J_j) - diag(dA_j) and diagonal couplings
// L_j = -diag(dC_j) (to layer j-1), U_j = -diag(dB_j) (to layer j+1).
//
// The factorisation (vk_lureg.cu: k_prep32 + k_lu32) works on the scaled
// system R A S, with per-layer power-of-two row scales R_j (row maxima of D_j)
// and column scales S_j (column maxima of R_j D_j), so the scaling itself is
// exact; each Schur-complemented scaled block
//     D~'_j = R_j D_j S_j - L~_j G~_{j-1} U~_{j-1}
// is inverted in FP32 and G~_j is stored in FP32 (half the bytes of FP64).
//
// k_refine (one column at a time per CTA) solves A x = b: x = 0, r = b; repeat
// { d = S M~^-1 R r  (FP32 forward/back sweeps with G~);  x += d (FP64);
//   r = b - A x  (FP64, matrix-free from the sparse -J and dA/dB/dC) }
// until max |d| / (|x| + |yscale| + 1e-10 n_0) <= tol or max sweeps; a
// column that does not converge is flagged for the FP64 path.
//
// Routing.  At large dt the scaled diagonal blocks of a near-steady column
// reach condition numbers of 1e10..1e16 (c0 -> 0 exposes the conserved and
// slow chemical modes), beyond what FP32 factors can precondition: refinement
// diverges.  A column whose refinement failed at step size dt therefore sends
// every later attempt with a step >= dt/4 straight to the FP64 path (thr64),
// and tries the mixed path again only after its step has dropped below that:
// the margin keeps a rejected attempt (dt halved) and the step-size rule's
// 0.5x..2x changes from retrying a factorisation that has just failed.
#include <cuda_runtime.h>
#include <math.h>

#include "vk_internal.cuh"
#include "vk_tma.cuh"

namespace vk {

constexpr double kRouteMargin = 0.25;   // FP64 from dt >= kRouteMargin x the failed step


// Iterative refinement of A x = b with the FP32 factors (one column at a time
// per CTA, columns from the work queue).
// The inverse blocks G~_j stream into shared memory by TMA (double-buffered)
// in the order the sweeps visit them: forward 0..nz-1, back nz-2..0.
// yscale (may be NULL) widens the convergence floor: k1/k2 enter sol next to y.
__global__ void __launch_bounds__(256)
k_refine(DevNet net, DevBatch b, const float *__restrict__ G32, const double *__restrict__ rsc,
         const double *__restrict__ csc, const double *__restrict__ jv,
         const double *__restrict__ dA, const double *__restrict__ dB,
         const double *__restrict__ dC, const double *__restrict__ dt,
         const double *__restrict__ rhs, double *__restrict__ x, double *__restrict__ res,
         float *__restrict__ zf, const double *__restrict__ yscale, double *__restrict__ yk2,
         const double *__restrict__ y, int max_sweeps, double tol, int *__restrict__ fallback,
         int *__restrict__ sweeps_out, int *__restrict__ status, double *__restrict__ err_out,
         double *__restrict__ thr64, int *act32, int *__restrict__ failed) {
    extern __shared__ __align__(16) unsigned char smr[];
    const int n = net.ni, NNP = block_stride32(n);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smr);           // [2]
    float *Gbuf = reinterpret_cast<float *>(smr + 16);           // [2][NNP]
    float *vin = Gbuf + 2 * NNP;                                 // [n]
    float *vout = vin + n;                                       // [n]
    __shared__ double red[8];
    __shared__ int s_col;
    const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const int nwarp = nth >> 5;
    const uint32_t bytes = (uint32_t)NNP * sizeof(float);
    const int tpr = 2 * n <= nth ? 2 : 1;          // lanes per matvec row
    const int mrow = tid / tpr, mhalf = tid - mrow * tpr;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    // copies issued / consumed by this CTA over all its columns (the same
    // count in every thread; thread 0 issues): copy k lands in buffer k&1
    int issued = 0, consumed = 0;
    for (int c; (c = next_column(b, &s_col)) >= 0;) {
        if (b.active && !b.active[c]) continue;
        const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
        const double c0 = 1.0 / (R_ROS * dt[c]);
        const size_t base = (size_t)l0 * n;
        const int per_sweep = 2 * nz - 1;            // blocks visited per sweep
        // visit v (within a sweep) -> layer
        auto layer_of = [&](int v) { return v < nz ? v : 2 * nz - 2 - v; };
        auto issue = [&](int v) {
            const int buf = issued & 1;
            if (tid == 0)
                tma_load_1d(Gbuf + buf * NNP, G32 + ((size_t)l0 + layer_of(v)) * NNP, bytes, &bar[buf]);
            ++issued;
        };
        for (int e = tid; e < nz * n; e += nth) {
            x[base + e] = 0.0;
            res[base + e] = rhs[base + e];
        }
        __syncthreads();
        issue(0);
        int sweep = 0, converged = 0, timed_out = 0;
        double m_prev = INFINITY;
        // per-layer vectors of a visit, loaded into registers one visit ahead
        // (the sweeps are a chain of dependent visits: nothing else hides the
        // global-memory latency)
        struct Visit { double rsc, a, bc, cscn, csc, x, ys, n0; float zf; };
        auto fetch = [&](int v) {
            Visit q{0, 0, 0, 0, 0, 0, 0, 0, 0.f};
            const int j = layer_of(v);
            const size_t l = (size_t)l0 + j;
            const bool fwd = v < nz;
            if (tid < n) {
                const size_t e = l * n + tid;
                q.rsc = rsc[e];
                if (fwd) {
                    q.a = res[e];
                    if (j > 0) { q.bc = dC[e]; q.cscn = csc[e - n]; }
                } else {
                    q.bc = dB[e];
                    q.cscn = csc[e + n];
                }
                if (!fwd || j == nz - 1) {
                    q.csc = csc[e];
                    q.x = x[e];
                    q.ys = yscale ? fabs(yscale[e]) : 0.0;
                    q.n0 = b.atm[l * VK_ATM_NF + VK_ATM_N0];
                }
            }
            if (!fwd && mrow < n && mhalf == 0) q.zf = zf[l * n + mrow];
            return q;
        };
        for (; sweep < max_sweeps && !converged && !timed_out; ++sweep) {
            // largest |d| / sc of the sweep as a fraction (num, den): compared by
            // cross-multiplication, divided once per thread after the sweep
            // (FP64 divisions are long FP64-pipe sequences on this chip)
            double dnum = 0.0, dden = 1.0;
            Visit cur = fetch(0);
            for (int v = 0; v < per_sweep; ++v) {
                const int j = layer_of(v);
                const size_t l = (size_t)l0 + j;
                const bool fwd = v < nz;
                Visit nxt = cur;
                if (v + 1 < per_sweep) nxt = fetch(v + 1);
                // right-hand side of this visit
                if (tid < n) {
                    double vi;
                    if (fwd) {
                        vi = cur.rsc * cur.a;
                        if (j > 0) vi += cur.rsc * cur.bc * cur.cscn * (double)vout[tid];
                    } else {
                        vi = cur.rsc * cur.bc * cur.cscn * (double)vout[tid];
                    }
                    vin[tid] = (float)vi;
                }
                const int buf = consumed & 1;
                const bool ok = mbar_wait(&bar[buf], (consumed >> 1) & 1);
                ++consumed;
                if (__syncthreads_or(!ok)) {
                    --consumed;                  // still in flight: drained below
                    timed_out = 1;
                    break;
                }
                // prefetch the next visit (possibly the first of the next sweep)
                if (v + 1 < per_sweep) issue(v + 1);
                else if (sweep + 1 < max_sweeps) issue(0);
                const float *G = Gbuf + buf * NNP;
                // matvec: tpr adjacent lanes per row, interleaved columns
                float sacc = 0.0f;
                if (mrow < n) {
                    float s0 = 0.0f, s1 = 0.0f;
                    const float *row = G + mrow * n;
                    int q = mhalf;
                    for (; q + tpr < n; q += 2 * tpr) {
                        s0 = fmaf(row[q], vin[q], s0);
                        s1 = fmaf(row[q + tpr], vin[q + tpr], s1);
                    }
                    if (q < n) s0 = fmaf(row[q], vin[q], s0);
                    sacc = s0 + s1;
                }
                if (tpr == 2) sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
                if (mrow < n && mhalf == 0) {
                    if (fwd) {
                        zf[l * n + mrow] = sacc;
                    } else {
                        sacc += cur.zf;
                    }
                    vout[mrow] = sacc;
                }
                __syncthreads();
                // the back sweep starts at the top layer: x~_{nz-1} = z~_{nz-1} (vout)
                if ((fwd && j == nz - 1) || !fwd) {
                    if (tid < n) {
                        const size_t e = l * n + tid;
                        const double d = cur.csc * (double)vout[tid];
                        const double xn = cur.x + d;
                        x[e] = xn;
                        const double sc = fabs(xn) + cur.ys + 1e-10 * cur.n0;
                        const double ad = fabs(d);
                        if (!isfinite(d)) { dnum = INFINITY; dden = 1.0; }
                        else if (ad * dden > dnum * sc) { dnum = ad; dden = sc; }
                    }
                }
                __syncthreads();
                cur = nxt;
            }
            if (timed_out) break;
            double dmax = dnum / dden;
            for (int o = 16; o; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
            if (lane == 0) red[warp] = dmax;
            __syncthreads();
            double m = red[0];
            for (int w = 1; w < nwarp; ++w) m = fmax(m, red[w]);
            __syncthreads();
            // converged; or stagnating at the FP64 residual's noise floor (the
            // correction stopped shrinking while already below 1e-6 of |x|+|y|)
            converged = (m <= tol) || (sweep >= 1 && m > 0.25 * m_prev && m <= 1e-6);
            if (!(m <= m_prev) && sweep >= 2) break;        // diverging: leave to the FP64 path
            m_prev = m;
            if (converged) break;
            // residual r = b - A x  (FP64, matrix-free; every (layer, species) at once)
            for (int q = tid; q < nz * n; q += nth) {
                const int j = q / n, sp = q - j * n;
                const size_t l = (size_t)l0 + j;
                const size_t e = base + q;
                const double *jl = jv + l * net.nnz;
                double ax = (c0 - dA[e]) * x[e];
                for (int k = net.jrowptr[sp]; k < net.jrowptr[sp + 1]; ++k) ax += jl[k] * x[l * n + net.jcol[k]];
                if (j > 0) ax -= dC[e] * x[e - n];
                if (j < nz - 1) ax -= dB[e] * x[e + n];
                res[e] = rhs[e] - ax;
            }
            __syncthreads();
        }
        // every issued copy lands before the column ends (bounded waits); a
        // copy that never lands ends this CTA's work with a timeout
        int lost = 0;
        while (consumed < issued) {
            lost |= !mbar_wait(&bar[consumed & 1], (consumed >> 1) & 1);
            ++consumed;
        }
        if (__syncthreads_or(lost)) timed_out = 1;
        if (tid == 0) {
            if (timed_out) status[c] = VK_ETIMEOUT;
            else {
                if (!converged) {
                    fallback[c] = 1;
                    act32[c] = 0;                   // later mixed launches of this attempt skip it
                    failed[c] = 1;                  // redone in FP64 after the routed columns
                    thr64[c] = fmin(thr64[c], kRouteMargin * dt[c]);
                }
                if (sweeps_out) atomicMax(sweeps_out, sweep + (converged ? 1 : 0));
                if (err_out) err_out[c] = fmax(err_out[c], m_prev);
            }
        }
        if (timed_out) return;
        __syncthreads();
        if (yk2) {
            for (int e = tid; e < nz * n; e += nth) yk2[base + e] = y[base + e] + x[base + e] / R_ROS;
        }
    }
}

// fallback[c] = 1: this attempt of column c is solved in FP64 (its step is at or
// above the size at which its refinement last failed); act32[c] = 1: mixed.
// Routing of one attempt: routed[c] = 1: solved in FP64 from the start (its
// step is at or above the size at which its refinement last failed, with the
// margin); act32[c] = 1: mixed; fallback[c] = every FP64 solve of the attempt
// (routed, and mixed columns whose refinement fails, which k_refine adds
// together with failed[c]).
__global__ void k_route(DevBatch b, const double *__restrict__ dt, const double *__restrict__ thr64,
                        int *__restrict__ fallback, int *__restrict__ act32, int *__restrict__ routed,
                        int *__restrict__ failed) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= b.ncols) return;
    const int a = b.active ? b.active[c] : 1;
    const int f64 = a && !(dt[c] < thr64[c]);
    fallback[c] = f64;
    routed[c] = f64;
    act32[c] = a && !f64;
    failed[c] = 0;
}

__global__ void k_reset_route(int ncols, double *__restrict__ thr64) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncols) thr64[c] = INFINITY;
}

void launch_route(const DevBatch &b, const Work &w, cudaStream_t s) {
    k_route<<<(b.ncols + 127) / 128, 128, 0, s>>>(b, w.dt, w.thr64, w.fallback, w.act32, w.routed,
                                                   w.failed);
}

void launch_reset_route(const Work &w, int ncols, cudaStream_t s) {
    if (w.thr64) k_reset_route<<<(ncols + 127) / 128, 128, 0, s>>>(ncols, w.thr64);
}

cudaError_t init_mixed_kernels(int n) {
    size_t sm = 16 + (size_t)2 * block_stride32(n) * sizeof(float) + 2 * n * sizeof(float);
    return cudaFuncSetAttribute(k_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
}

void launch_refine(const DevNet &net, const DevBatch &b, const Work &w, const double *rhs,
                   double *x, const double *yscale, double *yk2, int max_sweeps, double tol,
                   cudaStream_t s) {
    const int n = net.ni;
    size_t sm = 16 + (size_t)2 * block_stride32(n) * sizeof(float) + 2 * n * sizeof(float);
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    k_refine<<<column_grid(b, VK_TUNE_REFINE, 3), 256, sm, s>>>(net, b, w.G32, w.rs, w.cs, w.jv, w.dA, w.dB, w.dC, w.dt,
                                      rhs, x, w.r, w.zf, yscale, yk2, w.y, max_sweeps, tol,
                                      w.fallback, w.sweeps, w.status, w.refine_err, w.thr64,
                                      w.act32, w.failed);
}

}  // namespace vk
