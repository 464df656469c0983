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
// in the order the sweeps visit them: forward 0..nz-1, back nz-2..0.  A
// visit is FP32 only -- the product with G~_j, whose row r also yields row r
// of the next visit's input (one fma with the precomputed scaled coupling),
// so a visit costs one block barrier; everything in FP64 (the couplings, the
// scaled residual, x += S x~ and the correction size of the convergence
// test, the residual b - A x) runs in parallel passes over the whole column
// between the sweeps, off the chain of dependent visits.
// yscale (may be NULL) widens the convergence floor: k1/k2 enter sol next to y.
__global__ void __launch_bounds__(256)
k_refine(DevNet net, DevBatch b, const float *__restrict__ G32, const double *__restrict__ rsc,
         const double *__restrict__ csc, const double *__restrict__ jv,
         const double *__restrict__ dA, const double *__restrict__ dB,
         const double *__restrict__ dC, const double *__restrict__ dt,
         const double *__restrict__ rhs, double *__restrict__ x, double *__restrict__ res,
         float *__restrict__ zf, float *__restrict__ wcf, float *__restrict__ wcb,
         float *__restrict__ raf, float *__restrict__ xf,
         const double *__restrict__ yscale, double *__restrict__ yk2,
         const double *__restrict__ y, int max_sweeps, double tol, int *__restrict__ fallback,
         int *__restrict__ sweeps_out, int *__restrict__ status, double *__restrict__ err_out,
         double *__restrict__ thr64, int *act32, int *__restrict__ failed) {
    extern __shared__ __align__(16) unsigned char smr[];
    const int n = net.ni, NNP = block_stride32(n);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smr);           // [2]
    float *Gbuf = reinterpret_cast<float *>(smr + 16);           // [2][NNP]
    float *vin = Gbuf + 2 * NNP;                                 // [2][n] visit inputs
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
        // x = 0, r = b; the scaled couplings of the sweeps (FP32: they feed
        // the FP32 preconditioner) and the scaled first residual.  The
        // column-wide passes are unrolled so several elements' global loads
        // are in flight per thread.
#pragma unroll 4
        for (int e = tid; e < nz * n; e += nth) {
            const size_t g = base + e;
            const int j = e / n;
            x[g] = 0.0;
            res[g] = rhs[g];
            raf[g] = (float)(rsc[g] * rhs[g]);
            wcf[g] = j > 0 ? (float)(rsc[g] * dC[g] * csc[g - n]) : 0.f;
            wcb[g] = j < nz - 1 ? (float)(rsc[g] * dB[g] * csc[g + n]) : 0.f;
        }
        __syncthreads();
        issue(0);
        int sweep = 0, converged = 0, timed_out = 0;
        double m_prev = INFINITY;
        // per-row vectors of a visit (the row's coupling, scaled residual and
        // forward result), loaded into registers one visit ahead
        struct Visit { float w, ra, zf; };
        const bool rowt = mrow < n;          // this thread works on row mrow
        auto fetch = [&](int v) {
            Visit q{0.f, 0.f, 0.f};
            const size_t e = ((size_t)l0 + layer_of(v)) * n + mrow;
            if (rowt) {
                if (v < nz) { q.w = wcf[e]; q.ra = raf[e]; }
                else { q.w = wcb[e]; q.zf = zf[e]; }
            }
            return q;
        };
        int p = 0;                           // vin buffer of the current visit
        for (; sweep < max_sweeps && !converged && !timed_out; ++sweep) {
            Visit cur = fetch(0);
            if (rowt && mhalf == 0) vin[p * n + mrow] = cur.ra;     // layer 0: z~_0 = G~_0 R_0 r_0
            for (int v = 0; v < per_sweep; ++v) {
                const int j = layer_of(v);
                const size_t l = (size_t)l0 + j;
                const bool fwd = v < nz;
                Visit nxt = cur;
                if (v + 1 < per_sweep) nxt = fetch(v + 1);
                const int buf = consumed & 1;
                const bool ok = mbar_wait(&bar[buf], (consumed >> 1) & 1);
                ++consumed;
                // one block barrier per visit: the block has landed and every
                // row's input (written by its row thread last visit) is visible
                if (__syncthreads_or(!ok)) {
                    --consumed;                  // still in flight: drained below
                    timed_out = 1;
                    break;
                }
                // prefetch the next visit (possibly the first of the next sweep)
                if (v + 1 < per_sweep) issue(v + 1);
                else if (sweep + 1 < max_sweeps) issue(0);
                const float *G = Gbuf + buf * NNP;
                const float *xin = vin + p * n;
                // matvec: tpr adjacent lanes per row, interleaved columns
                float sacc = 0.0f;
                if (rowt) {
                    float s0 = 0.0f, s1 = 0.0f;
                    const float *row = G + mrow * n;
                    int q = mhalf;
                    for (; q + tpr < n; q += 2 * tpr) {
                        s0 = fmaf(row[q], xin[q], s0);
                        s1 = fmaf(row[q + tpr], xin[q + tpr], s1);
                    }
                    if (q < n) s0 = fmaf(row[q], xin[q], s0);
                    sacc = s0 + s1;
                }
                if (tpr == 2) sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
                if (rowt && mhalf == 0) {
                    if (fwd) zf[l * n + mrow] = sacc;
                    else sacc += cur.zf;
                    // the back sweep's result (it starts at the top layer:
                    // x~_{nz-1} = z~_{nz-1}), applied to x after the sweep
                    if (!fwd || j == nz - 1) xf[l * n + mrow] = sacc;
                    // the next visit's input row: a coupling times this row's
                    // result (+ the scaled residual going forward)
                    if (v + 1 < per_sweep)
                        vin[(p ^ 1) * n + mrow] = (v + 1 < nz) ? fmaf(nxt.w, sacc, nxt.ra) : nxt.w * sacc;
                }
                p ^= 1;
                cur = nxt;
            }
            if (timed_out) break;
            __syncthreads();                     // the last visit's results are visible
            // x += S x~ and the largest |d| / (|x| + |yscale| + 1e-10 n_0) of
            // the sweep, kept as a fraction (num, den) compared by
            // cross-multiplication and divided once per thread (FP64 divisions
            // are long FP64-pipe sequences on this chip)
            double dnum = 0.0, dden = 1.0;
#pragma unroll 4
            for (int e = tid; e < nz * n; e += nth) {
                const size_t g = base + e;
                const double d = csc[g] * (double)xf[g];
                const double xn = x[g] + d;
                x[g] = xn;
                const double n0 = b.atm[(size_t)(l0 + e / n) * VK_ATM_NF + VK_ATM_N0];
                const double sc = fabs(xn) + (yscale ? fabs(yscale[g]) : 0.0) + 1e-10 * n0;
                const double ad = fabs(d);
                if (!isfinite(d)) { dnum = INFINITY; dden = 1.0; }
                else if (ad * dden > dnum * sc) { dnum = ad; dden = sc; }
            }
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
            // residual r = b - A x  (FP64, matrix-free; every (layer, species)
            // at once) and its scaled FP32 copy for the next sweep
#pragma unroll 2
            for (int q = tid; q < nz * n; q += nth) {
                const int j = q / n, sp = q - j * n;
                const size_t l = (size_t)l0 + j;
                const size_t e = base + q;
                const double *jl = jv + l * net.nnz;
                double ax = (c0 - dA[e]) * x[e];
                for (int k = net.jrowptr[sp]; k < net.jrowptr[sp + 1]; ++k) ax += jl[k] * x[l * n + net.jcol[k]];
                if (j > 0) ax -= dC[e] * x[e - n];
                if (j < nz - 1) ax -= dB[e] * x[e + n];
                const double r = rhs[e] - ax;
                res[e] = r;
                raf[e] = (float)(rsc[e] * r);
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

__global__ void k_reset_route(int ncols, double *__restrict__ thr64, double route_dt0) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncols) thr64[c] = route_dt0;
}

void launch_route(const DevBatch &b, const Work &w, cudaStream_t s) {
    k_route<<<(b.ncols + 127) / 128, 128, 0, s>>>(b, w.dt, w.thr64, w.fallback, w.act32, w.routed,
                                                   w.failed);
}

void launch_reset_route(const Work &w, int ncols, double route_dt0, cudaStream_t s) {
    if (w.thr64) k_reset_route<<<(ncols + 127) / 128, 128, 0, s>>>(ncols, w.thr64, route_dt0);
}

cudaError_t init_mixed_kernels(int n) {
    size_t sm = 16 + (size_t)2 * block_stride32(n) * sizeof(float) + 2 * n * sizeof(float);
    return raise_smem_limit(k_refine, (int)sm);
}

void launch_refine(const DevNet &net, const DevBatch &b, const Work &w, const double *rhs,
                   double *x, const double *yscale, double *yk2, int max_sweeps, double tol,
                   cudaStream_t s) {
    const int n = net.ni;
    size_t sm = 16 + (size_t)2 * block_stride32(n) * sizeof(float) + 2 * n * sizeof(float);
    cudaMemsetAsync(b.queue, 0, sizeof(unsigned), s);
    k_refine<<<column_grid(b, VK_TUNE_REFINE, 3), 256, sm, s>>>(net, b, w.G32, w.rs, w.cs, w.jv, w.dA, w.dB, w.dC, w.dt,
                                      rhs, x, w.r, w.zf, w.wcf, w.wcb, w.raf, w.xf, yscale, yk2, w.y,
                                      max_sweeps, tol,
                                      w.fallback, w.sweeps, w.status, w.refine_err, w.thr64,
                                      w.act32, w.failed);
}

}  // namespace vk
