// Device-side step control for a batch of columns (one CTA per column).
//
// After each Ros2 attempt k_control does what the reference's Python does on
// the host after Ros2.solver:
//   clip + loss            op.py:2447-2487  (ODESolver.clip / loss)
//   step_ok / step_reject  op.py:2489-2534  (reject: y <- y_prev, dt *= 0.5,
//                                            give up at dt_min)
//   update_mu_dz           op.py:944-984    (every update_frq steps, from ymix)
//   hydrostatic renorm     op.py:914        (y = n_0 * ymix)
//   save_step              op.py:1087-1105  (t += dt, count += 1, history)
//   step_size              op.py:3105-3125
//   stop / conv            op.py:1018-1085  (checked before the next step)
// and backs up y for the next step.  Every column advances independently; a
// column whose step was accepted starts its next step in the next attempt.
#include <cuda_runtime.h>
#include <math.h>

#include "vk_internal.cuh"
#include "vk_control.cuh"
#include "vk_geo.cuh"

namespace vk {

constexpr double KB_ = 1.38064852E-16;
constexpr double NAVO_ = 6.02214086E+23;

__device__ __forceinline__ double block_sum(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double block_max(double v, double *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = red[0];
    for (int w = 1; w < nw; ++w) s = fmax(s, red[w]);
    __syncthreads();
    return s;
}

__device__ __forceinline__ int block_or(int v, int *redi) {
    v = __any_sync(0xffffffffu, v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) redi[threadIdx.x >> 5] = v;
    __syncthreads();
    int s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s |= redi[w];
    __syncthreads();
    return s;
}

// Element totals sum_i compo[i,a] sum_z y[z,i] of one column into out[natom].
__device__ void atom_totals(const DevNet &net, const double *y, int l0, int nz, double *out,
                            double *red) {
    const int n = net.ni;
    for (int a = 0; a < net.natom; ++a) {
        double s = 0.0;
        for (int e = threadIdx.x; e < nz * n; e += blockDim.x) {
            int i = e % n;
            s += net.compo[i * net.natom + a] * y[(size_t)l0 * n + e];
        }
        s = block_sum(s, red);
        if (threadIdx.x == 0) out[a] = s;
    }
}

// Steady-state test (Integration.conv) on the current state; thread 0 result.
__device__ int conv_test(const DevNet &net, const DevBatch &b, const RunState &rs,
                         const RunCtrl &cc, int c, int l0, int nz, double *red) {
    const int n = net.ni;
    const int R = cc.conv_step;
    const int count = rs.count[c];
    const double t = rs.t[c];
    // slope_min = clip(min(Kzz / (0.1 Hp)^2), 1e-10, 1e-8)
    double smin = 1e300;
    for (int j = threadIdx.x; j < nz - 1; j += blockDim.x) {
        double K = b.atm[(size_t)(l0 + j) * VK_ATM_NF + VK_ATM_KZZ];
        double H = b.atm[(size_t)(l0 + j) * VK_ATM_NF + VK_ATM_HP];
        smin = fmin(smin, K / ((0.1 * H) * (0.1 * H)));
    }
    smin = -block_max(-smin, red);
    double slope_min = fmax(fmin(smin, 1.e-8), 1.e-10);
    // history index closest to t * st_factor (first minimum), within the ring
    __shared__ int s_indx;
    if (threadIdx.x == 0) {
        const double target = t * cc.st_factor;
        const int lo = count - R > 0 ? count - R : 0;
        int best = lo;
        double bd = fabs(rs.hist_t[(size_t)c * R + (lo % R)] - target);
        for (int i = lo + 1; i < count; ++i) {
            double d = fabs(rs.hist_t[(size_t)c * R + (i % R)] - target);
            if (d < bd) { bd = d; best = i; }
        }
        if (best == count - 1) best -= 1;
        if (best < count - R) best = count - R;
        s_indx = best;
    }
    __syncthreads();
    const int indx = s_indx;
    const double *ynow = rs.hist_y + ((size_t)((count - 1) % R) * b.L) * n;
    const double *yref = rs.hist_y + ((size_t)(indx % R) * b.L) * n;
    double ld = 0.0;
    for (int e = threadIdx.x; e < nz * n; e += blockDim.x) {
        const size_t g = (size_t)l0 * n + e;
        const int i = e % n, j = e / n;
        const double ym = rs.ymix[g];
        const double yv = rs.y[g];
        if (!(ym > 0.0)) continue;
        if (ym < cc.mtol_conv || yv < cc.atol || rs.ignore[(size_t)c * n + i]) continue;
        const double n0 = b.atm[(size_t)(l0 + j) * VK_ATM_NF + VK_ATM_N0];
        ld = fmax(ld, fabs((ynow[g] - yref[g]) / n0) / ym);
    }
    double longdy = block_max(ld, red);
    int ok = 0;
    if (threadIdx.x == 0) {
        double dtt = rs.hist_t[(size_t)c * R + ((count - 1) % R)] - rs.hist_t[(size_t)c * R + (indx % R)];
        double longdydt = longdy / dtt;
        rs.longdy[c] = longdy;
        rs.longdydt[c] = longdydt;
        ok = ((longdy < cc.yconv_cri && longdydt < cc.slope_cri) ||
              (longdy < cc.yconv_min && longdydt < slope_min)) &&
             rs.aflux_change[c] < cc.flux_cri;
    }
    return ok;
}

// Check stop conditions and back up the state at the start of a step.
__device__ void start_step(const DevNet &net, const DevBatch &b, const RunState &rs,
                           const RunCtrl &cc, int c, int l0, int nz, double *red) {
    __shared__ int s_stop;
    if (threadIdx.x == 0) s_stop = 0;
    __syncthreads();
    const double t = rs.t[c];
    const int count = rs.count[c];
    int conv = 0;
    if (t > cc.trun_min && count > cc.count_min && count >= 2) conv = conv_test(net, b, rs, cc, c, l0, nz, red);
    if (threadIdx.x == 0) {
        int end = 0;
        if (conv) end = 1;
        else if (t > cc.runtime) end = 2;
        else if (count > cc.count_max) end = 3;
        if (end) { rs.end_case[c] = end; s_stop = 1; }
        else if (rs.steps_call[c] >= cc.max_steps) s_stop = 1;
        rs.active[c] = s_stop ? 0 : 1;
        rs.natt[c] = 0;
        for (int a = 0; a < net.natom; ++a) rs.loss_prev[c * VK_MAX_NATOM + a] = rs.loss[c * VK_MAX_NATOM + a];
    }
    __syncthreads();
    if (s_stop) return;
    const int n = net.ni;
    for (int e = threadIdx.x; e < nz * n; e += blockDim.x) {
        size_t g = (size_t)l0 * n + e;
        rs.y_prev[g] = rs.y[g];
    }
}

__global__ void __launch_bounds__(256) k_start(DevNet net, DevBatch b, RunState rs, RunCtrl cc) {
    __shared__ double red[8];
    const int c = blockIdx.x;
    if (rs.end_case[c] != 0) { if (threadIdx.x == 0) rs.active[c] = 0; return; }
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    if (threadIdx.x == 0) rs.steps_call[c] = 0;
    __syncthreads();
    start_step(net, b, rs, cc, c, l0, nz, red);
}

// update_mu_dz for one column (thread 0 runs the height recurrence).
__device__ void update_mu_dz(const DevNet &net, const DevBatch &b, const RunState &rs,
                             const RunCtrl &cc, int c, int l0, int nz, double *mu) {
    const int n = net.ni;
    const double *ms = b.spf + (size_t)c * VK_SP_NF * n + VK_SP_MS * n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int j = warp; j < nz; j += nwarp) {
        // mean_mass accumulates species by species: mu += m_i * ymix_i
        if (lane == 0) {
            double s = 0.0;
            for (int i = 0; i < n; ++i) s += ms[i] * rs.ymix[(size_t)(l0 + j) * n + i];
            mu[j] = s;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double *atm = rs.atm;
        auto A = [&](int j, int f) -> double & { return atm[(size_t)(l0 + j) * VK_ATM_NF + f]; };
        const int pref = rs.pref[c];
        double zco = 0.0;          // zco[pref] = 0 (reference level)
        // upward from the reference level
        for (int i = pref; i < nz; ++i) {
            double g = (i == pref) ? cc.gs : cc.gs * (cc.Rp / (cc.Rp + zco)) * (cc.Rp / (cc.Rp + zco));
            double Hp = KB_ * A(i, VK_ATM_TCO) / (mu[i] / NAVO_ * g);
            double dz = Hp * log(A(i, VK_ATM_PICO) / A(i, VK_ATM_PICOU));
            A(i, VK_ATM_G) = g;
            A(i, VK_ATM_HP) = Hp;
            A(i, VK_ATM_DZ) = dz;
            zco += dz;
        }
        // downward below the reference level
        double zup = 0.0;
        for (int i = pref - 1; i >= 0; --i) {
            double g = cc.gs * (cc.Rp / (cc.Rp + zup)) * (cc.Rp / (cc.Rp + zup));
            double Hp = KB_ * A(i, VK_ATM_TCO) / (mu[i] / NAVO_ * g);
            double dz = Hp * log(A(i, VK_ATM_PICO) / A(i, VK_ATM_PICOU));
            A(i, VK_ATM_G) = g;
            A(i, VK_ATM_HP) = Hp;
            A(i, VK_ATM_DZ) = dz;
            zup -= dz;
        }
        for (int i = 0; i < nz - 1; ++i) {
            A(i, VK_ATM_DZI) = 0.5 * (A(i + 1, VK_ATM_DZ) + A(i, VK_ATM_DZ));
            if (cc.flags & VK_F_MOLDIFF) A(i, VK_ATM_HPI) = 0.5 * (A(i, VK_ATM_HP) + A(i + 1, VK_ATM_HP));
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(256) k_control(DevNet net, DevBatch b, RunState rs, RunCtrl cc,
                                                 const double *__restrict__ sol,
                                                 const double *__restrict__ ymix_sol,
                                                 const double *__restrict__ delta,
                                                 const int *__restrict__ status,
                                                 const int *__restrict__ fallback,
                                                 double *__restrict__ geo) {
    __shared__ double red[8];
    __shared__ int redi[8];
    __shared__ double loss[VK_MAX_NATOM];
    __shared__ double mu[1024];
    __shared__ int s_ok, s_giveup;
    const int c = blockIdx.x;
    if (!rs.active[c]) return;
    const int n = net.ni;
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    const size_t base = (size_t)l0 * n;
    const int NE = nz * n;
    // clip: zero values in [nega_cut, pos_cut); zero negatives where ymix < mtol
    int neg = 0, bad = 0;
    for (int e = threadIdx.x; e < NE; e += blockDim.x) {
        double v = sol[base + e];
        if (v < cc.pos_cut && v >= cc.nega_cut) v = 0.0;
        if (ymix_sol[base + e] < cc.mtol && v < 0.0) v = 0.0;
        if (!isfinite(v)) bad = 1;
        if (v < 0.0) neg = 1;
        rs.y[base + e] = v;
    }
    neg = block_or(neg, redi);
    bad = block_or(bad, redi) || !isfinite(delta[c]);
    __syncthreads();
    atom_totals(net, rs.y, l0, nz, loss, red);
    __syncthreads();
    // ymix of the clipped state
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int j = warp; j < nz; j += nwarp) {
        double s = 0.0;
        for (int i = lane; i < n; i += 32) s += rs.y[base + (size_t)j * n + i];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        for (int i = lane; i < n; i += 32) rs.ymix[base + (size_t)j * n + i] = rs.y[base + (size_t)j * n + i] / s;
    }
    if (threadIdx.x == 0) {
        double dl = 0.0;
        for (int a = 0; a < net.natom; ++a) {
            double ini = rs.atom_ini[c * VK_MAX_NATOM + a];
            double lo = (loss[a] - ini) / ini;
            rs.loss[c * VK_MAX_NATOM + a] = lo;
            dl = fmax(dl, fabs(lo - rs.loss_prev[c * VK_MAX_NATOM + a]));
        }
        const double d = delta[c];
        rs.delta[c] = d;
        rs.natt[c] += 1;
        rs.counters[c * VK_NCOUNTERS + 0] += 1;
        if (fallback && fallback[c]) rs.counters[c * VK_NCOUNTERS + 4] += 1;
        int ok = (!neg) && (dl < cc.loss_eps) && (d <= cc.rtol);
        int giveup = 0;
        if (bad || status[c] != 0) {
            rs.end_case[c] = bad ? -VK_ENAN : -status[c];
            rs.active[c] = 0;
            ok = 0;
        } else if (!ok) {
            if (d > cc.rtol) rs.counters[c * VK_NCOUNTERS + 1] += 1;
            else if (neg) rs.counters[c * VK_NCOUNTERS + 2] += 1;
            else rs.counters[c * VK_NCOUNTERS + 3] += 1;
            double dt = rs.dt[c] * cc.dt_var_min;
            if (dt < cc.dt_min) { dt = cc.dt_min; giveup = 1; }
            rs.dt[c] = dt;
            if (rs.natt[c] >= cc.max_attempts && !giveup) {
                rs.end_case[c] = -VK_EMAXATTEMPT;
                rs.active[c] = 0;
            }
        }
        s_ok = ok;
        s_giveup = giveup;
    }
    __syncthreads();
    if (!rs.active[c]) return;
    if (!s_ok) {
        // reject: y <- y_prev (ymix keeps the clipped failed attempt, as the
        // reference's var.ymix does); give up: also zero negatives and accept
        for (int e = threadIdx.x; e < NE; e += blockDim.x) {
            double v = rs.y_prev[base + e];
            if (s_giveup && v < 0.0) v = 0.0;
            rs.y[base + e] = v;
        }
        if (!s_giveup) return;
        __syncthreads();
    }
    // ---- accepted step: finalise (Integration loop body after one_step)
    const int count = rs.count[c];
    if (count % cc.update_frq == 0) {
        update_mu_dz(net, b, rs, cc, c, l0, nz, mu);
        // the transport geometry depends on g, dzi, Hpi: rebuild this column's
        const GeoCol gc = make_geocol(rs.atm, b.Dzz, b.spf, b.col_off, b.col_end, c, n);
        for (int e = threadIdx.x; e < NE; e += blockDim.x) {
            const int j = e / n, i = e - j * n;
            double out[GEO_NF];
            geo_coef(gc, j, i, cc.flags, out);
            double *gl = geo + (size_t)(l0 + j) * GEO_NF * n;
            for (int k = 0; k < GEO_NF; ++k) gl[k * n + i] = out[k];
        }
        __syncthreads();
    }
    const double dtv = rs.dt[c];
    const double tn = rs.t[c] + dtv;
    const int R = cc.conv_step;
    double *hy = rs.hist_y + ((size_t)(count % R) * b.L) * n;
    for (int e = threadIdx.x; e < NE; e += blockDim.x) {
        const int j = e / n;
        double v = b.atm[(size_t)(l0 + j) * VK_ATM_NF + VK_ATM_N0] * rs.ymix[base + e];
        rs.y[base + e] = v;
        hy[base + e] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        rs.hist_t[(size_t)c * R + (count % R)] = tn;
        rs.t[c] = tn;
        rs.count[c] = count + 1;
        rs.steps_call[c] += 1;
        rs.counters[c * VK_NCOUNTERS + 5] += 1;
        double d = rs.delta[c];
        if (d == 0) d = 0.01 * cc.rtol;
        double hf = 0.9 * sqrt(cc.rtol / d);
        hf = fmin(fmax(hf, cc.dt_var_min), cc.dt_var_max);
        double h = dtv * hf;
        h = fmin(fmax(h, cc.dt_min), cc.dt_max);
        rs.dt[c] = h;
    }
    __syncthreads();
    start_step(net, b, rs, cc, c, l0, nz, red);
}

__global__ void k_count_active(const int *active, int ncols, int *nactive) {
    __shared__ int s;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    int v = 0;
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) v += active[c];
    atomicAdd(&s, v);
    __syncthreads();
    if (threadIdx.x == 0) *nactive = s;
}

void launch_start(const DevNet &net, const DevBatch &b, const RunState &rs, const RunCtrl &cc,
                  cudaStream_t s) {
    k_start<<<b.ncols, 256, 0, s>>>(net, b, rs, cc);
}

void launch_control(const DevNet &net, const DevBatch &b, const RunState &rs, const RunCtrl &cc,
                    const double *sol, const double *ymix_sol, const double *delta,
                    const int *status, const int *fallback, double *geo, cudaStream_t s) {
    k_control<<<b.ncols, 256, 0, s>>>(net, b, rs, cc, sol, ymix_sol, delta, status, fallback, geo);
}

// A column's start of a run (vk_set_columns, vk_refill): clock, steady-state
// statistics (the reference starts longdy = longdydt = 1, store.Variables),
// counters, conservation losses, status, routing threshold, dt = 1e-10
// (vulcan_cfg.dttry).
__global__ void k_reset_columns(RunState rs, int n, const int *__restrict__ cols,
                                double *__restrict__ dt, int *__restrict__ status,
                                double *__restrict__ thr64, double route_dt0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cols[i];
    rs.t[c] = 0.0;
    rs.aflux_change[c] = 0.0;
    rs.longdy[c] = 1.0;
    rs.longdydt[c] = 1.0;
    rs.count[c] = 0;
    rs.end_case[c] = 0;
    for (int k = 0; k < VK_NCOUNTERS; ++k) rs.counters[(size_t)c * VK_NCOUNTERS + k] = 0;
    for (int a = 0; a < VK_MAX_NATOM; ++a) rs.loss[(size_t)c * VK_MAX_NATOM + a] = 0.0;
    dt[c] = 1e-10;
    status[c] = 0;
    if (thr64) thr64[c] = route_dt0;
}

void launch_reset_columns(const RunState &rs, int n, const int *cols, double *dt, int *status,
                          double *thr64, double route_dt0, cudaStream_t s) {
    k_reset_columns<<<(n + 127) / 128, 128, 0, s>>>(rs, n, cols, dt, status, thr64, route_dt0);
}

void launch_count_active(const int *active, int ncols, int *nactive, cudaStream_t s) {
    k_count_active<<<1, 256, 0, s>>>(active, ncols, nactive);
}

}  // namespace vk
