// Photochemistry radiative transfer on the device: optical depth, two-stream
// actinic flux and photolysis rates for every column of a batch.
//
// Restates op.ODESolver.compute_tau (op.py:2580-2599), compute_flux
// (op.py:2603-2739, isotropic scattering, ag0 = 0 in phy_const.py) and
// compute_J (op.py:2751-2786) on the binned cross sections the host set-up
// provides (make_bins_read_cross, read_sflux).  The T-dependent branches of
// compute_tau (op.py:2591-2592) and compute_J (op.py:2770-2774) read
// per-layer tables where vk_photo_set_cross_T gave them.
//
//   k_photo_flux  one thread per (column, wavelength bin): tau from the top,
//                 single-scattering albedo, the downward then upward sweeps of
//                 the diffuse fluxes (the downward sweep reads the previous
//                 call's upward flux, as the reference's arrays persist), and
//                 the actinic flux of every layer.  Staggered arrays (nz+1
//                 interfaces) of column c start at row col_off[c] + c.
//   k_photo_J     one CTA per layer: J of every channel = sum over bins of
//                 actinic flux x (cross_J x bin weight), written times
//                 f_diurnal into the channel's k slot; the column's largest
//                 relative actinic-flux change (aflux_change) by atomicMax on
//                 the bit pattern (non-negative doubles order like integers).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "vk_internal.cuh"

namespace vk {

constexpr double kHC = 1.98644582E-9;        // erg nm (phy_const.py)

__global__ void __launch_bounds__(128)
k_photo_flux(DevNet net, DevBatch b, PhotoDev ph, const double *__restrict__ y,
             const double *__restrict__ ymix) {
    const int c = blockIdx.y;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= b.ncols || n >= ph.nbins) return;
    if (b.active && !b.active[c]) return;
    const int ni = net.ni;
    const int l0 = b.col_off[c], nz = b.col_end[c] - l0;
    const size_t s0 = (size_t)(l0 + c);                      // staggered rows of this column
    const int NB = ph.nbins;
    const double cosz = cos(ph.sl_angle);
    const double mu = -cosz;
    const double edd = ph.edd;
    const double ftop = ph.sflux_top[n];
    // tau from the top; w0 per layer
    double tau_up = 0.0;
    ph.tau[(s0 + nz) * NB + n] = 0.0;
    for (int j = nz - 1; j >= 0; --j) {
        const size_t l = (size_t)l0 + j;
        const double dz = b.atm[l * VK_ATM_NF + VK_ATM_DZ];
        double t = 0.0, tabs = 0.0, tsc = 0.0;
        for (int a = 0; a < ph.nabs; ++a) {
            const double cr = ph.cross[(size_t)a * NB + n];
            const int s = ph.abs_sp[a];
            const int ts = ph.abs_tslot ? ph.abs_tslot[a] : -1;
            const double crt = ts < 0 ? cr : ph.cross_T[((size_t)ts * ph.lstride + l) * NB + n];
            t += y[l * ni + s] * dz * crt;
            if (ph.abs_photo[a]) tabs += ymix[l * ni + s] * cr;
        }
        for (int a = 0; a < ph.nscat; ++a) {
            const double cr = ph.cross_scat[(size_t)a * NB + n];
            const int s = ph.scat_sp[a];
            t += y[l * ni + s] * dz * cr;
            tsc += ymix[l * ni + s] * cr;
        }
        tau_up += t;
        ph.tau[(s0 + j) * NB + n] = tau_up;
        // numpy's nan_to_num, then the cap below 1 (pure scatterers)
        double w0 = tsc / (tabs + tsc);
        if (isnan(w0)) w0 = 0.0;
        else if (isinf(w0)) w0 = w0 > 0 ? DBL_MAX : -DBL_MAX;
        ph.w0[l * NB + n] = fmin(w0, 1. - 1.E-8);
    }
    // layer coefficients (recomputed in each sweep from tau and w0)
    auto coef = [&](int j, double &chi, double &xi, double &phi, double &iu, double &id) {
        const size_t l = (size_t)l0 + j;
        const double w0 = ph.w0[l * NB + n];
        const double tj = ph.tau[(s0 + j) * NB + n], tj1 = ph.tau[(s0 + j + 1) * NB + n];
        const double dtau = tj - tj1;
        const double sq = sqrt(1. - w0);
        const double tran = exp(-1. / edd * sq * dtau);
        const double zp = 0.5 * (1. + sq), zm = 0.5 * (1. - sq);
        const double ll = -1. * w0 / (1. / (mu * mu) - 1. / (edd * edd) * (1. - w0));
        const double gp = 0.5 * (ll * (1. / edd + 1. / mu));
        const double gm = 0.5 * (ll * (1. / edd - 1. / mu));
        chi = zm * zm * tran * tran - zp * zp;
        xi = zp * zm * (1. - tran * tran);
        phi = (zm * zm - zp * zp) * tran;
        const double dlo = ftop * exp(-1. * tj / cosz) * cosz;     // direct flux, lower interface
        const double dhi = ftop * exp(-1. * tj1 / cosz) * cosz;    // upper interface
        iu = phi * gp * dlo - (xi * gm + chi * gp) * dhi;
        id = phi * gm * dhi - (chi * gm + xi * gp) * dlo;
    };
    double *Du = ph.dflux_u, *Dd = ph.dflux_d;
    for (int j = nz - 1; j >= 0; --j) {
        double chi, xi, phi, iu, id;
        coef(j, chi, xi, phi, iu, id);
        Dd[(s0 + j) * NB + n] = 1. / chi * (phi * Dd[(s0 + j + 1) * NB + n] - xi * Du[(s0 + j) * NB + n] + id / mu);
    }
    for (int j = 1; j <= nz; ++j) {
        double chi, xi, phi, iu, id;
        coef(j - 1, chi, xi, phi, iu, id);
        Du[(s0 + j) * NB + n] = 1. / chi * (phi * Du[(s0 + j - 1) * NB + n] - xi * Dd[(s0 + j) * NB + n] + iu / mu);
    }
    const double e = kHC / ph.bins[n];
    for (int j = 0; j < nz; ++j) {
        const size_t l = (size_t)l0 + j;
        const double slo = ftop * exp(-1. * ph.tau[(s0 + j) * NB + n] / cosz);
        const double shi = ftop * exp(-1. * ph.tau[(s0 + j + 1) * NB + n] / cosz);
        const double ave = 0.5 * (slo + shi);
        const double tot = ave + 0.5 * (Du[(s0 + j) * NB + n] + Du[(s0 + j + 1) * NB + n]
                                        + Dd[(s0 + j + 1) * NB + n] + Dd[(s0 + j) * NB + n]) / edd;
        ph.aflux_prev[l * NB + n] = ph.aflux[l * NB + n];
        ph.aflux[l * NB + n] = tot / e;
    }
}

__global__ void __launch_bounds__(256)
k_photo_J(DevNet net, DevBatch b, PhotoDev ph, double *k, unsigned long long *change) {
    __shared__ double red[8];
    const int l = blockIdx.x;
    const int c = b.lay_col[l];
    if (c < 0 || (b.active && !b.active[c])) return;
    const int NB = ph.nbins;
    const double *af = ph.aflux + (size_t)l * NB;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarp = blockDim.x >> 5;
    for (int ch = 0; ch < ph.nch; ++ch) {
        const int ts = ph.ch_tslot ? ph.ch_tslot[ch] : -1;
        const double *wj = ts < 0 ? ph.wcross_J + (size_t)ch * NB
                                  : ph.wcross_J_T + ((size_t)ts * ph.lstride + l) * NB;
        double s = 0.0;
        for (int n = tid; n < NB; n += blockDim.x) s += af[n] * wj[n];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[warp] = s;
        __syncthreads();
        if (tid == 0) {
            double J = 0.0;
            for (int w = 0; w < nwarp; ++w) J += red[w];
            ph.J[(size_t)l * ph.nch + ch] = J;
            k[(size_t)l * net.nr + ph.ch_kindex[ch] - 1] = J * ph.f_diurnal;
        }
        __syncthreads();
    }
    // relative change of the actinic flux where it exceeds flux_atol
    double m = 0.0;
    const double *ap = ph.aflux_prev + (size_t)l * NB;
    for (int n = tid; n < NB; n += blockDim.x)
        if (af[n] > ph.flux_atol) m = fmax(m, fabs(af[n] - ap[n]) / af[n]);
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m > 0.0) atomicMax(change + c, (unsigned long long)__double_as_longlong(m));
}

// zero the change of the columns this update covers
__global__ void k_photo_clear(DevBatch b, unsigned long long *change) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < b.ncols && (!b.active || b.active[c])) change[c] = 0ull;
}

void launch_photo_clear(const DevBatch &b, unsigned long long *change, cudaStream_t s) {
    k_photo_clear<<<(b.ncols + 127) / 128, 128, 0, s>>>(b, change);
}

void launch_photo(const DevNet &net, const DevBatch &b, const PhotoDev &ph, const double *y,
                  const double *ymix, double *k, unsigned long long *change, cudaStream_t s) {
    dim3 g1((ph.nbins + 127) / 128, b.ncols);
    k_photo_flux<<<g1, 128, 0, s>>>(net, b, ph, y, ymix);
    k_photo_J<<<b.L, 256, 0, s>>>(net, b, ph, k, change);
}

}  // namespace vk
