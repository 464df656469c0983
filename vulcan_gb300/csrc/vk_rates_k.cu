// Rate constants on the device for batches whose temperature varies by
// column (op.ReadRate.read_rate and rev_rate, op.py:63-309; the host
// restatement is network.Network.rate_constants).
//
//   forward  A T^B exp(-C/T)                       (two-body, k0-only three-body)
//            k0 / (1 + k0 M / k_inf)               (fall-off three-body)
//            the pressure-dependent OH + CH3 + M form (op.py:197-207)
//            photolysis / ionisation / condensation: the slot is left as uploaded
//            low-temperature caps (op.py:320-342), where set: at T <= T_max the
//            cap's Arrhenius or fall-off form replaces the forward rate
//   reverse  k_f / Keq,  Keq = exp(-(sum_p nu g_p - sum_r nu g_r)) (kB T / P0)^(n_r - n_p)
//            with g/RT from two-range NASA-9 polynomials switched at 1000 K
//            (chem_funs Gibbs / gibbs_sp), for pairs before '# reverse stops'.
//
// One CTA per layer: g/RT of every species into shared memory, then one
// thread per pair.  FP64 throughout (exp / pow / log of CUDA's math library).
#include <cuda_runtime.h>
#include <math.h>

#include <string>

#include "vk_internal.cuh"

namespace vk {

__device__ __forceinline__ double g_rt(double T, const double *a) {
    const double lnT = log(T);
    const double h = -a[0] / (T * T) + a[1] * lnT / T + a[2] + a[3] * T / 2. + a[4] * T * T / 3.
                     + a[5] * T * T * T / 4. + a[6] * T * T * T * T / 5. + a[8] / T;
    const double s = -a[0] / (T * T) / 2. - a[1] / T + a[2] * lnT + a[3] * T + a[4] * T * T / 2.
                     + a[5] * T * T * T / 3. + a[6] * T * T * T * T / 4. + a[9];
    return h - s;
}

__device__ __forceinline__ double arrhenius(double A, double B, double C, double T) {
    return A * pow(T, B) * exp(-C / T);
}

__device__ double special_oh_ch3(double T, double M) {
    const double k = 1.932E3 * pow(T, -9.88) * exp(-7544. / T) + 5.109E-11 * pow(T, -6.25) * exp(-1433. / T);
    const double kinf = 1.031E-10 * pow(T, -0.018) * exp(16.74 / T);
    const double Fc = 0.1855 * exp(-T / 155.8) + 0.8145 * exp(-T / 1675.) + exp(-4531. / T);
    const double nn = 0.75 - 1.27 * log(Fc);
    const double x = log(k * M / kinf) / nn;
    const double ff = exp(log(Fc) / (1. + x * x));
    return k / (1 + k * M / kinf) * ff;
}

__global__ void __launch_bounds__(128)
k_rate_consts(DevNet net, DevBatch b, const int *__restrict__ kind, const int *__restrict__ rev,
              const int *__restrict__ cap_kind, const double *__restrict__ cap_T,
              const double *__restrict__ cap_params, const double *__restrict__ params,
              const double *__restrict__ nasa9, double *k) {
    extern __shared__ double gs[];                       // [ni] g/RT of this layer
    const int l = blockIdx.x;
    if (b.lay_col[l] < 0) return;                        // gap layer of a slot
    const double *al = b.atm + (size_t)l * VK_ATM_NF;
    const double T = al[VK_ATM_TCO], M = al[VK_ATM_M];
    for (int s = threadIdx.x; s < net.ni; s += blockDim.x)
        gs[s] = g_rt(T, nasa9 + (size_t)s * 20 + (T < 1000. ? 0 : 10));
    __syncthreads();
    double *kl = k + (size_t)l * net.nr;
    for (int p = threadIdx.x; p < net.npair; p += blockDim.x) {
        const double *pp = params + (size_t)p * 6;
        double kf;
        switch (kind[p]) {
        case VK_K_ARRHENIUS: kf = arrhenius(pp[0], pp[1], pp[2], T); break;
        case VK_K_FALLOFF: {
            const double k0 = arrhenius(pp[0], pp[1], pp[2], T);
            const double kinf = arrhenius(pp[3], pp[4], pp[5], T);
            kf = k0 / (1 + k0 * M / kinf);
            break;
        }
        case VK_K_SPECIAL_OH_CH3: kf = special_oh_ch3(T, M); break;
        default: kf = kl[2 * p];                         // photolysis etc.: as uploaded
        }
        if (cap_kind && cap_kind[p] != VK_K_NONE && T <= cap_T[p]) {
            const double *cp = cap_params + (size_t)p * 6;
            double c = arrhenius(cp[0], cp[1], cp[2], T);
            if (cap_kind[p] == VK_K_FALLOFF) {
                const double cinf = arrhenius(cp[3], cp[4], cp[5], T);
                c = c / (1. + c * M / cinf);
            }
            kf = c;
        }
        kl[2 * p] = kf;
        if (rev[p]) {
            const PairDesc *pd = net.pairs + p;
            double dg = 0.0;
            int nr_ = 0, np_ = 0;
            for (int t = 0; t < pd->nf; ++t) { dg -= pd->fnu[t] * gs[pd->fsp[t]]; nr_ += pd->fnu[t]; }
            for (int t = 0; t < pd->nr; ++t) { dg += pd->rnu[t] * gs[pd->rsp[t]]; np_ += pd->rnu[t]; }
            double kq = exp(-dg);
            if (np_ != nr_) kq *= pow(VK_CORR * T, (double)(nr_ - np_));
            kl[2 * p + 1] = kf / kq;
        } else {
            kl[2 * p + 1] = 0.0;
        }
    }
}

void launch_rate_consts(const DevNet &net, const DevBatch &b, const int *kind, const int *rev,
                        const int *cap_kind, const double *cap_T, const double *cap_params,
                        const double *params, const double *nasa9, double *k, cudaStream_t s) {
    k_rate_consts<<<b.L, 128, net.ni * sizeof(double), s>>>(net, b, kind, rev, cap_kind, cap_T,
                                                            cap_params, params, nasa9, k);
}

}  // namespace vk
