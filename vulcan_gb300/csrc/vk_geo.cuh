// Transport-operator geometry: the parts of the eddy + molecular diffusion
// coefficients that do not depend on the state (op.py:1496-1597 diffdf,
// op.py:1438-1494 diffdf_no_mol, op.py:1973-2166 lhs_jac_tot / no_mol).
//
// For species i in layer j the reference's operator is
//     dy_j/dt = A y_j + B y_{j+1} + C y_{j-1}      (eddy A,B,C + molecular Ai,Bi,Ci)
// and every term has the form  g * (ysum_a + ysum_b) / (2 ysum_c) + p  with a
// state-free factor g and offset p.  Per (layer, species) we store
//     gU  factor of the upper-interface flux   (K_{j+1/2} + D_{j+1/2,i}) / (dz_ave dzi_j)
//     gD  factor of the lower-interface flux   (K_{j-1/2} + D_{j-1/2,i}) / (dz_ave dzi_{j-1})
//     pA, pB, pC  advection and thermal/gravitational molecular terms
// so that, with q = ysum ratios,
//     cA = -gU (ys_{j+1}+ys_j)/(2 ys_j) - gD (ys_j+ys_{j-1})/(2 ys_j) + pA
//     cB =  gU (ys_{j+1}+ys_j)/(2 ys_{j+1}) + pB
//     cC =  gD (ys_j+ys_{j-1})/(2 ys_{j-1}) + pC.
// The divisions then happen once per atmosphere update instead of per RHS.
#pragma once
#include <cuda_runtime.h>

#include "vk_internal.cuh"

namespace vk {

constexpr double GEO_KB = 1.38064852E-16;
constexpr double GEO_NAVO = 6.02214086E+23;
constexpr int GEO_NF = 5;           // gU, gD, pA, pB, pC

struct GeoCol {
    const double *atm;   // [layer][VK_ATM_NF]
    const double *Dzz;   // [layer][ni]
    const double *ms, *alpha;
    int l0, nz, ni;
    __device__ double a(int j, int f) const { return atm[(size_t)(l0 + j) * VK_ATM_NF + f]; }
    __device__ double dzz(int j, int i) const { return Dzz[(size_t)(l0 + j) * ni + i]; }
    __device__ double phi(int j, int i, double g) const {
        double Ti = a(j, VK_ATM_TI);
        return -1. / a(j, VK_ATM_HPI) + ms[i] * g / (GEO_NAVO * GEO_KB * Ti)
               + alpha[i] / Ti * (a(j + 1, VK_ATM_TCO) - a(j, VK_ATM_TCO)) / a(j, VK_ATM_DZI);
    }
};

__device__ __forceinline__ GeoCol make_geocol(const double *atm, const double *Dzz,
                                              const double *spf, const int *col_off,
                                              const int *col_end, int c, int ni) {
    GeoCol g;
    g.atm = atm;
    g.Dzz = Dzz;
    g.ms = spf + (size_t)c * VK_SP_NF * ni + VK_SP_MS * ni;
    g.alpha = spf + (size_t)c * VK_SP_NF * ni + VK_SP_ALPHA * ni;
    g.l0 = col_off[c];
    g.nz = col_end[c] - g.l0;
    g.ni = ni;
    return g;
}

// Geometry of species i in layer j -> out[0..4] = gU, gD, pA, pB, pC.
__device__ __forceinline__ void geo_coef(const GeoCol &cv, int j, int i, int flags, double *out) {
    const int nz = cv.nz;
    const bool mol = flags & VK_F_MOLDIFF;
    double gU = 0, gD = 0, pA = 0, pB = 0, pC = 0;
    if (j == 0) {
        double dzi = cv.a(0, VK_ATM_DZI), K = cv.a(0, VK_ATM_KZZ), vz = cv.a(0, VK_ATM_VZ);
        gU = 1. / dzi * (K / dzi);
        pA = -((vz > 0) * vz) / dzi;
        pB = -((vz < 0) * vz) / dzi;
        if (mol) {
            double D = cv.dzz(0, i), ph = cv.phi(0, i, cv.a(0, VK_ATM_G));
            gU += 1. / dzi * (D / dzi);
            pA += 1. / dzi * D / 2. * ph;
            pB += 1. / dzi * D / 2. * ph;
        }
    } else if (j == nz - 1) {
        int t = nz - 2;
        double dzi = cv.a(t, VK_ATM_DZI), K = cv.a(t, VK_ATM_KZZ), vz = cv.a(t, VK_ATM_VZ);
        gD = 1. / dzi * (K / dzi);
        pA = ((vz < 0) * vz) / dzi;
        pC = ((vz > 0) * vz) / dzi;
        if (mol) {
            double D = cv.dzz(t, i), ph = cv.phi(t, i, cv.a(nz - 1, VK_ATM_G));
            gD += 1. / dzi * (D / dzi);
            pA += -1. / dzi * D / 2. * ph;
            pC += -1. / dzi * D / 2. * ph;
        }
    } else {
        double dm = cv.a(j - 1, VK_ATM_DZI), dp = cv.a(j, VK_ATM_DZI);
        double Km = cv.a(j - 1, VK_ATM_KZZ), Kp = cv.a(j, VK_ATM_KZZ);
        double vm = cv.a(j - 1, VK_ATM_VZ), vp = cv.a(j, VK_ATM_VZ);
        double da = 0.5 * (dm + dp);
        double inv = mol ? 1. / da : 2. / (dm + dp);
        gU = inv * (Kp / dp);
        gD = inv * (Km / dm);
        pA = -((vp > 0) * vp - (vm < 0) * vm) / da;
        pB = -((vp < 0) * vp) / da;
        pC = ((vm > 0) * vm) / da;
        if (mol) {
            double Dm = cv.dzz(j - 1, i), Dp = cv.dzz(j, i);
            double gm = cv.a(j - 1, VK_ATM_G), g0 = cv.a(j, VK_ATM_G), gp = cv.a(j + 1, VK_ATM_G);
            gU += 1. / da * (Dp / dp);
            gD += 1. / da * (Dm / dm);
            pA += 1. / (2. * da) * (Dp * cv.phi(j, i, g0) - Dm * cv.phi(j - 1, i, g0));
            pB += 1. / (2. * da) * Dp * cv.phi(j, i, gp);
            pC += -1. / (2. * da) * Dm * cv.phi(j - 1, i, gm);
        }
    }
    out[0] = gU; out[1] = gD; out[2] = pA; out[3] = pB; out[4] = pC;
}

}  // namespace vk
