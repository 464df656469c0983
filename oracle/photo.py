"""CPU oracle of the reference's photochemistry radiative transfer.

Test infrastructure only (imported by tests/ and the smoke check): a numpy
restatement of op.ODESolver.compute_tau (op.py:2580-2599), compute_flux
(op.py:2603-2739, isotropic scattering ag0 = 0 as phy_const.py sets) and
compute_J (op.py:2751-2786) for one column, given the binned cross sections,
scattering cross sections and top-of-atmosphere flux that the reference's
make_bins_read_cross / read_sflux produce (recorded in tests/golden).
"""
from __future__ import annotations

import numpy as np

HC = 1.98644582E-9        # erg nm (phy_const.py)


def compute_tau(y, dz, absp_idx, cross, scat_idx, cross_scat, cross_T=None):
    """tau [nz+1, nbins]: absorbers (photo and ion species) and Rayleigh
    scatterers summed layer by layer from the top (op.py:2580-2599).
    cross_T {absorber position: [nz, nbins]}: the per-layer cross sections
    of the temperature-dependent absorbers (op.py:2591-2592)."""
    nz = y.shape[0]
    cross_T = cross_T or {}
    tau = np.zeros((nz + 1, cross.shape[1]))
    for j in range(nz - 1, -1, -1):
        for a, s in enumerate(absp_idx):
            tau[j] += y[j, s] * dz[j] * (cross_T[a][j] if a in cross_T else cross[a])
        for a, s in enumerate(scat_idx):
            tau[j] += y[j, s] * dz[j] * cross_scat[a]
        tau[j] += tau[j + 1]
    return tau


def compute_flux(tau, ymix, photo_idx, cross_photo, scat_idx, cross_scat, sflux_top, bins,
                 sl_angle, edd, dflux_u, dflux_d, aflux_prev=None, flux_atol=1.0):
    """Two-stream actinic flux (op.py:2603-2739).  dflux_u / dflux_d [nz+1,
    nbins] are the previous call's diffuse fluxes (the downward sweep reads the
    old upward flux) and are updated in place.  Returns (aflux [nz, nbins],
    sflux [nz+1, nbins], aflux_change)."""
    nz = ymix.shape[0]
    mu_ang = -1. * np.cos(sl_angle)
    delta_tau = (tau - np.roll(tau, -1, axis=0))[:-1]
    nb = len(bins)
    tot_abs, tot_scat = np.zeros((nz, nb)), np.zeros((nz, nb))
    for a, s in enumerate(photo_idx):
        tot_abs += np.vstack(ymix[:, s]) * cross_photo[a]
    for a, s in enumerate(scat_idx):
        tot_scat += np.vstack(ymix[:, s]) * cross_scat[a]
    with np.errstate(divide='ignore', invalid='ignore'):
        w0 = tot_scat / (tot_abs + tot_scat)
    w0 = np.nan_to_num(w0)
    w0 = np.minimum(w0, 1. - 1.E-8)
    sflux = sflux_top * np.exp(-1. * tau / np.cos(sl_angle))
    dir_flux = sflux * np.cos(sl_angle)
    tran = np.exp(-1. / edd * (1. - w0) ** 0.5 * delta_tau)
    zeta_p = 0.5 * (1. + (1. - w0) ** 0.5)
    zeta_m = 0.5 * (1. - (1. - w0) ** 0.5)
    ll = -1. * w0 / (1. / mu_ang ** 2 - 1. / edd ** 2 * (1. - w0))
    g_p = 0.5 * (ll * (1. / edd + 1. / mu_ang))
    g_m = 0.5 * (ll * (1. / edd - 1. / mu_ang))
    chi = zeta_m ** 2 * tran ** 2 - zeta_p ** 2
    xi = zeta_p * zeta_m * (1. - tran ** 2)
    phi = (zeta_m ** 2 - zeta_p ** 2) * tran
    i_u = phi * g_p * dir_flux[:-1] - (xi * g_m + chi * g_p) * dir_flux[1:]
    i_d = phi * g_m * dir_flux[1:] - (chi * g_m + xi * g_p) * dir_flux[:-1]
    for j in range(nz - 1, -1, -1):
        dflux_d[j] = 1. / chi[j] * (phi[j] * dflux_d[j + 1] - xi[j] * dflux_u[j] + i_d[j] / mu_ang)
    for j in range(1, nz + 1):
        dflux_u[j] = 1. / chi[j - 1] * (phi[j - 1] * dflux_u[j - 1] - xi[j - 1] * dflux_d[j]
                                         + i_u[j - 1] / mu_ang)
    ave_dir_flux = 0.5 * (sflux[:-1] + sflux[1:])
    tot_flux = ave_dir_flux + 0.5 * (dflux_u[:-1] + dflux_u[1:] + dflux_d[1:] + dflux_d[:-1]) / edd
    aflux = tot_flux / (HC / bins)
    change = np.nan
    if aflux_prev is not None:
        m = aflux > flux_atol
        with np.errstate(divide='ignore', invalid='ignore'):
            change = float(np.nanmax(np.abs(aflux - aflux_prev)[m] / aflux[m])) if m.any() else np.nan
    return aflux, sflux, change


def j_weights(nbins, i12, dbin1, dbin2):
    """Bin weights of the reference's J integral (op.py:2770-2773): flux x
    cross summed with dbin1 below the switch index, dbin2 from it on, minus
    half the end points of each part -- with Python's indexing, so i12 = -1
    (no switch inside the bins) reproduces the reference's sums exactly."""
    w = np.zeros(nbins)
    idx = np.arange(nbins)
    w[idx[:i12]] += dbin1
    w[idx[0]] -= 0.5 * dbin1
    w[idx[i12 - 1]] -= 0.5 * dbin1
    w[idx[i12:]] += dbin2
    w[idx[i12]] -= 0.5 * dbin2
    w[idx[-1]] -= 0.5 * dbin2
    return w


def compute_J(aflux, cross_J, weights, cross_J_T=None):
    """J [nch, nz] of every photolysis channel (op.py:2751-2786): sum over
    bins of aflux x cross_J x weights; cross_J_T {channel position: [nz,
    nbins]} replaces cross_J by per-layer cross sections for the channels of
    temperature-dependent species (op.py:2770-2774)."""
    J = (aflux[None, :, :] * cross_J[:, None, :] * weights[None, None, :]).sum(axis=2)
    for c, cj in (cross_J_T or {}).items():
        J[c] = (aflux * cj * weights[None, :]).sum(axis=1)
    return J
