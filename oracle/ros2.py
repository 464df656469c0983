"""Numpy restatement of the reference Ros2 kinetics-diffusion step (TEST ORACLE).

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, as the oracle results are compared
with or as the timed CPU path.

Follows, function by function (paths relative to the reference project):
  chemdf            make_chem_funs.py:113-430 (generated chemdf / v_j lambdas)
  neg_jac_blocks    make_chem_funs.py:686-717 (sympy Jacobian of df, negated)
  diffdf            op.py:1496-1597 (eddy + molecular diffusion RHS)
  diffdf_no_mol     op.py:1438-1494
  lhs_blocks        op.py:1973-2042 (lhs_jac_tot), op.py:2122-2166 (no_mol)
  band solve        op.py:2833-2858 (store_bandM) + scipy.linalg.solve_banded
                    (LAPACK ?gbsv, the reference's own dependency)
  ros2_attempt      op.py:2860-3007 (Ros2.solver)
  clip / loss       op.py:2447-2487
  step_ok/reject    op.py:2489-2534
  step_size         op.py:3105-3125
  integrate         op.py:808-936, 944-984, 1018-1105 (Integration loop,
                    update_mu_dz, conv, stop, save_step)
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

KB = 1.38064852E-16
NAVO = 6.02214086E+23
R_ROS = 1. + 1. / 2. ** 0.5


def parse_reaction(text):
    reac, prod, cur = [], [], None
    cur = reac
    for term in text.split():
        if term == '+':
            continue
        if term == '->':
            cur = prod
            continue
        p = term.split('*')
        cur.append((1, p[0]) if len(p) == 1 else (int(p[0]), p[1]))
    return reac, prod


@dataclass
class OracleNet:
    species: list
    reactions: list          # [(reac_terms, prod_terms)] in k order
    compo: np.ndarray        # [ni, natom] for the tracked atoms
    mass: np.ndarray

    @property
    def ni(self):
        return len(self.species)

    @classmethod
    def from_npz(cls, path, atom_list):
        d = np.load(path, allow_pickle=False)
        species = [str(s) for s in d['species']]
        atoms = [str(a) for a in d['compo_atoms']]
        comp = d['compo'][:, [atoms.index(a) for a in atom_list]]
        rx = [parse_reaction(str(t)) for t in d['text']]
        return cls(species, rx, np.asarray(comp, float), np.asarray(d['mass'], float))


# --------------------------------------------------------------- chemistry
def _side_value(kk, terms, y, M, sidx):
    v = kk
    for nu, name in terms:
        f = M if name == 'M' else y[:, sidx[name]]
        v = v * (f if nu == 1 else f ** nu)
    return v


def chemdf(net: OracleNet, y, M, k):
    """dy/dt of the mass-action network; k is [nr, nz] (row i-1 = k[i])."""
    sidx = {s: i for i, s in enumerate(net.species)}
    dydt = np.zeros_like(y)
    for p, (reac, prod) in enumerate(net.reactions):
        v = (_side_value(k[2 * p], reac, y, M, sidx)
             - _side_value(k[2 * p + 1], prod, y, M, sidx))
        for nu, name in reac:
            if name != 'M':
                dydt[:, sidx[name]] = dydt[:, sidx[name]] + (-nu) * v
        for nu, name in prod:
            if name != 'M':
                dydt[:, sidx[name]] = dydt[:, sidx[name]] + nu * v
    return dydt


def _merged(terms):
    m, mp = {}, 0
    for nu, name in terms:
        if name == 'M':
            mp += nu
        else:
            m[name] = m.get(name, 0) + nu
    return m, mp


def _dside(kk, merged, mp, y, M, sidx, q):
    """d/dy_q of kk * M^mp * prod y_s^e_s."""
    e = merged[q]
    v = kk * (M ** mp if mp else 1.0)
    for name, ex in merged.items():
        f = y[:, sidx[name]]
        if name == q:
            v = v * (e * f ** (ex - 1) if ex > 1 else 1.0)
        else:
            v = v * f ** ex
    return v


def neg_jac_blocks(net: OracleNet, y, M, k):
    """-d(chemdf)/dy per layer, [nz, ni, ni] (block l = rows/cols of layer l)."""
    sidx = {s: i for i, s in enumerate(net.species)}
    nz, ni = y.shape
    J = np.zeros((nz, ni, ni))
    for p, (reac, prod) in enumerate(net.reactions):
        fm, fmp = _merged(reac)
        rm, rmp = _merged(prod)
        nu = {}
        for n, s in reac:
            if s != 'M':
                nu[s] = nu.get(s, 0) - n
        for n, s in prod:
            if s != 'M':
                nu[s] = nu.get(s, 0) + n
        for q in set(fm) | set(rm):
            d = np.zeros(nz)
            if q in fm:
                d = d + _dside(k[2 * p], fm, fmp, y, M, sidx, q)
            if q in rm:
                d = d - _dside(k[2 * p + 1], rm, rmp, y, M, sidx, q)
            for s, n in nu.items():
                if n:
                    J[:, sidx[s], sidx[q]] += n * d
    return -J


# --------------------------------------------------------------- diffusion
@dataclass
class Flags:
    use_moldiff: bool = True
    use_topflux: bool = False
    use_botflux: bool = False
    fix_sp_bot_idx: tuple = ()
    fix_sp_bot_mix: tuple = ()


def _phi(atm, j, gj):
    """-1/Hpi + ms g/(Navo kb Ti) + alpha/Ti dT/dz at interface j, gravity gj."""
    return (-1. / atm['Hpi'][j] + atm['ms'] * gj / (NAVO * KB * atm['Ti'][j])
            + atm['alpha'] / atm['Ti'][j] * (atm['Tco'][j + 1] - atm['Tco'][j]) / atm['dzi'][j])


def diff_coeffs(y, atm, flags: Flags):
    """Eddy (A,B,C: [nz]) and molecular (Ai,Bi,Ci: [nz,ni]) coefficients."""
    nz, ni = y.shape
    ys = np.sum(y, axis=1)
    dzi, Kzz, vz = atm['dzi'], atm['Kzz'], atm['vz']
    A, B, C = np.zeros(nz), np.zeros(nz), np.zeros(nz)
    Ai, Bi, Ci = [np.zeros((nz, ni)) for _ in range(3)]
    if flags.use_moldiff:
        A[0] = -1. / (dzi[0]) * (Kzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[0]
        B[0] = 1. / (dzi[0]) * (Kzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[1]
        A[nz - 1] = -1. / (dzi[nz - 2]) * (Kzz[nz - 2] / dzi[nz - 2]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 1]
        C[nz - 1] = 1. / (dzi[nz - 2]) * (Kzz[nz - 2] / dzi[nz - 2]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 2]
    else:
        A[0] = -1. / (dzi[0]) * (Kzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[0]
        B[0] = 1. / (dzi[0]) * (Kzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[1]
        A[nz - 1] = -1. / (dzi[nz - 2]) * (Kzz[nz - 2] / dzi[nz - 2]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 1]
        C[nz - 1] = 1. / (dzi[nz - 2]) * (Kzz[nz - 2] / dzi[nz - 2]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 2]
    A[0] += -((vz[0] > 0) * vz[0]) / dzi[0]
    B[0] += -((vz[0] < 0) * vz[0]) / dzi[0]
    A[-1] += ((vz[-1] < 0) * vz[-1]) / dzi[-1]
    C[-1] += ((vz[-1] > 0) * vz[-1]) / dzi[-1]
    j = np.arange(1, nz - 1)
    dz_ave = 0.5 * (dzi[j - 1] + dzi[j])
    if flags.use_moldiff:
        A[j] = -1. / dz_ave * (Kzz[j] / dzi[j] * (ys[j + 1] + ys[j]) / 2. + Kzz[j - 1] / dzi[j - 1] * (ys[j] + ys[j - 1]) / 2.) / ys[j]
        B[j] = 1. / dz_ave * Kzz[j] / dzi[j] * (ys[j + 1] + ys[j]) / 2. / ys[j + 1]
        C[j] = 1. / dz_ave * Kzz[j - 1] / dzi[j - 1] * (ys[j] + ys[j - 1]) / 2. / ys[j - 1]
    else:
        A[j] = -2. / (dzi[j - 1] + dzi[j]) * (Kzz[j] / dzi[j] * (ys[j + 1] + ys[j]) / 2. + Kzz[j - 1] / dzi[j - 1] * (ys[j] + ys[j - 1]) / 2.) / ys[j]
        B[j] = 2. / (dzi[j - 1] + dzi[j]) * Kzz[j] / dzi[j] * (ys[j + 1] + ys[j]) / 2. / ys[j + 1]
        C[j] = 2. / (dzi[j - 1] + dzi[j]) * Kzz[j - 1] / dzi[j - 1] * (ys[j] + ys[j - 1]) / 2. / ys[j - 1]
    A[j] += -((vz[j] > 0) * vz[j] - (vz[j - 1] < 0) * vz[j - 1]) / dz_ave
    B[j] += -((vz[j] < 0) * vz[j]) / dz_ave
    C[j] += ((vz[j - 1] > 0) * vz[j - 1]) / dz_ave
    if flags.use_moldiff:
        Dzz, g = atm['Dzz'], atm['g']
        f0 = _phi(atm, 0, g[0])
        Ai[0] = -1. / (dzi[0]) * (Dzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[0] + 1. / (dzi[0]) * Dzz[0] / 2. * f0
        Bi[0] = 1. / (dzi[0]) * (Dzz[0] / dzi[0]) * (ys[1] + ys[0]) / 2. / ys[1] + 1. / (dzi[0]) * Dzz[0] / 2. * f0
        ft = _phi(atm, nz - 2, g[-1])
        Ai[nz - 1] = -1. / (dzi[-1]) * (Dzz[nz - 2] / dzi[-1]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 1] - 1. / (dzi[-1]) * Dzz[-1] / 2. * ft
        Ci[nz - 1] = 1. / (dzi[-1]) * (Dzz[nz - 2] / dzi[-1]) * (ys[nz - 1] + ys[nz - 2]) / 2. / ys[nz - 2] - 1. / (dzi[-1]) * Dzz[-1] / 2. * ft
        for jj in range(1, nz - 1):
            da = 0.5 * (dzi[jj - 1] + dzi[jj])
            Ai[jj] = -1. / da * (Dzz[jj] / dzi[jj] * (ys[jj + 1] + ys[jj]) / 2. + Dzz[jj - 1] / dzi[jj - 1] * (ys[jj] + ys[jj - 1]) / 2.) / ys[jj]
            Bi[jj] = 1. / da * Dzz[jj] / dzi[jj] * (ys[jj + 1] + ys[jj]) / 2. / ys[jj + 1]
            Ci[jj] = 1. / da * Dzz[jj - 1] / dzi[jj - 1] * (ys[jj] + ys[jj - 1]) / 2. / ys[jj - 1]
            Ai[jj] += 1. / (2. * da) * (Dzz[jj] * _phi(atm, jj, g[jj]) - Dzz[jj - 1] * _phi(atm, jj - 1, g[jj]))
            Bi[jj] += 1. / (2. * da) * Dzz[jj] * _phi(atm, jj, g[jj + 1])
            Ci[jj] += -1. / (2. * da) * Dzz[jj - 1] * _phi(atm, jj - 1, g[jj - 1])
    return A, B, C, Ai, Bi, Ci


def diffdf(y, atm, flags: Flags, coeffs=None):
    nz, ni = y.shape
    A, B, C, Ai, Bi, Ci = coeffs if coeffs is not None else diff_coeffs(y, atm, flags)
    diff = np.empty_like(y)
    diff[0] = (A[0] + Ai[0]) * y[0] + (B[0] + Bi[0]) * y[1]
    m = slice(1, nz - 1)
    diff[m] = (A[m, None] * y[1:nz - 1] + B[m, None] * y[2:nz] + C[m, None] * y[0:nz - 2])
    diff[m] += Ai[m] * y[1:nz - 1] + Bi[m] * y[2:nz] + Ci[m] * y[0:nz - 2]
    diff[nz - 1] = (A[nz - 1] + Ai[nz - 1]) * y[nz - 1] + (C[nz - 1] + Ci[nz - 1]) * y[nz - 2]
    if flags.use_topflux:
        diff[-1] += atm['top_flux'] / atm['dzi'][-1]
    if flags.use_botflux:
        diff[0] += (atm['bot_flux'] - y[0] * atm['bot_vdep']) / atm['dzi'][0]
    return diff


def lhs_blocks(net, y, M, k, dt, atm, flags: Flags, negjac=None, perturb=None):
    """Block-tridiagonal c0 I - J: diagonal blocks D [nz,ni,ni] and the
    diagonal vectors of the off-diagonal blocks U (j,j+1) and L (j,j-1).

    ``perturb=(eps, seed)`` multiplies every chemistry Jacobian entry by
    (1 + eps u), u ~ U(-1, 1): used to measure how far rounding-level changes
    of the matrix move the step (its conditioning floor)."""
    nz, ni = y.shape
    c0 = 1. / (R_ROS * dt)
    D = neg_jac_blocks(net, y, M, k) if negjac is None else negjac.copy()
    if perturb is not None:
        rng = np.random.default_rng(perturb[1])
        D = D * (1.0 + perturb[0] * rng.uniform(-1.0, 1.0, D.shape))
    idx = np.arange(ni)
    A, B, C, Ai, Bi, Ci = diff_coeffs(y, atm, flags)
    D[:, idx, idx] = c0 + D[:, idx, idx]
    # reference subtracts the eddy part, then the molecular part
    D[:, idx, idx] -= A[:, None]
    D[:, idx, idx] -= Ai
    if flags.use_botflux:
        D[0, idx, idx] -= -1. * atm['bot_vdep'] / atm['dzi'][0]
    U = -(B[:, None] + Bi)
    L = -(C[:, None] + Ci)
    U[-1] = 0.
    L[0] = 0.
    return D, U, L


def band_from_blocks(D, U, L):
    """LAPACK band storage ab[bw + i - j, j] = A[i, j], bw = 2 ni - 1."""
    nz, ni, _ = D.shape
    N = nz * ni
    bw = 2 * ni - 1
    ab = np.zeros((2 * bw + 1, N))
    lay = np.arange(nz)[:, None, None] * ni
    rows = lay + np.arange(ni)[None, :, None]
    cols = lay + np.arange(ni)[None, None, :]
    ab[(bw + rows - cols).ravel(), np.broadcast_to(cols, D.shape).ravel()] = D.ravel()
    i = np.arange(N - ni)
    ab[bw - ni, i + ni] = U[:-1].ravel()          # (i, i+ni)
    ab[bw + ni, i] = L[1:].ravel()                # (i+ni, i)
    return ab, bw


def block_thomas(D, U, L, b):
    """Block tridiagonal solve with explicit block inverses (numpy/LAPACK)."""
    nz, ni, _ = D.shape
    b = b.reshape(nz, ni)
    G = np.empty_like(D)
    z = np.empty((nz, ni))
    G[0] = np.linalg.inv(D[0])
    z[0] = G[0] @ b[0]
    for j in range(1, nz):
        Dp = D[j] - L[j][:, None] * G[j - 1] * U[j - 1][None, :]
        G[j] = np.linalg.inv(Dp)
        z[j] = G[j] @ (b[j] - L[j] * z[j - 1])
    x = np.empty_like(z)
    x[-1] = z[-1]
    for j in range(nz - 2, -1, -1):
        x[j] = z[j] - G[j] @ (U[j] * x[j + 1])
    return x


# ---------------------------------------------------------------- the step
@dataclass
class StepResult:
    k1: np.ndarray
    k2: np.ndarray
    yk2: np.ndarray
    sol: np.ndarray
    ymix: np.ndarray
    delta: float


@dataclass
class Tol:
    atol: float = 1.E-1
    mtol: float = 1.E-22
    mtol_conv: float = 1.E-20
    pos_cut: float = 0.
    nega_cut: float = -1.
    loss_eps: float = 1e-1
    rtol: float = 0.25
    dt_min: float = 1.E-14
    dt_max: float = 1.E17
    dt_var_min: float = 0.5
    dt_var_max: float = 2.
    yconv_cri: float = 0.01
    slope_cri: float = 1.e-4
    yconv_min: float = 0.1
    st_factor: float = 0.5
    conv_step: int = 500
    trun_min: float = 1e2
    count_min: int = 120
    count_max: int = int(3E4)
    runtime: float = 1.E22
    update_frq: int = 100


def ros2_attempt(net, y, ymix, dt, k, atm, flags: Flags, tol: Tol, solve='banded',
                 perturb=None):
    """One Rosenbrock-2 attempt from state (y, ymix) with step dt."""
    nz, ni = y.shape
    M = atm['M']
    r = R_ROS
    df = chemdf(net, y, M, k).flatten() + diffdf(y, atm, flags).flatten()
    D, U, L = lhs_blocks(net, y, M, k, dt, atm, flags, perturb=perturb)
    if solve == 'banded':
        ab, bw = band_from_blocks(D, U, L)
        k1_flat = scipy.linalg.solve_banded((bw, bw), ab, df)
    else:
        k1_flat = block_thomas(D, U, L, df).flatten()
    k1 = k1_flat.reshape(y.shape)
    yk2 = y + k1 / r
    df = chemdf(net, yk2, M, k).flatten() + diffdf(yk2, atm, flags).flatten()
    rhs = df - 2. / (r * dt) * k1_flat
    if solve == 'banded':
        k2 = scipy.linalg.solve_banded((bw, bw), ab, rhs)
    else:
        k2 = block_thomas(D, U, L, rhs).flatten()
    k2 = k2.reshape(y.shape)
    sol = y + 3. / (2. * r) * k1 + 1 / (2. * r) * k2
    if len(flags.fix_sp_bot_idx):
        sol[0, list(flags.fix_sp_bot_idx)] = np.asarray(flags.fix_sp_bot_mix) * atm['n_0'][0]
    delta = np.abs(sol - yk2)
    delta[ymix < tol.mtol] = 0
    delta[sol < tol.atol] = 0
    if flags.use_botflux or len(flags.fix_sp_bot_idx):
        delta[0] = 0
    pos = sol > 0
    delta = float(np.amax(delta[pos] / sol[pos])) if np.any(pos) else 0.0
    ymix_new = sol / np.vstack(np.sum(sol, axis=1))
    return StepResult(k1, k2, yk2, sol, ymix_new, delta)


def clip(y, ymix, tol: Tol):
    y = y.copy()
    y[np.logical_and(y < tol.pos_cut, y >= tol.nega_cut)] = 0.
    y[np.logical_and(ymix < tol.mtol, y < 0)] = 0.
    return y, y / np.vstack(np.sum(y, axis=1))


def atom_sums(net, y):
    return np.array([np.sum([net.compo[i, a] * y[:, i] for i in range(net.ni)])
                     for a in range(net.compo.shape[1])])


def step_size(dt, delta, tol: Tol):
    if delta == 0:
        delta = 0.01 * tol.rtol
    f = 0.9 * (tol.rtol / delta) ** 0.5
    f = min(max(f, tol.dt_var_min), tol.dt_var_max)
    return min(max(dt * f, tol.dt_min), tol.dt_max)


# ---------------------------------------------------------- outer loop
@dataclass
class ColState:
    y: np.ndarray
    ymix: np.ndarray
    dt: float
    t: float = 0.0
    count: int = 0
    atom_ini: np.ndarray = None
    atom_loss: np.ndarray = None
    delta: float = 0.0
    hist_y: list = field(default_factory=list)
    hist_t: list = field(default_factory=list)
    longdy: float = 1.0
    longdydt: float = 1.0
    end_case: int = 0
    attempts: int = 0
    nrej: int = 0


def one_step(net, st: ColState, k, atm, flags, tol, solve='banded', on_attempt=None):
    """op.Ros2.one_step: attempts until accepted (or dt floor reached)."""
    y_prev = st.y.copy()
    loss_prev = st.atom_loss.copy()
    ymix = st.ymix
    y = st.y
    dt = st.dt
    while True:
        res = ros2_attempt(net, y, ymix, dt, k, atm, flags, tol, solve)
        st.attempts += 1
        if on_attempt is not None:
            on_attempt(y, ymix, dt, res)
        y, ymix = clip(res.sol, res.ymix, tol)
        loss = (atom_sums(net, y) - st.atom_ini) / st.atom_ini
        st.delta = res.delta
        ok = (np.all(y >= 0) and np.amax(np.abs(loss - loss_prev)) < tol.loss_eps
              and res.delta <= tol.rtol)
        if ok:
            break
        st.nrej += 1
        y = y_prev.copy()
        dt *= tol.dt_var_min
        if dt < tol.dt_min:
            dt = tol.dt_min
            y[y < 0] = 0.
            break
    st.y, st.ymix, st.dt, st.atom_loss = y, ymix, dt, loss
    return st


def update_mu_dz(atm, mass, ymix, gs, Rp, pref, use_moldiff=True):
    """Integration.update_mu_dz restated (op.py:944-984)."""
    nz = ymix.shape[0]
    mu = np.zeros(nz)
    for i in range(ymix.shape[1]):
        mu += mass[i] * ymix[:, i]
    Tco, pico = atm['Tco'], atm['pico']
    g, Hp, dz, zco = atm['g'].copy(), atm['Hp'].copy(), atm['dz'].copy(), atm['zco'].copy()
    for i in range(pref, nz):
        if i == pref:
            g[i] = gs
            Hp[i] = KB * Tco[i] / (mu[i] / NAVO * gs)
        else:
            g[i] = gs * (Rp / (Rp + zco[i])) ** 2
            Hp[i] = KB * Tco[i] / (mu[i] / NAVO * g[i])
        dz[i] = Hp[i] * np.log(pico[i] / pico[i + 1])
        zco[i + 1] = zco[i] + dz[i]
    for i in range(pref - 1, -1, -1):
        g[i] = gs * (Rp / (Rp + zco[i + 1])) ** 2
        Hp[i] = KB * Tco[i] / (mu[i] / NAVO * g[i])
        dz[i] = Hp[i] * np.log(pico[i] / pico[i + 1])
        zco[i] = zco[i + 1] - dz[i]
    dzi = 0.5 * (dz + np.roll(dz, 1))
    atm = dict(atm, mu=mu, g=g, Hp=Hp, dz=dz, zco=zco, dzi=dzi[1:].copy())
    if use_moldiff:
        Hpi = 0.5 * (Hp + np.roll(Hp, -1))
        atm['Hpi'] = Hpi[:-1].copy()
    return atm


def conv(st: ColState, atm, tol: Tol, ignore_idx=()):
    """Steady-state test of Integration.conv (op.py:1018-1063)."""
    slope_min = min(np.amin(atm['Kzz'] / (0.1 * atm['Hp'][:-1]) ** 2), 1.e-8)
    slope_min = max(slope_min, 1.e-10)
    t_time = np.array(st.hist_t)
    count = st.count
    indx = int(np.abs(t_time - st.t * tol.st_factor).argmin())
    if indx == count - 1:
        indx -= 1
    indx = max(count - tol.conv_step, indx)
    longdy = np.abs((st.hist_y[count - 1] - st.hist_y[indx]) / np.vstack(atm['n_0']))
    longdy[st.ymix < tol.mtol_conv] = 0
    longdy[st.y < tol.atol] = 0
    for i in ignore_idx:
        longdy[:, i] = 0
    pos = st.ymix > 0
    longdy = float(np.amax(longdy[pos] / st.ymix[pos]))
    longdydt = longdy / (t_time[-1] - t_time[indx])
    st.longdy, st.longdydt = longdy, longdydt
    return (longdy < tol.yconv_cri and longdydt < tol.slope_cri) or \
           (longdy < tol.yconv_min and longdydt < slope_min)


def integrate(net, st: ColState, k, atm, flags, tol: Tol, gs, Rp, pref, max_steps=None,
              solve='banded', ignore_idx=(), on_step=None, on_attempt=None):
    """Integration.__call__ restated: run until steady state / limits."""
    n = 0
    while True:
        if st.t > tol.trun_min and st.count > tol.count_min and conv(st, atm, tol, ignore_idx):
            st.end_case = 1
            break
        if st.t > tol.runtime:
            st.end_case = 2
            break
        if st.count > tol.count_max:
            st.end_case = 3
            break
        if max_steps is not None and n >= max_steps:
            break
        one_step(net, st, k, atm, flags, tol, solve, on_attempt)
        if st.count % tol.update_frq == 0:
            atm = update_mu_dz(atm, net.mass, st.ymix, gs, Rp, pref, flags.use_moldiff)
        st.y = np.vstack(atm['n_0']) * st.ymix
        st.t += st.dt
        st.count += 1
        st.hist_y.append(st.y)
        st.hist_t.append(st.t)
        st.dt = step_size(st.dt, st.delta, tol)
        n += 1
        if on_step is not None:
            on_step(st, atm)
    return st, atm
