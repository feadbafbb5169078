"""NumPy restatement of PyVibDMC's walker step loop -- the CPU oracle.

TEST INFRASTRUCTURE ONLY: used by ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline legs as the checker / timed CPU baseline.  The
product package never imports it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the unmodified reference
engine (``pyvibdmc/pyvibdmc.py``) with the deterministic noise of
:class:`InjectedNoise` patched into ``np.random.normal`` / ``np.random.random``
and commits its outputs; ``tests/test_oracle_golden.py`` checks this module
against those fixtures.

Every function cites the reference file:line it restates (paths relative to
the reference project root).
"""
import numpy as np

__all__ = [
    "WAVENUMBERS", "ANGSTROMS", "AMU", "MASS_H", "MASS_O", "mass_au",
    "InjectedNoise", "splitmix64",
    "pes_ho", "pes_h2o_lm", "oh_stretch_harm", "reduced_mass_au", "pes_dimer", "grad_ho", "grad_h2o_lm", "grad_dimer",
    "h2o_internals", "TrialH2OGauss", "TrialHOGauss", "TrialDimerGauss", "finite_diff",
    "metropolis", "local_kin", "move_randomly", "birth_or_death_discrete",
    "continuous_update_and_branch", "argpartition_introselect", "introselect_adversary", "calc_vref", "calc_desc_wts",
    "OracleDMC", "ho_config", "h2o_config", "h2o_equilibrium", "h2o_trial_config", "dimer_config",
    "dimer_equilibrium", "inv_dist_descriptors",
]

# ---------------------------------------------------------------- constants
# pyvibdmc/simulation_utilities/Constants.py:65-69
WAVENUMBERS = 4.556335281212229e-6
ANGSTROMS = 1 / 0.529177
AMU = 1.000000000000000000 / 6.02213670000e23 / 9.10938970000e-28
# pyvibdmc/simulation_utilities/Constants.py:3 (H, O entries)
MASS_H = 1.00782503
MASS_O = 15.99491462


def mass_au(amu):
    """Constants.mass -> amu * AMU (Constants.py:85-98)."""
    return amu * AMU


# ------------------------------------------------------------ injected noise
_U64 = np.uint64
_MASK = 0xFFFFFFFFFFFFFFFF


def splitmix64(z):
    """SplitMix64 finaliser on a uint64 array (wrapping arithmetic)."""
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + _U64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> _U64(30))) * _U64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> _U64(27))) * _U64(0x94D049BB133111EB)
        z = z ^ (z >> _U64(31))
    return z


class InjectedNoise:
    """Deterministic, platform-independent noise stream.

    Replaces NumPy's legacy global ``RandomState`` draws in the reference's
    call order (``np.random.normal`` in ``move_randomly`` pyvibdmc.py:544 /
    ``imp_move_randomly`` :556, ``np.random.random`` in ``birth_or_death``
    :392 and the Metropolis test :601).  Only integer ops and correctly
    rounded IEEE additions are used, so the same bits come out on x86 and Arm.

    * uniform: ``(splitmix64(key + i) >> 11) * 2**-53`` in [0, 1)
    * "normal": Irwin-Hall(12) - 6, mean 0, variance 1 (a stand-in deviate:
      the parity tests need identical inputs, not exact Gaussianity).
    """

    def __init__(self, seed):
        self.seed = int(seed) & _MASK
        self.calls = 0

    def _key(self, call):
        with np.errstate(over="ignore"):
            k = splitmix64(np.array([(self.seed * 0x632BE59BD9B4E019 + call * 0x9E3779B97F4A7C15) & _MASK],
                                    dtype=np.uint64))[0]
        return k

    def standard_normal(self, shape):
        n = int(np.prod(shape))
        key = self._key(self.calls)
        self.calls += 1
        idx = np.arange(n, dtype=np.uint64) * _U64(12)
        acc = np.zeros(n, dtype=np.float64)
        with np.errstate(over="ignore"):
            for j in range(12):
                h = splitmix64(idx + _U64(j) + key)
                acc = acc + (h >> _U64(11)).astype(np.float64) * 2.0 ** -53
        return (acc - 6.0).reshape(shape)

    def uniform(self, n):
        key = self._key(self.calls)
        self.calls += 1
        with np.errstate(over="ignore"):
            h = splitmix64(np.arange(n, dtype=np.uint64) + key)
        return (h >> _U64(11)).astype(np.float64) * 2.0 ** -53

    # drop-in replacements for np.random.normal / np.random.random
    def normal(self, loc=0.0, scale=1.0, size=None):
        z = self.standard_normal(size)
        return loc + scale * z

    def random(self, size=None):
        return self.uniform(int(np.prod(size)))


# ------------------------------------------------------------------ PESs
def pes_ho(x, k):
    """Isotropic harmonic well V = 1/2 k |x|^2 over every coordinate, (N,A,3) -> (N,)."""
    x = np.asarray(x, dtype=np.float64)
    s = np.zeros(len(x))
    for a in range(x.shape[1]):
        for d in range(x.shape[2]):
            s = s + x[:, a, d] * x[:, a, d]
    return 0.5 * k * s


def grad_ho(x, k):
    return k * np.asarray(x, dtype=np.float64)


def reduced_mass_au(a_amu, b_amu):
    """Constants.reduced_mass (Constants.py:100-119): both masses to atomic
    units first, then m1 m2 / (m1 + m2)."""
    m1, m2 = mass_au(a_amu), mass_au(b_amu)
    return m1 * m2 / (m1 + m2)


def oh_stretch_harm(cds, kwargs=None):
    """The reference's 1D sample potential (sample_potentials/PythonPots/
    harmonicOscillator1D.py:13-17): 1/2 mu omega^2 x^2 with the O-H reduced
    mass and omega = 3700 cm^-1, (N,1,1) -> (N,); with ``kwargs`` the
    ``oh_stretch_harm_with_arg`` variant (:25-29), mass and frequency from
    kwargs['mass'], kwargs['freq']."""
    if kwargs is None:
        mu, w = reduced_mass_au(MASS_O, MASS_H), 3700.0 * WAVENUMBERS
    else:
        mu, w = kwargs["mass"], kwargs["freq"]
    return np.squeeze(0.5 * mu * w ** 2 * cds ** 2)


def h2o_internals(x, o=0, h1=1, h2=2):
    """r1=|H1-O|, r2=|H2-O|, cos(theta), theta; O is the vertex.

    Same conventions as the bond lengths / angle helpers the reference trial
    functions use (call_trl_h2o.py:26-35, analysis/analyze_wfn.py)."""
    d1 = x[:, h1] - x[:, o]
    d2 = x[:, h2] - x[:, o]
    r1 = np.sqrt(d1[:, 0] * d1[:, 0] + d1[:, 1] * d1[:, 1] + d1[:, 2] * d1[:, 2])
    r2 = np.sqrt(d2[:, 0] * d2[:, 0] + d2[:, 1] * d2[:, 1] + d2[:, 2] * d2[:, 2])
    dot = d1[:, 0] * d2[:, 0] + d1[:, 1] * d2[:, 1] + d1[:, 2] * d2[:, 2]
    c = np.clip(dot / (r1 * r2), -1.0, 1.0)
    return d1, d2, r1, r2, c, np.arccos(c)


def pes_h2o_lm(x, p, o=0, h1=1, h2=2):
    """H2O local-mode PES (O,H,H order): two OH Morse stretches, harmonic bend
    1/2 k_theta (theta-theta_e)^2 and k_rr (r1-re)(r2-re) coupling.
    p = dict(De, a, re, ktheta, theta_e, krr)."""
    _, _, r1, r2, c, th = h2o_internals(x, o, h1, h2)
    dr1 = r1 - p["re"]
    dr2 = r2 - p["re"]
    e1 = 1.0 - np.exp(-p["a"] * dr1)
    e2 = 1.0 - np.exp(-p["a"] * dr2)
    dth = th - p["theta_e"]
    return p["De"] * e1 * e1 + p["De"] * e2 * e2 + 0.5 * p["ktheta"] * dth * dth + p["krr"] * dr1 * dr2


def _h2o_int_first(d1, d2, r1, r2, c):
    """Cartesian first derivatives of r1, r2, theta for atoms (O, H1, H2):
    arrays (N,3) per atom; restates ChainRuleHelper.dr_dx / dcth_dx / dth_dx
    (imp_samp_helper.py:40-52, 68-107, 162-179)."""
    e1 = d1 / r1[:, None]
    e2 = d2 / r2[:, None]
    g = 1.0 / (r1 * r2)
    dc_h1 = d2 * g[:, None] - (c / r1)[:, None] * e1
    dc_h2 = d1 * g[:, None] - (c / r2)[:, None] * e2
    dc_o = -(dc_h1 + dc_h2)
    s = -1.0 / np.sqrt(1.0 - c * c)
    dr1 = (-e1, e1, np.zeros_like(e1))
    dr2 = (-e2, np.zeros_like(e2), e2)
    dth = (s[:, None] * dc_o, s[:, None] * dc_h1, s[:, None] * dc_h2)
    return e1, e2, g, dr1, dr2, dth, (dc_o, dc_h1, dc_h2), s


def grad_h2o_lm(x, p, o=0, h1=1, h2=2):
    """Analytic dV/dx of :func:`pes_h2o_lm`, (N,3,3)."""
    d1, d2, r1, r2, c, th = h2o_internals(x, o, h1, h2)
    _, _, _, dr1, dr2, dth, _, _ = _h2o_int_first(d1, d2, r1, r2, c)
    a, De, re = p["a"], p["De"], p["re"]
    x1 = np.exp(-a * (r1 - re))
    x2 = np.exp(-a * (r2 - re))
    dv_dr1 = 2 * De * (1 - x1) * a * x1 + p["krr"] * (r2 - re)
    dv_dr2 = 2 * De * (1 - x2) * a * x2 + p["krr"] * (r1 - re)
    dv_dth = p["ktheta"] * (th - p["theta_e"])
    g = np.zeros_like(x, dtype=np.float64)
    for slot, atom in enumerate((o, h1, h2)):
        g[:, atom] += dv_dr1[:, None] * dr1[slot] + dv_dr2[:, None] * dr2[slot] + dv_dth[:, None] * dth[slot]
    return g


def pes_dimer(x, p):
    """Water dimer (O1,H1,H2,O2,H3,H4): two local-mode monomers + O-O
    Lennard-Jones 4 eps[(s/r)^12-(s/r)^6] + intermolecular point charges."""
    x = np.asarray(x, dtype=np.float64)
    v = pes_h2o_lm(x, p, 0, 1, 2) + pes_h2o_lm(x, p, 3, 4, 5)
    doo = x[:, 3] - x[:, 0]
    roo = np.sqrt(doo[:, 0] ** 2 + doo[:, 1] ** 2 + doo[:, 2] ** 2)
    sr6 = (p["sigma"] / roo) ** 6
    v = v + 4.0 * p["eps"] * (sr6 * sr6 - sr6)
    q = [p["qO"], p["qH"], p["qH"]]
    for i in range(3):
        for j in range(3):
            dij = x[:, 3 + j] - x[:, i]
            rij = np.sqrt(dij[:, 0] ** 2 + dij[:, 1] ** 2 + dij[:, 2] ** 2)
            v = v + q[i] * q[j] / rij
    return v


def grad_dimer(x, p):
    x = np.asarray(x, dtype=np.float64)
    g = np.zeros_like(x)
    g += grad_h2o_lm(x, p, 0, 1, 2)
    g += grad_h2o_lm(x, p, 3, 4, 5)
    doo = x[:, 3] - x[:, 0]
    roo = np.sqrt((doo ** 2).sum(-1))
    sr6 = (p["sigma"] / roo) ** 6
    dv_dr = 4.0 * p["eps"] * (-12 * sr6 * sr6 + 6 * sr6) / roo
    g[:, 3] += (dv_dr / roo)[:, None] * doo
    g[:, 0] -= (dv_dr / roo)[:, None] * doo
    q = [p["qO"], p["qH"], p["qH"]]
    for i in range(3):
        for j in range(3):
            dij = x[:, 3 + j] - x[:, i]
            rij = np.sqrt((dij ** 2).sum(-1))
            f = (-q[i] * q[j] / rij ** 3)[:, None] * dij
            g[:, 3 + j] += f
            g[:, i] -= f
    return g


def inv_dist_descriptors(x):
    """Inverse distances 1/r_ij over the upper triangle (i<j) in
    itertools.combinations order -- the pair order DistIt uses
    (tensorflow_descriptors/distance_descriptors.py:66-68, 102-113)."""
    x = np.asarray(x, dtype=np.float64)
    A = x.shape[1]
    out = []
    for i in range(A):
        for j in range(i + 1, A):
            d = x[:, i] - x[:, j]
            out.append(1.0 / np.sqrt((d ** 2).sum(-1)))
    return np.stack(out, axis=1)


# ------------------------------------------------------------- trial psi
class TrialH2OGauss:
    """psi_T = prod_q (alpha_q/pi)^(1/4) exp(-alpha_q (q - q_e)^2 / 2) over
    q = (r1, r2, theta), the direct-product form of call_trl_h2o.py:43-78.
    ``derivs`` returns (dpsi/dx / psi, d2psi/dx2 / psi) per Cartesian
    component, the contract of ImpSampManager.call_derivs
    (imp_samp_manager.py:202-224), built with the chain rule of
    ChainRuleHelper.dpsidx / d2psidx2 (imp_samp_helper.py:10-38)."""

    def __init__(self, alpha, qe, o=0, h1=1, h2=2):
        self.alpha = np.asarray(alpha, dtype=np.float64)
        self.qe = np.asarray(qe, dtype=np.float64)
        self.idx = (o, h1, h2)

    def psi(self, x):
        _, _, r1, r2, c, th = h2o_internals(np.asarray(x, dtype=np.float64), *self.idx)
        out = np.ones(len(r1))
        for q, a, qe in zip((r1, r2, th), self.alpha, self.qe):
            out = out * ((a / np.pi) ** 0.25 * np.exp(-a * (q - qe) ** 2 / 2))
        return out

    def derivs(self, x):
        x = np.asarray(x, dtype=np.float64)
        d1, d2, r1, r2, c, th = h2o_internals(x, *self.idx)
        e1, e2, g, dr1, dr2, dth, dc, s = _h2o_int_first(d1, d2, r1, r2, c)
        L = [-self.alpha[0] * (r1 - self.qe[0]), -self.alpha[1] * (r2 - self.qe[1]),
             -self.alpha[2] * (th - self.qe[2])]
        # second derivatives (diagonal) of r1, r2, cos(theta)
        d2r1 = ((1 - e1 * e1) / r1[:, None],) * 2 + (np.zeros_like(e1),)
        d2r2 = ((1 - e2 * e2) / r2[:, None], np.zeros_like(e2), (1 - e2 * e2) / r2[:, None])
        cc = c[:, None]
        gg = g[:, None]
        rr1 = r1[:, None]
        rr2 = r2[:, None]
        h = e1 / rr1 + e2 / rr2
        d2c_o = 2 * gg - 2 * (d1 + d2) * gg * h + cc * (h * h + (2 * e1 * e1 - 1) / rr1 ** 2
                                                        + (2 * e2 * e2 - 1) / rr2 ** 2)
        d2c_h1 = cc * (3 * e1 * e1 - 1) / rr1 ** 2 - 2 * d2 * e1 / (rr1 ** 2 * rr2)
        d2c_h2 = cc * (3 * e2 * e2 - 1) / rr2 ** 2 - 2 * d1 * e2 / (rr2 ** 2 * rr1)
        d2th_dc2 = (-c / (1 - c * c) ** 1.5)[:, None]
        ss = s[:, None]
        d2th = tuple(d2th_dc2 * dci * dci + ss * d2ci for dci, d2ci in zip(dc, (d2c_o, d2c_h1, d2c_h2)))
        first = np.zeros_like(x)
        sec = np.zeros_like(x)
        for slot, atom in enumerate(self.idx):
            qd = (dr1[slot], dr2[slot], dth[slot])
            qdd = (d2r1[slot], d2r2[slot], d2th[slot])
            f = np.zeros_like(e1)
            t = np.zeros_like(e1)
            for q in range(3):
                f = f + L[q][:, None] * qd[q]
                t = t - self.alpha[q] * qd[q] * qd[q] + L[q][:, None] * qdd[q]
            first[:, atom] = f
            sec[:, atom] = f * f + t
        return first, sec


class TrialDimerGauss:
    """Trial for the water dimer (O,H,H,O,H,H) of the GPU engine: the
    TrialH2OGauss of each monomer times (alpha_R/pi)^(1/4)
    exp(-alpha_R (R_OO - R_e)^2 / 2).  The reference ships no dimer trial;
    this restates the engine's, with the same derivative contract as
    TrialH2OGauss (imp_samp_manager.py:202-224).  alpha = (a_r1, a_r2,
    a_theta, a_R), qe = (r1e, r2e, theta_e, R_e)."""

    def __init__(self, alpha, qe):
        self.mono = (TrialH2OGauss(alpha[:3], qe[:3], 0, 1, 2), TrialH2OGauss(alpha[:3], qe[:3], 3, 4, 5))
        self.aR, self.Re = float(alpha[3]), float(qe[3])

    def _oo(self, x):
        v = x[:, 3] - x[:, 0]
        R = np.sqrt((v * v).sum(1))
        return v, R

    def psi(self, x):
        x = np.asarray(x, dtype=np.float64)
        _, R = self._oo(x)
        g = (self.aR / np.pi) ** 0.25 * np.exp(-self.aR * (R - self.Re) ** 2 / 2)
        return self.mono[0].psi(x) * self.mono[1].psi(x) * g

    def derivs(self, x):
        x = np.asarray(x, dtype=np.float64)
        f = np.zeros_like(x)
        t = np.zeros_like(x)
        for m in self.mono:
            fm, sm = m.derivs(x)
            f += fm
            t += sm - fm * fm  # d2 ln psi_m / dx2 (zero outside the monomer)
        v, R = self._oo(x)
        e = v / R[:, None]
        L = (-self.aR * (R - self.Re))[:, None]
        too = -self.aR * e * e + L * (1 - e * e) / R[:, None]
        f[:, 3] += L * e
        f[:, 0] -= L * e
        t[:, 3] += too
        t[:, 0] += too
        return f, f * f + t


class TrialHOGauss:
    """Separable Cartesian Gaussian psi_T = prod_k (a_k/pi)^(1/4) exp(-a_k x_k^2/2),
    a_k = m_atom * omega (the harmonic trial of harm_trial_wfn.py:6-40 in 3D)."""

    def __init__(self, alpha_atoms):
        self.alpha = np.asarray(alpha_atoms, dtype=np.float64)

    def psi(self, x):
        x = np.asarray(x, dtype=np.float64)
        a = self.alpha[None, :, None]
        return np.prod(np.prod((a / np.pi) ** 0.25 * np.exp(-a * x * x / 2), axis=1), axis=1)

    def derivs(self, x):
        x = np.asarray(x, dtype=np.float64)
        a = self.alpha[None, :, None]
        return -a * x, a * a * x * x - a


def finite_diff(cds, trial_func, dx=0.001):
    """3-point central finite differences of psi, restating ImpSamp.finite_diff
    (imp_samp.py:55-76): returns (dpsi/dx, d2psi/dx2, psi) NOT divided by psi."""
    cds = np.array(cds, dtype=np.float64, copy=True)
    first = np.zeros(cds.shape)
    sec = np.zeros(cds.shape)
    tmp = np.zeros((len(cds), 3))
    tmp[:, 1] = trial_func(cds)
    for a in range(cds.shape[1]):
        for d in range(cds.shape[-1]):
            cds[:, a, d] -= dx
            tmp[:, 0] = trial_func(cds)
            cds[:, a, d] += 2.0 * dx
            tmp[:, 2] = trial_func(cds)
            cds[:, a, d] -= dx
            first[:, a, d] = (tmp[:, 2] - tmp[:, 0]) / (2 * dx)
            sec[:, a, d] = (tmp[:, 0] - 2.0 * tmp[:, 1] + tmp[:, 2]) / dx ** 2
    return first, sec, tmp[:, 1]


def metropolis(sigma_trip, trial_x, trial_y, disp_x, disp_y, D_x, D_y, dt):
    """Green's-function Metropolis ratio, imp_samp.py:28-47 (3D branch)."""
    psi_ratio = (trial_y / trial_x) ** 2
    term_1 = np.exp(-1 * (disp_x - disp_y - D_y * dt) ** 2 / (2 * sigma_trip ** 2))
    term_2 = np.exp(-1 * (disp_y - disp_x - D_x * dt) ** 2 / (2 * sigma_trip ** 2))
    accep = term_1 / term_2
    accep = np.prod(np.prod(accep, axis=1), axis=1) * psi_ratio
    accep[np.where(trial_x * trial_y <= 0)[0]] = 0.0
    return accep


def local_kin(inv_masses_trip, sec_deriv):
    """imp_samp.py:49-53."""
    return -0.5 * np.sum(np.sum(inv_masses_trip * sec_deriv, axis=1), axis=1)


# ------------------------------------------------------------ step pieces
def move_randomly(x, sigmas, noise):
    """pyvibdmc.py:540-547: normal(0, sigma_a) drawn as (N,3,A), transposed."""
    disps = noise.normal(0.0, sigmas, size=np.shape(x.transpose(0, 2, 1))).transpose(0, 2, 1)
    x += disps
    return x


def birth_or_death_discrete(pots, vref, dt, rand_nums, pop_hi):
    """Weights and integer counts of pyvibdmc.py:391-417.  Returns
    (walker_idx, counts, births, deaths) or raises ValueError like :397-413."""
    weights = np.exp(-1. * (pots - vref) * dt)
    if not np.all(np.isfinite(weights)) or np.any(weights > pop_hi + 1):
        raise ValueError("Massive walker birth or death event!!!!!!! Dying...")
    counts = np.floor(weights).astype(np.int64)
    counts += rand_nums < (weights - counts)
    deaths = int(np.count_nonzero(counts == 0))
    births = int(np.sum(np.maximum(counts - 1, 0)))
    return np.repeat(np.arange(len(counts)), counts), counts, births, deaths


def _msb(n):
    """npy_get_msb: index of the highest set bit of n > 0."""
    d = 0
    while n > 1:
        n >>= 1
        d += 1
    return d


def argpartition_introselect(v, kth, less=None, stats=None):
    """``np.argpartition(v, kth)`` as NumPy's portable introselect computes it.

    The reference picks the walkers to replace above the upper weight
    threshold with ``np.argpartition(w, k)[:k]`` (pyvibdmc.py:443-445), so the
    ORDER of that list -- which decides which walker is cloned into which slot
    by the sequential ``_branch`` -- is NumPy's.  NumPy (numpy/_core/src/
    npysort/selection.cpp, functions ``introselect_``, ``dumb_select_``,
    ``median3_swap_``, ``unguarded_partition_``, ``median_of_median5_`` and
    ``median5_``; same algorithm in NumPy 1.x and 2.x) runs this introselect
    on every platform without a SIMD select kernel, e.g. aarch64, and on x86
    when the x86-simd-sort dispatch targets are switched off
    (``NPY_DISABLE_CPU_FEATURES``); on x86 with AVX2/AVX-512 NumPy 2.x
    substitutes a SIMD select whose order differs.  The algorithm:

    * kth - low < 3: selection sort of positions 0..kth (first minimum wins);
    * kth == num - 1: swap the last maximum into the last position;
    * otherwise quickselect with a median-of-3 pivot (median3_swap_: the
      median to ``low``, the smallest to ``low + 1``, the largest to
      ``high``), Hoare's unguarded partition and, once ``2 * msb(num)``
      partitions have not finished, a median-of-medians-of-5 pivot.

    ``less`` overrides the comparison (used by the adversary test);
    ``stats`` (a dict) counts the median-of-medians pivots taken.
    Returns the permutation as a list.
    """
    t = list(range(len(v)))
    if less is None:
        vals = list(v)

        def lt(i, j):
            return vals[t[i]] < vals[t[j]]

        def lt_val(i, pv):
            return vals[t[i]] < pv

        def val_lt(pv, i):
            return pv < vals[t[i]]

        def val(i):
            return vals[t[i]]
    else:
        def lt(i, j):
            return less(t[i], t[j])

        def lt_val(i, pv):
            return less(t[i], pv)

        def val_lt(pv, i):
            return less(pv, t[i])

        def val(i):  # the element id stands for its value
            return t[i]

    def swap(i, j):
        t[i], t[j] = t[j], t[i]

    def dumb_select(off, num, k):
        for i in range(k + 1):
            mi = i
            for q in range(i + 1, num):
                if lt(off + q, off + mi):
                    mi = q
            swap(off + i, off + mi)

    def median3_swap(low, mid, high):
        if lt(high, mid):
            swap(high, mid)
        if lt(high, low):
            swap(high, low)
        if lt(low, mid):
            swap(low, mid)
        swap(mid, low + 1)

    def median5(off):
        if lt(off + 1, off + 0):
            swap(off + 1, off + 0)
        if lt(off + 4, off + 3):
            swap(off + 4, off + 3)
        if lt(off + 3, off + 0):
            swap(off + 3, off + 0)
        if lt(off + 4, off + 1):
            swap(off + 4, off + 1)
        if lt(off + 2, off + 1):
            swap(off + 2, off + 1)
        if lt(off + 3, off + 2):
            return 1 if lt(off + 3, off + 1) else 3
        return 2

    def median_of_median5(off, num):
        nmed = num // 5
        for i in range(nmed):
            m = median5(off + 5 * i)
            swap(off + 5 * i + m, off + i)
        if nmed > 2:
            introselect(off, nmed, nmed // 2, top=False)
        return nmed // 2

    def introselect(off, num, kth, top):
        low, high = 0, num - 1
        if kth - low < 3:
            dumb_select(off + low, high - low + 1, kth - low)
            return
        if kth == num - 1:  # inexact types only (float64 weights)
            mi = low
            for q in range(low + 1, num):
                if not lt(off + q, off + mi):  # !(v[q] < max): the last maximum wins
                    mi = q
            swap(off + kth, off + mi)
            return
        depth = _msb(num) * 2
        while low + 1 < high:
            ll, hh = low + 1, high
            if depth > 0 or hh - ll < 5:
                median3_swap(off + low, off + low + (high - low) // 2, off + high)
            else:
                mid = ll + median_of_median5(off + ll, hh - ll)
                swap(off + mid, off + low)
                ll -= 1
                hh += 1
                if stats is not None:
                    stats["mom5"] = stats.get("mom5", 0) + 1
            depth -= 1
            pv = val(off + low)
            while True:  # unguarded_partition_
                ll += 1
                while lt_val(off + ll, pv):
                    ll += 1
                hh -= 1
                while val_lt(pv, off + hh):
                    hh -= 1
                if hh < ll:
                    break
                swap(off + ll, off + hh)
            swap(off + low, off + hh)
            if hh >= kth:
                high = hh - 1
            if hh <= kth:
                low = ll
        if high == low + 1 and lt(off + high, off + low):
            swap(off + high, off + low)

    n = len(t)
    if not 0 <= kth < n:
        raise ValueError(f"kth(={kth}) out of bounds ({n})")
    introselect(0, n, kth, top=True)
    return t


def introselect_adversary(n, kth):
    """Weights on which :func:`argpartition_introselect` takes poor median-of-3
    pivots until it falls back to median-of-medians pivots: McIlroy's "killer
    adversary" (Software: Practice and Experience 29, 341 (1999)) fixes the
    values lazily while the select runs -- of two undecided elements compared,
    the pivot candidate is frozen to the next smallest value -- and the frozen
    values then replay the same path.  Test input for the selection's rare
    branch."""
    gas = 1 << 40
    val = [gas] * n
    st = {"solid": 0, "cand": 0}

    def less(a, b):
        if val[a] == gas and val[b] == gas:
            z = a if a == st["cand"] else b
            val[z] = st["solid"]
            st["solid"] += 1
        if val[a] == gas:
            st["cand"] = a
        elif val[b] == gas:
            st["cand"] = b
        return val[a] < val[b]

    argpartition_introselect(list(range(n)), kth, less=less)
    nxt = st["solid"]
    for i in range(n):
        if val[i] == gas:
            val[i] = nxt
            nxt += 1
    return np.array(val, dtype=np.float64)


def continuous_update_and_branch(st, dt, thresh_lower, thresh_upper=None):
    """pyvibdmc.py:432-454 with _branch :340-356.  ``st`` is a dict of
    walker-aligned arrays with at least 'x', 'v', 'w' (and optionally 'who',
    'f', 'psi', 'ke').  The walkers replaced above the upper threshold are
    ``np.argpartition(w, k)[:k]`` in the order of NumPy's portable
    introselect (:func:`argpartition_introselect`)."""
    w = st["w"]
    w *= np.exp(-1.0 * (st["v"] - st["vref"]) * dt)
    keys = [k for k in ("x", "v", "who", "f", "psi", "ke") if st.get(k) is not None]

    def _branch(kill):
        for walker in kill:
            m = np.argmax(w)
            for k in keys:
                st[k][walker] = np.copy(st[k][m])
            w[m] /= 2.0
            w[walker] = np.copy(w[m])

    kill = np.where(w < thresh_lower)[0]
    _branch(kill)
    n_up = 0
    if thresh_upper is not None:
        n_up = int(np.sum(w > thresh_upper))
        if n_up:
            _branch(argpartition_introselect(w, n_up)[:n_up])
    return len(kill) + n_up, float(np.amax(w)), float(np.amin(w))


def calc_vref(pots, n0, alpha, weights=None):
    """pyvibdmc.py:651-661."""
    if weights is None:
        v_bar = np.average(pots)
        correction = (len(pots) - n0) / n0
    else:
        v_bar = np.average(pots, weights=weights)
        correction = (np.sum(weights) - n0) / n0
    return v_bar - (alpha * correction)


def calc_desc_wts(who_from, n_parent, weights=None):
    """pyvibdmc.py:663-672."""
    desc = np.zeros(n_parent)
    if weights is None:
        unique, counts = np.unique(who_from, return_counts=True)
        desc[unique] = counts
    else:
        for q in range(n_parent):
            desc[q] = np.sum(weights[who_from == q])
    return desc


# --------------------------------------------------------------- engine
class OracleDMC:
    """Restates ``DMC_Sim.propagate`` (pyvibdmc.py:701-876) minus file I/O:
    step-0 potential + vref (:760-769), move (:540-547) or importance-sampled
    move (:549-612), potential (:785-793), local energy (:807-809),
    discrete birth/death (:380-431) or continuous weights (:432-454, :833-837),
    vref (:651-661), sim arrays (:674-682) and descendant weighting
    (:739-747, :856-872).  ``noise`` supplies normal/random draws in the
    reference's call order."""

    def __init__(self, x0, masses, dt, pes, noise, num_walkers=None, weighting="discrete",
                 trial=None, alpha=None, equil_steps=None, wfn_every=None, desc_wt_steps=None,
                 cont_wt_thresh=None, start_cont_wts=None, branch_every=1):
        self.x = np.array(x0, dtype=np.float64, copy=True)
        self.branch_every = int(branch_every)  # branching on steps t % branch_every == 0 (pyvibdmc.py:139)
        self.n0 = len(self.x) if num_walkers is None else num_walkers
        self.masses = np.asarray(masses, dtype=np.float64)
        self.dt = dt
        self.pes = pes
        self.noise = noise
        self.weighting = weighting
        self.trial = trial
        self.sigmas = np.sqrt(self.dt / self.masses)
        self.alpha = 1.0 / (2.0 * self.dt) if alpha is None else alpha
        self.pop_thresh = [self.n0 - self.n0 * 0.5, self.n0 + self.n0 * 0.5]
        self.v = None
        self.vref = None
        self.who = None
        self.desc_active = False
        self.wfns = []
        if weighting == "continuous":
            self.w = np.ones(len(self.x)) if start_cont_wts is None else np.array(start_cont_wts, dtype=float)
            if cont_wt_thresh is None:
                self.thr = (1 / self.n0, None)
            elif isinstance(cont_wt_thresh, (int, float)):
                self.thr = (cont_wt_thresh, None)
            else:
                self.thr = (cont_wt_thresh[0], cont_wt_thresh[1] if len(cont_wt_thresh) == 2 else None)
        else:
            self.w = None
        if trial is not None:
            A = self.x.shape[1]
            self.inv_m3 = (1 / np.repeat(self.masses, 3)).reshape(A, 3)[None]
            self.sig3 = np.repeat(self.sigmas, 3).reshape(A, 3)[None]
            self.f_x = self.psi = self.sd = None
            self.eff_ts = []
        n_steps_guess = 0
        self.wfn_start = set()
        self.wfn_end = set()
        if equil_steps is not None:
            self.equil_steps, self.wfn_every, self.desc_steps = equil_steps, wfn_every, desc_wt_steps
        else:
            self.equil_steps = None
        self.vref_hist = []
        self.pop_hist = []
        self.counters = []

    def _schedule(self, nsteps):
        if self.equil_steps is None:
            return set(), set()
        s = np.arange(self.equil_steps, nsteps + self.wfn_every, self.wfn_every)
        return set(int(v) for v in s), set(int(v) for v in s + self.desc_steps)

    def _drift(self, x):
        f, sd = self.trial.derivs(x)
        return f, self.trial.psi(x), sd

    def run(self, nsteps):
        wfn_start, wfn_end = self._schedule(nsteps)
        for t in range(nsteps):
            if self.weighting == "discrete":
                if len(self.x) < self.pop_thresh[0] or len(self.x) > self.pop_thresh[1]:
                    raise ValueError("Massive walker birth or death event!!!!!!! Dying...")
            if t in wfn_start:
                self.parent = np.copy(self.x)
                self.parent_w = None if self.w is None else np.copy(self.w)
                self.who = np.arange(len(self.x))
                self.desc_active = True
            if t == 0:
                self.v = self.pes(self.x)
                if self.trial is not None:
                    _, _, sd0 = self._drift(self.x)
                    self.sd = sd0
                    self.v = self.v + local_kin(self.inv_m3, self.sd)
                self._vref()
            rej = 0
            if self.trial is None:
                move_randomly(self.x, self.sigmas, self.noise)
            else:
                rej = self._imp_move()
            self.v = self.pes(self.x)
            if self.trial is not None:
                self.v = self.v + local_kin(self.inv_m3, self.sd)
            branch = t % self.branch_every == 0
            dt = self.dt
            if self.trial is not None and (branch or self.weighting == "continuous"):
                # update_effetive_timestep (pyvibdmc.py:386-387, :832-834)
                dt = self.dt * self.dt_factor
                self.eff_ts.append(dt if t == 0 else self.eff_ts[-1] + dt)
            if not branch:
                # off the branching schedule (pyvibdmc.py:828-837): discrete walkers
                # are not weighted; continuous weights are updated, nothing replaced
                if self.weighting == "continuous":
                    self.w *= np.exp(-1.0 * (self.v - self.vref) * dt)
                self.counters.append((0, 0, len(self.x), rej))
            elif self.weighting == "discrete":
                u = self.noise.random(size=len(self.x))
                idx, counts, births, deaths = birth_or_death_discrete(self.v, self.vref, dt, u,
                                                                      self.pop_thresh[1])
                final_pop = int(np.sum(counts))
                if final_pop < self.pop_thresh[0] or final_pop > self.pop_thresh[1]:
                    raise ValueError("Massive walker birth or death event!!!!!!! Dying...")
                self.x = self.x[idx]
                self.v = self.v[idx]
                if self.trial is not None:
                    self.f_x = self.f_x[idx]
                    self.psi = self.psi[idx]
                    self.sd = self.sd[idx]
                if self.desc_active:
                    self.who = self.who[idx]
                self.counters.append((births, deaths, final_pop, rej))
            else:
                st = dict(x=self.x, v=self.v, w=self.w, vref=self.vref,
                          who=self.who if self.desc_active else None,
                          f=self.f_x if self.trial is not None else None,
                          psi=self.psi if self.trial is not None else None,
                          ke=self.sd if self.trial is not None else None)
                nb, wmax, wmin = continuous_update_and_branch(st, dt, *self.thr)
                self.counters.append((nb, wmax, wmin, rej))
            self._vref()
            self.vref_hist.append(self.vref)
            self.pop_hist.append(len(self.x) if self.w is None else float(np.sum(self.w)))
            if t + 1 in wfn_end:
                self.desc_active = False
                self.wfns.append(dict(start=t + 1 - self.desc_steps, coords=self.parent,
                                      desc_wts=calc_desc_wts(self.who, len(self.parent), self.w),
                                      parent_wts=self.parent_w))
        return self

    def _vref(self):
        self.vref = calc_vref(self.v, self.n0, self.alpha, self.w)

    def _imp_move(self):
        """pyvibdmc.py:549-612."""
        if self.f_x is None or self.psi is None:
            self.f_x, self.psi, self.sd = self._drift(self.x)
        disps = self.noise.normal(0.0, self.sigmas,
                                  size=np.shape(self.x.transpose(0, 2, 1))).transpose(0, 2, 1)
        d_x = self.inv_m3 * self.f_x
        y = self.x + disps + d_x * self.dt
        f_y, psi_y, sd_y = self._drift(y)
        d_y = self.inv_m3 * f_y
        met = metropolis(self.sig3, self.psi, psi_y, self.x, y, d_x, d_y, self.dt)
        u = self.noise.random(size=len(self.x))
        accept = np.argwhere(met > u)
        self.dt_factor = len(accept) / len(self.x)
        self.x[accept] = y[accept]
        self.f_x[accept] = f_y[accept]
        self.psi[accept] = psi_y[accept]
        self.sd[accept] = sd_y[accept]
        return len(self.x) - len(accept)


# ------------------------------------------------------------- configs
def ho_config():
    """3D isotropic HO: 1 atom of 1.00782505 amu, omega = 3000 cm^-1."""
    m = 1.00782505 * AMU
    omega = 3000.0 * WAVENUMBERS
    return dict(mass=m, omega=omega, k=m * omega * omega, masses=[m])


def h2o_config():
    """Local-mode H2O PES parameters (O,H,H)."""
    p = dict(De=0.1869, a=1.2, re=1.81, ktheta=0.16, theta_e=np.deg2rad(104.5), krr=0.01)
    masses = [mass_au(MASS_O), mass_au(MASS_H), mass_au(MASS_H)]
    return p, masses


def h2o_equilibrium(p=None):
    p = p or h2o_config()[0]
    re, th = p["re"], p["theta_e"]
    return np.array([[0.0, 0.0, 0.0],
                     [re, 0.0, 0.0],
                     [re * np.cos(th), re * np.sin(th), 0.0]])


def h2o_trial_config(p=None):
    """Gaussian widths from 3800/3800/1600 cm^-1: alpha_r = mu_OH omega,
    alpha_theta = omega_theta / G_thth (G-matrix element as in
    call_trl_h2o.py:38-46)."""
    p = p or h2o_config()[0]
    mo, mh = mass_au(MASS_O), mass_au(MASS_H)
    mu = mo * mh / (mo + mh)
    re, th = p["re"], p["theta_e"]
    g = 1 / (mh * re ** 2) + 1 / (mh * re ** 2) + (1 / mo) * (2 / re ** 2 - 2 * np.cos(th) / (re * re))
    alpha = [mu * 3800.0 * WAVENUMBERS, mu * 3800.0 * WAVENUMBERS, 1600.0 * WAVENUMBERS / g]
    return alpha, [re, re, th]


def dimer_config():
    p, _ = h2o_config()
    p = dict(p, eps=2.4e-4, sigma=5.95, qH=0.417, qO=-0.834)
    mo, mh = mass_au(MASS_O), mass_au(MASS_H)
    return p, [mo, mh, mh, mo, mh, mh]


def dimer_equilibrium():
    """Minimum of :func:`pes_dimer` (E = -0.0108784 Eh, R_OO = 5.152 bohr),
    found once with scipy BFGS from random donor/acceptor starts."""
    return np.array([
    [0.000000000000, 0.000000000000, 0.000000000000],
    [1.427477952458, -0.371496091643, 1.058267415716],
    [-0.475355230876, -1.624174243271, -0.657060123398],
    [-0.890893874743, 4.517468473284, -2.310760800984],
    [-2.231456348667, 5.100851802863, -1.249695023025],
    [-0.483907575038, 2.882598047543, -1.568314000679]])
