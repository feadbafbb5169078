"""Initial conditions: harmonic analysis and initial ensembles.

``HarmonicAnalysis`` keeps the interface and the finite-difference stencils of
the reference's ``HarmonicAnalysis``
(simulation_utilities/initial_conditioner/harmonic_analysis.py:10-129, with
``MolFiniteDifference``, finite_difference.py:6-68): 3- or 5-point mixed first
derivatives above the diagonal and 3- or 5-point second derivatives on it,
step dx (1e-3 bohr), then the mass-weighted Hessian diagonalised.  The
reference calls ``getpot`` once per Hessian element; here every stencil
geometry of the whole Hessian is built first and evaluated in ONE potential
call -- for a :class:`Potential_GPU` one kernel launch over
9 (3A)(3A-1)/2 + 5 (3A) geometries -- and the differences are taken on the
host with the reference's weights and summation order.

``InitialConditioner`` keeps the reference's ``InitialConditioner``
(initial_conditioner.py:7-108): ``harmonic_sampling`` draws Gaussian
normal-mode displacements with widths 1/sqrt(omega) and maps them back to
Cartesians; ``permute_atoms`` shuffles like atoms per walker.  Both use
NumPy's global generator, as the reference does, so a seeded script draws
the same ensemble.
"""
import itertools as itt

import numpy as np

from .constants import Constants

__all__ = ["HarmonicAnalysis", "InitialConditioner", "fd_weights"]


def fd_weights(der, num_points):
    """Stencil weights of finite_difference.py:8-13 (der 1 or 2; 3 or 5 points)."""
    if der == 1:
        return {3: np.array([-1 / 2, 0, 1 / 2]), 5: np.array([1 / 12, -2 / 3, 0, 2 / 3, -1 / 12])}[num_points]
    return {3: np.array([1, -2, 1]), 5: np.array([-1 / 12, 4 / 3, -5 / 2, 4 / 3, -1 / 12])}[num_points]


def _displace(eq_geom, atm_cd, dx, num_disps):
    """MolFiniteDifference.displace_molecule (finite_difference.py:15-54)."""
    half = num_disps // 2
    steps = np.arange(-half, half + 1) * dx
    if len(atm_cd) == 2:
        out = np.repeat(eq_geom[None], len(steps), axis=0)
        out[:, atm_cd[0], atm_cd[1]] += steps
        return out
    a1, c1, a2, c2 = atm_cd
    out = np.repeat(eq_geom[None], len(steps) ** 2, axis=0)
    out[:, a1, c1] += np.repeat(steps, len(steps))
    out[:, a2, c2] += np.tile(steps, len(steps))
    return out


class HarmonicAnalysis:
    """Mass-weighted Cartesian Hessian by finite differences and its normal modes.

    :param eq_geom: (A, 3) geometry in bohr
    :param atoms: A atom symbols (masses from :class:`Constants` unless given)
    :param potential: object with ``getpot(cds) -> (N,)``, e.g. a Potential_GPU
    :param dipole: optional object whose ``getpot`` returns (N, 3) dipoles
    """

    def __init__(self, eq_geom, atoms, potential, masses=None, dx=1.0e-3, points_diag=5, points_off_diag=3,
                 dipole=None):
        self.eq_geom = np.asarray(eq_geom, dtype=np.float64)
        self.atoms = atoms
        self.potential = potential
        self.masses = np.array([Constants.mass(a) for a in atoms]) if masses is None else np.asarray(masses, float)
        self.dx = dx
        self.points_diag = points_diag
        self.points_off_diag = points_off_diag
        self.num_elems = 3 * len(atoms)
        self.dipole = dipole

    def _stencils(self):
        A = len(self.atoms)
        n = self.num_elems
        off = list(itt.combinations(range(n), 2))
        geoms, where = [], []
        for i, j in off:
            geoms.append(_displace(self.eq_geom, (i // 3, i % 3, j // 3, j % 3), self.dx, self.points_off_diag))
            where.append(("off", i, j))
        for k in range(n):
            geoms.append(_displace(self.eq_geom, (k // 3, k % 3), self.dx, self.points_diag))
            where.append(("diag", k, k))
        assert len(geoms) == n * (n - 1) // 2 + n and A * 3 == n
        return geoms, where

    def generate_hessian(self):
        geoms, where = self._stencils()
        sizes = [len(g) for g in geoms]
        v = np.asarray(self.potential.getpot(np.concatenate(geoms)), dtype=np.float64)  # one batched call
        w1 = fd_weights(1, self.points_off_diag) / self.dx
        w2 = fd_weights(2, self.points_diag) / self.dx ** 2
        hess = np.zeros((self.num_elems, self.num_elems))
        pos = 0
        diag = []
        for (kind, i, j), m in zip(where, sizes):
            vals = v[pos:pos + m]
            pos += m
            if kind == "off":
                p = self.points_off_diag
                hess[i, j] = np.dot(w1, np.dot(w1, vals.reshape(p, p)))
            else:
                diag.append((i, np.dot(w2, vals)))
        hess = hess + hess.T
        for i, val in diag:
            hess[i, i] = val
        return hess

    def dipole_derivs(self):
        """d(dipole)/dx per Cartesian displacement (5-point), one batched dipole call."""
        geoms = [_displace(self.eq_geom, (k // 3, k % 3), self.dx, 5) for k in range(self.num_elems)]
        d = np.asarray(self.dipole.getpot(np.concatenate(geoms)), dtype=np.float64).reshape(self.num_elems, 5, 3)
        w = fd_weights(1, 5) / self.dx
        return np.stack([np.dot(w, d[k]) for k in range(self.num_elems)])

    def diagonalize(self, hessian):
        m = np.repeat(self.masses, 3)
        hess_mw = hessian / np.sqrt(m) / np.sqrt(m[:, np.newaxis])
        freqs, normal_modes = np.linalg.eigh(hess_mw)
        freqs_cm = Constants.convert(np.sqrt(np.abs(freqs)) * np.sign(freqs), "wavenumbers", to_AU=False)
        return freqs_cm, normal_modes

    def run(self):
        return self.diagonalize(self.generate_hessian())


class InitialConditioner:
    """Preliminary ensemble from a minimum geometry: ``harmonic_sampling``
    (technique_kwargs: freqs, normal_modes, scaling_factor, ensemble) or
    ``permute_atoms`` (technique_kwargs: like_atoms, ensemble)."""

    def __init__(self, coord, atoms, num_walkers, technique, technique_kwargs, masses=None):
        self.coord = np.asarray(coord, dtype=np.float64)
        self.atoms = atoms
        self.masses = masses
        self.num_walkers = num_walkers
        self.technique = technique.lower()
        self.technique_kwargs = technique_kwargs
        if self.technique == "harmonic_sampling":
            self.run_func = self.run_harm
        elif self.technique == "permute_atoms":
            self.run_func = self.run_permute
        else:
            raise NotImplementedError("Choose another initial condition: harmonic_sampling or permute_atoms")

    def displace_along_nms(self, freqs_au, nms, masses, ensemble):
        """initial_conditioner.py:36-62: widths 1/sqrt(omega) along the 3A-6 modes."""
        three_n = len(freqs_au) + 6
        disp = np.random.normal(loc=0, scale=1 / np.sqrt(freqs_au), size=(self.num_walkers, len(freqs_au)))
        carts = np.matmul(disp, nms.T[np.newaxis, :, :]).squeeze()
        carts = np.reshape(carts, (-1, three_n // 3, 3)) / np.sqrt(masses)[:, np.newaxis]
        base = np.tile(self.coord, (self.num_walkers, 1, 1)) if ensemble is None else ensemble
        return base + carts

    def run_harm(self):
        kw = self.technique_kwargs
        masses = np.array([Constants.mass(a) for a in self.atoms]) if self.masses is None else np.asarray(self.masses)
        freqs_au = Constants.convert(np.asarray(kw["freqs"])[6:], "wavenumbers", to_AU=True) / kw["scaling_factor"]
        return self.displace_along_nms(freqs_au, np.asarray(kw["normal_modes"])[:, 6:], masses, kw["ensemble"])

    def run_permute(self):
        kw = self.technique_kwargs
        walkers = np.tile(self.coord, (self.num_walkers, 1, 1)) if kw["ensemble"] is None else kw["ensemble"]
        for like in kw["like_atoms"]:
            sub = walkers[:, like]
            for row in sub:
                np.random.shuffle(row)
            walkers[:, like] = sub
        return walkers

    def run(self):
        return self.run_func()
