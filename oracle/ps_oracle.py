"""NumPy restatement of the Partridge-Schwenke water PES that the reference
ships as its Fortran sample potential -- TEST INFRASTRUCTURE ONLY (see
``oracle/__init__.py``).

Follows ``calc_hoh_pot`` (sample_potentials/FortPots/Partridge_Schwenke_H2O/
calc_h2o_pot.f:1-30: r1, r2 from the O atom, theta = acos(ct / r1 / r2)) and
``vibpot`` (h2opes_v2.f:466-491: the power table fmat, the term-by-term sum
over j = 2..245, the damping exponential and the OH/HH two-body terms) in the
Fortran's own order of operations.  The coefficients are the reference's
DATA statements after vibpot's first-call scaling (h2opes_v2.f:420-458),
stored by ``pyvibdmc_gb300/csrc/gen_ps_pes.py`` in ``ps_pes_data.npz``.

gfortran is not available, so the Fortran itself cannot run here: parity is
pinned by (i) re-parsing the Fortran source in a CPU test (when the reference
is present) and (ii) the reference's own sample runs on this PES
(sample_sim_data/tutorial_water_*_log.txt: per-step mean potential energy of
8000 walkers), reproduced statistically on the GPU.
"""
import os

import numpy as np

__all__ = ["ps_data", "pes_ps"]

_DATA = None


def ps_data():
    global _DATA
    if _DATA is None:
        with np.load(os.path.join(os.path.dirname(__file__), "ps_pes_data.npz")) as z:
            _DATA = {k: z[k] for k in z.files}
    return _DATA


def pes_ps(x, order="OHH"):
    """V (hartree) of walkers x (N, 3, 3) in bohr; order 'OHH' or 'HHO'."""
    d = ps_data()
    x = np.asarray(x, dtype=np.float64)
    o, h1, h2 = (0, 1, 2) if order == "OHH" else (2, 0, 1)
    # calc_hoh_pot: d1 = x(O) - x(H1), d2 = x(O) - x(H2) (calc_h2o_pot.f:17-25)
    d1 = x[:, o] - x[:, h1]
    d2 = x[:, o] - x[:, h2]
    r1 = np.sqrt((d1 ** 2).sum(1))
    r2 = np.sqrt((d2 ** 2).sum(1))
    ct = (d1 * d2).sum(1)
    th = np.arccos(ct / r1 / r2)
    reoh, ce = float(d["reoh"]), float(d["ce"])
    x1 = (r1 - reoh) / reoh
    x2 = (r2 - reoh) / reoh
    x3 = np.cos(th) - ce
    rhh = np.sqrt(r1 ** 2 + r2 ** 2 - 2.0 * r1 * r2 * np.cos(th))
    vhh = float(d["phh1"]) * np.exp(-float(d["phh2"]) * rhh)
    ex = np.exp(-float(d["alphaoh"]) * (r1 - float(d["roh"])))
    voh1 = float(d["deoh"]) * ex * (ex - 2.0)
    ex = np.exp(-float(d["alphaoh"]) * (r2 - float(d["roh"])))
    voh2 = float(d["deoh"]) * ex * (ex - 2.0)
    n = len(x)
    fmat = np.ones((15, 3, n))
    for j in range(1, 15):
        fmat[j, 0] = fmat[j - 1, 0] * x1
        fmat[j, 1] = fmat[j - 1, 1] * x2
        fmat[j, 2] = fmat[j - 1, 2] * x3
    c, idx = d["c"], d["idx"] - 1
    v = np.zeros(n)
    for j in range(1, 245):
        a, b, k = idx[j]
        term = c[j] * (fmat[a, 0] * fmat[b, 1] + fmat[b, 0] * fmat[a, 1]) * fmat[k, 2]
        v = v + term
    return v * np.exp(-float(d["b1"]) * ((r1 - reoh) ** 2 + (r2 - reoh) ** 2)) + c[0] + voh1 + voh2 + vhh
