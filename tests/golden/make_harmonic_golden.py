"""Golden fixture for the harmonic analysis and the initial conditioner, from
the UNMODIFIED reference (``HarmonicAnalysis``, ``InitialConditioner``) with
the oracle's NumPy PESs plugged in through ``Potential_Direct``:

    python tests/golden/make_harmonic_golden.py <reference checkout>   (or set GBDMC_REFERENCE)

Writes ``tests/golden/harmonic.npz``: Hessians, frequencies and normal modes
of the local-mode water (O,H,H at its minimum) and of the Partridge-Schwenke
water (H,H,O at the geometry of the reference's own harmonic-analysis test,
test_initial_conditions.py), plus seeded harmonic-sampling and
atom-permutation ensembles.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _import_reference, ROOT  # noqa: E402

sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle.ps_oracle import pes_ps  # noqa: E402


def main(ref):
    pv = _import_reference(ref)
    out = {}
    p, _ = oracle.h2o_config()
    lm_eq = oracle.h2o_equilibrium(p)
    ha = pv.HarmonicAnalysis(eq_geom=lm_eq, atoms=["O", "H", "H"], potential=pv.Potential_Direct(
        lambda c: oracle.pes_h2o_lm(c, p)), dx=1e-3)
    out["lm_geom"] = lm_eq
    out["lm_hess"] = ha.generate_hessian()
    out["lm_freqs"], out["lm_nms"] = ha.diagonalize(out["lm_hess"])
    ps_geom = pv.Constants.convert(np.array([[0.9578400, 0.0, 0.0], [-0.2399535, 0.9272970, 0.0], [0.0, 0.0, 0.0]]),
                                   "angstroms", to_AU=True)
    ha = pv.HarmonicAnalysis(eq_geom=ps_geom, atoms=["H", "H", "O"],
                             potential=pv.Potential_Direct(lambda c: pes_ps(c, "HHO")), dx=1e-3)
    out["ps_geom"] = ps_geom
    out["ps_hess"] = ha.generate_hessian()
    out["ps_freqs"], out["ps_nms"] = ha.diagonalize(out["ps_hess"])
    np.random.seed(11)
    ic = pv.InitialConditioner(coord=ps_geom, atoms=["H", "H", "O"], num_walkers=64, technique="harmonic_sampling",
                               technique_kwargs=dict(freqs=out["ps_freqs"], normal_modes=out["ps_nms"],
                                                     scaling_factor=1.0, ensemble=None))
    out["harm_walkers"] = ic.run()
    geo = np.arange(18, dtype=float).reshape(6, 3) * 0.1
    np.random.seed(12)
    ic = pv.InitialConditioner(coord=geo[None], atoms=["C", "H", "H", "H", "H", "H"], num_walkers=40,
                               technique="permute_atoms",
                               technique_kwargs=dict(like_atoms=[[0], [1, 2, 3, 4, 5]], ensemble=None))
    out["perm_geom"] = geo
    out["perm_walkers"] = ic.run()
    np.savez_compressed(os.path.join(HERE, "harmonic.npz"), **out)
    print("ps harmonic frequencies (cm-1):", out["ps_freqs"][6:], "lm:", out["lm_freqs"][6:])


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBDMC_REFERENCE")
    if not ref:
        sys.exit("usage: %s <reference checkout>  (or set GBDMC_REFERENCE)" % sys.argv[0])
    main(ref)
