"""Harmonic analysis and initial conditions against the reference's own
HarmonicAnalysis / InitialConditioner (golden fixture from
tests/golden/make_harmonic_golden.py)."""
import os

import numpy as np
import pytest

import oracle
from oracle.ps_oracle import pes_ps
import pyvibdmc_gb300 as pg

G = os.path.join(os.path.dirname(__file__), "golden", "harmonic.npz")


class _NumpyPES:
    def __init__(self, f):
        self.f = f

    def getpot(self, cds):
        return self.f(np.asarray(cds))


@pytest.fixture(scope="module")
def gold():
    with np.load(G) as z:
        return {k: z[k] for k in z.files}


def test_hessian_and_modes_equal_the_reference(gold):
    """Same potential values, same stencils and weights: equal to the reference's Hessian
    (bit for bit where NumPy's exp/arccos are the fixture machine's; their last bits
    differ between x86 and Arm builds of NumPy, and a 1-ulp change of V ~ 0.4 Eh
    becomes ~1e-10 in a Hessian element through the 1/dx^2 = 1e6 stencil weights)."""
    p, _ = oracle.h2o_config()
    ha = pg.HarmonicAnalysis(gold["lm_geom"], ["O", "H", "H"], _NumpyPES(lambda c: oracle.pes_h2o_lm(c, p)))
    np.testing.assert_allclose(ha.generate_hessian(), gold["lm_hess"], rtol=1e-9, atol=1e-9)
    ha = pg.HarmonicAnalysis(gold["ps_geom"], ["H", "H", "O"], _NumpyPES(lambda c: pes_ps(c, "HHO")))
    h = ha.generate_hessian()
    np.testing.assert_allclose(h, gold["ps_hess"], rtol=1e-9, atol=1e-9)
    f, nm = ha.diagonalize(h)
    # the six near-zero translation/rotation "frequencies" are square roots of round-off
    np.testing.assert_allclose(f[6:], gold["ps_freqs"][6:], rtol=0, atol=1e-6)


def test_initial_conditioner_equals_the_reference(gold):
    np.random.seed(11)
    ic = pg.InitialConditioner(gold["ps_geom"], ["H", "H", "O"], 64, "harmonic_sampling",
                               dict(freqs=gold["ps_freqs"], normal_modes=gold["ps_nms"], scaling_factor=1.0,
                                    ensemble=None))
    np.testing.assert_array_equal(ic.run(), gold["harm_walkers"])
    np.random.seed(12)
    ic = pg.InitialConditioner(gold["perm_geom"][None], ["C", "H", "H", "H", "H", "H"], 40, "permute_atoms",
                               dict(like_atoms=[[0], [1, 2, 3, 4, 5]], ensemble=None))
    np.testing.assert_array_equal(ic.run(), gold["perm_walkers"])


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["lm", "ps"])
def test_hessian_on_the_gpu_pes_matches_the_reference(gold, which):
    """All stencil geometries of the Hessian in one batched GPU potential call."""
    if which == "lm":
        ha = pg.HarmonicAnalysis(gold["lm_geom"], ["O", "H", "H"], pg.h2o_local_mode())
    else:
        ha = pg.HarmonicAnalysis(gold["ps_geom"], ["H", "H", "O"], pg.partridge_schwenke(atom_order="HHO"))
    f, _ = ha.run()
    np.testing.assert_allclose(ha.generate_hessian(), gold[f"{which}_hess"], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(f[6:], gold[f"{which}_freqs"][6:], rtol=0, atol=1e-3)
