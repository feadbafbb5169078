"""Host-side configuration: constants and PES/trial parameters agree with the
oracle's restatement of the reference's units (no GPU needed)."""
import numpy as np

import oracle
import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import _capi


def test_constants_match_reference_values():
    C = pg.Constants
    assert C.atomic_units["wavenumbers"] == oracle.WAVENUMBERS
    assert C.atomic_units["amu"] == oracle.AMU
    assert C.mass("H") == oracle.mass_au(oracle.MASS_H)
    assert C.mass("O") == oracle.mass_au(oracle.MASS_O)
    assert pg.get_atomic_num(["H", "O"]) == [1, 10]  # reference table order (H, D, T, He, ...)
    assert abs(C.convert(C.convert(3000.0, "wavenumbers"), "wavenumbers", to_AU=False) - 3000.0) < 1e-9


def test_pes_parameters_match_oracle_configs():
    p, _ = oracle.h2o_config()
    pot = pg.Potential_GPU("h2o_local_mode", dict(p))
    st = pot.pes_struct()
    assert st.kind == _capi.PES_H2O_LM and st.natoms == 3
    assert list(st.p[:6]) == [p["De"], p["a"], p["re"], p["ktheta"], p["theta_e"], p["krr"]]
    ho = oracle.ho_config()
    assert pg.harmonic_oscillator().params["k"] == ho["k"]
    assert pg.h2o_local_mode().params == p
    pd, _ = oracle.dimer_config()
    assert pg.water_dimer().params == pd


def test_trial_parameters_match_oracle():
    a, qe = oracle.h2o_trial_config()
    t = pg.h2o_gaussian_trial()
    np.testing.assert_allclose(t.alpha, a, rtol=1e-15)
    np.testing.assert_allclose(t.qe, qe, rtol=1e-15)
    st = t.trial_struct()
    assert st.kind == _capi.TRIAL_H2O_GAUSS


def test_bad_pes_kind_rejected():
    import pytest
    with pytest.raises(ValueError):
        pg.Potential_GPU("lennard_jones", {})
    with pytest.raises(ValueError):
        pg.Potential_GPU("h2o_local_mode", {"De": 1.0})
