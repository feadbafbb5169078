"""Potentials written in Python inside the GPU engine: DMC_Sim moves and
branches the walkers on the GPU (gbdmc_sim_move / gbdmc_sim_branch through the
C ABI) and calls the potential's getpot on the moved walkers each step, as
the reference's propagate does (pyvibdmc.py:785-793).

Pins:
* the reference's own 1D sample potential (harmonicOscillator1D.py, restated in
  the oracle) through pyvibdmc_gb300.Potential_Direct, against fixtures of the
  unmodified reference running that sample file: walkers, populations and
  descendant weights bit-exact, vref 1e-12;
* the same with pot_kwargs and pass_timestep;
* a Python surface equal to a built-in GPU surface gives the fused step's
  trajectory: same Philox deviates and branching uniforms, walkers bit-exact,
  vref 1e-12 (the two evaluations of V differ in the last bits)."""
import os

import numpy as np
import pytest
import torch

import oracle
import pyvibdmc_gb300 as pg

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with np.load(os.path.join(G, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def _run_1d(g, pot, **kw):
    sim = pg.DMC_Sim(sim_name="t", output_folder="/tmp/gbdmc_ext", weighting=kw.pop("weighting", "discrete"),
                     num_walkers=int(g["n"]), num_timesteps=int(g["nsteps"]), equil_steps=int(g["equil"]),
                     chkpt_every=10 ** 6, wfn_every=10 ** 6, desc_wt_steps=int(g["desc"]), atoms=["O-H"],
                     delta_t=float(g["dt"]), potential=pot, start_structures=np.zeros((1, 1, 1)),
                     rng=oracle.InjectedNoise(int(g["seed"])), write_files=False, **kw)
    sim.run()
    return sim


def test_oracle_restates_the_reference_sample_potential():
    g = load("oh_1d")
    assert np.array_equal(oracle.oh_stretch_harm(g["probe"]), g["probe_v"])
    kw = {"mass": float(g["kw_mass"]), "freq": float(g["kw_freq"])}
    assert np.array_equal(oracle.oh_stretch_harm(g["probe"], kw), g["probe_v_kwargs"])


def test_reference_sample_potential_discrete_vs_reference():
    g = load("oh_1d")
    sim = _run_1d(g, pg.Potential_Direct(oracle.oh_stretch_harm))
    np.testing.assert_array_equal(sim.masses, g["masses"])
    assert np.array_equal(sim.walkers, g["x_final"])
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    assert len(sim.wfns) == 1
    assert np.array_equal(sim.wfns[0]["coords"], g["wfn0_coords"])
    assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])


def test_reference_sample_potential_continuous_vs_reference():
    g = load("oh_1d_cont")
    sim = _run_1d(g, pg.Potential_Direct(oracle.oh_stretch_harm), weighting="continuous",
                  cont_wt_thresh=[float(t) for t in g["thresh"]])
    x, w = sim.walkers
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(w, g["w_final"], rtol=1e-12)
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(sim._pop_vs_tau, g["pop"], rtol=1e-12)
    np.testing.assert_allclose(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"], rtol=1e-12)


def test_pot_kwargs_and_pass_timestep_vs_reference():
    g = load("oh_1d_kwargs")
    g0 = load("oh_1d")
    kw = {"mass": float(g0["kw_mass"]), "freq": float(g0["kw_freq"])}
    seen = []

    def f(cds, kwargs):
        seen.append(kwargs["timestep"])
        return oracle.oh_stretch_harm(cds, kwargs)

    pot = pg.Potential_Direct(f, pot_kwargs=dict(kw), pass_timestep=True)
    sim = _run_1d(g, pot)
    assert np.array_equal(sim.walkers, g["x_final"])
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    assert seen == list(range(int(g["nsteps"]) + 1))  # step 0's call, then one per step


@pytest.mark.parametrize("weighting", ["discrete", "continuous"])
def test_python_surface_reproduces_the_fused_step(weighting):
    p, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(31).standard_normal((3000, 3, 3))
    kw = dict(num_walkers=3000, num_timesteps=40, equil_steps=10, wfn_every=10 ** 6, desc_wt_steps=20,
              atoms=["O", "H", "H"], masses=m, delta_t=10.0, start_structures=x0, seed=5, write_files=False,
              weighting=weighting)
    if weighting == "continuous":
        kw["cont_wt_thresh"] = [0.05, 3.0]
    fused = pg.DMC_Sim(potential=pg.h2o_local_mode(), fused_steps=0, **kw)  # the per-step kernels' noise
    fused.run()
    ext = pg.DMC_Sim(potential=pg.Potential_Direct(lambda c: oracle.pes_h2o_lm(c, p)), **kw)
    ext.run()
    if weighting == "discrete":
        np.testing.assert_array_equal(ext._pop_vs_tau, fused._pop_vs_tau)
        assert np.array_equal(ext.walkers, fused.walkers)
        assert np.array_equal(ext.wfns[0]["desc_wts"], fused.wfns[0]["desc_wts"])
    else:
        (xe, we), (xf, wf) = ext.walkers, fused.walkers
        assert np.array_equal(xe, xf)
        np.testing.assert_allclose(we, wf, rtol=1e-12)
        np.testing.assert_allclose(ext._pop_vs_tau, fused._pop_vs_tau, rtol=1e-12)
    np.testing.assert_allclose(ext._vref_vs_tau, fused._vref_vs_tau, rtol=0, atol=1e-12)


class TorchHO:
    """A harmonic well written in torch: getpot_device keeps the walkers on the GPU."""

    def __init__(self, k):
        self.k = k
        self.calls = 0

    def getpot_device(self, x):
        self.calls += 1
        return 0.5 * self.k * (x * x).sum(dim=(1, 2))

    def getpot(self, cds, timeit=False):  # the reference contract, for completeness
        return 0.5 * self.k * np.sum(np.asarray(cds) ** 2, axis=(1, 2))


def test_device_tensor_potential_reproduces_the_fused_step():
    ho = oracle.ho_config()
    x0 = 0.1 * oracle.InjectedNoise(33).standard_normal((2000, 1, 3))
    kw = dict(num_walkers=2000, num_timesteps=30, equil_steps=10 ** 6, atoms=["H"], masses=ho["masses"],
              delta_t=10.0, start_structures=x0, seed=9, write_files=False)
    fused = pg.DMC_Sim(potential=pg.harmonic_oscillator(), fused_steps=0, **kw)
    fused.run()
    pot = TorchHO(ho["k"])
    ext = pg.DMC_Sim(potential=pot, **kw)
    ext.run()
    assert pot.calls == 31
    np.testing.assert_array_equal(ext._pop_vs_tau, fused._pop_vs_tau)
    assert np.array_equal(ext.walkers, fused.walkers)
    np.testing.assert_allclose(ext._vref_vs_tau, fused._vref_vs_tau, rtol=0, atol=1e-12)


def test_python_potential_population_guard_raises():
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[50:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])  # V = 2 Eh for half the walkers: the weight guard trips
    sim = pg.DMC_Sim(num_walkers=100, num_timesteps=5, equil_steps=1000, atoms=["H"], masses=ho["masses"],
                     delta_t=10.0, potential=pg.Potential_Direct(lambda c: oracle.pes_ho(c, ho["k"])),
                     start_structures=x0, seed=3, write_files=False)
    with pytest.raises(ValueError, match="Massive walker"):
        sim.run()
