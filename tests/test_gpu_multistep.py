"""The multi-step kernel (gbdmc_sim_run: many plain DMC steps per launch, the
walkers resident in shared memory, one grid barrier per step) against the
per-step kernels (gbdmc_sim_step).  Both draw the same Philox deviates and
branching uniforms, so the trajectories agree: populations, walkers,
ancestor indices and descendant weights bit for bit, vref within 1e-12 Eh
(the multi-step kernel sums the per-block partials in another order)."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
import pyvibdmc_gb300 as pg

pytestmark = pytest.mark.gpu


def _pair(**kw):
    runs = []
    for fused in (64, 0):
        sim = pg.DMC_Sim(write_files=False, fused_steps=fused, **kw)
        sim.run()
        runs.append(sim)
    return runs


def _same(a, b):
    np.testing.assert_array_equal(a._pop_vs_tau, b._pop_vs_tau)
    np.testing.assert_allclose(a._vref_vs_tau, b._vref_vs_tau, rtol=0, atol=1e-12)
    assert np.array_equal(a.walkers, b.walkers)


@pytest.mark.parametrize("n", [31, 33, 1025, 20000])
def test_multi_step_kernel_follows_the_per_step_trajectory_h2o(n):
    p, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(5).standard_normal((n, 3, 3))
    steps = 200 if n > 1000 else 100
    a, b = _pair(num_walkers=n, num_timesteps=steps, equil_steps=30, wfn_every=1000, desc_wt_steps=50,
                 atoms=["O", "H", "H"], masses=m, delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0,
                 seed=17)
    assert a._multi_used and not b._multi_used
    _same(a, b)
    assert np.array_equal(a.wfns[0]["desc_wts"], b.wfns[0]["desc_wts"])


@pytest.mark.parametrize("system", ["ho", "dimer", "ps"])
def test_multi_step_kernel_follows_the_per_step_trajectory(system):
    if system == "ho":
        ho = oracle.ho_config()
        kw = dict(atoms=["H"], masses=ho["masses"], potential=pg.harmonic_oscillator(),
                  start_structures=0.1 * oracle.InjectedNoise(6).standard_normal((5000, 1, 3)), num_walkers=5000)
    elif system == "dimer":
        dm = [pg.Constants.mass(a) for a in ("O", "H", "H", "O", "H", "H")]
        kw = dict(atoms=["O", "H", "H"] * 2, masses=dm, potential=pg.water_dimer(),
                  start_structures=pg.WATER_DIMER_EQ[None], num_walkers=3000)
    else:
        _, m = oracle.h2o_config()
        x0 = np.array([[0.0, 0.0, 0.0], [1.81, 0.0, 0.0], [-0.45, 1.75, 0.0]])
        kw = dict(atoms=["O", "H", "H"], masses=m, potential=pg.partridge_schwenke(), num_walkers=4000,
                  start_structures=x0[None] + 0.03 * oracle.InjectedNoise(7).standard_normal((4000, 3, 3)))
    a, b = _pair(num_timesteps=150, equil_steps=10 ** 6, delta_t=10.0, seed=23, **kw)
    _same(a, b)


def test_copies_that_pile_up_in_a_few_blocks_are_split_evenly():
    """The walkers of the first blocks sit at the bottom of a harmonic well and the
    others high up its side, so the first blocks' walkers multiply by a fifth every
    step while the population stays near N0: every step splits the branched
    population evenly over the blocks again, one launch runs all 40 steps, and
    the trajectory is the per-step kernels'."""
    ho = oracle.ho_config()
    n = 2000
    x0 = np.zeros((n, 1, 3))
    x0[200:, 0, 0] = np.sqrt(2 * 0.02 / ho["k"])  # V = 0.02 Eh
    a, b = _pair(num_walkers=n, num_timesteps=40, equil_steps=10 ** 6, atoms=["H"], masses=ho["masses"],
                 delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=29)
    _same(a, b)
    assert a._multi_launches == 1


def test_multi_step_guards_stop_with_the_moved_walkers():
    """A tripped guard stops the launch at that step with the moved, unbranched
    walkers in the output, as the per-step kernels leave them."""
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])
    x0[37, 0, 0] = 0.0  # a huge weight for walker 37 on the first step
    out = []
    for fused in (64, 0):
        sim = pg.DMC_Sim(num_walkers=100, num_timesteps=20, equil_steps=1000, atoms=["H"], masses=ho["masses"],
                         delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=3,
                         write_files=False, fused_steps=fused)
        with pytest.raises(ValueError, match="Massive walker"):
            sim.run()
        c = sim._read_ctrl()
        out.append((int(c.n), int(c.err_step), sim._coords_host()))
    assert out[0][0] == out[1][0] == 100 and out[0][1] == out[1][1] == 0
    assert np.array_equal(out[0][2], out[1][2])


def test_sim_run_entry_point_checks_its_arguments():
    L = pg._capi.load()
    s = pg._capi.Sim(natoms=3, weighting=pg._capi.CONTINUOUS, ld=1000, n0=100)
    s.pes.kind, s.pes.natoms = pg._capi.PES_H2O_LM, 3
    w = pg._capi.Walkers(x=16, v=16)
    rc = L.gbdmc_sim_run(C.byref(s), C.byref(w), C.byref(pg._capi.Walkers(x=32, v=32)), C.c_void_p(16),
                         C.c_void_p(16), 10, 4, None)
    assert rc == pg._capi.ERR_ARG and b"discrete" in L.gbdmc_last_error()
    torch.cuda.synchronize()
