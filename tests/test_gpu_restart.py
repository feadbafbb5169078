"""Checkpoint and restart (pyvibdmc.py:892-965): a run written to disk,
reloaded with dmc_restart and extended, follows the trajectory of the same
run done in one go.  The deviates are keyed by (seed, step, walker), so the
populations and walkers agree bit for bit; vref agrees to 1e-12 Eh (the
restart recomputes the first vref from the saved walkers, which sums them in
another order)."""
import numpy as np
import pytest

import oracle
import pyvibdmc_gb300 as pg

pytestmark = pytest.mark.gpu

T = 60


def _kw(tmp_path, name, nsteps, **kw):
    p, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium(p)[None] + 0.08 * oracle.InjectedNoise(11).standard_normal((3000, 3, 3))
    return dict(sim_name=name, output_folder=str(tmp_path / name), num_walkers=3000, num_timesteps=nsteps,
                equil_steps=10 ** 6, wfn_every=10 ** 6, desc_wt_steps=1, atoms=["O", "H", "H"], masses=m,
                delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=7, **kw)


def _same(c, a):
    np.testing.assert_array_equal(c._pop_vs_tau, a._pop_vs_tau)
    np.testing.assert_allclose(c._vref_vs_tau, a._vref_vs_tau, rtol=0, atol=1e-12)
    assert np.array_equal(c.walkers, a.walkers)


@pytest.fixture(scope="module")
def whole(tmp_path_factory):
    a = pg.DMC_Sim(**_kw(tmp_path_factory.mktemp("a"), "a", T, chkpt_every=10 ** 6, write_files=False))
    a.run()
    return a


def test_restart_after_a_finished_run(tmp_path, whole):
    b = pg.DMC_Sim(**_kw(tmp_path, "b", 25, chkpt_every=10 ** 6, write_files=True))
    b.run()
    c = pg.dmc_restart(pg.h2o_local_mode(), str(tmp_path / "b"), "b", additional_timesteps=T - 25)
    assert c.cur_timestep == 25 and c.num_timesteps == T
    c.run()
    _same(c, whole)


def test_restart_from_a_checkpoint_of_an_interrupted_run(tmp_path, whole, monkeypatch):
    b = pg.DMC_Sim(**_kw(tmp_path, "b", T, chkpt_every=20, write_files=True))
    run_steps = b._run_steps

    def crash_at_40(n):  # the host side fails before step 40 (after the checkpoint of step 40)
        if b.cur_timestep == 40:
            raise RuntimeError("interrupted")
        return run_steps(n)

    monkeypatch.setattr(b, "_run_steps", crash_at_40)
    with pytest.raises(RuntimeError, match="interrupted"):
        b.run()
    c = pg.dmc_restart(pg.h2o_local_mode(), str(tmp_path / "b"), "b")
    assert c.cur_timestep == 40
    c.run()
    _same(c, whole)


@pytest.mark.parametrize("weighting", ["discrete", "continuous"])
def test_run_writes_the_reference_files(tmp_path, weighting):
    """sim_info, wave functions, checkpoint and log under output_folder, with
    the reference's names and keys (pyvibdmc.py:856-872, 897-922)."""
    import os

    from pyvibdmc_gb300 import archive

    kw = _kw(tmp_path, "f", 30, chkpt_every=15, write_files=True)
    kw.update(equil_steps=10, wfn_every=10, desc_wt_steps=5, weighting=weighting)
    s = pg.DMC_Sim(**kw)
    s.run()
    out = str(tmp_path / "f")
    info = archive.load_h5(f"{out}/f_sim_info.hdf5")
    assert sorted(info) == ["atomic_masses", "atomic_nums", "pop_vs_tau", "vref_vs_tau"]
    np.testing.assert_array_equal(info["vref_vs_tau"][:, 0], np.arange(30) * 10.0)
    np.testing.assert_array_equal(info["vref_vs_tau"][:, 1], s._vref_vs_tau)
    np.testing.assert_array_equal(info["pop_vs_tau"][:, 1], s._pop_vs_tau)
    assert [w["start"] for w in s.wfns] == [10, 20]
    keys = ["coords", "desc_wts"] + (["parent_wts"] if weighting == "continuous" else [])
    for w in s.wfns:
        f = archive.load_h5(f"{out}/wfns/f_wfn_{w['start']}ts.hdf5")
        assert sorted(f) == sorted(keys)
        for k in keys:
            np.testing.assert_array_equal(f[k], w[k])
        if weighting == "discrete":  # every walker at the window's end descends from one parent
            assert w["desc_wts"].sum() == s._pop_vs_tau[w["start"] + 4]
    assert sorted(os.listdir(f"{out}/chkpts")) == ["f_29.pickle"]
    assert "Simulation has finished." in open(f"{out}/f_log.txt").read()


def _golden(name):
    import os
    with np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", ["restart_oh_cont", "restart_h2o_disc"])
def test_restart_from_a_checkpoint_the_reference_wrote(name, tmp_path):
    """dmc_restart reads the reference's own checkpoint (its pickled DMC_Sim, written
    by the unmodified reference) and continues it as the reference's dmc_restart
    does: the run restarted here matches the reference's restarted run on the same
    deviates -- walkers bit for bit, weights, vref and descendant weights of the
    window left open in the checkpoint within 1e-12."""
    g = _golden(name)
    folder = tmp_path / name
    (folder / "chkpts").mkdir(parents=True)
    (folder / "chkpts" / f"{name}_{int(g['chkpt_step'])}.pickle").write_bytes(g["pickle"].tobytes())
    if name == "restart_oh_cont":
        pot = pg.Potential_Direct(oracle.oh_stretch_harm)
    else:
        p, _ = oracle.h2o_config()
        pot = pg.Potential_Direct(lambda c: oracle.pes_h2o_lm(c, p))
    sim = pg.dmc_restart(pot, str(folder), name, additional_timesteps=int(g["additional"]),
                         rng=oracle.InjectedNoise(int(g["seed2"])), write_files=False)
    assert sim.cur_timestep == int(g["chkpt_step"])
    sim.run()
    if sim.weighting == "continuous":
        x, w = sim.walkers
        np.testing.assert_allclose(w, g["w_final"], rtol=1e-12)
        np.testing.assert_allclose(sim._pop_vs_tau, g["pop"], rtol=1e-12)
        np.testing.assert_allclose(sim.wfns[0]["parent_wts"], g["wfn0_parent_wts"], rtol=1e-12)
        np.testing.assert_allclose(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"], rtol=1e-12)
    else:
        x = sim.walkers
        np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
        assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    assert np.array_equal(sim.wfns[0]["coords"], g["wfn0_coords"])
