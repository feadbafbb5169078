"""Host logic without a GPU: the output files and checkpoint housekeeping
(simulation_utilities/sim_archive.py, file_manager.py, sim_logger.py), the
DMC_Sim options the GPU engine refuses (pyvibdmc.py:67-98), and the loud
failure of the engine where no CUDA device is present."""
import os
import types

import numpy as np
import pytest
import torch

import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import archive


def test_save_h5_round_trip(tmp_path):
    f = str(tmp_path / "wfns" / "w_wfn_100ts.hdf5")
    archive.create_filesystem(str(tmp_path))
    for sub in ("chkpts", "wfns"):
        assert os.path.isdir(tmp_path / sub)
    x = np.arange(24.0).reshape(4, 2, 3)
    d = np.array([1.0, 0.0, 2.0, 1.0])
    path = archive.save_h5(f, ["coords", "desc_wts"], [x, d])
    assert os.path.exists(path)
    back = archive.load_h5(f)
    assert sorted(back) == ["coords", "desc_wts"]
    assert np.array_equal(back["coords"], x) and np.array_equal(back["desc_wts"], d)
    with pytest.raises(FileNotFoundError):
        archive.load_h5(str(tmp_path / "missing.hdf5"))


def _touch(p):
    os.makedirs(os.path.dirname(p), exist_ok=True)
    open(p, "wb").close()


def test_checkpoint_housekeeping(tmp_path):
    root = str(tmp_path)
    for t in (5, 10, 20):
        _touch(f"{root}/chkpts/sim_{t}.pickle")
    _touch(f"{root}/chkpts/sim_final.pickle")  # no step in the name: left alone
    _touch(f"{root}/chkpts/other_3.pickle")
    for t in (8, 30):
        _touch(f"{root}/wfns/sim_wfn_{t}ts.hdf5.npz")
    assert archive.checkpoint_step(f"{root}/chkpts/sim_20.pickle") == 20
    assert archive.checkpoint_step(f"{root}/chkpts/sim_final.pickle") is None

    archive.delete_older_checkpoints(root, "sim", 10)  # file_manager.py:29-38: steps before 10
    assert sorted(os.listdir(f"{root}/chkpts")) == ["other_3.pickle", "sim_10.pickle", "sim_20.pickle",
                                                     "sim_final.pickle"]
    archive.delete_future_checkpoints(root, "sim", 10)  # file_manager.py:11-26: steps after 10
    assert sorted(os.listdir(f"{root}/chkpts")) == ["other_3.pickle", "sim_10.pickle", "sim_final.pickle"]
    assert os.listdir(f"{root}/wfns") == ["sim_wfn_8ts.hdf5.npz"]


def test_sim_logger_writes_the_reference_lines(tmp_path):
    sim = types.SimpleNamespace(sim_name="w", cur_timestep=0, potential_info={"kind": "h2o_local_mode", "_x": 1},
                                num_walkers=100, num_timesteps=50, weighting="discrete", branch_every=1,
                                delta_t=10.0, masses=np.array([1.0, 2.0]), equil_steps=10, chkpt_every=25,
                                wfn_every=5)
    f = str(tmp_path / "w_log.txt")
    lg = archive.SimLogger(f, overwrite=True)
    lg.beginning(sim)
    z = np.zeros(4)
    h = dict(vmean=z, vmax=z, vmin=z, births=np.array([0, 0, 0, 2]), deaths=np.array([0, 0, 0, 1]),
             pop=np.array([100.0, 100.0, 100.0, 101.0]), rejected=np.array([0, 0, 0, 4]))
    lg.step_block(3, "discrete", h)  # the device history always carries `rejected`; no IS, no Metropolis line
    lg.step_block(2, "discrete", dict(h, pop_before=np.array([0, 0, 100, 0]), rejected=np.array([0, 0, 5, 0])))
    lg.finish(1.5)
    text = open(f).read()
    assert text.count("Metropolis rejected") == 1 and "Metropolis rejected 5 of 100 walkers (5.00 %)" in text
    for line in ("Simulation w starting at step 0", "\tkind: h2o_local_mode", "Num Walkers: 100",
                 "Delta Tau: 10.0 a.u.", "Time step 3", "\tWalker Births: 2", "\tWalker Deaths: 1",
                 "\tNumber of Walkers: 101", "Simulation has finished.", "Simulation took 1.5 seconds."):
        assert line in text, line
    assert "_x" not in text  # private potential attributes are not logged


@pytest.mark.parametrize("opt", [dict(imp_samp_oned=True), dict(second_impsamp_displacement=True),
                                 dict(excited_state_imp_samp=True), dict(adiabatic_dmc={"steps": 1}),
                                 dict(fixed_node={"g": 1}), dict(DEBUG_mass_change={"factor": 2}),
                                 dict(DEBUG_save_desc_wt_tracker=True), dict(DEBUG_save_before_bod=True),
                                 dict(branch_every=2, imp_samp="trial")])
def test_unsupported_reference_options_raise(opt):
    x0 = np.zeros((1, 3, 3))
    if opt.get("imp_samp") == "trial":  # branch_every > 1 is refused only with importance-sampled discrete weights
        opt = dict(opt, imp_samp=pg.h2o_gaussian_trial(device="cpu"))
    with pytest.raises(NotImplementedError):
        pg.DMC_Sim(num_walkers=10, atoms=["O", "H", "H"], potential=pg.h2o_local_mode(), start_structures=x0,
                   write_files=False, **opt)


def test_branch_every_must_be_positive():
    with pytest.raises(ValueError, match="branch_every"):
        pg.DMC_Sim(num_walkers=10, atoms=["O", "H", "H"], potential=pg.h2o_local_mode(),
                   start_structures=np.zeros((1, 3, 3)), write_files=False, branch_every=0)


def test_potential_must_be_a_gpu_potential():
    with pytest.raises(TypeError):
        pg.DMC_Sim(num_walkers=10, atoms=["O", "H", "H"], potential=object(), start_structures=np.zeros((1, 3, 3)),
                   write_files=False)


def test_walker_layout_round_trip_and_empty_input():
    from pyvibdmc_gb300.potentials import from_soa, to_soa
    x = np.arange(2 * 3 * 3, dtype=np.float64).reshape(2, 3, 3)
    s = to_soa(x, "cpu")
    assert s.shape == (9, 2) and s[4, 1].item() == x[1, 1, 1]  # component 3*atom + dim of walker i
    assert np.array_equal(from_soa(s, 2, 3), x)
    e = to_soa(np.zeros((0, 3, 3)), "cpu")
    assert e.shape == (9, 0) and from_soa(e, 0, 3).shape == (0, 3, 3)


def test_getpot_checks_the_walker_shape_first():
    with pytest.raises(ValueError, match="cds must be"):
        pg.h2o_local_mode().getpot(np.zeros((5, 2, 3)))


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")
def test_engine_fails_loudly_without_cuda():
    with pytest.raises(RuntimeError, match="CUDA device"):
        pg.DMC_Sim(num_walkers=10, atoms=["O", "H", "H"], potential=pg.h2o_local_mode(),
                   start_structures=np.zeros((1, 3, 3)), write_files=False)


# DMC_Sim keywords, defaults and order of pyvibdmc.py:67-98
REFERENCE_KEYWORDS = [
    ("sim_name", "DMC_Sim"), ("output_folder", "exSimResults"), ("weighting", "discrete"), ("num_walkers", 10000),
    ("num_timesteps", 20000), ("equil_steps", 2000), ("chkpt_every", 1000), ("wfn_every", 1000),
    ("desc_wt_steps", 100), ("atoms", []), ("delta_t", 1), ("potential", None), ("masses", None),
    ("start_structures", None), ("start_cont_wts", None), ("branch_every", 1), ("log_every", 1),
    ("cur_timestep", 0), ("cont_wt_thresh", None), ("imp_samp", None), ("imp_samp_oned", False),
    ("second_impsamp_displacement", False), ("excited_state_imp_samp", False), ("adiabatic_dmc", None),
    ("fixed_node", None), ("DEBUG_alpha", None), ("DEBUG_save_desc_wt_tracker", None),
    ("DEBUG_save_training_every", None), ("DEBUG_save_before_bod", False), ("DEBUG_mass_change", None)]


def test_dmc_sim_keeps_the_reference_constructor():
    import inspect
    params = list(inspect.signature(pg.DMC_Sim.__init__).parameters.values())[1:]
    positional = [p for p in params if p.kind == p.POSITIONAL_OR_KEYWORD]
    assert [(p.name, p.default) for p in positional] == REFERENCE_KEYWORDS
    assert all(p.kind == p.KEYWORD_ONLY for p in params[len(positional):])  # extras only by keyword
    for name in ("DMC_Sim", "dmc_restart", "Constants", "Potential_GPU", "ImpSampManager_GPU", "NN_Potential_GPU",
                 "HarmonicAnalysis", "InitialConditioner"):
        assert hasattr(pg, name), name


def _golden(name):
    with np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("name", ["restart_oh_cont", "restart_h2o_disc"])
def test_reference_checkpoints_load_without_the_reference(name, tmp_path):
    from pyvibdmc_gb300 import archive
    g = _golden(name)
    path = tmp_path / "c.pickle"
    path.write_bytes(g["pickle"].tobytes())
    st = archive.load_checkpoint(str(path))
    assert isinstance(st, archive.ReferenceCheckpoint)
    assert int(st.cur_timestep) == int(g["chkpt_step"]) and st.sim_name == name
    assert st._walker_coords.ndim == 3 and st._desc_wt  # saved inside a descendant-weighting window
    assert len(st._who_from) == len(st._walker_coords)


def test_checkpoint_loader_refuses_foreign_globals(tmp_path):
    import pickle
    from pyvibdmc_gb300 import archive
    path = tmp_path / "evil.pickle"
    with open(path, "wb") as fh:
        pickle.dump({"f": os.path.join}, fh, protocol=4)  # a function global: not checkpoint data
    with pytest.raises(pickle.UnpicklingError):
        archive.load_checkpoint(str(path))


@pytest.mark.skipif(not os.environ.get("GBDMC_REFERENCE"), reason="set GBDMC_REFERENCE to a reference checkout")
def test_the_reference_shipped_restart_fixture_loads():
    # the reference's own restart fixture (sample_sim_data/chkpts/pytest_364.pickle,
    # used by tests/test_pyvibdmc.py:152-169)
    from pyvibdmc_gb300 import archive
    st = archive.load_checkpoint(os.path.join(os.environ["GBDMC_REFERENCE"],
                                              "pyvibdmc/sample_sim_data/chkpts/pytest_364.pickle"))
    assert int(st.cur_timestep) == 364 and st.weighting == "continuous" and st._walker_coords.shape == (5000, 1, 1)
    assert list(st._atm_nums) == [-1] and st.cont_wt_thresh == [0.002, 15]
