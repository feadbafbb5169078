"""The potential managers for Python potentials (pyvibdmc_gb300.potential_manager),
with the reference's names and arguments (potential_manager.py:12-253): the
function is found by file and name, pot_kwargs is its second argument,
pass_timestep counts the calls, timeit returns (v, seconds), and the pool
splits the walkers into num_cores chunks.  CPU only."""
import os
import textwrap

import numpy as np
import pytest

import pyvibdmc_gb300 as pg

MODULE = textwrap.dedent('''
    import numpy as np
    SCALE = float(open("scale.txt").read())   # read at import, relative to the module's directory

    def harm(cds):
        return SCALE * np.sum(cds * cds, axis=(1, 2))

    def harm_kw(cds, kw):
        return kw["k"] * np.sum(cds * cds, axis=(1, 2)) + kw.get("timestep", 0)

    def harm_file(cds):
        return float(open("scale.txt").read()) * np.sum(cds * cds, axis=(1, 2))

    def nn(cds, model, kw=None):
        return model["w"] * np.sum(cds, axis=(1, 2)) + (0 if kw is None else kw["b"])
''')


@pytest.fixture()
def potdir(tmp_path):
    d = tmp_path / "pots"
    d.mkdir()
    (d / "mypot.py").write_text(MODULE)
    (d / "scale.txt").write_text("0.5")
    return str(d)


def _cds(n=10, a=2):
    return np.random.default_rng(0).normal(size=(n, a, 3))


def test_potential_direct_kwargs_timestep_and_timeit():
    calls = []

    def f(cds, kw):
        calls.append(dict(kw))
        return np.full(len(cds), kw["timestep"], dtype=float)

    pot = pg.Potential_Direct(f, pot_kwargs={"k": 1.0}, pass_timestep=True)
    assert pot.pot_kwargs == {"k": 1.0, "timestep": 0}
    assert pot.getpot(_cds())[0] == 0.0
    v, secs = pot.getpot(_cds(), timeit=True)
    assert v[0] == 1.0 and secs >= 0.0
    assert [c["timestep"] for c in calls] == [0, 1] and pot.pot_kwargs["timestep"] == 2
    plain = pg.Potential_Direct(lambda c: np.zeros(len(c)))
    assert plain.getpot(_cds(4)).shape == (4,)


def test_potential_nomp_imports_by_file_and_name(potdir):
    x = _cds()
    pot = pg.Potential_NoMP("harm", potdir, "mypot.py")
    np.testing.assert_array_equal(pot.getpot(x), 0.5 * np.sum(x * x, axis=(1, 2)))
    here = os.getcwd()
    with pytest.raises(FileNotFoundError):  # reads scale.txt relative to the working directory
        pg.Potential_NoMP("harm_file", potdir, "mypot.py").getpot(x)
    assert os.getcwd() == here
    chd = pg.Potential_NoMP("harm_file", potdir, "mypot.py", ch_dir=True)
    np.testing.assert_array_equal(chd.getpot(x), 0.5 * np.sum(x * x, axis=(1, 2)))
    assert os.getcwd() == here
    kw = pg.Potential_NoMP("harm_kw", potdir, "mypot.py", pot_kwargs={"k": 2.0}, pass_timestep=True)
    v0, v1 = kw.getpot(x), kw.getpot(x)
    np.testing.assert_allclose(v1 - v0, np.ones(len(x)), rtol=0, atol=1e-12)


def test_nn_potential_passes_the_model(potdir):
    x = _cds()
    pot = pg.NN_Potential("nn", potdir, "mypot.py", model={"w": 3.0})
    np.testing.assert_array_equal(pot.getpot(x), 3.0 * np.sum(x, axis=(1, 2)))
    pot = pg.NN_Potential("nn", potdir, "mypot.py", model={"w": 1.0}, pot_kwargs={"b": 5.0})
    np.testing.assert_array_equal(pot.getpot(x), np.sum(x, axis=(1, 2)) + 5.0)


def test_pool_potential_splits_over_worker_processes(potdir):
    x = _cds(37)
    pot = pg.Potential("harm_kw", potdir, "mypot.py", num_cores=2, pot_kwargs={"k": 0.25}, pass_timestep=True)
    try:
        v0 = pot.getpot(x)
        v1, secs = pot.getpot(x, timeit=True)
        np.testing.assert_allclose(v0, 0.25 * np.sum(x * x, axis=(1, 2)), rtol=0, atol=0)
        np.testing.assert_allclose(v1 - v0, np.ones(len(x)), rtol=0, atol=1e-12)
        assert pot.pool is not None and secs >= 0.0
    finally:
        pot.mp_close()


def test_engine_refuses_an_object_without_getpot():
    with pytest.raises(TypeError, match="getpot"):
        pg.DMC_Sim(num_walkers=10, atoms=["H"], potential=object(), start_structures=np.zeros((1, 1, 3)),
                   write_files=False)
