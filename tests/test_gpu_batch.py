"""Batched replicas (gbdmc_batch_*): every replica of a batch is the same
simulation the single-replica engine runs with that replica's Philox stream
and tile width, so their vref histories agree bit for bit; the autotuner picks
a tile width per walker-count bucket; replica ZPEs agree with each other
within their blocking error bars."""
import numpy as np
import pytest

import oracle
import pyvibdmc_gb300 as pg

pytestmark = pytest.mark.gpu


def starts(ns, seed):
    p, _ = oracle.h2o_config()
    eq = oracle.h2o_equilibrium(p)
    g = np.random.default_rng(seed)
    return [eq[None] + 0.05 * g.standard_normal((n, 3, 3)) for n in ns]


@pytest.mark.parametrize("imp", [False, True])
def test_batch_replicas_equal_single_runs(imp):
    _, m = oracle.h2o_config()
    ns = [700, 1800, 5000]
    x0 = starts(ns, 3)
    trial = pg.h2o_gaussian_trial() if imp else None
    nsteps = 40
    b = pg.DMC_Batch(pg.h2o_local_mode(), ns, x0, m, 10.0, nsteps, imp_samp=trial, seed=99, block_threads=64,
                     graph_steps=8)
    b.init()
    b.run(nsteps)
    vb = b.vref_history()
    pb = b.pop_history()
    for r, n in enumerate(ns):
        sim = pg.DMC_Sim(num_walkers=n, num_timesteps=nsteps, equil_steps=10 ** 6, atoms=["O", "H", "H"],
                         masses=m, delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0[r], seed=99,
                         replica_id=r, block_threads=64, imp_samp=trial, capacity=b.caps[r], write_files=False)
        sim.run()
        assert np.array_equal(sim._pop_vs_tau, pb[r]), f"replica {r} population differs"
        assert np.array_equal(sim._vref_vs_tau, vb[r]), f"replica {r} vref differs"
        assert np.array_equal(sim.walkers, b.walkers(r)), f"replica {r} walkers differ"


def test_batch_autotune_and_zpe_consistency():
    _, m = oracle.h2o_config()
    rng = np.random.default_rng(0)
    ns = [int(v) for v in rng.integers(1000, 20001, size=12)]
    p, _ = oracle.h2o_config()
    b = pg.DMC_Batch(pg.h2o_local_mode(), ns, oracle.h2o_equilibrium(p)[None], m, 10.0, 1500, seed=5,
                     start_noise=0.05, buckets=(4096, 1 << 40))
    b.init()
    tune = b.autotune(steps_per_candidate=3)
    gl, gus, gtable = tune.pop("graph_steps")
    assert gl in gtable and set(gtable) == {8, 16, 32} and b.graph_steps == gl and gus > 0
    assert len(tune) == len(b.buckets)
    for tpb, us, table in tune.values():
        assert tpb in pg.DMC_Batch.CANDIDATES and us > 0
    b.run(1500 - b.step)
    z, e = b.zpe(start=400)
    zbar = np.average(z, weights=1 / e ** 2)
    chi2 = np.sum(((z - zbar) / e) ** 2)
    assert chi2 / (len(z) - 1) < 4.0, (z, e)
    # sanity: local-mode water ZPE well above 4000 cm^-1 and below 5500 cm^-1
    assert 4000 < zbar < 5500
    assert b.walker_steps(0, b.step) > 0
