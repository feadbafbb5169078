"""The multi-step kernel (gbdmc_sim_run: many plain DMC steps per launch, the
walkers resident in shared memory, the grid-wide reduction of a step behind
the next step's move) against its walk replayed by the per-step kernels
(gbdmc_sim_step on the same lineage-keyed Philox noise, tests/lineage_harness.py):
populations, walkers and ancestor ids bit for bit, vref within 1e-12 Eh (the
multi-step kernel adds the per-block sums in another order)."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
import pyvibdmc_gb300 as pg
from lineage_harness import replay

pytestmark = pytest.mark.gpu
K = 64  # steps per launch (fused_steps)


def _fused(**kw):
    sim = pg.DMC_Sim(write_files=False, fused_steps=K, **kw)
    sim.run()
    return sim


def _who(sim):
    sim._compact()
    n = int(sim._read_ctrl().n)
    return sim._bufs[sim._cur]["who"][:n].cpu().numpy()


def _same(a, b, steps, who=True):
    """a: the multi-step kernel's run, b: the replay."""
    assert a._multi_used
    pa = a._hist["pop"].cpu().numpy()[:steps]
    pb = b._hist["pop"].cpu().numpy()[:steps]
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_allclose(a._hist["vref"].cpu().numpy()[:steps], b._hist["vref"].cpu().numpy()[:steps],
                               rtol=0, atol=1e-12)
    assert np.array_equal(a.walkers, b.walkers)
    if who:
        assert np.array_equal(_who(a), _who(b))


@pytest.mark.parametrize("n", [31, 33, 1025, 20000])
def test_multi_step_kernel_follows_its_replayed_walk_h2o(n):
    p, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(5).standard_normal((n, 3, 3))
    steps = 200 if n > 1000 else 100
    kw = dict(num_walkers=n, num_timesteps=steps, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m,
              delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=17)
    a = _fused(**kw)
    b, stopped = replay(steps, **kw)
    assert not stopped
    _same(a, b, steps)


@pytest.mark.parametrize("system", ["ho", "dimer", "ps"])
def test_multi_step_kernel_follows_its_replayed_walk(system):
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
    kw.update(num_timesteps=150, equil_steps=10 ** 6, delta_t=10.0, seed=23)
    a = _fused(**kw)
    b, stopped = replay(150, **kw)
    assert not stopped
    _same(a, b, 150)


def test_descendant_windows_split_the_launches_not_the_walk():
    """Events end launches: a descendant-weighting window from step 30 to 80
    gives launches [0, 30), [30, 80), [80, 144), [144, 200); the lineage keys
    travel with the walkers, so the walk is the replayed one, and the window's
    descendant weights come from the ancestor ids the kernel carries."""
    p, m = oracle.h2o_config()
    n = 3000
    x0 = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(15).standard_normal((n, 3, 3))
    kw = dict(num_walkers=n, num_timesteps=200, equil_steps=30, wfn_every=1000, desc_wt_steps=50,
              atoms=["O", "H", "H"], masses=m, delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0,
              seed=19)
    a = _fused(**kw)
    assert a._multi_launches == 4
    b, _ = replay(200, **dict(kw, equil_steps=10 ** 6))
    _same(a, b, 200, who=False)  # the window restarts the ancestor ids at step 30
    assert len(a.wfns) == 1
    d = a.wfns[0]["desc_wts"]
    assert d.sum() == int(a._hist["pop"].cpu().numpy()[79]) and len(d) == len(a.wfns[0]["coords"])


def test_copies_that_pile_up_in_a_few_blocks_are_split_evenly():
    """The walkers of the first blocks sit at the bottom of a harmonic well and
    the others high up its side, so the first blocks' walkers multiply by a
    fifth every step while the population stays near N0: the runs are split
    evenly again whenever the largest would take another warp, one launch runs
    all 40 steps, and the walk is the replayed one."""
    ho = oracle.ho_config()
    n = 2000
    x0 = np.zeros((n, 1, 3))
    x0[200:, 0, 0] = np.sqrt(2 * 0.02 / ho["k"])  # V = 0.02 Eh
    kw = dict(num_walkers=n, num_timesteps=40, equil_steps=10 ** 6, atoms=["H"], masses=ho["masses"],
              delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=29)
    a = _fused(**kw)
    b, _ = replay(40, **kw)
    _same(a, b, 40)
    assert a._multi_launches == 1


def test_multi_step_guards_stop_with_the_moved_walkers():
    """A tripped guard stops the launch at that step with the moved, unbranched
    walkers in the output, as the per-step kernels leave them."""
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])
    x0[37, 0, 0] = 0.0  # a huge weight for walker 37 on the first step
    kw = dict(num_walkers=100, num_timesteps=20, equil_steps=1000, atoms=["H"], masses=ho["masses"],
              delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=3)
    sim = pg.DMC_Sim(write_files=False, fused_steps=K, **kw)
    with pytest.raises(ValueError, match="Massive walker"):
        sim.run()
    c = sim._read_ctrl()
    b, stopped = replay(20, **kw)
    assert stopped
    cb = b._read_ctrl()
    assert int(c.n) == int(cb.n) == 100 and int(c.err_step) == int(cb.err_step) == 0
    assert int(c.status) == int(cb.status)
    assert np.array_equal(sim._coords_host(), b._coords_host())


def test_sim_run_entry_point_checks_its_arguments():
    L = pg._capi.load()
    s = pg._capi.Sim(natoms=3, weighting=pg._capi.CONTINUOUS, ld=1000, n0=100)
    s.pes.kind, s.pes.natoms = pg._capi.PES_H2O_LM, 3
    w = pg._capi.Walkers(x=16, v=16)
    rc = L.gbdmc_sim_run(C.byref(s), C.byref(w), C.byref(pg._capi.Walkers(x=32, v=32)), C.c_void_p(16),
                         C.c_void_p(16), 10, 4, None)
    assert rc == pg._capi.ERR_ARG and b"discrete" in L.gbdmc_last_error()
    torch.cuda.synchronize()


@pytest.mark.parametrize("mode", ["philox32", "philox64"])
def test_lineage_noise_matches_the_oracle_stream(mode):
    """gbdmc_lineage_noise (the multi-step kernel's noise) against the oracle's
    restatement of the lineage-keyed Philox stream: every deviate (8 fp32 ulps
    in philox32, whose log/sin/cos differ from NumPy's in the last bits; 1e-12
    in philox64) and every branching uniform exactly."""
    from oracle.philox_oracle import philox_normals, lineage_key
    L = pg._capi.load()
    n, seed, step = 4096, 0x0123456789ABCDEF, 77
    keys = lineage_key(np.arange(n, dtype=np.uint64) * np.uint64(7919), np.arange(n) % 3, 12)
    s = pg._capi.Sim(natoms=3, seed=seed, replica_id=5)
    s.noise_mode = pg._capi.NOISE_PHILOX32 if mode == "philox32" else pg._capi.NOISE_PHILOX64
    kd = torch.as_tensor(keys.view(np.int64), device="cuda")
    z = torch.empty((9, n), dtype=torch.float64, device="cuda")
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    pg._capi.check(L.gbdmc_lineage_noise(C.byref(s), C.c_void_p(kd.data_ptr()), n, step, C.c_void_p(z.data_ptr()), n,
                                         C.c_void_p(u.data_ptr()), None))
    torch.cuda.synchronize()
    zr, st = philox_normals(seed, step, keys, 9, mode, replica=5, lineage=True)
    tol = dict(rtol=1e-6, atol=1e-6) if mode == "philox32" else dict(rtol=0, atol=1e-12)
    np.testing.assert_allclose(z.cpu().numpy(), zr, **tol)
    np.testing.assert_array_equal(u.cpu().numpy(), st.uniform53())


@pytest.mark.parametrize("pad", [0, 64])
def test_host_walker_entry_point_follows_the_device_resident_walk(pad):
    """gbdmc_sim_run_host -- the walkers in page-locked host memory between
    calls, one call per 50-step window -- against DMC_Sim's device-resident
    launches of the same walk: vref history, populations and walkers bit for
    bit (the lineage keys travel through the host arrays).  pad 0: host arrays
    with the device's leading dimension, read by the launch in place; pad 64:
    another leading dimension, copied in first."""
    p, m = oracle.h2o_config()
    n = 3000
    x0 = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(41).standard_normal((n, 3, 3))
    kw = dict(num_walkers=n, num_timesteps=200, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m, delta_t=10.0,
              potential=pg.h2o_local_mode(), start_structures=x0, seed=31)
    a = pg.DMC_Sim(write_files=False, fused_steps=50, **kw)  # the same launch boundaries: the same vref sums
    a.run()
    assert a._multi_used
    b = pg.DMC_Sim(write_files=False, fused_steps=50, **kw)
    b._init_device()
    L = pg._capi.load()
    ld = int(b._sim.ld)
    hld = ld + pad
    scratch = torch.zeros(L.gbdmc_sim_run_scratch_bytes(b.capacity), dtype=torch.uint8, device="cuda")
    hx = torch.zeros((9, hld), dtype=torch.float64).pin_memory()
    hv = torch.zeros(hld, dtype=torch.float64).pin_memory()
    hw = torch.zeros(hld, dtype=torch.int32).pin_memory()
    hk = torch.zeros(hld, dtype=torch.int64).pin_memory()
    hc = torch.zeros(C.sizeof(pg._capi.Ctrl), dtype=torch.uint8).pin_memory()
    hh = torch.zeros((2, 50), dtype=torch.float64).pin_memory()
    b0, b1 = b._bufs[b._cur], b._bufs[1 - b._cur]
    n0 = int(b._read_ctrl().n)
    hx[:, :n0].copy_(b0["x"][:, :n0])
    hw[:n0].copy_(b0["who"][:n0])
    hk[:n0].copy_(b0["key"][:n0])
    hc.copy_(b._ctrl)
    torch.cuda.synchronize()
    ctrl = pg._capi.Ctrl.from_address(hc.data_ptr())
    host = pg._capi.HostWalkersC(x=hx.data_ptr(), v=hv.data_ptr(), who=hw.data_ptr(), key=hk.data_ptr(), ld=hld)
    ws, wd = b._walker_struct(b0, False), b._walker_struct(b1, False)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    vref, pop = [], []
    for _ in range(4):
        step = int(ctrl.step)
        pg._capi.check(L.gbdmc_sim_run_host(C.byref(b._sim), C.byref(host), C.byref(ws), C.byref(wd),
                                            C.c_void_p(b._ctrl.data_ptr()), C.byref(ctrl),
                                            C.c_void_p(scratch.data_ptr()), step + 50, 50, C.c_void_p(hh.data_ptr()),
                                            stream))
        assert ctrl.status == 0 and ctrl.step == step + 50
        vref.append(hh[0].numpy().copy())
        pop.append(hh[1].numpy().copy())
    assert np.array_equal(np.concatenate(vref), a._hist["vref"].cpu().numpy()[:200])
    assert np.array_equal(np.concatenate(pop), a._hist["pop"].cpu().numpy()[:200])
    nn = int(ctrl.n)
    xb = np.ascontiguousarray(hx[:, :nn].numpy().T).reshape(nn, 3, 3)
    assert np.array_equal(xb, a.walkers)
    assert np.array_equal(hw[:nn].numpy(), _who(a))
