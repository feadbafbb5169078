"""GPU parity: libgbdmc kernels (through the C ABI) against the oracle and the
golden fixtures of the reference engine.

Tolerances: coordinates, populations, branch counts and descendant weights
bit-exact; potentials 1e-12 Eh; vref 1e-12 Eh; importance-sampled runs 1e-10
(the adjoint derivatives differ from the reference's NumPy chain rule in
the last bits, which moves proposals by ~1e-16 bohr)."""
import ctypes as C
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


def geoms(n, seed=3, scale=0.08):
    p, _ = oracle.h2o_config()
    return oracle.h2o_equilibrium(p)[None] + scale * oracle.InjectedNoise(seed).standard_normal((n, 3, 3))


def dimer_geoms(n, seed=4):
    x = geoms(2 * n, seed)
    return np.concatenate([x[:n], x[n:] + np.array([5.6, 0.2, -0.3])], axis=1)


# ---------------------------------------------------------------- kernels
@pytest.mark.parametrize("n", [1, 31, 33, 1025, 20000])
def test_h2o_pes_matches_oracle(n):
    p, _ = oracle.h2o_config()
    x = geoms(n)
    v = pg.h2o_local_mode().getpot(x)
    np.testing.assert_allclose(v, oracle.pes_h2o_lm(x, p), rtol=0, atol=1e-12)


def test_getpot_keeps_the_plugin_contract():
    # potential_manager.py:71-99: (N, A, 3) bohr -> (N,) float64 hartree, or (v, seconds) with timeit
    pot = pg.h2o_local_mode()
    x = geoms(100)
    v = pot.getpot(x)
    v2, secs = pot.getpot(x, timeit=True)
    assert v.shape == (100,) and v.dtype == np.float64
    assert np.array_equal(v, v2) and secs >= 0.0
    assert pot.getpot(np.zeros((0, 3, 3))).shape == (0,)  # no walkers
    assert vars(pot)["kind"] == "h2o_local_mode"  # the reference engine logs vars(potential)


def test_ho_and_dimer_pes_match_oracle():
    ho = oracle.ho_config()
    x1 = 0.3 * oracle.InjectedNoise(5).standard_normal((777, 1, 3))
    np.testing.assert_allclose(pg.harmonic_oscillator().getpot(x1), oracle.pes_ho(x1, ho["k"]), rtol=1e-14, atol=0)
    x3 = 0.3 * oracle.InjectedNoise(6).standard_normal((300, 3, 3))
    pot3 = pg.Potential_GPU("harmonic_oscillator", {"k": ho["k"]}, natoms=3)
    np.testing.assert_allclose(pot3.getpot(x3), oracle.pes_ho(x3, ho["k"]), rtol=1e-14, atol=0)
    pd, _ = oracle.dimer_config()
    xd = dimer_geoms(513)
    np.testing.assert_allclose(pg.water_dimer().getpot(xd), oracle.pes_dimer(xd, pd), rtol=0, atol=1e-12)


def test_pes_adjoint_matches_oracle_fd_and_autograd():
    p, _ = oracle.h2o_config()
    x = geoms(257)
    pot = pg.h2o_local_mode()
    v, g = pot.getgrad(x)
    np.testing.assert_allclose(g, oracle.grad_h2o_lm(x, p), rtol=0, atol=1e-12)
    # central finite differences, h = 1e-3 bohr as the reference's ImpSamp.finite_diff
    h = 1e-3
    for a in range(3):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[:, a, d] += h
            xm[:, a, d] -= h
            fd = (pot.getpot(xp) - pot.getpot(xm)) / (2 * h)
            np.testing.assert_allclose(g[:, a, d], fd, rtol=0, atol=2e-6)
    # torch autograd of a float64 torch restatement of the PES
    xt = torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
    d1 = xt[:, 1] - xt[:, 0]
    d2 = xt[:, 2] - xt[:, 0]
    r1, r2 = d1.norm(dim=1), d2.norm(dim=1)
    th = torch.acos((d1 * d2).sum(1) / (r1 * r2))
    vt = (p["De"] * (1 - torch.exp(-p["a"] * (r1 - p["re"]))) ** 2 + p["De"] * (1 - torch.exp(-p["a"] * (r2 - p["re"]))) ** 2
          + 0.5 * p["ktheta"] * (th - p["theta_e"]) ** 2 + p["krr"] * (r1 - p["re"]) * (r2 - p["re"]))
    gt, = torch.autograd.grad(vt.sum(), xt)
    np.testing.assert_allclose(g, gt.cpu().numpy(), rtol=0, atol=1e-12)
    # the autograd.Function wrapper routes backward through the adjoint kernel
    xg = torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=True)
    vv = pg.PESFunction.apply(xg, pot)
    (vv * 2.0).sum().backward()
    np.testing.assert_allclose(xg.grad.cpu().numpy(), 2.0 * g, rtol=0, atol=1e-12)
    pd, _ = oracle.dimer_config()
    xd = dimer_geoms(129)
    _, gd = pg.water_dimer().getgrad(xd)
    np.testing.assert_allclose(gd, oracle.grad_dimer(xd, pd), rtol=0, atol=1e-12)


def test_trial_adjoint_matches_chain_rule_helper_golden():
    g = load("h2o_trial_derivs")
    t = pg.ImpSampManager_GPU("h2o_gauss", g["alpha"], g["qe"])
    np.testing.assert_allclose(t.call_trial(g["geo"]), g["psi"], rtol=1e-13)
    d1, d2 = t.call_derivs(g["geo"])
    np.testing.assert_allclose(d1, g["d1"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(d2, g["d2"], rtol=0, atol=1e-10)
    # against the reference's central finite differences (h = 1e-3)
    np.testing.assert_allclose(d1, g["fd1"] / g["fpsi"][:, None, None], rtol=0, atol=1e-4)
    np.testing.assert_allclose(d2, g["fd2"] / g["fpsi"][:, None, None], rtol=0, atol=2e-3)
    # and torch autograd through the TrialFunction adjoint
    xg = torch.tensor(g["geo"], dtype=torch.float64, device="cuda", requires_grad=True)
    psi = pg.TrialFunction.apply(xg, t)
    psi.sum().backward()
    np.testing.assert_allclose(xg.grad.cpu().numpy(), d1 * g["psi"][:, None, None], rtol=1e-10, atol=1e-14)


def test_dimer_trial_matches_oracle():
    """gbdmc_trial_eval with the dimer trial (FP64) against the oracle's restatement."""
    t = pg.dimer_gaussian_trial()
    tr = oracle.TrialDimerGauss(t.alpha, t.qe)
    x = oracle.dimer_equilibrium()[None] + 0.08 * oracle.InjectedNoise(6).standard_normal((1025, 6, 3))
    np.testing.assert_allclose(t.call_trial(x), tr.psi(x), rtol=1e-12)
    d1, d2 = t.call_derivs(x)
    o1, o2 = tr.derivs(x)
    np.testing.assert_allclose(d1, o1, rtol=0, atol=1e-10)
    np.testing.assert_allclose(d2, o2, rtol=0, atol=1e-8)


def ps_geoms(n, seed=7, scale=0.08):
    from oracle.ps_oracle import ps_data
    d = ps_data()
    re_, th = float(d["reoh"]), np.arccos(float(d["ce"]))
    eq = np.array([[0, 0, 0], [re_, 0, 0], [re_ * np.cos(th), re_ * np.sin(th), 0]], dtype=float)
    return eq[None] + scale * oracle.InjectedNoise(seed).standard_normal((n, 3, 3))


@pytest.mark.parametrize("order", ["OHH", "HHO"])
@pytest.mark.parametrize("n", [1, 33, 4097])
def test_partridge_schwenke_matches_oracle(order, n):
    """The Partridge-Schwenke kernel (nested-Horner polynomial, cos(theta) and r_HH from
    the bond vectors) against the term-by-term restatement of vibpot, and its adjoint
    against central differences of the oracle."""
    from oracle.ps_oracle import pes_ps
    x = ps_geoms(n)
    if order == "HHO":
        x = x[:, [1, 2, 0]]
    pot = pg.partridge_schwenke(atom_order=order)
    np.testing.assert_allclose(pot.getpot(x), pes_ps(x, order), rtol=0, atol=1e-12)
    v, g = pot.getgrad(x)
    h = 1e-5
    fd = np.zeros_like(x)
    for a in range(3):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[:, a, d] += h
            xm[:, a, d] -= h
            fd[:, a, d] = (pes_ps(xp, order) - pes_ps(xm, order)) / (2 * h)
    np.testing.assert_allclose(g, fd, rtol=0, atol=2e-7)


def test_partridge_schwenke_dmc_reproduces_the_reference_sample_runs():
    """The reference's own sample runs on this PES (tutorial_water_0..4: 8000 walkers,
    dt = 5, 5000 steps, discrete) print the ensemble's mean potential after each move;
    its average over steps 500-4999, over five runs, against five GPU runs."""
    import json
    ref = json.load(open(os.path.join(G, "ps_tutorial_reference.json")))
    r0 = ref["runs"][0]
    mref = np.array([r["mean_v_cm"] for r in ref["runs"]])
    x0 = ps_geoms(1, scale=0.0)[:, [1, 2, 0]]
    ours = []
    for seed in range(5):
        sim = pg.DMC_Sim(num_walkers=r0["walkers"], num_timesteps=r0["steps"], equil_steps=10 ** 9,
                         atoms=["H", "H", "O"], masses=r0["masses"], delta_t=r0["dt"],
                         potential=pg.partridge_schwenke(atom_order="HHO"), start_structures=x0, seed=100 + seed,
                         write_files=False, graph_steps=32)
        sim._init_device()
        sim._run_steps(r0["steps"])
        torch.cuda.synchronize()
        assert int(sim._read_ctrl().status) == 0
        vm = sim._hist["vmean"].cpu().numpy()[ref["first_step"]:r0["steps"]]
        ours.append(pg.Constants.convert(vm, "wavenumbers", to_AU=False).mean())
    ours = np.array(ours)
    d = ours.mean() - mref.mean()
    err = np.hypot(ours.std(ddof=1) / np.sqrt(len(ours)), mref.std(ddof=1) / np.sqrt(len(mref)))
    assert abs(d) < 0.5 + 4.0 * err, (ours, mref, d, err)


# ----------------------------------------------------------------- engine
def _sim(x0, masses, atoms, pot, seed, nsteps, **kw):
    return pg.DMC_Sim(sim_name="t", output_folder="/tmp/gbdmc_test", num_walkers=len(x0), num_timesteps=nsteps,
                      equil_steps=kw.pop("equil", nsteps + 10), wfn_every=kw.pop("wfn_every", 10 ** 6),
                      desc_wt_steps=kw.pop("desc", 1), chkpt_every=10 ** 6, atoms=atoms, masses=masses,
                      delta_t=10.0, potential=pot, start_structures=x0, rng=oracle.InjectedNoise(seed),
                      write_files=False, **kw)


def test_engine_ho_discrete_bit_exact_vs_reference():
    g = load("ho_discrete")
    ho = oracle.ho_config()
    sim = _sim(g["x0"], ho["masses"], ["H"], pg.harmonic_oscillator(), int(g["seed"]), int(g["nsteps"]))
    sim.run()
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    x = sim.walkers
    assert np.array_equal(x, g["x_final"])  # coordinates bit-exact


def test_engine_h2o_discrete_descendants_bit_exact_vs_reference():
    g = load("h2o_discrete")
    _, m = oracle.h2o_config()
    sim = _sim(g["x0"], m, ["O", "H", "H"], pg.h2o_local_mode(), int(g["seed"]), int(g["nsteps"]),
               equil=int(g["equil"]), wfn_every=int(g["wfn_every"]), desc=int(g["desc"]))
    sim.run()
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    assert np.array_equal(sim.walkers, g["x_final"])
    assert len(sim.wfns) == 2
    for i, w in enumerate(sim.wfns):
        assert np.array_equal(w["coords"], g[f"wfn{i}_coords"])
        assert np.array_equal(w["desc_wts"], g[f"wfn{i}_desc_wts"])


def test_engine_continuous_vs_reference():
    g = load("h2o_continuous")
    _, m = oracle.h2o_config()
    sim = _sim(g["x0"], m, ["O", "H", "H"], pg.h2o_local_mode(), int(g["seed"]), int(g["nsteps"]),
               weighting="continuous", cont_wt_thresh=float(g["thresh"]))
    sim.run()
    x, w = sim.walkers
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(w, g["w_final"], rtol=1e-12)
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(sim._pop_vs_tau, g["pop"], rtol=1e-13)


def test_engine_importance_sampling_vs_reference():
    g = load("h2o_is")
    _, m = oracle.h2o_config()
    sim = _sim(g["x0"], m, ["O", "H", "H"], pg.h2o_local_mode(), int(g["seed"]), int(g["nsteps"]),
               imp_samp=pg.ImpSampManager_GPU("h2o_gauss", g["alpha"], g["qe"]))
    sim.run()
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(sim._eff_ts, g["eff_ts"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(sim.walkers, g["x_final"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("surface", ["fused", "python"])
def test_engine_branch_every_vs_reference(surface):
    """Branching on every third step (discrete, with a descendant window) and
    every fourth (continuous) only, as the unmodified reference runs them with
    branch_every (pyvibdmc.py:139, :828-837): the built-in surface fused into
    the step kernel and the same surface as a Python getpot."""
    p, m = oracle.h2o_config()

    def pot():
        return pg.h2o_local_mode() if surface == "fused" else pg.Potential_Direct(lambda c: oracle.pes_h2o_lm(c, p))

    g = load("h2o_branch_every")
    sim = _sim(g["x0"], m, ["O", "H", "H"], pot(), int(g["seed"]), int(g["nsteps"]), equil=int(g["equil"]),
               wfn_every=1000, desc=int(g["desc"]), branch_every=int(g["branch_every"]))
    sim.run()
    np.testing.assert_array_equal(sim._pop_vs_tau, g["pop"])
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    assert np.array_equal(sim.walkers, g["x_final"])
    assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])
    g = load("h2o_cont_branch_every")
    sim = _sim(g["x0"], m, ["O", "H", "H"], pot(), int(g["seed"]), int(g["nsteps"]), weighting="continuous",
               cont_wt_thresh=float(g["thresh"]), branch_every=int(g["branch_every"]))
    sim.run()
    x, w = sim.walkers
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(w, g["w_final"], rtol=1e-12)
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)


def test_engine_dimer_importance_sampling_vs_oracle():
    """Importance-sampled dimer DMC (dimer trial) against the oracle step loop on the same
    injected deviates; tolerances as for the water IS case."""
    p, m = oracle.dimer_config()
    t = pg.dimer_gaussian_trial()
    x0 = oracle.dimer_equilibrium()[None] + 0.03 * oracle.InjectedNoise(17).standard_normal((600, 6, 3))
    nsteps = 12
    ref = oracle.OracleDMC(x0, m, 10.0, lambda c: oracle.pes_dimer(c, p), oracle.InjectedNoise(23),
                           trial=oracle.TrialDimerGauss(t.alpha, t.qe)).run(nsteps)
    sim = _sim(x0, m, ["O", "H", "H", "O", "H", "H"], pg.water_dimer(), 23, nsteps, imp_samp=t)
    sim.run()
    np.testing.assert_array_equal(sim._pop_vs_tau, np.array(ref.pop_hist))
    np.testing.assert_allclose(sim._vref_vs_tau, np.array(ref.vref_hist), rtol=0, atol=1e-10)
    np.testing.assert_allclose(sim.walkers, ref.x, rtol=0, atol=1e-10)


def test_population_guard_raises_value_error():
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[50:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])  # V = 2 Eh for half the walkers -> w ~ e^10
    sim = _sim(x0, ho["masses"], ["H"], pg.harmonic_oscillator(), 3, 20)
    with pytest.raises(ValueError, match="Massive walker"):
        sim.run()
    assert sim.cur_timestep == 0


@pytest.mark.parametrize("imp", [False, True])
def test_weight_guard_sees_every_walker_of_a_tile(imp):
    """A single walker with a huge weight trips the weight guard (pyvibdmc.py:397) when it
    is not the first walker of its tile: every thread's guard bits reach the control
    block.  Plain step (counting in the move kernel) and importance-sampled step (the
    counting pass), 100 HO walkers at V = 2 Eh except walker 37 at V = 0."""
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])
    x0[37, 0, 0] = 0.0  # w_37 ~ exp(vref dt) with vref ~ 2 Eh
    kw = dict(imp_samp=pg.ho_gaussian_trial(ho["masses"], 1500.0)) if imp else {}
    sim = _sim(x0, ho["masses"], ["H"], pg.harmonic_oscillator(), 3, 20, **kw)
    with pytest.raises(ValueError, match="Massive walker"):
        sim.run()
    assert sim.cur_timestep == 0


def test_philox_graph_batching_is_deterministic():
    _, m = oracle.h2o_config()
    x0 = geoms(4000, seed=11, scale=0.05)
    runs = []
    for gs in (2, 32):
        sim = pg.DMC_Sim(num_walkers=4000, num_timesteps=100, equil_steps=1000, atoms=["O", "H", "H"], masses=m,
                         delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=123,
                         graph_steps=gs, write_files=False, fused_steps=0)
        sim.run()
        runs.append((sim._vref_vs_tau.copy(), sim.walkers))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("imp,graph,pipelined", [(False, False, False), (False, True, False), (True, True, False),
                                                 (False, True, True), (True, True, True)])
def test_host_resident_step_matches_device_step(imp, graph, pipelined):
    """gbdmc_sim_step_host (walkers in page-locked host memory, read and written by
    the kernels) reproduces the device-resident step bit for bit, one step per call
    (step) and with the 20 steps queued back to back (run)."""
    _, m = oracle.h2o_config()
    x0 = geoms(3000, seed=8, scale=0.05)

    def mk():
        return pg.DMC_Sim(num_walkers=3000, num_timesteps=50, equil_steps=1000, atoms=["O", "H", "H"], masses=m,
                          delta_t=10.0, potential=pg.h2o_local_mode(),
                          imp_samp=pg.h2o_gaussian_trial() if imp else None, start_structures=x0, seed=77,
                          write_files=False)

    a, b = mk(), mk()
    a._init_device()
    b._init_device()
    hw = pg.HostWalkers(b, graph=graph)
    for _ in range(20):
        a._cur, a._lazy = a._launch_step(a._cur, a._lazy)
        if not pipelined:
            n = hw.step()
    if pipelined:
        n = hw.run(20)
    a._compact()
    na = int(a._read_ctrl().n)
    assert n == na
    ba = a._bufs[a._cur]
    for k in ("x", "v", "who") + (("f", "psi", "ke") if imp else ()):
        got = hw.host[k][..., :n].numpy()
        want = ba[k][..., :n].cpu().numpy()
        assert np.array_equal(got, want), k
    hw.close()
    assert b.cur_timestep == 20 and np.array_equal(b._coords_host(), a._coords_host())


@pytest.mark.parametrize("rng", ["philox32", "philox64"])
def test_philox_noise_and_branching_match_oracle_stream(rng):
    """Two steps of water in a Philox mode.  Each step's moved walkers (pre-branch
    slots) are x_src + sigma*z with z the oracle's restatement of the walker's
    Philox stream (walker = destination index, step = step counter); the branch
    index equals np.repeat(arange(N), counts) with counts from the oracle's
    branch uniforms.  fp32 normals: 8 fp32 ulps (device and NumPy log/sin/cos
    differ in the last bits); fp64 normals: 1e-12."""
    from oracle.philox_oracle import philox_normals, philox_branch_uniform
    _, m = oracle.h2o_config()
    n, seed, dt = 3000, 0x123456789ABC, 10.0
    sim = pg.DMC_Sim(num_walkers=n, num_timesteps=10, equil_steps=1000, atoms=["O", "H", "H"], masses=m,
                     delta_t=dt, potential=pg.h2o_local_mode(), start_structures=geoms(n, seed=5, scale=0.05),
                     seed=seed, rng=rng, write_files=False)
    sim._init_device()
    sig = np.repeat([sim._sim.sigma[a] for a in range(3)], 3)[:, None]
    tol = dict(rtol=1e-6, atol=1e-6) if rng == "philox32" else dict(rtol=0, atol=1e-12)
    prev = sim._bufs[sim._cur]["x"][:, :n].cpu().numpy()
    for step in range(2):
        c = sim._read_ctrl()
        assert c.step == step and c.n == n
        sim._cur, sim._lazy = sim._launch_step(sim._cur, sim._lazy)
        b = sim._bufs[sim._cur]
        moved = b["x"][:, :n].cpu().numpy()
        z_gpu = (moved - prev) / sig
        z, _ = philox_normals(seed, step, np.arange(n), 9, rng)
        np.testing.assert_allclose(z_gpu, z, **tol)
        v = b["v"][:n].cpu().numpy()
        w = np.exp(-(v - c.vref) * dt)
        u = philox_branch_uniform(seed, step, np.arange(n), 9, rng)
        counts = np.floor(w).astype(np.int64) + (u < w - np.floor(w))
        n = int(sim._read_ctrl().n)
        assert n == counts.sum()
        idx = b["idx"][:n].cpu().numpy()
        np.testing.assert_array_equal(idx, np.repeat(np.arange(len(counts)), counts))
        prev = moved[:, idx]


@pytest.mark.parametrize("rng", ["philox32", "philox64"])
def test_ho_zpe_analytic(rng):
    """3D HO, omega = 3000 cm^-1: ZPE = 4500 cm^-1."""
    ho = oracle.ho_config()
    x0 = 0.1 * oracle.InjectedNoise(12).standard_normal((10000, 1, 3))
    sim = pg.DMC_Sim(num_walkers=10000, num_timesteps=6000, equil_steps=10 ** 6, atoms=["H"], masses=ho["masses"],
                     delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=7, rng=rng,
                     write_files=False)
    sim.run()
    # The walk is exact for the Trotter-split propagator exp(-dt V) exp(-dt T),
    # whose ground-state growth rate for this oscillator is known in closed form:
    # E(dt) = 3/(2 dt) arccosh(1 + (omega dt)^2 / 2) = 4496.5 cm^-1 at dt = 10
    # (4500 cm^-1 as dt -> 0).  Bar: 3 standard errors of 20 block means.
    w = pg.Constants.convert(3000.0, "wavenumbers")
    e_dt = pg.Constants.convert(1.5 / 10.0 * np.arccosh(1.0 + (w * 10.0) ** 2 / 2.0), "wavenumbers", to_AU=False)
    v = pg.Constants.convert(sim._vref_vs_tau[1000:], "wavenumbers", to_AU=False)
    blocks = v.reshape(20, -1).mean(1)
    err = blocks.std(ddof=1) / np.sqrt(len(blocks))
    assert abs(e_dt - 4496.5) < 0.1
    assert abs(v.mean() - e_dt) < 3 * err, (v.mean(), e_dt, err)


def test_is_and_plain_converge_at_small_time_step():
    """Importance-sampled and plain DMC carry time-step biases of opposite sign
    (plain -7, IS +4.6 cm^-1 at dt = 10 for this trial); at dt = 2.5 they agree
    to within the statistical error."""
    _, m = oracle.h2o_config()
    x0 = geoms(20000, seed=9, scale=0.05)
    z = {}
    for tag, trial in (("plain", None), ("is", pg.h2o_gaussian_trial())):
        sm = pg.DMC_Sim(num_walkers=20000, num_timesteps=24000, equil_steps=10 ** 9, atoms=["O", "H", "H"],
                        masses=m, delta_t=2.5, potential=pg.h2o_local_mode(), imp_samp=trial, start_structures=x0,
                        seed=21, write_files=False, graph_steps=32)
        sm._init_device()
        sm._run_steps(24000)
        torch.cuda.synchronize()
        vr = pg.Constants.convert(sm._hist["vref"].cpu().numpy()[6000:], "wavenumbers", to_AU=False)
        z[tag] = pg.blocking_error(vr, 30)
    d = z["is"][0] - z["plain"][0]
    err = float(np.hypot(z["is"][1], z["plain"][1]))
    assert abs(d) < 1.0 + 4.0 * err, (z, d, err)


def test_full_size_workload_step_properties():
    """The benchmark workload at its full size (water, 20000 walkers, Philox32, dt = 10),
    three consecutive steps, checked through size-independent properties: every deviate
    equals the oracle's Philox restatement (8 fp32 ulps), every branch count equals
    floor(w) + [u < w - floor(w)] with the oracle's uniform, the branch index is
    np.repeat(arange(N), counts), and vref equals the mean potential of the branched
    population minus the population term (1e-12 relative)."""
    from oracle.philox_oracle import philox_normals, philox_branch_uniform
    _, m = oracle.h2o_config()
    n, seed, dt = 20000, 20240611, 10.0
    sim = pg.DMC_Sim(num_walkers=n, num_timesteps=10, equil_steps=1000, atoms=["O", "H", "H"], masses=m,
                     delta_t=dt, potential=pg.h2o_local_mode(), start_structures=geoms(n, seed=19, scale=0.05),
                     seed=seed, rng="philox32", write_files=False)
    sim._init_device()
    sig = np.repeat([sim._sim.sigma[a] for a in range(3)], 3)[:, None]
    alpha = 1.0 / (2.0 * dt)
    prev = sim._bufs[sim._cur]["x"][:, :n].cpu().numpy()
    for step in range(3):
        c = sim._read_ctrl()
        sim._cur, sim._lazy = sim._launch_step(sim._cur, sim._lazy)
        b = sim._bufs[sim._cur]
        moved = b["x"][:, :n].cpu().numpy()
        z, _ = philox_normals(seed, step, np.arange(n), 9, "philox32")
        np.testing.assert_allclose((moved - prev) / sig, z, rtol=1e-6, atol=1e-6)
        v = b["v"][:n].cpu().numpy()
        w = np.exp(-(v - c.vref) * dt)
        u = philox_branch_uniform(seed, step, np.arange(n), 9, "philox32")
        counts = np.floor(w).astype(np.int64) + (u < w - np.floor(w))
        c2 = sim._read_ctrl()
        n2 = int(c2.n)
        idx = b["idx"][:n2].cpu().numpy()
        np.testing.assert_array_equal(idx, np.repeat(np.arange(n), counts))
        vref = v[idx].mean() - alpha * (n2 - 20000) / 20000
        np.testing.assert_allclose(c2.vref, vref, rtol=1e-12, atol=0)
        n, prev = n2, moved[:, idx]


def test_host_resident_step_failure_keeps_the_host_walkers():
    """A step that trips the weight guard raises the reference's ValueError and leaves
    the host walkers as they were before the step."""
    ho = oracle.ho_config()
    x0 = np.zeros((100, 1, 3))
    x0[50:, 0, 0] = np.sqrt(2 * 2.0 / ho["k"])  # V = 2 Eh for half the walkers -> w ~ e^10
    sim = pg.DMC_Sim(num_walkers=100, num_timesteps=5, equil_steps=1000, atoms=["H"], masses=ho["masses"],
                     delta_t=10.0, potential=pg.harmonic_oscillator(), start_structures=x0, seed=3, write_files=False)
    sim._init_device()
    hw = pg.HostWalkers(sim)
    before = hw.host["x"][:, :100].clone()
    with pytest.raises(ValueError, match="Massive walker"):
        hw.step()
    assert torch.equal(hw.host["x"][:, :100], before)
    # queued steps: the first trips the guard, the device skips the rest
    with pytest.raises(ValueError, match="Massive walker"):
        hw.run(4)
    assert torch.equal(hw.host["x"][:, :100], before)


def _cont_upper(name):
    g = load(name)
    p, m = oracle.h2o_config()
    if g["x0"].size == 0:  # regenerated from its seed (make_golden.py keeps the large fixture small)
        n = len(g["wfn0_desc_wts"])
        g["x0"] = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(700 + int(g["seed"])).standard_normal(
            (n, 3, 3))
    return g, p, m


@pytest.mark.parametrize("name", ["h2o_cont_upper", "h2o_cont_upper_1500"])
def test_engine_continuous_upper_threshold_vs_reference(name):
    # both thresholds (pyvibdmc.py:432-454): the walkers replaced above the upper
    # threshold come in np.argpartition order (block_argpartition), so which walker
    # is cloned into which slot is the reference's.  Walkers bit-exact; weights,
    # weight sums, vref and descendant weights within 1e-12 (CUDA's exp vs NumPy's)
    g, p, m = _cont_upper(name)
    thr = [float(t) for t in g["thresh"]]
    sim = _sim(g["x0"], m, ["O", "H", "H"], pg.h2o_local_mode(), int(g["seed"]), int(g["nsteps"]),
               weighting="continuous", cont_wt_thresh=thr, equil=int(g["equil"]), desc=int(g["desc"]))
    sim.run()
    x, w = sim.walkers
    assert np.array_equal(x, g["x_final"])
    np.testing.assert_allclose(w, g["w_final"], rtol=1e-12)
    np.testing.assert_allclose(sim._vref_vs_tau, g["vref"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(sim._pop_vs_tau, g["pop"], rtol=1e-12)
    assert len(sim.wfns) == 1
    np.testing.assert_allclose(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(sim.wfns[0]["parent_wts"], g["wfn0_parent_wts"], rtol=1e-12, atol=0)


def _argpartition_cases():
    rng = np.random.default_rng(3)
    cases = []
    for n in (1, 2, 3, 5, 31, 1023, 1024, 1025, 3000, 20000):
        for k in sorted({0, 1, 2, 3, 4, n // 2, n - 2, n - 1} & set(range(n))):
            v = rng.random(n)
            cases.append((f"rand{n}/{k}", v, k))
            cases.append((f"ties{n}/{k}", np.round(v * 8) / 8, k))
    cases.append(("equal5000", np.full(5000, 0.5), 2500))
    for n, k in ((200, 100), (1000, 37), (2500, 1250), (777, 700)):
        cases.append((f"adversary{n}/{k}", oracle.introselect_adversary(n, k), k))
    return cases


def test_argpartition_kernel_matches_numpy_introselect():
    # the block-wide select against the oracle's restatement of NumPy's
    # introselect (itself pinned on np.argpartition): random weights, heavy ties,
    # a constant array, several 1024-element chunks, kth in every branch of the
    # algorithm (selection sort, last element, quickselect) and adversarial inputs
    # that take the median-of-medians pivots
    L = pg._capi.load()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for label, v, k in _argpartition_cases():
        n = len(v)
        w = torch.as_tensor(v, device="cuda")
        perm = torch.empty(n, dtype=torch.int32, device="cuda")
        lpos = torch.empty(n, dtype=torch.int32, device="cuda")
        fl = torch.empty(n, dtype=torch.uint8, device="cuda")
        pg._capi.check(L.gbdmc_argpartition(C.c_void_p(w.data_ptr()), n, k, C.c_void_p(perm.data_ptr()),
                                            C.c_void_p(lpos.data_ptr()), C.c_void_p(fl.data_ptr()), st),
                       "gbdmc_argpartition")
        got = perm.cpu().numpy()
        ref = np.array(oracle.argpartition_introselect(v, k))
        assert np.array_equal(got[:k], ref[:k]), label
        if k >= 3:
            assert np.array_equal(got, ref), label


@pytest.mark.parametrize("thresh", [0.3, 0.9])
def test_continuous_kills_many_and_tied_vs_oracle(thresh):
    """Continuous weighting where many walkers die each step against the
    oracle's sequential argmax cloning (pyvibdmc.py:340-356) on the same
    injected deviates.  The walkers start on a few shared geometries, so many
    weights tie (the first index wins, np.argmax). With the threshold at 0.9
    nearly every weight falls below it, and the largest weight can be a walker
    still waiting to die, the case where the kernel copies in kill order.
    Walkers bit-exact, weights to 1e-12 (CUDA's exp vs NumPy's)."""
    p, m = oracle.h2o_config()
    base = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(71).standard_normal((8, 3, 3))
    x0 = np.repeat(base, 64, axis=0)  # 512 walkers on 8 geometries: tied weights at the first step
    nsteps = 6
    ref = oracle.OracleDMC(x0, m, 10.0, lambda c: oracle.pes_h2o_lm(c, p), oracle.InjectedNoise(31),
                           weighting="continuous", cont_wt_thresh=thresh).run(nsteps)
    sim = _sim(x0, m, ["O", "H", "H"], pg.h2o_local_mode(), 31, nsteps, weighting="continuous",
               cont_wt_thresh=thresh)
    sim.run()
    x, w = sim.walkers
    assert np.array_equal(x, ref.x)
    np.testing.assert_allclose(w, ref.w, rtol=1e-12)
