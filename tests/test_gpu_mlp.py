"""MLP surrogate kernels (BF16 tensor cores, FP32 accumulation) against a
plain PyTorch fp32 reference and the NumPy oracle of the force-matching loss.

Tolerances: GEMMs with bf16-rounded operands agree with torch fp32 on the same
rounded operands to 1e-4 relative; quantities that round activations to bf16
between layers agree with the fp64 oracle to a few 1e-2 relative (bf16 keeps
8 mantissa bits)."""
import numpy as np
import pytest
import torch

import oracle
from oracle import mlp_oracle as mo
import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import _capi
from pyvibdmc_gb300.surrogate import MLPSurrogate, NNDMC, harvest_training_data, _p, _s

pytestmark = pytest.mark.gpu


def bf(t):
    return t.to(torch.bfloat16).float()


@pytest.mark.parametrize("engine", ["mma_sync", "tcgen05"])
@pytest.mark.parametrize("K", [16, 128])
@pytest.mark.parametrize("M", [1, 37, 1000, 4096])
def test_gemm_xw_matches_torch(K, M, engine):
    L = _capi.load()
    gemm = L.gbdmc_mlp_gemm if engine == "mma_sync" else L.gbdmc_mlp_gemm_tc
    g = torch.Generator(device="cuda").manual_seed(K + M)
    X = torch.randn(M, K, device="cuda", generator=g)
    W = torch.randn(K, 128, device="cuda", generator=g) / np.sqrt(K)
    b = torch.randn(128, device="cuda", generator=g)
    Wt = W.t().contiguous().to(torch.bfloat16).view(torch.int16)
    Y = torch.empty(M, 128, device="cuda")
    _capi.check(gemm(_p(X), M, K, _p(Wt), _p(b), _p(Y), _s()))
    ref = bf(X) @ bf(W) + b
    torch.testing.assert_close(Y, ref, rtol=1e-4, atol=1e-4)
    assert L.gbdmc_mlp_gemm_status(1) == 0


@pytest.mark.parametrize("engine", ["mma_sync", "tcgen05"])
@pytest.mark.parametrize("K", [16, 128])
@pytest.mark.parametrize("M", [5, 64, 3001])
def test_gemm_tn_matches_torch(K, M, engine):
    L = _capi.load()
    gemm_tn = L.gbdmc_mlp_gemm_tn if engine == "mma_sync" else L.gbdmc_mlp_gemm_tn_tc
    g = torch.Generator(device="cuda").manual_seed(7 * K + M)
    X = torch.randn(M, K, device="cuda", generator=g)
    D = torch.randn(M, 128, device="cuda", generator=g)
    G = torch.ones(K, 128, device="cuda")
    _capi.check(gemm_tn(_p(X), _p(D), M, K, _p(G), _s()))
    ref = 1.0 + bf(X).t() @ bf(D)
    torch.testing.assert_close(G, ref, rtol=1e-4, atol=1e-3)
    assert L.gbdmc_mlp_gemm_status(1) == 0


@pytest.mark.parametrize("engine", [0, 1])
@pytest.mark.parametrize("K", [16, 128])
@pytest.mark.parametrize("M", [37, 8192])
def test_gemm_pairs_match_single_calls(K, M, engine):
    """gbdmc_mlp_gemm_pair gives each operand set's single-call result bit for
    bit (one bias or none); gbdmc_mlp_gemm_tn_pair accumulates both sets."""
    L = _capi.load()
    gemm = L.gbdmc_mlp_gemm if engine == 0 else L.gbdmc_mlp_gemm_tc
    g = torch.Generator(device="cuda").manual_seed(3 * K + M + engine)
    X0, X1 = (torch.randn(M, K, device="cuda", generator=g) for _ in range(2))
    D0, D1 = (torch.randn(M, 128, device="cuda", generator=g) for _ in range(2))
    W = torch.randn(K, 128, device="cuda", generator=g) / np.sqrt(K)
    b = torch.randn(128, device="cuda", generator=g)
    Wt = W.t().contiguous().to(torch.bfloat16).view(torch.int16)
    Y0, Y1, R0, R1 = (torch.empty(M, 128, device="cuda") for _ in range(4))
    _capi.check(L.gbdmc_mlp_gemm_pair(_p(X0), _p(X1), M, K, _p(Wt), _p(b), None, _p(Y0), _p(Y1), engine, _s()))
    _capi.check(gemm(_p(X0), M, K, _p(Wt), _p(b), _p(R0), _s()))
    _capi.check(gemm(_p(X1), M, K, _p(Wt), None, _p(R1), _s()))
    assert torch.equal(Y0, R0) and torch.equal(Y1, R1)
    G = torch.ones(K, 128, device="cuda")
    _capi.check(L.gbdmc_mlp_gemm_tn_pair(_p(X0), _p(D0), _p(X1), _p(D1), M, K, _p(G), engine, _s()))
    ref = 1.0 + bf(X0).t() @ bf(D0) + bf(X1).t() @ bf(D1)
    torch.testing.assert_close(G, ref, rtol=1e-4, atol=2e-3)
    assert L.gbdmc_mlp_gemm_status(1) == 0
    assert L.gbdmc_mlp_gemm_pair(_p(X0), _p(X1), M, K, _p(Wt), None, None, _p(Y0), _p(Y1), 2, _s()) == _capi.ERR_ARG


def _group_copies(x):
    """Each geometry under one of the eight permutations of like atoms (the
    hydrogens of either water, the two waters), cycling through them."""
    perms = []
    for g in (False, True):
        for a in (False, True):
            for b in (False, True):
                w1, w2 = ([0, 2, 1] if a else [0, 1, 2]), ([3, 5, 4] if b else [3, 4, 5])
                perms.append((w2 + w1) if g else (w1 + w2))
    perms = np.array(perms)
    return x[np.arange(len(x))[:, None], perms[np.arange(len(x)) % 8]]


@pytest.mark.parametrize("sort", [False, True])
def test_features_match_oracle(sort):
    """Descriptors and their directional derivatives against the oracle (with
    sort: DistIt's sorted atom order, which the oracle restates and the
    reference's own DistIt pins).  The kernel decides the order in fp32: the
    walkers whose decisions are within 1e-4 of a tie (relative, by the
    oracle's fp64 norms) are left out, and at least 90 % remain."""
    x = oracle.dimer_equilibrium()[None] + 0.1 * oracle.InjectedNoise(3).standard_normal((300, 6, 3))
    x = _group_copies(x)
    v = oracle.InjectedNoise(4).standard_normal((300, 6, 3))
    p, _ = oracle.dimer_config()
    grad = oracle.grad_dimer(x, p)
    f_ref, t_ref = mo.inv_dist_features(x, v, sort=sort)
    keep = mo.dimer_sort_perm(x)[1].min(1) > 1e-4 if sort else np.ones(300, bool)
    assert keep.mean() > 0.9
    mu = torch.linspace(0.1, 0.3, 16, device="cuda")
    isd = torch.linspace(1.0, 2.0, 16, device="cuda")
    L = _capi.load()
    xs, vs, gs = (pg.to_soa(a, "cuda") for a in (x, v, grad))
    feat = torch.empty(300, 16, device="cuda")
    tang = torch.empty(300, 16, device="cuda")
    et = torch.empty(300, device="cuda")
    _capi.check(L.gbdmc_dimer_features(_p(xs), 300, 300, _p(mu), _p(isd), _p(vs), _p(gs), 0.01, _p(feat), _p(tang),
                                       _p(et), int(sort), _s()))
    mu_, isd_ = mu.cpu().numpy()[:15], isd.cpu().numpy()[:15]
    np.testing.assert_allclose(feat.cpu().numpy()[keep, :15], ((f_ref - mu_) * isd_)[keep], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(tang.cpu().numpy()[keep, :15], (t_ref * isd_)[keep], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(et.cpu().numpy(), (grad * v).sum((1, 2)) / 0.01, rtol=1e-4, atol=1e-4)


def _small_model(seed=0):
    m = MLPSurrogate(seed=seed)
    x = oracle.dimer_equilibrium()[None] + 0.1 * oracle.InjectedNoise(seed + 10).standard_normal((2048, 6, 3))
    p, _ = oracle.dimer_config()
    xs = pg.to_soa(x, "cuda")
    v = torch.as_tensor(oracle.pes_dimer(x, p), device="cuda")
    g = pg.to_soa(oracle.grad_dimer(x, p), "cuda")
    m.set_normalisation(xs, v)
    return m, x, xs, v, g


@pytest.mark.parametrize("train_engine", ["auto", "mma_sync", "tcgen05"])
def test_training_gradients_match_oracle(train_engine):
    """One training step's gradients against the oracle of the training
    kernels' arithmetic (bf16 GEMM operands, fp32 buffers and accumulation).
    What remains is the fp32 summation order of the tensor cores and the
    atomics (and expf's last bits, which move a few bf16 roundings by one
    step): about 1e-5 of the gradient norm, where the sums cancel, and less
    of the summed terms' magnitudes, the scale of an fp32 summation error.
    Measured on a GB300: at most 4.2e-5 of the norm (layer 1, whose gradients
    collect the flips of all later layers) and 9.5e-6 of the magnitudes.  The
    fp64 gradients without the rounding are only a bf16-sized match, and a
    planted mistake in the oracle (descriptor columns 3 and 4 swapped) is far
    outside the bars."""
    m, x, xs, v, g = _small_model(1)
    m.train_engine = train_engine  # the training GEMMs' engines
    P0 = {k: t.detach().cpu().double().numpy() for k, t in m.P.items()}
    m.loss_gradients(xs, v, g)
    Gg = {k: t.detach().cpu().double().numpy() for k, t in m.grads.items()}
    b = m.buf
    D = b["feat"].cpu().double().numpy()
    U = b["tang"].cpu().double().numpy()
    e = b["e"].cpu().double().numpy()  # the kernels take the targets shifted by b4
    et = b["et"].cpu().double().numpy()

    def errors(G, scale=None):
        G["W1"][15] = 0.0
        out = {}
        for k in G:
            d = np.linalg.norm(Gg[k].ravel() - np.ravel(G[k]))
            out[k] = d / max(np.linalg.norm(np.ravel(G[k] if scale is None else scale[k])), 1e-30)
        return out

    P0["b4"] = P0["b4"][0]
    Gt, _, Gm = mo.mlp_loss_grads_bf16(P0, D, U, e, et, 1.0, 0.5, magnitudes=True)
    rel, mag = errors(dict(Gt)), errors(dict(Gt), Gm)
    print("relative to the gradient norm:", rel, "\nrelative to the summed magnitudes:", mag)
    assert max(rel.values()) < 1e-4, rel
    assert max(mag.values()) < 2e-5, mag
    loose = errors(mo.mlp_loss_grads(dict(P0, b4=0.0), D, U, e, et, 1.0, 0.5)[0])
    assert max(loose.values()) < 5e-2, loose
    Dp = D.copy()
    Dp[:, [3, 4]] = Dp[:, [4, 3]]
    planted = errors(mo.mlp_loss_grads_bf16(P0, Dp, U, e, et, 1.0, 0.5)[0])
    assert min(planted.values()) > 1e-3, planted
    m.train_batch(xs, v, g, lr=0.0)  # Adam with lr 0 leaves the parameters and clears the gradients
    for k, t in m.P.items():
        np.testing.assert_array_equal(t.detach().cpu().double().numpy().ravel(), np.ravel(P0[k]))
    assert not any(bool(t.any()) for t in m.grads.values())


def test_inference_kernel_matches_oracle_forward():
    """The tcgen05 inference kernel against the oracle of its arithmetic (bf16
    operands and activations where the kernel rounds, exact tanh where the
    kernel uses tanh.approx): the remaining differences are tanh.approx's and
    rsqrtf's last bits, which move a fraction of the bf16 roundings by one
    bf16 step.  Bars in units of the energy scale, and a planted mistake in the
    oracle (two atoms swapped, which permutes descriptor columns) shows what
    they catch."""
    m, x, xs, v, g = _small_model(2)
    for _ in range(30):
        m.train_batch(xs, v, g, lr=2e-3)
    P = {k: t.detach().cpu().double().numpy() for k, t in m.P.items()}
    mu, isd = m.mu.cpu().double().numpy(), m.inv_sd.cpu().double().numpy()
    assert m.sort_atoms
    keep = mo.dimer_sort_perm(x)[1].min(1) > 1e-4  # fp32 order decisions away from a tie
    assert keep.mean() > 0.9
    ref = mo.mlp_energy_tc(P, x, mu, isd, m.e_mean, m.e_scale, sort=True)
    got = m.energy(x)
    err = (np.abs(got - ref) / m.e_scale)[keep]
    assert np.median(err) < 1e-3 and err.max() < 1e-2, (np.median(err), err.max())
    # the fp64 forward without the rounding (a looser oracle) for scale
    f, _ = mo.inv_dist_features(x, sort=True)
    D = np.zeros((len(x), 16))
    D[:, :15] = (f - mu[:15]) * isd[:15]
    E, _, _ = mo.mlp_forward(dict(P, b4=P["b4"][0]), D)
    loose = (np.abs(got - (m.e_mean + m.e_scale * E)) / m.e_scale)[keep]
    assert np.median(err) < np.median(loose)
    x_bad = x.copy()
    x_bad[:, [3, 4]] = x_bad[:, [4, 3]]  # an oxygen and a hydrogen exchanged: other descriptors
    bad = np.abs(got - mo.mlp_energy_tc(P, x_bad, mu, isd, m.e_mean, m.e_scale, sort=True)) / m.e_scale
    assert np.median(bad) > 10 * 1e-3
    # every copy of a geometry under the permutations of like atoms gets the same energy, bit for bit
    # (the same pair values in the same canonical places), away from the order's ties
    got8 = m.energy(_group_copies(np.repeat(x[:64], 8, axis=0)))
    k64 = keep[:64]
    same = got8.reshape(64, 8)
    assert np.array_equal(same[k64], np.repeat(same[k64, :1], 8, axis=1))
    # and the unsorted descriptor does not have that property
    m.sort_atoms = False
    un8 = m.energy(_group_copies(np.repeat(x[:64], 8, axis=0))).reshape(64, 8)
    assert np.median(np.abs(un8 - un8[:, :1]).max(1)) / m.e_scale > 1e-3


def test_training_reduces_loss_and_surrogate_dmc_runs():
    p, masses = oracle.dimer_config()
    pot = pg.water_dimer()
    x, v, g, _ = harvest_training_data(pot, 4000, 120, 10, pg.WATER_DIMER_EQ[None], masses, seed=3, equil=20)
    m = MLPSurrogate(seed=0).fit(x, v, g, epochs=12, batch=2048, lr=3e-3)
    h = m.history
    assert h[-1]["mse_e"] < 0.2 * h[0]["mse_e"]
    assert h[-1]["mse_f"] < 0.5 * h[0]["mse_f"]
    nd = NNDMC(m, pot, 3000, pg.WATER_DIMER_EQ[None], masses, 10.0, 200, seed=1, audit_every=10).init()
    nd.run(200)
    a = nd.audit()
    assert a["audited"] > 0
    assert np.isfinite(nd.vref_history()).all()
    assert len(nd.walkers()) == int(nd.ctrl().n)

    # online bias control.  A network shifted by +d whose correction starts at +d follows
    # the same trajectory as the unshifted one (corrected energies agree to rounding), and
    # its correction stays exactly d above the unshifted run's.
    w = pg.Constants.atomic_units["wavenumbers"]
    runs = []
    for shift in (0.0, 150.0):
        nb = NNDMC(m, pot, 3000, pg.WATER_DIMER_EQ[None], masses, 10.0, 200, seed=5, audit_every=10,
                   bias_control=0.2)
        e0 = float(nb._net.e_mean)
        nb._net.e_mean += shift * w
        nb._audit[4] = float(nb._net.e_mean) - e0  # the shift as the float32 e_mean holds it
        nb.init().run(200)
        runs.append((nb.audit(), nb.vref_history(), nb.pop_history(), float(nb._net.e_mean) - e0))
    (a0, v0, p0, _), (a1, v1, p1, d) = runs
    assert a0["bias_correction_cm"] != 0.0
    np.testing.assert_array_equal(p0, p1)
    np.testing.assert_allclose(v0, v1, rtol=0, atol=1e-9)
    assert abs((a1["bias_correction_cm"] - a0["bias_correction_cm"]) * w - d) < 1e-9
    assert abs((a1["mean_cm"] - a0["mean_cm"]) * w - d) < 1e-9
    # bias_control = 0 leaves the correction at zero
    nz = NNDMC(m, pot, 3000, pg.WATER_DIMER_EQ[None], masses, 10.0, 20, seed=5, audit_every=10, bias_control=0.0)
    nz.init().run(20)
    assert nz.audit()["bias_correction_cm"] == 0.0


def test_tcgen05_forward_matches_mma_sync_forward():
    """The tcgen05/TMEM inference kernel computes the same BF16 network as the
    mma.sync kernel (same operand rounding; fp32 accumulation order differs)."""
    m, x, xs, v, g = _small_model(3)
    for _ in range(20):
        m.train_batch(xs, v, g, lr=2e-3)
    xx = oracle.dimer_equilibrium()[None] + 0.1 * oracle.InjectedNoise(77).standard_normal((1000, 6, 3))
    e0 = m.energy(xx, engine=0)
    e1 = m.energy(xx, engine=1)
    rel = np.abs(e1 - e0) / m.e_scale
    assert np.median(rel) < 2e-4 and rel.max() < 5e-3, (np.median(rel), rel.max())


@pytest.fixture(scope="module")
def dimer_model():
    """A surrogate fitted well enough for ZPE comparisons (about 1M harvested samples)."""
    p, masses = oracle.dimer_config()
    pot = pg.water_dimer()
    x, v, g, _ = harvest_training_data(pot, 100000, 210, 20, pg.WATER_DIMER_EQ[None], masses, seed=3, equil=20)
    m = MLPSurrogate(seed=0).fit(x, v, g, epochs=15, batch=8192, lr=2e-3)
    return m, pot, masses


def test_surrogate_is_start_state_matches_fp64_trial(dimer_model):
    """The fp32 trial of the surrogate IS path (ln psi, drift, local KE written at step 0)
    against the FP64 oracle trial at the same (fp32-rounded) coordinates."""
    m, pot, masses = dimer_model
    t = pg.dimer_gaussian_trial()
    x0 = (oracle.dimer_equilibrium()[None] + 0.05 * oracle.InjectedNoise(4).standard_normal((3000, 6, 3)))
    x0 = x0.astype(np.float32).astype(np.float64)
    nd = NNDMC(m, pot, 3000, x0, masses, 10.0, 4, seed=1, imp_samp=t).init()
    torch.cuda.synchronize()
    b = nd._bufs[nd._cur]
    tr = oracle.TrialDimerGauss(t.alpha, t.qe)
    d1, d2 = tr.derivs(x0)
    lnorm = 2 * 0.25 * np.log(np.prod(t.alpha[:3]) / np.pi ** 3) + 0.25 * np.log(t.alpha[3] / np.pi)
    lp = np.log(tr.psi(x0)) - lnorm
    ke = -0.5 * (d2 / np.asarray(masses)[None, :, None]).sum((1, 2))
    got_f = b["f"][:, :3000].cpu().numpy().T.reshape(3000, 6, 3)
    np.testing.assert_allclose(b["lnpsi"][:3000].cpu().numpy(), lp, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(got_f, d1, rtol=1e-3, atol=2e-3)
    np.testing.assert_allclose(b["ke"][:3000].cpu().numpy(), ke, rtol=1e-3, atol=1e-5)
    v = b["v"][:3000].cpu().numpy()
    np.testing.assert_allclose(v - b["ke"][:3000].cpu().numpy(), oracle.pes_dimer(x0, oracle.dimer_config()[0]),
                               rtol=0, atol=1e-10)


@pytest.mark.parametrize("imp", [False, True])
def test_surrogate_replica_batch_equals_single_runs(dimer_model, imp):
    """Replica r of a batch reproduces a single run with replica_id = r bit for bit
    (bias control off, so no statistic is shared between replicas)."""
    m, pot, masses = dimer_model
    t = pg.dimer_gaussian_trial() if imp else None
    ns = [700, 3000, 1500]
    b = NNDMC(m, pot, ns, pg.WATER_DIMER_EQ[None], masses, 10.0, 40, seed=9, bias_control=0.0, imp_samp=t)
    b.init().run(40)
    for r, n in enumerate(ns):
        s = NNDMC(m, pot, n, pg.WATER_DIMER_EQ[None], masses, 10.0, 40, seed=9, bias_control=0.0, imp_samp=t,
                  replica_id=r)
        s.init().run(40)
        np.testing.assert_array_equal(b.pop_history()[r], s.pop_history())
        np.testing.assert_array_equal(b.vref_history()[r], s.vref_history())
        assert np.array_equal(b.walkers(r), s.walkers())


def test_surrogate_is_zpe_agrees_with_fp64_is(dimer_model):
    """Importance-sampled surrogate DMC against importance-sampled FP64 analytic DMC of
    the dimer (same trial, dt, walkers)."""
    m, pot, masses = dimer_model
    t = pg.dimer_gaussian_trial()
    nd = NNDMC(m, pot, 50000, pg.WATER_DIMER_EQ[None], masses, 10.0, 3000, seed=3, imp_samp=t).init()
    nd.run(3000)
    z_nn = nd.zpe(start=750)
    acc = 1.0  # the acceptance is checked through the FP64 run's rejected counts below
    fp = pg.DMC_Sim(num_walkers=50000, num_timesteps=3000, equil_steps=10 ** 9, atoms=["O", "H", "H"] * 2,
                    masses=masses, delta_t=10.0, potential=pot, imp_samp=t, start_structures=pg.WATER_DIMER_EQ[None],
                    seed=3, write_files=False)
    fp._init_device()
    fp._run_steps(3000)
    torch.cuda.synchronize()
    vv = pg.Constants.convert(fp._hist["vref"].cpu().numpy()[750:3000], "wavenumbers", to_AU=False)
    z_fp = pg.blocking_error(vv, 20)
    rej = fp._hist["rejected"].cpu().numpy()[:3000].sum() / (50000.0 * 3000)
    assert rej < 0.2 and acc > 0
    d = z_nn[0] - z_fp[0]
    err = float(np.hypot(z_nn[1], z_fp[1]))
    assert abs(d) < 3.0 + 4.0 * err, (z_nn, z_fp, nd.audit())


def test_trained_surrogate_gains_over_the_fp64_pes(dimer_model):
    """What the trained network gains over the method without it: one surrogate DMC
    step of 200000 dimer walkers against one step of the FP64 analytic PES, same
    walkers, dt and branching (graph-replayed steps, CUDA events).  The ZPE agreement
    of the two is checked in the statistical tests above and in the bench extras."""
    m, pot, masses = dimer_model
    nd = NNDMC(m, pot, 200000, pg.WATER_DIMER_EQ[None], masses, 10.0, 200, seed=4).init()
    fp = pg.DMC_Sim(num_walkers=200000, num_timesteps=200, equil_steps=10 ** 9, atoms=["O", "H", "H"] * 2,
                    masses=masses, delta_t=10.0, potential=pot, start_structures=pg.WATER_DIMER_EQ[None], seed=4,
                    write_files=False, graph_steps=16)
    fp._init_device()
    nd.run(32)
    fp._run_steps(32)
    torch.cuda.synchronize()
    times = []
    for run in (nd.run, fp._run_steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run(64)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 64)
    assert times[0] < 0.85 * times[1], times


@pytest.mark.parametrize("nwalk", [300, 70000])
def test_step_kernel_energies_equal_the_energy_kernel(dimer_model, nwalk):
    """The DMC step kernel (move + descriptors + network in 128-walker tile groups, four
    groups per CTA) gives each moved walker the same surrogate energy as the energy
    kernel evaluated on the moved coordinates (audit and bias correction off)."""
    m, pot, masses = dimer_model
    nd = NNDMC(m, pot, nwalk, pg.WATER_DIMER_EQ[None], masses, 10.0, 4, seed=8, audit_every=0,
               bias_control=0.0).init()
    nd.run(1)
    torch.cuda.synchronize()
    b = nd._bufs[nd._cur]  # pre-branch moved walkers in slots 0..N-1
    x = b["x"][:, :nwalk].contiguous()
    v_step = b["v"][:nwalk].cpu().numpy()
    v_ref, outside = m.energy_soa(x, nwalk, engine=1)
    keep = outside.cpu().numpy() == 0
    assert keep.mean() > 0.5
    np.testing.assert_array_equal(v_step[keep], v_ref.cpu().numpy()[keep])


def test_surrogate_branch_counts_match_the_oracle_draws(dimer_model):
    """The surrogate path's counting kernel (fp32 weight from the fp64 exponent, the
    Philox branching uniform compared with the fractional weight on the integer pipes,
    per-tile sums of c (V - vref) in fp32) against the oracle: fp64 weights from the
    same energies and the oracle's 53-bit uniforms of the same Philox stream.  The
    counts are read back from the branching index; walkers whose uniform lies within
    1e-5 of the fractional weight (fp32 exp) may go either way.  vref to 1e-9 hartree."""
    from oracle.philox_oracle import PhiloxStream
    m, pot, masses = dimer_model
    n0, seed, dt = 20000, 21, 10.0
    nd = NNDMC(m, pot, n0, pg.WATER_DIMER_EQ[None], masses, dt, 8, seed=seed, audit_every=0,
               bias_control=0.0).init()
    nd.run(3)
    torch.cuda.synchronize()
    c0 = nd.ctrl()
    n, step, vref = int(c0.n), int(c0.step), float(c0.vref)
    assert c0.dt_eff == dt
    nd.run(1)
    torch.cuda.synchronize()
    c1 = nd.ctrl()
    b = nd._bufs[nd._cur]
    v = b["v"][:n].cpu().numpy()
    idx = b["idx"][:int(c1.n)].cpu().numpy()
    cnt = np.bincount(idx, minlength=n)
    assert len(cnt) == n and cnt.sum() == c1.n
    st = PhiloxStream(seed, step, np.arange(n), replica=0)
    st.slot = 64
    u = st.uniform53()
    w = np.exp(-(v - vref) * dt)
    fl = np.floor(w)
    want = fl.astype(np.int64) + (u < w - fl)
    amb = (np.abs(u - (w - fl)) < 1e-5) | (np.abs(w - np.round(w)) < 1e-5)
    assert amb.sum() < 0.002 * n
    np.testing.assert_array_equal(cnt[~amb], want[~amb])
    nn = int(c1.n)
    vref_want = (cnt * v).sum() / nn - (1.0 / (2.0 * dt)) * (nn - n0) / n0
    assert abs(c1.vref - vref_want) < 1e-9, (c1.vref, vref_want)


def test_audit_energies_match_the_fp64_oracle(dimer_model):
    """With every walker audited (audit_every = 1) each moved walker's energy is the
    fp32 analytic dimer energy of the audit pass; against the FP64 oracle PES at the
    same (fp32) coordinates it agrees to 2e-7 hartree (0.04 cm^-1), far inside the
    surrogate error the audit measures."""
    m, pot, masses = dimer_model
    p, _ = oracle.dimer_config()
    n = 3000
    nd = NNDMC(m, pot, n, pg.WATER_DIMER_EQ[None], masses, 10.0, 4, seed=12, audit_every=1,
               bias_control=0.0).init()
    nd.run(1)
    torch.cuda.synchronize()
    b = nd._bufs[nd._cur]  # pre-branch moved walkers in slots 0..N-1
    x = b["x"][:, :n].cpu().numpy().astype(np.float64).T.reshape(n, 6, 3)
    v = b["v"][:n].cpu().numpy()
    np.testing.assert_allclose(v, oracle.pes_dimer(x, p), rtol=0, atol=2e-7)
    assert nd.audit()["audited"] >= n


@pytest.mark.parametrize("n0", [100, 5000])
def test_surrogate_injected_step_matches_the_oracle(dimer_model, n0):
    """One surrogate step with injected deviates and uniforms (a one-tile replica of 100
    walkers and one of 5000): every moved walker is x + sigma z in fp32, and the gather
    index expands the counts floor(w) + [u < w - floor(w)] of the oracle's fp64 weights
    from the step's own energies and the injected uniforms (walkers whose uniform lies
    within 1e-5 of the fractional weight may go either way); vref to 1e-9 hartree."""
    m, pot, masses = dimer_model
    seed, dt = 31, 10.0
    nd = NNDMC(m, pot, n0, pg.WATER_DIMER_EQ[None], masses, dt, 4, rng=oracle.InjectedNoise(seed), audit_every=0,
               bias_control=0.0).init()
    torch.cuda.synchronize()
    c0 = nd.ctrl()
    n, vref = int(c0.n), float(c0.vref)
    x_old = nd._bufs[nd._cur]["x"][:, :n].cpu().numpy()
    twin = oracle.InjectedNoise(seed)
    z = np.asarray(twin.standard_normal((n, 3, 6)), dtype=np.float64).transpose(2, 1, 0).reshape(18, n)
    u = twin.uniform(n)
    nd.run(1)
    torch.cuda.synchronize()
    c1 = nd.ctrl()
    b = nd._bufs[nd._cur]
    sig = np.repeat(np.sqrt(dt / np.asarray(masses)), 3).astype(np.float32)[:, None]
    want_x = x_old + sig * z.astype(np.float32)
    np.testing.assert_allclose(b["x"][:, :n].cpu().numpy(), want_x, rtol=0, atol=2e-6)
    v = b["v"][:n].cpu().numpy()
    nn = int(c1.n)
    cnt = np.bincount(b["idx"][:nn].cpu().numpy(), minlength=n)
    assert len(cnt) == n and cnt.sum() == nn
    w = np.exp(-(v - vref) * dt)
    fl = np.floor(w)
    want = fl.astype(np.int64) + (u < w - fl)
    amb = (np.abs(u - (w - fl)) < 1e-5) | (np.abs(w - np.round(w)) < 1e-5)
    assert amb.sum() < max(3, 0.002 * n)
    np.testing.assert_array_equal(cnt[~amb], want[~amb])
    vref_want = (cnt * v).sum() / nn - (1.0 / (2.0 * dt)) * (nn - n0) / n0
    assert abs(c1.vref - vref_want) < 1e-9, (c1.vref, vref_want)


def test_dmc_sim_with_a_surrogate_potential_runs_the_fused_step():
    """DMC_Sim(potential=NN_Potential_GPU(model, fallback=water_dimer())) runs the
    fused surrogate step: the same trajectory as NNDMC with the same seed, plus
    the descendant-weighting windows and files of DMC_Sim; without a fallback the
    surrogate is called through getpot like any Python potential."""
    p, masses = oracle.dimer_config()
    pot = pg.water_dimer()
    x, v, g, _ = harvest_training_data(pot, 3000, 60, 10, pg.WATER_DIMER_EQ[None], masses, seed=3, equil=10)
    m = MLPSurrogate(seed=0).fit(x, v, g, epochs=4, batch=2048, lr=3e-3)
    sim = pg.DMC_Sim(num_walkers=3000, num_timesteps=80, equil_steps=20, wfn_every=1000, desc_wt_steps=30,
                     atoms=["O", "H", "H"] * 2, masses=masses, delta_t=10.0,
                     potential=pg.NN_Potential_GPU(m, fallback=pot), start_structures=pg.WATER_DIMER_EQ[None],
                     seed=5, write_files=False)
    sim.run()
    nd = NNDMC(m, pot, 3000, pg.WATER_DIMER_EQ[None], masses, 10.0, 80, seed=5).init()
    nd.run(80)
    np.testing.assert_array_equal(sim._vref_vs_tau, nd.vref_history())
    np.testing.assert_array_equal(sim._pop_vs_tau, nd.pop_history())
    assert np.array_equal(sim.walkers, nd.walkers().astype(np.float64))
    assert len(sim.wfns) == 1 and sim.wfns[0]["desc_wts"].sum() == sim._pop_vs_tau[49]
    slow = pg.DMC_Sim(num_walkers=500, num_timesteps=5, equil_steps=100, atoms=["O", "H", "H"] * 2, masses=masses,
                      delta_t=10.0, potential=pg.NN_Potential_GPU(m), start_structures=pg.WATER_DIMER_EQ[None],
                      seed=5, write_files=False)
    slow.run()
    assert slow._external and np.all(np.isfinite(slow._vref_vs_tau))
