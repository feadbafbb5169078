"""The oracle (oracle/dmc_oracle.py) against fixtures produced by running the
unmodified reference engine (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import oracle

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with np.load(os.path.join(G, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def test_injected_noise_is_deterministic():
    a = oracle.InjectedNoise(7)
    b = oracle.InjectedNoise(7)
    z1, u1 = a.standard_normal((5, 3, 2)), a.uniform(9)
    z2, u2 = b.standard_normal((5, 3, 2)), b.uniform(9)
    assert np.array_equal(z1, z2) and np.array_equal(u1, u2)
    big = oracle.InjectedNoise(1).standard_normal((200000,))
    assert abs(big.mean()) < 0.01 and abs(big.std() - 1) < 0.01


def test_ho_discrete_matches_reference():
    g = load("ho_discrete")
    ho = oracle.ho_config()
    sim = oracle.OracleDMC(g["x0"], ho["masses"], float(g["dt"]), lambda c: oracle.pes_ho(c, ho["k"]),
                           oracle.InjectedNoise(int(g["seed"]))).run(int(g["nsteps"]))
    assert np.array_equal(np.array(sim.vref_hist), g["vref"])
    assert np.array_equal(np.array(sim.pop_hist), g["pop"])
    assert np.array_equal(sim.x, g["x_final"])
    assert np.array_equal(sim.v, g["v_final"])


def test_h2o_discrete_and_descendants_match_reference():
    g = load("h2o_discrete")
    p, m = oracle.h2o_config()
    sim = oracle.OracleDMC(g["x0"], m, float(g["dt"]), lambda c: oracle.pes_h2o_lm(c, p),
                           oracle.InjectedNoise(int(g["seed"])), equil_steps=int(g["equil"]),
                           wfn_every=int(g["wfn_every"]), desc_wt_steps=int(g["desc"])).run(int(g["nsteps"]))
    assert np.array_equal(np.array(sim.vref_hist), g["vref"])
    assert np.array_equal(sim.x, g["x_final"])
    assert len(sim.wfns) == 2
    for i, w in enumerate(sim.wfns):
        assert np.array_equal(w["coords"], g[f"wfn{i}_coords"])
        assert np.array_equal(w["desc_wts"], g[f"wfn{i}_desc_wts"])


def test_h2o_continuous_matches_reference():
    g = load("h2o_continuous")
    p, m = oracle.h2o_config()
    sim = oracle.OracleDMC(g["x0"], m, float(g["dt"]), lambda c: oracle.pes_h2o_lm(c, p),
                           oracle.InjectedNoise(int(g["seed"])), weighting="continuous",
                           cont_wt_thresh=float(g["thresh"])).run(int(g["nsteps"]))
    assert np.array_equal(np.array(sim.vref_hist), g["vref"])
    assert np.array_equal(sim.x, g["x_final"])
    assert np.array_equal(sim.w, g["w_final"])
    assert sum(c[0] for c in sim.counters) > 0  # branching happened


def test_branch_every_matches_reference():
    """Branching on every third (discrete) and fourth (continuous) step only."""
    p, m = oracle.h2o_config()
    g = load("h2o_branch_every")
    sim = oracle.OracleDMC(g["x0"], m, float(g["dt"]), lambda c: oracle.pes_h2o_lm(c, p),
                           oracle.InjectedNoise(int(g["seed"])), equil_steps=int(g["equil"]), wfn_every=1000,
                           desc_wt_steps=int(g["desc"]), branch_every=int(g["branch_every"])).run(int(g["nsteps"]))
    # vref within a few ulps: NumPy's SIMD sums peel for the array's address alignment
    np.testing.assert_allclose(np.array(sim.vref_hist), g["vref"], rtol=0, atol=5e-17)
    assert np.array_equal(np.array(sim.pop_hist), g["pop"])
    assert np.array_equal(sim.x, g["x_final"])
    assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])
    pops = np.array(sim.pop_hist)
    assert (pops[1::3] == pops[0::3][:len(pops[1::3])]).all() and (pops[2::3] == pops[1::3][:len(pops[2::3])]).all()
    g = load("h2o_cont_branch_every")
    sim = oracle.OracleDMC(g["x0"], m, float(g["dt"]), lambda c: oracle.pes_h2o_lm(c, p),
                           oracle.InjectedNoise(int(g["seed"])), weighting="continuous",
                           cont_wt_thresh=float(g["thresh"]), branch_every=int(g["branch_every"])).run(int(g["nsteps"]))
    np.testing.assert_allclose(np.array(sim.vref_hist), g["vref"], rtol=0, atol=5e-17)
    assert np.array_equal(sim.x, g["x_final"])
    np.testing.assert_allclose(sim.w, g["w_final"], rtol=1e-13)  # the vref ulps, compounded over 24 steps


def _cont_upper_fixture(name):
    g = load(name)
    p, m = oracle.h2o_config()
    if g["x0"].size == 0:  # regenerated from its seed (make_golden.py keeps the large fixture small)
        n = len(g["wfn0_desc_wts"])
        g["x0"] = oracle.h2o_equilibrium(p)[None] + 0.05 * oracle.InjectedNoise(700 + int(g["seed"])).standard_normal(
            (n, 3, 3))
    return g, p, m


def _numpy_without_simd_env():
    """Environment that switches NumPy's SIMD dispatch off, as make_golden.py does
    when it runs the reference for the upper-threshold fixtures (the SIMD kernels
    also change the association of NumPy's float sums in the last bits)."""
    import subprocess
    import sys
    feats = subprocess.run([sys.executable, "-c", "import numpy._core._multiarray_umath as m; "
                            "print(' '.join(getattr(m, '__cpu_dispatch__', [])))"],
                           capture_output=True, text=True, check=True).stdout.strip()
    return dict(os.environ, NPY_DISABLE_CPU_FEATURES=feats)


def _in_numpy_without_simd(code, timeout=600):
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-c", f"import sys; sys.path[:0] = [{os.path.dirname(here)!r}, {here!r}]\n"
                        + code], capture_output=True, text=True, env=_numpy_without_simd_env(), timeout=timeout)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r.stdout


@pytest.mark.parametrize("name", ["h2o_cont_upper", "h2o_cont_upper_1500"])
def test_h2o_continuous_upper_threshold_matches_reference(name):
    # both thresholds: the walkers replaced above the upper threshold come in
    # np.argpartition order (portable introselect); walkers, weights, potentials,
    # vref, the weight sums and the descendant weights of a window spanning the
    # replacements are all bit-equal to the unmodified reference's, with NumPy's
    # arithmetic set up as it was when the fixture was made
    out = _in_numpy_without_simd(f"import test_oracle_golden as t; t.check_cont_upper({name!r}); print('OK')")
    assert out.strip().endswith("OK")


def check_cont_upper(name):
    g, p, m = _cont_upper_fixture(name)
    pes = lambda c: oracle.pes_h2o_lm(c, p)  # noqa: E731

    def run(thresh):
        return oracle.OracleDMC(g["x0"], m, float(g["dt"]), pes, oracle.InjectedNoise(int(g["seed"])),
                                weighting="continuous", cont_wt_thresh=thresh, equil_steps=int(g["equil"]),
                                wfn_every=10 ** 6, desc_wt_steps=int(g["desc"])).run(int(g["nsteps"]))

    sim = run(list(g["thresh"]))
    assert np.array_equal(sim.x, g["x_final"])
    assert np.array_equal(sim.w, g["w_final"])
    assert np.array_equal(sim.v, g["v_final"])
    assert np.array_equal(np.array(sim.vref_hist), g["vref"])
    assert np.array_equal(np.array(sim.pop_hist), g["pop"])
    assert len(sim.wfns) == 1
    assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])
    assert np.array_equal(sim.wfns[0]["parent_wts"], g["wfn0_parent_wts"])
    if "wfn0_coords" in g:
        assert np.array_equal(sim.wfns[0]["coords"], g["wfn0_coords"])
    assert min(c[0] for c in sim.counters) > 5  # every step branched above the upper threshold
    low = run(float(g["thresh"][0]))  # the upper threshold changed the walkers
    assert not np.array_equal(low.x, sim.x)


@pytest.mark.parametrize("name", ["oh_1d", "oh_1d_cont", "oh_1d_kwargs"])
def test_reference_sample_potential_runs_match_reference(name):
    # the reference's 1D sample potential (harmonicOscillator1D.py) run by the
    # unmodified reference on (N, 1, 1) walkers: the oracle with its restatement
    # of the sample function reproduces walkers, populations, vref and the
    # descendant weights bit for bit
    out = _in_numpy_without_simd(f"import test_oracle_golden as t; t.check_oh_1d({name!r}); print('OK')")
    assert out.strip().endswith("OK")


def check_oh_1d(name):
    g = load(name)
    g0 = load("oh_1d")
    kw = {"mass": float(g0["kw_mass"]), "freq": float(g0["kw_freq"])}
    pes = (lambda c: oracle.oh_stretch_harm(c, kw)) if name == "oh_1d_kwargs" else oracle.oh_stretch_harm
    assert np.array_equal(oracle.oh_stretch_harm(g0["probe"]), g0["probe_v"])
    assert np.array_equal(oracle.oh_stretch_harm(g0["probe"], kw), g0["probe_v_kwargs"])
    n = int(g["n"])
    cont = g["thresh"].size > 0
    sim = oracle.OracleDMC(np.zeros((n, 1, 1)), g["masses"], float(g["dt"]), pes, oracle.InjectedNoise(int(g["seed"])),
                           weighting="continuous" if cont else "discrete",
                           cont_wt_thresh=list(g["thresh"]) if cont else None, equil_steps=int(g["equil"]),
                           wfn_every=10 ** 6, desc_wt_steps=int(g["desc"])).run(int(g["nsteps"]))
    assert np.array_equal(sim.x, g["x_final"])
    assert np.array_equal(np.array(sim.vref_hist), g["vref"])
    assert np.array_equal(np.array(sim.pop_hist), g["pop"])
    assert np.array_equal(sim.wfns[0]["desc_wts"], g["wfn0_desc_wts"])
    if cont:
        assert np.array_equal(sim.w, g["w_final"])


def test_continuous_replacement_rules_by_hand():
    # pyvibdmc.py:340-356, 432-454: below `lower` in slot order, then
    # np.argpartition(w, n_up)[:n_up], each replaced by a copy of the current
    # largest weight (first slot on ties), both halved
    x = np.arange(5.0)[:, None, None] * np.ones((5, 1, 3))
    st = dict(x=x, v=np.arange(5.0), w=np.array([0.1, 3.0, 0.5, 3.0, 2.0]), vref=0.0)
    nb, wmax, wmin = oracle.continuous_update_and_branch(st, 0.0, 0.2, 1.4)
    # slot 0 <- 1 (w 1.5 each); then n_up = 4 = N - 1: argpartition swaps the first
    # maximum (slot 3) to the end, so slots 0, 1, 2, 4 <- 3, 4, 0, 3
    assert (nb, wmax, wmin) == (5, 1.0, 0.75)
    assert np.array_equal(st["w"], [0.75, 1.0, 0.75, 0.75, 0.75])
    assert np.array_equal(st["x"][:, 0, 0], [3.0, 4.0, 3.0, 3.0, 3.0])
    assert np.array_equal(st["v"], [3.0, 4.0, 3.0, 3.0, 3.0])


def test_upper_threshold_order_is_introselect_not_ascending():
    # seven weights, three above the threshold: argpartition(w, 3)[:3] = [6, 1, 4]
    # by dumb_select_ (kth < 3 is not the case: kth = 3 takes the quickselect loop)
    w = np.array([5.0, 0.9, 4.0, 6.0, 0.8, 7.0, 0.7])
    order = oracle.argpartition_introselect(w, 3)[:3]
    assert sorted(order) == [1, 4, 6]
    assert order != sorted(order)


_PIN_SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from oracle import argpartition_introselect as aps, introselect_adversary as adversary
rng = np.random.default_rng(11)
bad = []
for trial in range(600):
    n = int(rng.integers(1, 1500))
    v = rng.random(n)
    if trial % 3 == 0:
        v = np.round(v * 8) / 8          # many ties
    if trial % 13 == 0:
        v[:] = 0.25                     # all equal
    k = int(rng.integers(0, n))
    if not np.array_equal(np.argpartition(v, k), aps(v, k)):
        bad.append((n, k))

mom5 = 0
for n, k in ((200, 100), (1000, 37), (2500, 1250), (777, 700)):
    v = adversary(n, k)
    stats = {}
    if not np.array_equal(np.argpartition(v, k), aps(v, k, stats=stats)):
        bad.append(("adversary", n, k))
    mom5 += stats.get("mom5", 0)
print("BAD", bad, "MOM5", mom5)
"""


def test_introselect_restatement_matches_numpy_argpartition():
    # pins oracle.argpartition_introselect on np.argpartition itself, with NumPy's
    # SIMD select dispatch switched off (the portable introselect that aarch64 runs),
    # on random weights, heavy ties, constant arrays and adversarial inputs that
    # force the median-of-medians pivot
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _PIN_SCRIPT, root], capture_output=True, text=True,
                       env=_numpy_without_simd_env(), timeout=600)
    assert r.returncode == 0, r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("BAD")][-1]
    assert line.startswith("BAD [] "), line
    assert int(line.split("MOM5")[1]) > 0


def test_h2o_importance_sampling_matches_reference():
    g = load("h2o_is")
    p, m = oracle.h2o_config()
    tr = oracle.TrialH2OGauss(g["alpha"], g["qe"])
    sim = oracle.OracleDMC(g["x0"], m, float(g["dt"]), lambda c: oracle.pes_h2o_lm(c, p),
                           oracle.InjectedNoise(int(g["seed"])), trial=tr).run(int(g["nsteps"]))
    # the oracle's chain rule differs from ChainRuleHelper's evaluation order at 1e-15
    np.testing.assert_allclose(np.array(sim.vref_hist), g["vref"], rtol=0, atol=1e-12)
    assert sim.x.shape == g["x_final"].shape
    np.testing.assert_allclose(sim.x, g["x_final"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(np.array(sim.eff_ts), g["eff_ts"], rtol=0, atol=1e-12)


def test_trial_derivatives_match_chain_rule_helper():
    g = load("h2o_trial_derivs")
    tr = oracle.TrialH2OGauss(g["alpha"], g["qe"])
    d1, d2 = tr.derivs(g["geo"])
    np.testing.assert_allclose(tr.psi(g["geo"]), g["psi"], rtol=1e-13)
    np.testing.assert_allclose(d1, g["d1"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(d2, g["d2"], rtol=0, atol=1e-11)
    # reference finite differences (h = 1e-3 bohr) agree to their truncation error
    fd1, fd2, fpsi = oracle.finite_diff(g["geo"], tr.psi)
    np.testing.assert_allclose(fd1, g["fd1"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(fd1 / fpsi[:, None, None], d1, rtol=0, atol=1e-4)
    np.testing.assert_allclose(fd2 / fpsi[:, None, None], d2, rtol=0, atol=2e-3)


def test_metropolis_and_local_kin_match_reference():
    g = load("h2o_metropolis")
    a, qe = oracle.h2o_trial_config()
    tr = oracle.TrialH2OGauss(a, qe)
    m = g["masses"]
    sig3 = np.repeat(np.sqrt(10.0 / m), 3).reshape(3, 3)[None]
    inv3 = (1 / np.repeat(m, 3)).reshape(3, 3)[None]
    fa, _ = tr.derivs(g["xa"])
    fb, sdb = tr.derivs(g["xb"])
    met = oracle.metropolis(sig3, tr.psi(g["xa"]), tr.psi(g["xb"]), g["xa"], g["xb"], inv3 * fa, inv3 * fb, 10.0)
    np.testing.assert_allclose(met, g["met"], rtol=1e-10)
    np.testing.assert_allclose(oracle.local_kin(inv3, sdb), g["ke"], rtol=1e-12)


def test_pes_gradients_match_finite_differences():
    p, _ = oracle.h2o_config()
    rng = oracle.InjectedNoise(9)
    x = oracle.h2o_equilibrium(p)[None] + 0.05 * rng.standard_normal((16, 3, 3))
    g = oracle.grad_h2o_lm(x, p)
    h = 1e-5
    fd = np.zeros_like(x)
    for a in range(3):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[:, a, d] += h
            xm[:, a, d] -= h
            fd[:, a, d] = (oracle.pes_h2o_lm(xp, p) - oracle.pes_h2o_lm(xm, p)) / (2 * h)
    np.testing.assert_allclose(g, fd, atol=1e-8)
    pd, _ = oracle.dimer_config()
    xd = np.concatenate([x[:4], x[:4] + np.array([5.5, 0.3, 0.2])], axis=1)
    gd = oracle.grad_dimer(xd, pd)
    fdd = np.zeros_like(xd)
    for a in range(6):
        for d in range(3):
            xp, xm = xd.copy(), xd.copy()
            xp[:, a, d] += h
            xm[:, a, d] -= h
            fdd[:, a, d] = (oracle.pes_dimer(xp, pd) - oracle.pes_dimer(xm, pd)) / (2 * h)
    np.testing.assert_allclose(gd, fdd, atol=1e-8)


def test_philox_restatement_known_answers():
    """Philox4x32-10 against the published known-answer vectors (Salmon et al., SC'11)."""
    from oracle.philox_oracle import philox4x32_10
    kat = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
           ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
           ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
            (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in kat:
        got = philox4x32_10(*[np.array([v], dtype=np.uint64) for v in ctr], *key)
        assert tuple(int(g[0]) for g in got) == want


def test_philox_normals_are_standard_normal():
    from oracle.philox_oracle import philox_normals, philox_branch_uniform
    for mode in ("philox32", "philox64"):
        z, _ = philox_normals(99, 3, np.arange(200000), 9, mode)
        assert abs(z.mean()) < 3e-3 and abs(z.std() - 1.0) < 3e-3
        u = philox_branch_uniform(99, 3, np.arange(200000), 9, mode)
        assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 3e-3


def test_dimer_trial_derivatives_match_finite_differences():
    """The dimer trial's analytic d psi/psi and d2 psi/psi against central differences."""
    from pyvibdmc_gb300.imp_samp import dimer_gaussian_trial
    t = dimer_gaussian_trial()
    tr = oracle.TrialDimerGauss(t.alpha, t.qe)
    x = oracle.dimer_equilibrium()[None] + 0.05 * oracle.InjectedNoise(5).standard_normal((40, 6, 3))
    f, d2 = tr.derivs(x)
    h = 1e-4
    psi0 = tr.psi(x)
    for a in range(6):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[:, a, d] += h
            xm[:, a, d] -= h
            pp, pm = tr.psi(xp), tr.psi(xm)
            np.testing.assert_allclose(f[:, a, d], (pp - pm) / (2 * h) / psi0, rtol=1e-6, atol=1e-6)
            np.testing.assert_allclose(d2[:, a, d], (pp - 2 * psi0 + pm) / (h * h) / psi0, rtol=1e-4, atol=1e-3)


# the reference checkout, when the environment names it (GBDMC_REFERENCE)
REF_PS = os.path.join(os.environ.get("GBDMC_REFERENCE", ""),
                      "pyvibdmc/sample_potentials/FortPots/Partridge_Schwenke_H2O/h2opes_v2.f")


@pytest.mark.skipif(not os.environ.get("GBDMC_REFERENCE") or not os.path.exists(REF_PS),
                    reason="set GBDMC_REFERENCE to a reference checkout to pin the coefficients on its source")
def test_ps_coefficients_match_the_fortran_source():
    """The committed Partridge-Schwenke tables against an independent read of the
    Fortran DATA statements and vibpot's first-call scaling (h2opes_v2.f:420-458)."""
    import re
    from oracle.ps_oracle import ps_data
    src = open(REF_PS).read()

    def block(name):
        m = re.search(r"data \(" + name + r"\(i\),i=1,245\)/(.*?)/", src, re.S)
        return np.array([float(t.replace("D", "e")) for t in re.findall(r"-?\d\.\d+D[-+]\d+", m.group(1))])

    c5z, cb, cc, cr = (block(n) for n in ("c5z", "cbasis", "ccore", "crest"))
    c = (0.99967788500000 * c5z + 0.15860145369897 * cb - 1.6351695982132 * cc + 1.0 * cr) * 4.556335e-6
    c[0] *= 2.0
    d = ps_data()
    np.testing.assert_allclose(d["c"], c, rtol=1e-14, atol=1e-20)
    assert d["idx"].shape == (245, 3) and d["idx"].min() == 1 and d["idx"][:, 2].max() <= 15


def test_ps_oracle_is_near_zero_at_its_expansion_centre():
    from oracle.ps_oracle import pes_ps, ps_data
    d = ps_data()
    re_, th = float(d["reoh"]), np.arccos(float(d["ce"]))
    ohh = np.array([[0, 0, 0], [re_, 0, 0], [re_ * np.cos(th), re_ * np.sin(th), 0]], dtype=float)[None]
    v = pes_ps(ohh)
    assert abs(v[0]) < 1.0 * oracle.WAVENUMBERS
    np.testing.assert_allclose(pes_ps(ohh[:, [1, 2, 0]], order="HHO"), v, rtol=0, atol=1e-15)


def test_lineage_keys_stay_distinct_through_branching():
    """The multi-step kernel's walkers are named by lineage keys (copy 0 keeps
    its parent's key, copy r >= 1 derives one from the parent's key, r and the
    step): through 300 steps of random births and deaths every key in the
    population stays distinct, including for walkers that branch at several
    steps, so no two walkers ever share a Philox stream."""
    from oracle.philox_oracle import lineage_key
    g = np.random.default_rng(3)
    keys = np.arange(2000, dtype=np.uint64)
    for step in range(300):
        c = g.choice([0, 0, 1, 1, 1, 1, 2, 3], size=len(keys), p=None)  # mean 9/8
        if c.sum() > 3000:  # population control, as vref does
            c[np.flatnonzero(c > 1)[: c.sum() - 2000]] = 1
        a = np.repeat(np.arange(len(keys)), c)
        first = np.searchsorted(a, a, side="left")
        keys = lineage_key(keys[a], np.arange(len(a)) - first, step)
        assert len(np.unique(keys)) == len(keys), step
