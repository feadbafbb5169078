"""Generate the golden fixtures by running the UNMODIFIED reference engine.

Run from the repository root with the reference checkout available::

    python tests/golden/make_golden.py <reference checkout> [fixture,fixture,...]

(or set GBDMC_REFERENCE to the checkout and omit the first argument).

What it does:

* stubs ``h5py`` (in-memory ``File`` that records every dataset written by
  ``SimArchivist.save_h5``) and ``matplotlib`` -- neither is installed and the
  reference uses them only for output files and plots;
* imports ``pyvibdmc`` from the given checkout;
* replaces ``np.random.normal`` / ``np.random.random`` with
  :class:`oracle.InjectedNoise` (deterministic, platform independent), so the
  reference and the GPU engine consume identical deviates in the reference's
  call order;
* runs small DMC simulations through the reference's own plug-in path
  (``Potential_Direct`` for the PES, ``ImpSampManager_NoMP`` for the trial
  wave function, whose derivative function uses the reference's
  ``ChainRuleHelper``), and ``ImpSamp.finite_diff`` / ``ChainRuleHelper`` on
  the reference test geometry;
* writes ``tests/golden/*.npz``.

NumPy's SIMD select is switched off (``NPY_DISABLE_CPU_FEATURES`` set to every
dispatch target of the running NumPy, before NumPy is imported), so the
reference's ``np.argpartition`` (pyvibdmc.py:443-445) runs NumPy's portable
introselect, the algorithm NumPy uses on every platform without a SIMD
select kernel (aarch64 among them).  On x86 with AVX2/AVX-512 NumPy 2.x would
otherwise substitute a SIMD select whose output order differs.

The fixtures hold the seeds, the inputs and the reference outputs.
"""
import os
import subprocess
import sys
import tempfile
import types


def _numpy_dispatch_targets():
    r = subprocess.run([sys.executable, "-c", "import numpy._core._multiarray_umath as m; "
                        "print(' '.join(getattr(m, '__cpu_dispatch__', [])))"],
                       capture_output=True, text=True, check=True)
    return r.stdout.strip()


if __name__ == "__main__" and "NPY_DISABLE_CPU_FEATURES" not in os.environ:
    feats = _numpy_dispatch_targets()
    if feats:
        os.environ["NPY_DISABLE_CPU_FEATURES"] = feats
        os.execv(sys.executable, [sys.executable] + sys.argv)

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

H5_STORE = {}


def _install_stubs():
    h5 = types.ModuleType("h5py")

    class File:
        def __init__(self, fname, mode="r"):
            self.fname = fname
            self.mode = mode
            if "w" in mode:
                H5_STORE[fname] = {}

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def create_dataset(self, key, data):
            H5_STORE[self.fname][key] = np.array(data, copy=True)

        def __getitem__(self, key):
            return H5_STORE[self.fname][key]

    h5.File = File
    sys.modules["h5py"] = h5
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.rcParams = {}
    mpl.pyplot = plt
    mpl.use = lambda *a, **k: None
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt


def _import_reference(path):
    _install_stubs()
    sys.path.insert(0, path)
    import pyvibdmc as pv
    return pv


class _Patch:
    def __init__(self, noise):
        self.noise = noise

    def __enter__(self):
        self.saved = (np.random.normal, np.random.random)
        np.random.normal = self.noise.normal
        np.random.random = self.noise.random
        return self

    def __exit__(self, *a):
        np.random.normal, np.random.random = self.saved


TRIAL_MODULE = '''
import numpy as np
import pyvibdmc as pv

ALPHA = {alpha!r}
QE = {qe!r}


def _internals(cds):
    an = pv.AnalyzeWfn(cds)
    r1 = an.bond_length(1, 0)
    r2 = an.bond_length(2, 0)
    th = an.bond_angle(1, 0, 2)
    return r1, r2, th


def trial(cds):
    qs = _internals(cds)
    out = np.ones(len(cds))
    for q, a, qe in zip(qs, ALPHA, QE):
        out = out * ((a / np.pi) ** 0.25 * np.exp(-a * (q - qe) ** 2 / 2))
    return out


def derivs(cds):
    """dpsi/dx/psi, d2psi/dx2/psi through the reference ChainRuleHelper,
    mirroring call_trl_h2o.py:101-149 for one water (O,H,H)."""
    qs = _internals(cds)
    dpsi_dr = np.stack([-a * (q - qe) for q, a, qe in zip(qs, ALPHA, QE)])
    d2psi_dr2 = np.stack([(a * (q - qe)) ** 2 - a for q, a, qe in zip(qs, ALPHA, QE)])
    crh = pv.ChainRuleHelper(cds, np)
    ohs = [[0, 1], [0, 2]]
    hoh = [1, 0, 2]
    cos_theta = np.cos(qs[2])
    dr_dxs = np.stack([crh.dr_dx(oh) for oh in ohs])
    d2r_dx2s = np.stack([crh.d2r_dx2(oh, dr_dx=dr_dxs[n]) for n, oh in enumerate(ohs)])
    dcth_dx = crh.dcth_dx(hoh, cos_theta=cos_theta, dr_da=dr_dxs[0], dr_dc=dr_dxs[1])
    dth_dx = crh.dth_dx(hoh, cos_theta=cos_theta, dcth_dx=dcth_dx, dr_da=dr_dxs[0], dr_dc=dr_dxs[1])
    d2th_dx2 = crh.d2th_dx2(hoh, cos_theta=cos_theta, dcth_dx=dcth_dx, dr_da=dr_dxs[0],
                            dr_dc=dr_dxs[1], d2r_da2=d2r_dx2s[0], d2r_dc2=d2r_dx2s[1])
    dint = np.stack([dr_dxs[0], dr_dxs[1], dth_dx])
    d2int = np.stack([d2r_dx2s[0], d2r_dx2s[1], d2th_dx2])
    return crh.dpsidx(dpsi_dr, dint), crh.d2psidx2(d2psi_dr2, d2int, dpsi_dr, dint)
'''


def run_reference(pv, out_dir, name, x0, atoms, masses, dt, nsteps, pes, seed, weighting="discrete",
                  imp=None, equil=None, wfn_every=None, desc=None, thresh=None, branch_every=1):
    noise = oracle.InjectedNoise(seed)
    kw = dict(sim_name=name, output_folder=os.path.join(out_dir, name), weighting=weighting,
              num_walkers=len(x0), num_timesteps=nsteps, equil_steps=equil if equil is not None else nsteps + 10,
              chkpt_every=10 ** 6, wfn_every=wfn_every or 10 ** 6, desc_wt_steps=desc or 1,
              atoms=atoms, masses=masses, delta_t=dt, potential=pv.Potential_Direct(pes),
              start_structures=np.array(x0, copy=True), log_every=10 ** 6, cont_wt_thresh=thresh,
              imp_samp=imp, branch_every=branch_every)
    sim = pv.DMC_Sim(**kw)
    with _Patch(noise):
        sim.run()
    out = dict(vref=np.array(sim._vref_vs_tau), pop=np.array(sim._pop_vs_tau),
               x_final=np.array(sim._walker_coords), v_final=np.array(sim._walker_pots),
               n_noise_calls=noise.calls)
    if weighting == "continuous":
        out["w_final"] = np.array(sim._cont_wts)
    if imp is not None:
        out["eff_ts"] = np.array(sim.eff_ts)
        out["psi_final"] = np.array(sim.psi_1)
        out["f_final"] = np.array(sim.f_x)
    wfns = sorted(k for k in H5_STORE if "/wfns/" in k and k.startswith(kw["output_folder"]))
    for i, k in enumerate(wfns):
        for key, val in H5_STORE[k].items():
            out[f"wfn{i}_{key}"] = val
    return out


def main(ref_path, only=None):  # noqa: C901
    pv = _import_reference(ref_path)
    tmp = tempfile.mkdtemp(prefix="gbdmc_golden_")
    fixtures = {}

    # --- config-1 family: 3D HO, discrete, 40 steps
    ho = oracle.ho_config()
    n = 256
    x0 = 0.1 * oracle.InjectedNoise(101).standard_normal((n, 1, 3))
    pes = lambda c, k=ho["k"]: oracle.pes_ho(c, k)
    r = run_reference(pv, tmp, "ho", x0, ["H"], ho["masses"], 10.0, 40, pes, seed=1)
    fixtures["ho_discrete"] = dict(x0=x0, seed=1, dt=10.0, nsteps=40, **r)

    # --- config-2 family: H2O local mode, discrete + descendant weights
    p, masses = oracle.h2o_config()
    eq = oracle.h2o_equilibrium(p)
    n = 384
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(202).standard_normal((n, 3, 3))
    pes = lambda c, p=p: oracle.pes_h2o_lm(c, p)
    r = run_reference(pv, tmp, "h2o", x0, ["O", "H", "H"], masses, 10.0, 60, pes, seed=2,
                      equil=20, wfn_every=30, desc=10)
    fixtures["h2o_discrete"] = dict(x0=x0, seed=2, dt=10.0, nsteps=60, equil=20, wfn_every=30, desc=10, **r)

    # --- continuous weights (lower threshold only), H2O
    n = 192
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(303).standard_normal((n, 3, 3))
    r = run_reference(pv, tmp, "h2o_cont", x0, ["O", "H", "H"], masses, 10.0, 40, pes, seed=3,
                      weighting="continuous", thresh=0.2)
    fixtures["h2o_continuous"] = dict(x0=x0, seed=3, dt=10.0, nsteps=40, thresh=0.2, **r)

    # --- branching every third (discrete, with a descendant window) and every fourth
    # (continuous) step only (pyvibdmc.py:139, :828-837): off the schedule discrete
    # walkers are not weighted and continuous weights are updated without replacements
    n = 256
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(404).standard_normal((n, 3, 3))
    r = run_reference(pv, tmp, "h2o_be", x0, ["O", "H", "H"], masses, 10.0, 30, pes, seed=21, equil=8,
                      wfn_every=1000, desc=12, branch_every=3)
    fixtures["h2o_branch_every"] = dict(x0=x0, seed=21, dt=10.0, nsteps=30, equil=8, desc=12, branch_every=3, **r)
    n = 192
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(405).standard_normal((n, 3, 3))
    r = run_reference(pv, tmp, "h2o_cbe", x0, ["O", "H", "H"], masses, 10.0, 24, pes, seed=22,
                      weighting="continuous", thresh=0.2, branch_every=4)
    fixtures["h2o_cont_branch_every"] = dict(x0=x0, seed=22, dt=10.0, nsteps=24, thresh=0.2, branch_every=4, **r)

    # --- continuous weights with both thresholds.  The reference replaces the walkers
    # above the upper threshold in np.argpartition order (portable introselect, see the
    # module docstring), so these fixtures pin which walker is cloned into which slot.
    # The thresholds are the 2 % and 90 % (85 %) quantiles of the first step's weights,
    # so every step branches a few walkers below and more above than the lower
    # branching halves; a descendant-weighting window follows the walkers' ancestors
    # through the replacements.  The 1500-walker case spans two 1024-walker chunks
    # of the GPU's block-wide select.
    for name, n, nsteps, seed, q_hi in (("h2o_cont_upper", 192, 6, 7, 0.9),
                                         ("h2o_cont_upper_1500", 1500, 3, 8, 0.85)):
        x0 = eq[None] + 0.05 * oracle.InjectedNoise(700 + seed).standard_normal((n, 3, 3))
        probe = oracle.OracleDMC(x0, masses, 10.0, pes, oracle.InjectedNoise(seed), weighting="continuous",
                                 cont_wt_thresh=[1e-300, 1e300]).run(1)
        thr = [float(q) for q in np.quantile(probe.w, [0.02, q_hi])]
        r = run_reference(pv, tmp, name, x0, ["O", "H", "H"], masses, 10.0, nsteps, pes, seed=seed,
                          weighting="continuous", thresh=thr, equil=1, wfn_every=10 ** 6, desc=nsteps - 2)
        if n > 1000:  # kept small: x0 is regenerated from its seed, the parents are x after step 1
            r.pop("wfn0_coords")
        fixtures[name] = dict(x0=x0 if n <= 1000 else np.zeros(0), seed=seed, dt=10.0, nsteps=nsteps,
                              thresh=np.array(thr), equil=1, desc=nsteps - 2, numpy_version=np.__version__,
                              npy_disable_cpu_features=os.environ.get("NPY_DISABLE_CPU_FEATURES", ""), **r)

    # --- the reference's own 1D sample potential (sample_potentials/PythonPots/
    # harmonicOscillator1D.py), imported from the checkout, as its tests run it
    # (tests/test_pyvibdmc.py:14-48: atoms ["O-H"], (1,1,1) start): discrete with a
    # descendant window, continuous with both thresholds, and the pot_kwargs +
    # pass_timestep variant through Potential_Direct.  Energies of probe geometries
    # pin the oracle's restatement of the sample functions.
    sys.path.insert(0, os.path.join(ref_path, "pyvibdmc", "sample_potentials", "PythonPots"))
    import harmonicOscillator1D as ho1d  # noqa: E402
    probe = 0.3 * oracle.InjectedNoise(808).standard_normal((64, 1, 1))
    kw = {"mass": float(pv.Constants.reduced_mass("O-H")), "freq": float(pv.Constants.convert(3700.0, "wavenumbers"))}
    n = 200
    x0 = np.zeros((1, 1, 1))
    runs = {}
    for name, pot, weighting, thresh, seed in (
            ("oh_1d", pv.Potential_Direct(ho1d.oh_stretch_harm), "discrete", None, 8),
            ("oh_1d_cont", pv.Potential_Direct(ho1d.oh_stretch_harm), "continuous", [0.05, 2.5], 9),
            ("oh_1d_kwargs", pv.Potential_Direct(ho1d.oh_stretch_harm_with_arg, pot_kwargs=dict(kw),
                                                 pass_timestep=True), "discrete", None, 10)):
        noise = oracle.InjectedNoise(seed)
        kwd = dict(sim_name=name, output_folder=os.path.join(tmp, name), weighting=weighting, num_walkers=n,
                   num_timesteps=60, equil_steps=20, chkpt_every=10 ** 6, wfn_every=10 ** 6, desc_wt_steps=15,
                   atoms=["O-H"], delta_t=5.0, potential=pot, start_structures=x0.copy(), log_every=10 ** 6,
                   cont_wt_thresh=thresh)
        sim = pv.DMC_Sim(**kwd)
        with _Patch(noise):
            sim.run()
        r = dict(vref=np.array(sim._vref_vs_tau), pop=np.array(sim._pop_vs_tau), x_final=np.array(sim._walker_coords),
                 v_final=np.array(sim._walker_pots), seed=seed, n=n, dt=5.0, nsteps=60, equil=20, desc=15,
                 thresh=np.array(thresh if thresh else []), masses=np.array(sim.masses))
        if weighting == "continuous":
            r["w_final"] = np.array(sim._cont_wts)
        wf = [k for k in H5_STORE if "/wfns/" in k and k.startswith(kwd["output_folder"])]
        for key, val in H5_STORE[sorted(wf)[0]].items():
            r[f"wfn0_{key}"] = val
        if name == "oh_1d":
            r.update(probe=probe, probe_v=ho1d.oh_stretch_harm(probe.copy()),
                     probe_v_kwargs=ho1d.oh_stretch_harm_with_arg(probe.copy(), dict(kw)),
                     kw_mass=kw["mass"], kw_freq=kw["freq"])
        runs[name] = r
    fixtures.update(runs)

    # --- checkpoints the reference writes (SimArchivist.chkpt: its pickled DMC_Sim) and
    # the reference's own dmc_restart continuing from them: a 1D continuous-weight run
    # checkpointed inside an open descendant-weighting window (like the reference's
    # restart fixture chkpts/pytest_364.pickle), and a 3D discrete water run.  The
    # checkpoint is the one a finished run leaves (written after its last step, with
    # cur_timestep = that step; the reference's restart runs that step again).  The
    # fixture keeps the checkpoint file's bytes and the restarted run's results.
    p, masses = oracle.h2o_config()
    eq = oracle.h2o_equilibrium(p)
    for name, pot_fn, atoms, x0, weighting, thresh, steps, chk, add, s1, s2, dt in (
            ("restart_oh_cont", ho1d.oh_stretch_harm, ["O-H"], np.zeros((1, 1, 1)), "continuous", [0.05, 2.5],
             30, 29, 20, 11, 12, 5.0),
            ("restart_h2o_disc", lambda c, p=p: oracle.pes_h2o_lm(c, p), ["O", "H", "H"],
             eq[None] + 0.05 * oracle.InjectedNoise(909).standard_normal((256, 3, 3)), "discrete", None,
             30, 29, 10, 13, 14, 10.0)):
        folder = os.path.join(tmp, name)
        n = 200 if len(x0) == 1 else len(x0)
        kwd = dict(sim_name=name, output_folder=folder, weighting=weighting, num_walkers=n, num_timesteps=steps,
                   equil_steps=5, chkpt_every=10 ** 6, wfn_every=1000, desc_wt_steps=30, atoms=atoms, delta_t=dt,
                   potential=pv.Potential_Direct(pot_fn), start_structures=np.array(x0, copy=True),
                   log_every=10 ** 6, cont_wt_thresh=thresh, masses=None if atoms == ["O-H"] else masses)
        sim = pv.DMC_Sim(**kwd)
        with _Patch(oracle.InjectedNoise(s1)):
            sim.run()
        ck = os.path.join(folder, "chkpts", f"{name}_{chk}.pickle")
        blob = np.frombuffer(open(ck, "rb").read(), dtype=np.uint8).copy()
        for k in [k for k in H5_STORE if k.startswith(folder)]:
            del H5_STORE[k]
        r2 = pv.dmc_restart(pv.Potential_Direct(pot_fn), folder, name, additional_timesteps=add)
        with _Patch(oracle.InjectedNoise(s2)):
            r2.run()
        out = dict(pickle=blob, chkpt_step=chk, additional=add, seed2=s2, vref=np.array(r2._vref_vs_tau),
                   pop=np.array(r2._pop_vs_tau), x_final=np.array(r2._walker_coords))
        if weighting == "continuous":
            out["w_final"] = np.array(r2._cont_wts)
        wf = sorted(k for k in H5_STORE if "/wfns/" in k and k.startswith(folder))
        for key, val in H5_STORE[wf[0]].items():
            out[f"wfn0_{key}"] = val
        fixtures[name] = out

    # --- config-3 family: importance sampling with the Gaussian internal trial
    alpha, qe = oracle.h2o_trial_config(p)
    mod_dir = os.path.join(tmp, "trialmod")
    os.makedirs(mod_dir)
    with open(os.path.join(mod_dir, "gauss_trial_h2o.py"), "w") as fh:
        fh.write(TRIAL_MODULE.format(alpha=list(alpha), qe=list(qe)))
    imp = pv.ImpSampManager_NoMP(trial_function="trial", trial_directory=mod_dir,
                                 python_file="gauss_trial_h2o.py", deriv_function="derivs")
    n = 256
    x0 = eq[None] + 0.03 * oracle.InjectedNoise(404).standard_normal((n, 3, 3))
    r = run_reference(pv, tmp, "h2o_is", x0, ["O", "H", "H"], masses, 10.0, 30, pes, seed=4, imp=imp)
    fixtures["h2o_is"] = dict(x0=x0, seed=4, dt=10.0, nsteps=30, alpha=np.array(alpha), qe=np.array(qe), **r)

    # --- derivative pins on the reference test geometry (test_imp_samp_helper.py:8-11),
    # reordered O,H,H, plus random displacements
    wc = np.array([[1.81005599, 0., 0.], [-0.45344658, 1.75233806, 0.], [0., 0., 0.]]) * 1.01
    wc = wc[[2, 0, 1]]
    geo = wc[None] + 0.05 * oracle.InjectedNoise(505).standard_normal((64, 3, 3))
    sys.path.insert(0, mod_dir)
    import gauss_trial_h2o as gt  # noqa: E402
    d1, d2 = gt.derivs(geo)
    fd1, fd2, fpsi = pv.ImpSamp.finite_diff(np.array(geo, copy=True), gt.trial)
    fixtures["h2o_trial_derivs"] = dict(geo=geo, psi=gt.trial(geo), d1=d1, d2=d2, fd1=fd1, fd2=fd2,
                                        fpsi=fpsi, alpha=np.array(alpha), qe=np.array(qe))

    # --- Metropolis / local KE pins through the reference's static methods
    ns = oracle.InjectedNoise(606)
    xa = geo
    xb = geo + 0.02 * ns.standard_normal(geo.shape)
    sig = np.sqrt(10.0 / np.asarray(masses))
    sig3 = np.repeat(sig, 3).reshape(3, 3)[None]
    inv3 = (1 / np.repeat(masses, 3)).reshape(3, 3)[None]
    fa, _ = gt.derivs(xa)
    fb, sdb = gt.derivs(xb)
    met = pv.ImpSamp.metropolis(sig3, gt.trial(xa), gt.trial(xb), xa, xb, inv3 * fa, inv3 * fb, 10.0)
    ke = pv.ImpSamp.local_kin(inv3, sdb)
    fixtures["h2o_metropolis"] = dict(xa=xa, xb=xb, met=met, ke=ke, masses=np.asarray(masses))

    for name, d in fixtures.items():
        if only and name not in only:
            continue
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in d.items()})
        print(f"wrote {path} ({os.path.getsize(path)} bytes)")


if __name__ == "__main__":
    # optional second argument: comma-separated fixture names to write (default: all)
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBDMC_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> [fixture,...]  (or set GBDMC_REFERENCE)")
    main(ref, set(sys.argv[2].split(",")) if len(sys.argv) > 2 else None)
