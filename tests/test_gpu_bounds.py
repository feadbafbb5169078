"""The bounds-checked build (libgbdmc_bc.so, -DGBDMC_BOUNDS_CHECK) on the tiny
and edge-size cases: every data-dependent index of the step kernels is
checked against its range, and none of these runs may set an error bit.

The cases run in a child process that loads the checked library
(GBDMC_BOUNDS_CHECK=1): the plain step on injected deviates against the oracle
at N = 1, 31, 33 and 1025 (bit-exact, or the same population-guard stop), the
multi-step kernel against its replayed walk, continuous weighting with
both thresholds and importance sampling against the reference fixtures, a
Python getpot through gbdmc_sim_move / gbdmc_sim_branch, and the surrogate
step.  One more case feeds gbdmc_walkers_compact a gather index that lies
inside the buffers but outside the previous population: the checker flags
exactly that site (an in-range access, so the unchecked build reads a stale
walker rather than faulting)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r'''
import json, sys, ctypes as C
sys.path[:0] = [ROOT, HERE]
import numpy as np, torch
import oracle
import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import _capi
L = _capi.load()
assert L.gbdmc_bounds_check_enabled() == 1
out = {}
p, m = oracle.h2o_config()
eq = oracle.h2o_equilibrium(p)

def load(name):
    with np.load(f"{HERE}/golden/{name}.npz") as z:
        return {k: z[k] for k in z.files}

def sim(x0, pot, **kw):
    base = dict(num_walkers=len(x0), num_timesteps=20, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m,
                delta_t=10.0, potential=pot, start_structures=x0, write_files=False)
    base.update(kw)
    return pg.DMC_Sim(**base)

# the plain step on injected deviates against the oracle
for n in (1, 31, 33, 1025):
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(40 + n).standard_normal((n, 3, 3))
    s = sim(x0, pg.h2o_local_mode(), rng=oracle.InjectedNoise(n))
    try:
        ref = oracle.OracleDMC(x0, m, 10.0, lambda c: oracle.pes_h2o_lm(c, p), oracle.InjectedNoise(n)).run(20)
        ref_err = None
    except ValueError as e:
        ref, ref_err = None, str(e)
    try:
        s.run()
        err = None
    except ValueError as e:
        err = str(e)
    if ref_err is None:
        ok = err is None and np.array_equal(s._pop_vs_tau, np.array(ref.pop_hist)) and np.array_equal(s.walkers, ref.x)
    else:
        ok = err is not None
    out[f"plain_{n}"] = [bool(ok), int(L.gbdmc_bounds_errors(1))]

# the multi-step kernel against its walk replayed by the per-step kernels
from lineage_harness import replay
for n in (31, 33, 1025):
    x0 = eq[None] + 0.05 * oracle.InjectedNoise(60 + n).standard_normal((n, 3, 3))
    a = sim(x0, pg.h2o_local_mode(), num_timesteps=100, seed=11, fused_steps=64)
    a.run()
    kw = dict(num_walkers=n, num_timesteps=100, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m,
              delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=11)
    b, _ = replay(100, **kw)
    ok = a._multi_used and np.array_equal(a._hist["pop"].cpu().numpy()[:100],
                                          b._hist["pop"].cpu().numpy()[:100]) and np.array_equal(a.walkers, b.walkers)
    out[f"multi_{n}"] = [bool(ok), int(L.gbdmc_bounds_errors(1))]

# continuous weighting with both thresholds (the reference fixture)
g = load("h2o_cont_upper")
s = pg.DMC_Sim(sim_name="t", output_folder="/tmp/gbdmc_bc", weighting="continuous", num_walkers=len(g["x0"]),
               num_timesteps=int(g["nsteps"]), equil_steps=int(g["equil"]), chkpt_every=10 ** 6, wfn_every=10 ** 6,
               desc_wt_steps=int(g["desc"]), atoms=["O", "H", "H"], masses=m, delta_t=float(g["dt"]),
               potential=pg.h2o_local_mode(), start_structures=g["x0"], rng=oracle.InjectedNoise(int(g["seed"])),
               cont_wt_thresh=[float(t) for t in g["thresh"]], write_files=False)
s.run()
x, w = s.walkers
out["continuous_upper"] = [bool(np.array_equal(x, g["x_final"])), int(L.gbdmc_bounds_errors(1))]

# importance sampling (the reference fixture)
g = load("h2o_is")
s = sim(g["x0"], pg.h2o_local_mode(), num_timesteps=int(g["nsteps"]), rng=oracle.InjectedNoise(int(g["seed"])),
        imp_samp=pg.ImpSampManager_GPU("h2o_gauss", g["alpha"], g["qe"]))
s.run()
out["importance_sampling"] = [bool(np.allclose(s.walkers, g["x_final"], rtol=0, atol=1e-10)),
                              int(L.gbdmc_bounds_errors(1))]

# a Python getpot between the move and branching kernels
x0 = eq[None] + 0.05 * oracle.InjectedNoise(77).standard_normal((33, 3, 3))
a = sim(x0, pg.Potential_Direct(lambda c: oracle.pes_h2o_lm(c, p)), rng=oracle.InjectedNoise(5))
b = sim(x0, pg.h2o_local_mode(), rng=oracle.InjectedNoise(5))
a.run(); b.run()
out["external"] = [bool(np.array_equal(a.walkers, b.walkers)), int(L.gbdmc_bounds_errors(1))]

# the surrogate step (a briefly trained network: only the indices are checked here)
from pyvibdmc_gb300.surrogate import MLPSurrogate, NNDMC
pd, dm = oracle.dimer_config()
xd = oracle.dimer_equilibrium()[None] + 0.05 * oracle.InjectedNoise(8).standard_normal((2048, 6, 3))
mdl = MLPSurrogate(seed=0)  # trained briefly, as the inference tests do
xs, vd = pg.to_soa(xd, "cuda"), torch.as_tensor(oracle.pes_dimer(xd, pd), device="cuda")
gd = pg.to_soa(oracle.grad_dimer(xd, pd), "cuda")
mdl.set_normalisation(xs, vd)
for _ in range(30):
    mdl.train_batch(xs, vd, gd, lr=2e-3)
nd = NNDMC(mdl, pg.water_dimer(), [1025, 33], pg.WATER_DIMER_EQ[None], dm, 10.0, 30, seed=2, audit_every=5).init()
nd.run(30, check=False)
torch.cuda.synchronize()
out["surrogate"] = [True, int(L.gbdmc_bounds_errors(1))]

# a gather index inside the buffers but past the previous population
n = 64
s = sim(eq[None] + 0.05 * oracle.InjectedNoise(9).standard_normal((n, 3, 3)), pg.h2o_local_mode(), fused_steps=0)
s._init_device()
s._run_steps(1)
torch.cuda.synchronize()
c = s._read_ctrl()
if s._lazy:
    b = s._bufs[s._cur]
    b["idx"][0] = int(c.n_prev) + 3  # < capacity: an in-range read of a walker that is not in the population
    s._compact()
    out["planted_compact_gather"] = [True, int(L.gbdmc_bounds_errors(1))]
print("RESULT " + json.dumps(out))
'''


def test_bounds_checked_build_finds_no_bad_index():
    env = dict(os.environ, GBDMC_BOUNDS_CHECK="1")
    code = "ROOT, HERE = %r, %r\n" % (ROOT, HERE) + CHILD
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    line = [s for s in r.stdout.splitlines() if s.startswith("RESULT ")]
    assert r.returncode == 0 and line, r.stdout[-3000:] + r.stderr[-3000:]
    res = json.loads(line[-1][len("RESULT "):])
    planted = res.pop("planted_compact_gather", None)
    for name, (ok, bits) in res.items():
        assert ok, f"{name}: results differ under the bounds-checked build"
        assert bits == 0, f"{name}: bounds-check bits {bits:#x}"
    assert planted is not None and planted[1] == 1 << 2, planted  # kBcCompactGather only
