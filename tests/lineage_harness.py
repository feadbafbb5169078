"""The multi-step kernel's walk replayed by the per-step kernels.

gbdmc_sim_run draws every walker's deviates and branching uniform from the
Philox stream of its lineage key (the walkers' logical indices at the
simulation's start; copy 0 keeps its parent's key, copy r >= 1 of a walker
with key k branching at step s takes lineage_key(k, r, s)); the keys travel
with the walkers from
launch to launch.  This harness runs the same walk through gbdmc_sim_step on
injected noise: before every step it draws the walkers' noise with
gbdmc_lineage_noise from their keys, and after it it follows the branching
(the gather index of the branched population, np.repeat order) to the next
keys.  Both use the device's own Philox, Box-Muller, move, potential and
branching code, so the two walks agree bit for bit (vref within 1e-12: the
sums are added in another order)."""
import ctypes as C

import numpy as np
import torch

import pyvibdmc_gb300 as pg
from oracle.philox_oracle import lineage_key
from pyvibdmc_gb300 import _capi


class _NoHostDraws:
    """Marks the simulation's noise as injected; the harness supplies it."""

    def standard_normal(self, shape):
        raise AssertionError("the harness injects the noise itself")

    def uniform(self, n):
        raise AssertionError("the harness injects the noise itself")


def replay(nsteps, noise="philox32", **kw):
    """DMC_Sim(**kw) stepped nsteps times by gbdmc_sim_step on the multi-step
    kernel's noise; returns the simulation (stopped at a guard as the engine
    stops) and whether a guard tripped."""
    sim = pg.DMC_Sim(rng=_NoHostDraws(), write_files=False, **kw)
    sim._init_device()
    L = _capi.load()
    s = _capi.Sim.from_buffer_copy(sim._sim)
    s.noise_mode = _capi.NOISE_PHILOX32 if noise == "philox32" else _capi.NOISE_PHILOX64
    nc = sim._ncoord
    keys = np.arange(int(sim._read_ctrl().n), dtype=np.uint64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for t in range(nsteps):
        c = sim._read_ctrl()
        if c.status:
            return sim, True
        n = int(c.n)
        kd = torch.as_tensor(keys.view(np.int64), device=sim.device)
        normal = torch.empty((nc, max(n, 1)), dtype=torch.float64, device=sim.device)
        u = torch.empty(max(n, 1), dtype=torch.float64, device=sim.device)
        _capi.check(L.gbdmc_lineage_noise(C.byref(s), C.c_void_p(kd.data_ptr()), n, int(c.step),
                                          C.c_void_p(normal.data_ptr()), max(n, 1), C.c_void_p(u.data_ptr()),
                                          stream), "gbdmc_lineage_noise")
        nz = _capi.Noise()
        nz.normal, nz.u_branch, nz.ld_noise = normal.data_ptr(), u.data_ptr(), max(n, 1)
        sim._cur, sim._lazy = sim._launch_step(sim._cur, sim._lazy, nz)
        torch.cuda.synchronize()
        c = sim._read_ctrl()
        if c.status:  # the step's moved, unbranched walkers, compact in its output
            sim._lazy = False
            return sim, True
        a = sim._bufs[sim._cur]["idx"][:int(c.n)].cpu().numpy().astype(np.int64)
        first = np.searchsorted(a, a, side="left")
        keys = lineage_key(keys[a], np.arange(len(a)) - first, int(c.step) - 1)
    return sim, False
