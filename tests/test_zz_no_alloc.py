"""The allocation-free step entry point, gbdmc_sim_step_static.

Some callers cannot allocate device memory: code running under a framework
whose caching allocator owns the device, or a plug-in that only receives its
input and output buffers.  gbdmc_sim_step_static runs
the same walker step as gbdmc_sim_step, but its scratch lives in a static
device array inside libgbdmc.so instead of a caller-provided buffer.  This
test drives both entry points through the C ABI on identical walkers for two
steps in a row and requires the same results: populations and coordinates
bit for bit, vref within the 1e-12 Eh tolerance of the other parity tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import _capi

pytestmark = pytest.mark.gpu


def _sim(seed):
    _, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium()[None] + 0.05 * oracle.InjectedNoise(21).standard_normal((3000, 3, 3))
    sim = pg.DMC_Sim(num_walkers=3000, num_timesteps=8, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m,
                     delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=seed,
                     write_files=False)
    sim._init_device()
    return sim


def _two_steps(sim, static):
    L = _capi.load()
    for _ in range(2):
        src = sim._walker_struct(sim._bufs[sim._cur], sim._lazy)
        dst = sim._walker_struct(sim._bufs[1 - sim._cur], True)
        ctrl = C.c_void_p(sim._ctrl.data_ptr())
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        if static:
            rc = L.gbdmc_sim_step_static(C.byref(sim._sim), C.byref(src), C.byref(dst), ctrl, None, stream)
        else:
            rc = L.gbdmc_sim_step(C.byref(sim._sim), C.byref(src), C.byref(dst), ctrl,
                                  C.c_void_p(sim._scratch.data_ptr()), None, stream)
        _capi.check(rc, "step")
        sim._cur, sim._lazy = 1 - sim._cur, True
    torch.cuda.synchronize()
    c = sim._read_ctrl()
    assert c.status == 0 and c.step == 2
    return int(c.n), float(c.vref), sim._hist["vref"][:2].cpu().numpy(), sim.walkers


def test_static_scratch_step_matches_caller_scratch_step():
    n_a, vref_a, hist_a, x_a = _two_steps(_sim(17), static=False)
    n_b, vref_b, hist_b, x_b = _two_steps(_sim(17), static=True)
    assert n_a == n_b
    assert abs(vref_a - vref_b) <= 1e-12
    np.testing.assert_allclose(hist_a, hist_b, rtol=0, atol=1e-12)
    assert np.array_equal(x_a, x_b)


def test_static_scratch_rejects_oversized_capacity():
    L = _capi.load()
    sim = _sim(3)
    big = _capi.Sim.from_buffer_copy(bytes(sim._sim))
    big.ld = int(L.gbdmc_sim_step_static_max_ld()) + 1
    src = sim._walker_struct(sim._bufs[0], False)
    dst = sim._walker_struct(sim._bufs[1], True)
    rc = L.gbdmc_sim_step_static(C.byref(big), C.byref(src), C.byref(dst), C.c_void_p(sim._ctrl.data_ptr()), None,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _capi.ERR_CAPACITY
    assert b"static scratch" in L.gbdmc_last_error()


def _sim_cont(seed, n=3000):
    _, m = oracle.h2o_config()
    x0 = oracle.h2o_equilibrium()[None] + 0.05 * oracle.InjectedNoise(22).standard_normal((n, 3, 3))
    sim = pg.DMC_Sim(num_walkers=n, num_timesteps=8, equil_steps=10 ** 6, atoms=["O", "H", "H"], masses=m,
                     delta_t=10.0, potential=pg.h2o_local_mode(), start_structures=x0, seed=seed,
                     weighting="continuous", write_files=False)
    sim._init_device()
    return sim


def test_static_scratch_after_another_shape_and_continuous_weighting():
    """The static array left dirty by steps of another shape (500 walkers,
    continuous weighting) changes nothing: discrete and continuous steps
    through the static scratch then match the caller-scratch steps."""
    _two_steps(_sim_cont(5, n=500), static=True)
    n_a, vref_a, _, x_a = _two_steps(_sim(17), static=False)
    n_b, vref_b, _, x_b = _two_steps(_sim(17), static=True)
    assert n_a == n_b and abs(vref_a - vref_b) <= 1e-12 and np.array_equal(x_a, x_b)
    n_a, vref_a, _, (x_a, w_a) = _two_steps(_sim_cont(9), static=False)
    n_b, vref_b, _, (x_b, w_b) = _two_steps(_sim_cont(9), static=True)
    assert n_a == n_b and abs(vref_a - vref_b) <= 1e-12
    assert np.array_equal(x_a, x_b) and np.array_equal(w_a, w_b)
