"""Forward walking of the surrogate's error (gbdmc_mlp_fw_begin / _end) and
the pure-weighted bias control built on it.

The kernels are checked against the same sums formed on the host from the
device's own arrays: at a window's start every live walker's ancestor id is
its slot and its error is the network energy minus the analytic energy; at
the window's end the descendant-weighted sum is the live walkers' errors
looked up through their ancestor ids (sum_s D_s delta_s, D_s from a bincount
of the ids)."""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
import pyvibdmc_gb300 as pg
from pyvibdmc_gb300 import _capi
from pyvibdmc_gb300.surrogate import MLPSurrogate, NNDMC, _p, _s

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    _, masses = oracle.dimer_config()
    x, v, g, _ = pg.harvest_training_data(pg.water_dimer(), 4000, 120, 10, pg.WATER_DIMER_EQ[None], masses, seed=3,
                                          equil=20)
    return MLPSurrogate(seed=0).fit(x, v, g, epochs=12, batch=2048, lr=3e-3)


def _live(nd):
    return np.concatenate([np.arange(nd.offs[r], nd.offs[r] + int(c.n)) for r, c in enumerate(nd.ctrls())])


def test_forward_walking_kernels_match_host_sums(model):
    _, masses = oracle.dimer_config()
    pot = pg.water_dimer()
    nd = NNDMC(model, pot, [700, 1500, 300], pg.WATER_DIMER_EQ[None], masses, 10.0, 120, seed=3, audit_every=10,
               bias_weighting="mixed").init()
    nd.run(40)
    L = _capi.load()
    reps, nrep = nd._rep_args()
    nd._compact()
    b = nd._bufs[nd._cur]
    w = nd._w(b, False)
    ld = nd.ld
    vnn = torch.zeros(ld, dtype=torch.float64, device="cuda")
    out = torch.zeros(ld, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    delta = torch.full((ld,), np.nan, dtype=torch.float64, device="cuda")
    part = torch.zeros(2 * _capi.FW_BLOCKS, dtype=torch.float64, device="cuda")
    _capi.check(L.gbdmc_mlp_energy(C.byref(nd._net), _p(b["x"]), ld, ld, _p(vnn), _p(out), _p(st), _s()))
    _capi.check(L.gbdmc_mlp_fw_begin(C.byref(nd._sim), reps, nrep, C.byref(w), _p(nd._ctrl), _p(vnn), _p(out),
                                     _p(delta), _p(part), _s()))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    live = _live(nd)
    who = b["who"].cpu().numpy()
    np.testing.assert_array_equal(who[live], live)
    d = delta.cpu().numpy()
    x = b["x"][:, torch.as_tensor(live, device="cuda")].double()
    exact = pot.eval_soa(x.contiguous(), len(live)).cpu().numpy()
    ref = np.where(out.cpu().numpy()[live] != 0, 0.0, vnn.cpu().numpy()[live] - exact)
    np.testing.assert_allclose(d[live], ref, rtol=0, atol=2e-7)  # the fp32 analytic energy: ~1e-7 relative
    pr = part.cpu().numpy().reshape(-1, 2)
    assert pr[:, 1].sum() == len(live)
    np.testing.assert_allclose(pr[:, 0].sum(), d[live].sum(), rtol=1e-12, atol=1e-13)
    # 60 steps later: the descendant-weighted sum
    nd.run(60)
    nd._compact()
    b2 = nd._bufs[nd._cur]
    _capi.check(L.gbdmc_mlp_fw_end(C.byref(nd._sim), reps, nrep, C.byref(nd._w(b2, False)), _p(nd._ctrl),
                                   _p(delta), _p(part), _s()))
    torch.cuda.synchronize()
    live2 = _live(nd)
    anc = b2["who"].cpu().numpy()[live2]
    assert set(anc) <= set(live)  # every walker descends from a walker alive at the start
    D = np.bincount(anc, minlength=ld)
    assert D.sum() == len(live2) and (D > 1).any() and (D[live] == 0).any()
    pr = part.cpu().numpy().reshape(-1, 2)
    assert pr[:, 1].sum() == len(live2)
    np.testing.assert_allclose(pr[:, 0].sum(), (D[live] * d[live]).sum(), rtol=1e-12, atol=1e-13)


def test_pure_weighted_bias_control(model):
    """Windows close on schedule, the offset is their running mean, it enters
    the applied correction, and a constant shift of the network (which moves
    the pure and mixed averages alike) leaves the offset unchanged.  The
    training box is opened wide here: a walker outside it takes the analytic
    energy, so its error would not move with the shift."""
    _, masses = oracle.dimer_config()
    pot = pg.water_dimer()
    w = pg.Constants.atomic_units["wavenumbers"]
    runs = []
    margin, model.hull_margin = model.hull_margin, 1e6
    for shift in (0.0, 150.0):
        nd = NNDMC(model, pot, [900, 1300], pg.WATER_DIMER_EQ[None], masses, 10.0, 400, seed=7, audit_every=10,
                   bias_control=0.2, fw_time=320.0)
        assert nd._fw_len == 32
        e0 = float(nd._net.e_mean)
        nd._net.e_mean += shift * w
        nd._audit[4] = float(nd._net.e_mean) - e0
        nd.init().run(200)
        runs.append((nd, float(nd._net.e_mean) - e0))
    model.hull_margin = margin
    (a, _), (b, d) = runs
    h = a.fw_history()
    assert len(h) == 200 // 32 - 1 and np.array_equal(h[:, 0], np.arange(2, 200 // 32 + 1) * 32)
    r = h[:, 2] - h[:, 1]
    off = 0.0
    for k, rk in enumerate(r, 1):
        off += max(1.0 / k, 0.25) * (rk - off)
    au = a.audit()
    assert abs(au["pure_offset_cm"] - off) < 1e-9
    assert au["pure_offset_cm"] != 0.0
    assert abs(au["bias_correction_cm"] - (float(a._audit[4].item()) / w + off)) < 1e-9
    hb = b.fw_history()
    np.testing.assert_allclose(hb[:, 1:] - h[:, 1:], d / w, rtol=0, atol=1e-6)
    np.testing.assert_allclose(b.audit()["pure_offset_cm"], au["pure_offset_cm"], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(a.pop_history(), b.pop_history())
