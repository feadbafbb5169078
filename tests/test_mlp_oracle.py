"""The MLP oracle on the CPU: its fp64 gradients are the derivatives of its
loss (central differences), its bf16 conversion rounds to nearest even, and
its emulation of the training kernels' rounding stays within bf16 error of
the exact gradients."""
import numpy as np

from oracle import mlp_oracle as mo


def _net(seed, M=64):
    g = np.random.default_rng(seed)
    P = {"W1": 0.3 * g.standard_normal((16, 128)), "b1": 0.1 * g.standard_normal(128),
         "W2": 0.1 * g.standard_normal((128, 128)), "b2": 0.1 * g.standard_normal(128),
         "W3": 0.1 * g.standard_normal((128, 128)), "b3": 0.1 * g.standard_normal(128),
         "w4": 0.1 * g.standard_normal(128), "b4": 0.05}
    D = g.standard_normal((M, 16))
    D[:, 15] = 0.0
    U = g.standard_normal((M, 16))
    U[:, 15] = 0.0
    return P, D, U, g.standard_normal(M), g.standard_normal(M)


def _loss(P, D, U, e, et, wE=1.0, wF=0.5):
    E, Et, _ = mo.mlp_forward(P, D, U)
    return wE * np.mean((E - e) ** 2) + wF * np.mean((Et - et) ** 2)


def test_fp64_gradients_are_the_derivatives_of_the_loss():
    P, D, U, e, et = _net(0)
    G, _ = mo.mlp_loss_grads(P, D, U, e, et)
    g = np.random.default_rng(1)
    h = 1e-6
    for k in ("W1", "b1", "W2", "b3", "w4"):
        for _ in range(3):
            idx = tuple(int(g.integers(0, n)) for n in np.shape(P[k]))
            if k == "W1":
                idx = (int(g.integers(0, 15)), idx[1])
            Pp = {q: np.array(v, copy=True) for q, v in P.items()}
            Pm = {q: np.array(v, copy=True) for q, v in P.items()}
            Pp[k][idx] += h
            Pm[k][idx] -= h
            fd = (_loss(Pp, D, U, e, et) - _loss(Pm, D, U, e, et)) / (2 * h)
            assert abs(G[k][idx] - fd) < 1e-6 * max(1.0, abs(fd)), (k, idx, G[k][idx], fd)
    fd = (_loss(dict(P, b4=P["b4"] + h), D, U, e, et) - _loss(dict(P, b4=P["b4"] - h), D, U, e, et)) / (2 * h)
    assert abs(G["b4"][0] - fd) < 1e-6


def test_bf16_rounds_to_nearest_even():
    one = 1.0
    step = 2.0 ** -7  # bf16 spacing just above 1
    assert mo.bf16(one + step / 2) == one  # tie to the even neighbour (1.0)
    assert mo.bf16(one + 1.5 * step) == one + 2 * step  # tie to the even neighbour (1 + 2 step)
    assert mo.bf16(one + 0.5001 * step) == one + step
    assert mo.bf16(-3.0) == -3.0 and mo.bf16(0.0) == 0.0


def test_bf16_emulation_is_within_bf16_error_of_the_exact_gradients():
    P, D, U, e, et = _net(2, M=256)
    exact, _ = mo.mlp_loss_grads(dict(P, b4=0.0), D, U, e - P["b4"], et)
    emul, _ = mo.mlp_loss_grads_bf16(P, D, U, e - P["b4"], et)
    for k in exact:
        rel = np.linalg.norm(np.ravel(emul[k]) - np.ravel(exact[k])) / np.linalg.norm(np.ravel(exact[k]))
        assert 1e-5 < rel < 3e-2, (k, rel)  # bf16-sized: neither exact nor off


def _golden_distit():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "distit_dimer.npz"))


def _pair_charges():
    z = mo.DIMER_Z
    return np.array([z[i] * z[j] for i in range(6) for j in range(i + 1, 6)])


def test_sorted_dimer_descriptor_matches_the_reference_distit():
    """The oracle's canonical atom order against the reference's own DistIt
    (method 'coulomb', sorted_atoms=[[0],[1,2],[3],[4,5]],
    sorted_groups=[[0,1,2],[3,4,5]]) on 512 displaced dimers, each under one of
    the eight permutations of like atoms (tests/golden/make_distit_golden.py):
    the sorted and the unsorted Coulomb descriptors agree to rounding, and the
    sorting changes the descriptor of most of them."""
    d = _golden_distit()
    zz = _pair_charges()
    f, _ = mo.inv_dist_features(d["x"], sort=True)
    np.testing.assert_allclose(f * zz, d["sorted"], rtol=1e-13, atol=0)
    f0, _ = mo.inv_dist_features(d["x"])
    np.testing.assert_allclose(f0 * zz, d["unsorted"], rtol=1e-13, atol=0)
    assert np.mean(np.any(d["sorted"] != d["unsorted"], axis=1)) > 0.5


def test_sorted_descriptor_is_invariant_under_the_dimer_permutations():
    """All eight copies of a geometry under exchange of the hydrogens of either
    water and of the two waters get the same sorted descriptor and derivative;
    a planted mistake (an oxygen exchanged with a hydrogen) does not."""
    d = _golden_distit()
    x = d["x"][:32]
    v = np.random.default_rng(5).standard_normal(x.shape)
    f0, t0 = mo.inv_dist_features(x, v, sort=True)
    for g in (False, True):
        for a in (False, True):
            for b in (False, True):
                w1, w2 = ([0, 2, 1] if a else [0, 1, 2]), ([3, 5, 4] if b else [3, 4, 5])
                p = (w2 + w1) if g else (w1 + w2)
                f, t = mo.inv_dist_features(x[:, p], v[:, p], sort=True)
                np.testing.assert_allclose(f, f0, rtol=1e-15, atol=0)
                np.testing.assert_allclose(t, t0, rtol=1e-12, atol=1e-15)
    fb, _ = mo.inv_dist_features(x[:, [0, 1, 2, 4, 3, 5]], sort=True)
    assert np.all(np.abs(fb - f0).max(1) > 1e-3)
