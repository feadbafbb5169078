"""NumPy (float64) reference of the MLP surrogate and its force-matching loss.

TEST INFRASTRUCTURE ONLY (checker for the GPU training and inference
kernels).  The network maps the normalised descriptor row D (16, last entry
zero) to E = h3 . w4 + b4 with h_l = silu(h_{l-1} W_l + b_l).  The tangent
stream carries the directional derivative along u (the descriptor change for
a Cartesian direction): Et = dE/dD . u.  Loss
    L = wE mean (E - e)^2 + wF mean (Et - et)^2
and its gradient with respect to every parameter (the tangent part needs
silu'').
"""
import numpy as np

__all__ = ["mlp_forward", "mlp_loss_grads", "silu", "dsilu", "d2silu", "inv_dist_features", "bf16", "f32",
           "mlp_energy_tc", "mlp_loss_grads_bf16", "dimer_sort_perm", "DIMER_Z"]

DIMER_Z = np.array([8.0, 1.0, 1.0, 8.0, 1.0, 1.0])  # O, H, H, O, H, H


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def d2silu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 - s) * (2.0 + z * (1.0 - 2.0 * s))


def mlp_forward(P, D, U=None):
    """Returns E, Et and the cache of pre-activations/activations."""
    cache = {"H0": D, "Ht0": U}
    h, ht = D, U
    for l in (1, 2, 3):
        z = h @ P[f"W{l}"] + P[f"b{l}"]
        cache[f"Z{l}"] = z
        if ht is not None:
            zt = ht @ P[f"W{l}"]
            cache[f"Zt{l}"] = zt
            ht = dsilu(z) * zt
        h = silu(z)
        cache[f"H{l}"], cache[f"Ht{l}"] = h, ht
    E = h @ P["w4"] + P["b4"]
    Et = ht @ P["w4"] if ht is not None else None
    return E, Et, cache


def mlp_loss_grads(P, D, U, e, et, wE=1.0, wF=0.5):
    M = len(D)
    E, Et, c = mlp_forward(P, D, U)
    dE = 2.0 * wE * (E - e) / M
    dEt = 2.0 * wF * (Et - et) / M
    G = {"w4": c["H3"].T @ dE + c["Ht3"].T @ dEt, "b4": np.array([dE.sum()])}
    hb = np.outer(dE, P["w4"])
    htb = np.outer(dEt, P["w4"])
    for l in (3, 2, 1):
        z, zt = c[f"Z{l}"], c[f"Zt{l}"]
        zb = dsilu(z) * hb + d2silu(z) * zt * htb
        ztb = dsilu(z) * htb
        G[f"W{l}"] = c[f"H{l-1}"].T @ zb + c[f"Ht{l-1}"].T @ ztb
        G[f"b{l}"] = zb.sum(0)
        hb = zb @ P[f"W{l}"].T
        htb = ztb @ P[f"W{l}"].T
    loss = (((E - e) ** 2).sum(), ((Et - et) ** 2).sum())
    return G, loss


def dimer_sort_perm(x):
    """Canonical atom order of water dimers, (N,6,3) -> (N,6) permutations
    (position p holds atom perm[:, p]) and the relative margins of the three
    decisions (N,3), restating DistIt with method 'coulomb',
    sorted_atoms=[[0],[1,2],[3],[4,5]] and sorted_groups=[[0,1,2],[3,4,5]]
    (tensorflow_descriptors/distance_descriptors.py:115-152, 177-213):
      - Coulomb matrix M_ij = z_i z_j / r_ij, M_ii = z_i^2.4 / 2 (:154-165);
      - sort_atoms (:115-131): within each group of like atoms, descending
        column norm of M (NumPy's argsort of -norm over six entries is an
        insertion sort, so ties keep the given order);
      - sort_groups (:133-152), on the atom-sorted matrix: the groups by
        descending sum of their columns' norms (the same sums, since atom
        sorting permutes columns within a group)."""
    x = np.asarray(x, dtype=np.float64)
    z = DIMER_Z
    d = x[:, :, None, :] - x[:, None, :, :]
    r = np.sqrt((d ** 2).sum(-1))
    n = len(x)
    M = np.empty((n, 6, 6))
    off = ~np.eye(6, dtype=bool)
    M[:, off] = (np.outer(z, z)[off])[None] / r[:, off]
    M[:, np.arange(6), np.arange(6)] = 0.5 * z ** 2.4
    cn = np.linalg.norm(M, axis=1)
    perm = np.tile(np.arange(6), (n, 1))
    sa = cn[:, 2] > cn[:, 1]
    sb = cn[:, 5] > cn[:, 4]
    perm[sa, 1], perm[sa, 2] = 2, 1
    perm[sb, 4], perm[sb, 5] = 5, 4
    ta, tb = cn[:, :3].sum(1), cn[:, 3:].sum(1)
    sg = tb > ta
    perm[sg] = perm[sg][:, [3, 4, 5, 0, 1, 2]]
    marg = np.stack([np.abs(cn[:, 2] - cn[:, 1]) / cn[:, 1], np.abs(cn[:, 5] - cn[:, 4]) / cn[:, 4],
                     np.abs(tb - ta) / ta], 1)
    return perm, marg


def inv_dist_features(x, v=None, sort=False):
    """1/r_ij (15 pairs, i<j) and their directional derivative along v, (N,6,3)
    inputs; with sort, of the atoms in the canonical order of dimer_sort_perm."""
    if sort:
        perm, _ = dimer_sort_perm(x)
        rows = np.arange(len(x))[:, None]
        x = np.asarray(x)[rows, perm]
        v = None if v is None else np.asarray(v)[rows, perm]
    f, t = [], []
    for i in range(6):
        for j in range(i + 1, 6):
            d = x[:, i] - x[:, j]
            r = np.sqrt((d ** 2).sum(-1))
            f.append(1.0 / r)
            if v is not None:
                dv = v[:, i] - v[:, j]
                t.append(-(d * dv).sum(-1) / r ** 3)
    return np.stack(f, 1), (np.stack(t, 1) if v is not None else None)


def f32(a):
    """Round to float32 (returned as float64)."""
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def bf16(a):
    """Round to bfloat16, nearest even (the conversion the kernels' bf16 packs use),
    returned as float64."""
    u = np.asarray(a, dtype=np.float64).astype(np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def mlp_energy_tc(P, x, mu, inv_sd, e_mean, e_scale, sort=False):
    """The tcgen05 inference kernel's arithmetic with its rounding points
    (gbdmc_mlp_tc.cu): fp32 walkers; descriptors 1/r scaled to (1/r - mu)/sd in
    fp32 and rounded to bf16 as the A operand; hidden layers with the weights
    rounded to bf16 and halved (exact), the bias as a bf16 pair b_hi + b_lo of
    b/2, products summed exactly (the tensor cores accumulate in fp32); the
    accumulator is h = z/2 and silu(z) = h + h tanh(h) (exact tanh here: the
    kernel's tanh.approx.f32 differs by at most 2^-10.99 relative); the
    activations of layers 1 and 2 rounded to bf16, layer 3's kept in fp32;
    the output h3 . w4 + b4 and V = e_mean + e_scale * output.  (N, 6, 3)
    fp64 coordinates in, V (N,) out; sort as in inv_dist_features."""
    x = f32(x)
    f, _ = inv_dist_features(x, sort=sort)
    scale = f32(inv_sd[:15])
    shift = f32(-f32(mu[:15]) * scale)
    D = np.zeros((len(x), 16))
    D[:, :15] = bf16(f32(f32(f) * scale + shift))
    h = D
    for l in (1, 2, 3):
        W = bf16(P[f"W{l}"]) * 0.5
        hb = f32(0.5 * f32(P[f"b{l}"]))
        b_hi = bf16(hb)
        b_lo = bf16(f32(hb - b_hi))
        z2 = h @ W + b_hi + b_lo
        a = z2 + z2 * np.tanh(z2)
        h = bf16(a) if l < 3 else f32(a)
    e = h @ f32(P["w4"])
    return float(e_mean) + float(e_scale) * (e + float(np.asarray(P["b4"]).ravel()[0]))


def mlp_loss_grads_bf16(P, D, U, e, et, wE=1.0, wF=0.5, magnitudes=False):
    """The training kernels' arithmetic with their rounding points
    (gbdmc_mlp.cu: k_gemm_xw, k_silu_fwd, k_head, k_silu_bwd, k_gemm_tn): every
    GEMM operand rounded to bf16 (activations, tangents, back-propagated
    signals and the weights), products summed exactly and the sum rounded to
    fp32 (the tensor cores accumulate in fp32), the bias added in fp32; every
    buffer the kernels store is fp32; the logistic function 1 / (1 + exp(-z))
    in fp32; a layer's bias gradient is the column sum of the SiLU
    backward's fp32 output (before its bf16 rounding as a GEMM operand).  The
    output bias enters as a shift of the targets (e here is already shifted),
    so the head adds nothing.  D, U are the kernels' (M, 16)
    descriptor and tangent rows, e, et their (M,) targets.  Returns the
    gradients and the two loss sums; with ``magnitudes`` also the sums of the
    magnitudes of the terms each gradient entry adds up (the scale of the
    fp32 summation error, which cancellation leaves in place)."""
    M = len(D)
    Wb = {l: bf16(P[f"W{l}"]) for l in (1, 2, 3)}
    w4 = f32(P["w4"])
    h, ht = f32(D), f32(U)
    cache = {}
    for l in (1, 2, 3):
        z = f32(f32(bf16(h) @ Wb[l]) + f32(P[f"b{l}"]))
        zt = f32(bf16(ht) @ Wb[l])
        s = f32(1.0 / f32(1.0 + f32(np.exp(-z))))
        cache[l] = (h, ht, z, zt, s)
        h = f32(z * s)
        ht = f32(f32(s * f32(1.0 + f32(z * f32(1.0 - s)))) * zt)
    E = f32(h @ w4)
    Et = f32(ht @ w4)
    dE = f32(2.0 * wE * f32(E - f32(e)) / M)
    dEt = f32(2.0 * wF * f32(Et - f32(et)) / M)
    G = {"w4": h.T @ dE + ht.T @ dEt, "b4": np.array([dE.sum()])}
    Gm = {"w4": np.abs(h).T @ np.abs(dE) + np.abs(ht).T @ np.abs(dEt), "b4": np.array([np.abs(dE).sum()])}
    hb = f32(np.outer(dE, w4))
    htb = f32(np.outer(dEt, w4))
    for l in (3, 2, 1):
        hin, htin, z, zt, s = cache[l]
        d1 = f32(s * f32(1.0 + f32(z * f32(1.0 - s))))
        d2 = f32(f32(s * f32(1.0 - s)) * f32(2.0 + f32(z * f32(1.0 - f32(2.0 * s)))))
        zb32 = f32(d1 * hb + f32(d2 * zt) * htb)  # the SiLU backward's fp32 output
        zb = bf16(zb32)  # as a GEMM operand
        ztb = bf16(f32(d1 * htb))
        G[f"W{l}"] = bf16(hin).T @ zb + bf16(htin).T @ ztb
        G[f"b{l}"] = zb32.sum(0)  # summed by the SiLU backward itself, in fp32
        Gm[f"W{l}"] = np.abs(bf16(hin)).T @ np.abs(zb) + np.abs(bf16(htin)).T @ np.abs(ztb)
        Gm[f"b{l}"] = np.abs(zb32).sum(0)
        hb = f32(zb @ Wb[l].T)
        htb = f32(ztb @ Wb[l].T)
    loss = (float(((E - f32(e)) ** 2).sum()), float(((Et - f32(et)) ** 2).sum()))
    return (G, loss, Gm) if magnitudes else (G, loss)
