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

__all__ = ["mlp_forward", "mlp_loss_grads", "silu", "dsilu", "d2silu", "inv_dist_features"]


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


def inv_dist_features(x, v=None):
    """1/r_ij (15 pairs, i<j) and their directional derivative along v, (N,6,3) inputs."""
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
