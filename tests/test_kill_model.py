"""The continuous-weighting kill algorithm of the GPU kernel (fast_kills in
pyvibdmc_gb300/csrc/gbdmc_step.cu), modelled step for step in NumPy, against
the oracle's sequential kills (pyvibdmc.py:340-356, :432-439): the final
weights bit for bit and the walker every slot ends up holding.

The model keeps the kernel's choices: weights compared as their 64-bit
patterns; chunks of 2^k weights with k from the kernel's load-count model;
per-chunk maxima (first index on ties); after a kill, the largest walker's
chunk scanned again and the killed slot's chunk updated with the half (or
scanned again when its largest was the killed slot); copies deferred along
the chain of sources, unless the largest weight fell below the threshold,
when they run in kill order.  The GPU tests check the kernel itself against
the oracle; this pins the argument that the chunked, deferred form is the
sequential algorithm, at sizes and tie patterns beyond them."""
import numpy as np
import pytest

from oracle import dmc_oracle as od


def _chunk_log(n, lo=6, max_chunks=2048):
    lk = lo
    while (n + (1 << lk) - 1) >> lk > max_chunks:
        lk += 1

    def cost(q):
        ch = (n + (1 << q) - 1) >> q
        return 2 * ((ch + 31) >> 5) + (((1 << q) + 31) >> 5)

    q = lk + 1
    while q < 20 and cost(q) < cost(lk):
        lk, q = q, q + 1
    return lk


def _chunk_best(key, lo, hi):
    seg = key[lo:hi]
    j = int(np.argmax(seg))  # the first index of the largest key
    return int(seg[j]), lo + j


def model_kills(w, thresh, counts=None):
    """(final weights, final walker of each slot) of the kernel's algorithm;
    ``counts`` (a dict) receives how often each branch of it was taken."""
    w = w.copy()
    n = len(w)
    kill = np.flatnonzero(w < thresh)
    holder = np.arange(n)
    if len(kill) == 0 or len(kill) == n:
        return None  # the kernel takes its block-wide path here
    lk = _chunk_log(n)
    nch = (n + (1 << lk) - 1) >> lk
    key = w.view(np.int64)  # non-negative doubles order like their patterns
    cv, ci = zip(*(_chunk_best(key, c << lk, min((c + 1) << lk, n)) for c in range(nch)))
    cv, ci = list(cv), list(ci)
    thr_key = int(np.array([thresh]).view(np.int64)[0])
    src = {}
    patho = False
    for to in kill:
        best = max(range(nch), key=lambda c: (cv[c], -ci[c]))
        bk, m = cv[best], ci[best]
        if bk < thr_key:
            patho = True
        h = w[m] * 0.5
        w[m] = h
        w[to] = h
        src[to] = m
        cm, ct = m >> lk, to >> lk
        cv[cm], ci[cm] = _chunk_best(key, cm << lk, min((cm + 1) << lk, n))
        if ct != cm:
            hk = int(key[to])
            if ci[ct] == to:
                cv[ct], ci[ct] = _chunk_best(key, ct << lk, min((ct + 1) << lk, n))
                if counts is not None:
                    counts["rescan"] = counts.get("rescan", 0) + 1
            elif hk > cv[ct] or (hk == cv[ct] and to < ci[ct]):
                cv[ct], ci[ct] = hk, int(to)
    killed = set(int(t) for t in kill)
    if counts is not None:
        counts["patho"] = patho
        counts["chained"] = sum(1 for to in kill if int(src[to]) in killed)
    if not patho:
        for to in kill:
            s = src[to]
            while s in killed:
                s = src[s]
            holder[to] = s
    else:
        for to in kill:
            holder[to] = holder[src[to]]
    return w, holder


def oracle_kills(w, thresh):
    st = {"w": w.copy(), "v": np.zeros(len(w)), "vref": 0.0, "x": np.arange(len(w), dtype=np.float64)}
    od.continuous_update_and_branch(st, 0.0, thresh)
    return st["w"], st["x"].astype(np.int64)


@pytest.mark.parametrize("n", [100, 2000, 20000, 70000])
@pytest.mark.parametrize("ties", [False, True])
def test_chunked_kills_are_the_sequential_kills(n, ties):
    rng = np.random.default_rng(n + ties)
    if ties:  # few distinct values: the first-index rule decides most picks
        w = rng.choice(np.array([0.25, 0.5, 1.0, 2.0, 4.0]) / n, size=n, p=[0.03, 0.27, 0.4, 0.2, 0.1])
        thresh = 0.3 / n
    else:
        w = rng.lognormal(0.0, 1.0, size=n) / n
        thresh = np.quantile(w, 0.03)
    counts = {}
    got = model_kills(w, thresh, counts)
    assert got is not None and not counts["patho"]
    assert ties or n < 1000 or counts["chained"] > 0  # sources that were killed earlier
    ref = oracle_kills(w, thresh)
    assert np.array_equal(got[0].view(np.int64), ref[0].view(np.int64))
    assert np.array_equal(got[1], ref[1])


def test_a_chunk_below_the_threshold():
    """A run of light walkers, heaviest first: a killed slot can be the largest
    of its chunk, whose maximum is then scanned again."""
    n = 20000
    rng = np.random.default_rng(11)
    w = rng.lognormal(0.0, 1.0, size=n) / n
    thresh = np.quantile(w, 0.02)
    w[3000:3700] = np.sort(rng.uniform(0.05, 0.9, size=700))[::-1] * thresh
    counts = {}
    got = model_kills(w, thresh, counts)
    assert counts.get("rescan", 0) > 0 and not counts["patho"]
    ref = oracle_kills(w, thresh)
    assert np.array_equal(got[0].view(np.int64), ref[0].view(np.int64))
    assert np.array_equal(got[1], ref[1])


def test_every_weight_below_the_threshold_keeps_the_kill_order():
    """When the largest weight falls below the threshold, a slot still waiting
    to be killed can be a source: the copies then run in kill order."""
    n = 3000
    rng = np.random.default_rng(7)
    w = rng.uniform(0.5, 1.0, size=n) / n
    w[::3] *= 4.0  # two thirds of the slots below the threshold, halvings drag the rest below it
    thresh = 1.9 / n
    counts = {}
    got = model_kills(w, thresh, counts)
    assert counts["patho"] and counts["chained"] > 0
    ref = oracle_kills(w, thresh)
    assert np.array_equal(got[0].view(np.int64), ref[0].view(np.int64))
    assert np.array_equal(got[1], ref[1])


def test_chunk_size_follows_the_load_model():
    assert _chunk_log(2000) == 6 and _chunk_log(20000) == 7 and _chunk_log(24000) == 8
    assert (10 ** 6 + (1 << _chunk_log(10 ** 6)) - 1) >> _chunk_log(10 ** 6) <= 2048
