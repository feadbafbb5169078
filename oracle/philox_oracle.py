"""NumPy restatement of the GPU walker step's counter-based noise.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The reference draws its displacements from NumPy's global generator
(``np.random.normal`` in ``pyvibdmc/pyvibdmc.py:544-547``, branching uniforms
from ``np.random.random`` at ``pyvibdmc.py:392-403``).  A per-walker
counter-based stream replaces it on the GPU so that walkers can be moved in
any order and replicas never share deviates.  This module restates that
stream so the GPU noise layout is checked, value by value:

* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
  as 1, 2, 3", SC'11), pinned by the published known-answer vectors in
  ``tests/test_oracle_golden.py``;
* counter = (walker index, step low word, block slot | replica << 8,
  step high word ^ (walker >> 31)), key = (seed low word, seed high word);
* ``philox32``: two normals per two 32-bit draws, Box-Muller in fp32
  (u1 = fl32(a * 2^-32 + 2^-33) in (0, 1], u2 = (b >> 8) * 2^-24);
* ``philox64``: Box-Muller in fp64 from 53-bit uniforms;
* branch uniform: 53 bits from the next two 32-bit draws.

The fp32 transcendental functions (log, sqrt, sin/cos of pi*x) of the device
and of NumPy may differ in the last bits, so comparisons of the fp32 normals
use a relative tolerance of a few fp32 ulps; the Philox words are exact.
"""
import numpy as np

__all__ = ["philox4x32_10", "PhiloxStream", "philox_normals", "philox_branch_uniform", "lineage_key"]

_M32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 on uint32-valued arrays; returns four uint64 arrays of 32-bit words."""
    c = [np.asarray(v, dtype=np.uint64) & _M32 for v in (c0, c1, c2, c3)]
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    m0, m1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    w0, w1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    for _ in range(10):
        p0 = m0 * c[0]
        p1 = m1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & _M32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _M32
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
        k0 = (k0 + w0) & _M32
        k1 = (k1 + w1) & _M32
    return c


class PhiloxStream:
    """The 32-bit draws of walkers ``walkers`` at step ``step`` (vectorised).
    With ``lineage`` the walkers are 64-bit lineage keys (the multi-step
    kernel's streams): counter = (key low word, key high word, step low word,
    slot | replica << 8 | 1 << 31)."""

    def __init__(self, seed, step, walkers, replica=0, lineage=False):
        self.k0 = int(seed) & 0xFFFFFFFF
        self.k1 = (int(seed) >> 32) & 0xFFFFFFFF
        self.i = np.asarray(walkers, dtype=np.uint64)
        self.s_lo = int(step) & 0xFFFFFFFF
        self.s_hi = (int(step) >> 32) & 0xFFFFFFFF
        self.rep = int(replica)
        self.lineage = bool(lineage)
        self.slot = 0
        self.buf = None
        self.used = 4

    def _block(self):
        n = self.i.shape
        if self.lineage:
            c = philox4x32_10(self.i & _M32, self.i >> np.uint64(32), np.full(n, self.s_lo, np.uint64),
                              np.full(n, self.slot | (self.rep << 8) | 0x80000000, np.uint64), self.k0, self.k1)
        else:
            c = philox4x32_10(self.i, np.full(n, self.s_lo, np.uint64),
                              np.full(n, self.slot | (self.rep << 8), np.uint64),
                              np.full(n, self.s_hi, np.uint64) ^ (self.i >> np.uint64(31)), self.k0, self.k1)
        self.slot += 1
        return c

    def next32(self):
        if self.used == 4:
            self.buf = self._block()
            self.used = 0
        v = self.buf[self.used]
        self.used += 1
        return v

    def uniform53(self):
        hi, lo = self.next32(), self.next32()
        return ((hi << np.uint64(21)) | (lo >> np.uint64(11))).astype(np.float64) * 2.0 ** -53

    def normal2_f32(self):
        a, b = self.next32(), self.next32()
        u1 = a.astype(np.float32) * np.float32(2.0 ** -32) + np.float32(2.0 ** -33)
        u2 = (b >> np.uint64(8)).astype(np.float32) * np.float32(2.0 ** -24)
        rad = np.sqrt(np.float32(-2.0) * np.log(u1))
        ang = np.pi * (2.0 * u2.astype(np.float64))
        c = np.cos(ang).astype(np.float32)
        s = np.sin(ang).astype(np.float32)
        return rad * c, rad * s

    def normal2_f64(self):
        u1 = 1.0 - self.uniform53()
        u2 = self.uniform53()
        rad = np.sqrt(-2.0 * np.log(u1))
        ang = np.pi * (2.0 * u2)
        return rad * np.cos(ang), rad * np.sin(ang)


def philox_normals(seed, step, walkers, ncoord, mode="philox32", replica=0, lineage=False):
    """(ncoord, len(walkers)) normals as the move kernel draws them, plus the stream
    positioned for the branch uniform."""
    st = PhiloxStream(seed, step, walkers, replica, lineage)
    out = np.empty((ncoord, len(st.i)), dtype=np.float64)
    for k in range(0, ncoord, 2):
        a, b = st.normal2_f32() if mode == "philox32" else st.normal2_f64()
        out[k] = a
        if k + 1 < ncoord:
            out[k + 1] = b
    return out, st


def philox_branch_uniform(seed, step, walkers, ncoord, mode="philox32", replica=0):
    """The branching uniform of each walker: the draw after its ncoord normals."""
    _, st = philox_normals(seed, step, walkers, ncoord, mode, replica)
    return st.uniform53()


def lineage_key(k, r, step):
    """Lineage keys of the multi-step kernel's walkers: copy r of a walker with
    key k, branching at step ``step``, keeps k for r = 0 and takes the
    SplitMix64 finaliser (Steele, Lea, Flood 2014; Vigna's constants) of
    k + r * 0x9E3779B97F4A7C15 + step * 0xD1B54A32D192ED03 for r >= 1 (uint64
    arrays, wrapping arithmetic)."""
    k = np.asarray(k, dtype=np.uint64)
    r = np.asarray(r, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = k + r * np.uint64(0x9E3779B97F4A7C15) + np.uint64(int(step) & 0xFFFFFFFFFFFFFFFF) * \
            np.uint64(0xD1B54A32D192ED03)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return np.where(r == 0, k, z)
