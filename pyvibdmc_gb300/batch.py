"""Batched ensembles of independent DMC replicas with uneven walker counts.

All replicas share one set of SoA walker arrays (replica r owns slots
[off_r, off_r + cap_r)).  Replicas are grouped into walker-count buckets; a
bucket is stepped by one persistent launch per phase (``gbdmc_batch_step``:
move+PES+weights, then the branch index), with its tile width chosen by a
small autotuner that times the candidate widths on the device.  Buckets run
on their own streams and a whole batch of steps of all buckets is captured
into one CUDA graph.

Each replica is the same simulation ``DMC_Sim`` would run with
``replica_id = r`` and the bucket's ``block_threads`` (same Philox stream,
same tiles), so a replica can be re-run on its own and compared step by step.
"""
import ctypes as C

import numpy as np
import torch

from . import _capi
from .constants import Constants
from .potentials import Potential_GPU, default_device, to_soa, from_soa

__all__ = ["DMC_Batch", "blocking_error"]

_MASSIVE = "Massive walker birth or death event!!!!!!! Dying..."


def blocking_error(series, nblocks=20):
    """Mean and standard error of a correlated series from `nblocks` block means."""
    s = np.asarray(series, dtype=np.float64)
    nb = max(2, min(nblocks, len(s) // 2))
    m = s[: len(s) // nb * nb].reshape(nb, -1).mean(1)
    return float(s.mean()), float(m.std(ddof=1) / np.sqrt(nb))


class DMC_Batch:
    """Independent replicas of one system run together.

    :param potential: a :class:`Potential_GPU`
    :param num_walkers: list of target populations, one per replica
    :param start_structures: (1, A, 3) geometry copied to every walker, or a
        list of (n_r, A, 3) arrays
    :param masses: atomic masses (a.u.)
    :param delta_t: time step (a.u.)
    :param num_timesteps: steps of history kept per replica
    :param imp_samp: optional :class:`ImpSampManager_GPU` (importance sampling)
    :param buckets: upper bounds of the walker-count buckets
    :param block_threads: fixed tile width for every bucket (skips the tuner)
    """

    CANDIDATES = (64, 128, 192, 256)

    def __init__(self, potential, num_walkers, start_structures, masses, delta_t, num_timesteps, imp_samp=None,
                 seed=0, rng="philox32", buckets=(4096, 16384, 1 << 40), block_threads=None, graph_steps=16,
                 start_noise=0.0, device=None, stats=False):
        if not isinstance(potential, Potential_GPU):
            raise TypeError("potential must be a Potential_GPU")
        if rng not in ("philox32", "philox64"):
            raise ValueError("DMC_Batch draws its deviates with Philox ('philox32' or 'philox64')")
        self.potential = potential
        self.imp_samp = imp_samp
        self.n0 = [int(n) for n in num_walkers]
        if not self.n0 or len(self.n0) > 4 * _capi.MAX_REPLICAS * 16:
            raise ValueError("need at least one replica")
        self.R = len(self.n0)
        self.masses = np.asarray(masses, dtype=np.float64)
        self.A = potential.natoms
        self.dt = float(delta_t)
        self.T = int(num_timesteps)
        self.seed = int(seed)
        self.noise_mode = _capi.NOISE_PHILOX32 if rng == "philox32" else _capi.NOISE_PHILOX64
        self.graph_steps = max(2, int(graph_steps) // 2 * 2)
        self.device = torch.device(device) if device is not None else default_device()
        self.fixed_tpb = block_threads
        self.stats = stats
        self.caps = [((int(np.floor(n + n * 0.5)) + 1) + 31) // 32 * 32 for n in self.n0]
        # bucket replicas by walker count (stable within a bucket), then lay out slots
        bidx = [int(np.searchsorted(np.asarray(buckets), n, side="left")) for n in self.n0]
        self.order = sorted(range(self.R), key=lambda r: (bidx[r], r))
        self.offs = [0] * self.R
        off = 0
        for r in self.order:
            self.offs[r] = off
            off += self.caps[r]
        self.ld = off
        self._alloc(start_structures, start_noise)
        self.buckets = []
        for b in sorted(set(bidx)):
            reps = [r for r in self.order if bidx[r] == b]
            for k in range(0, len(reps), _capi.MAX_REPLICAS):
                self.buckets.append(self._make_bucket(reps[k:k + _capi.MAX_REPLICAS]))
        self._graphs = {}
        self.tuning = {}

    # ------------------------------------------------------------ set-up
    def _alloc(self, start, noise_scale):
        dev, ld, A = self.device, self.ld, self.A
        f64 = dict(dtype=torch.float64, device=dev)
        IS = self.imp_samp is not None
        self._bufs = []
        for _ in range(2):
            b = dict(x=torch.zeros(3 * A, ld, **f64), v=torch.zeros(ld, **f64),
                     who=torch.zeros(ld, dtype=torch.int32, device=dev),
                     idx=torch.zeros(ld, dtype=torch.int32, device=dev))
            if IS:
                b.update(f=torch.zeros(3 * A, ld, **f64), psi=torch.zeros(ld, **f64), ke=torch.zeros(ld, **f64))
            self._bufs.append(b)
        gen = np.random.default_rng(self.seed ^ 0x5EED)
        for r in range(self.R):
            n = self.n0[r]
            if isinstance(start, (list, tuple)):
                x0 = np.asarray(start[r], dtype=np.float64)
            else:
                x0 = np.repeat(np.asarray(start, dtype=np.float64).reshape(1, A, 3), n, axis=0)
                if noise_scale:
                    x0 = x0 + noise_scale * gen.standard_normal(x0.shape)
            self._bufs[0]["x"][:, self.offs[r]:self.offs[r] + n] = to_soa(x0, dev)
        self._cur, self._lazy = 0, False
        self._ctrl = torch.zeros(self.R, C.sizeof(_capi.Ctrl), dtype=torch.uint8, device=dev)
        ctrl = (_capi.Ctrl * self.R)()
        for j, r in enumerate(self.order):
            ctrl[j].n = self.n0[r]
        self._ctrl.copy_(torch.frombuffer(bytearray(bytes(ctrl)), dtype=torch.uint8).view(self.R, -1))
        T = max(self.T, 1)
        self._hist = dict(vref=torch.zeros(self.R, T, **f64), pop=torch.zeros(self.R, T, **f64))
        if self.stats:
            self._hist.update(vmin=torch.zeros(self.R, T, **f64), vmax=torch.zeros(self.R, T, **f64),
                              vmean=torch.zeros(self.R, T, **f64))

    def _make_bucket(self, reps):
        """Replicas `reps` (contiguous in self.order) stepped by one launch per phase."""
        j0 = self.order.index(reps[0])
        table = (_capi.Replica * len(reps))()
        for k, r in enumerate(reps):
            table[k].off, table[k].cap, table[k].n0, table[k].stream = self.offs[r], self.caps[r], self.n0[r], r
        L = _capi.load()
        scratch = torch.zeros(L.gbdmc_batch_scratch_bytes(table, len(reps)), dtype=torch.uint8, device=self.device)
        bk = dict(reps=reps, j0=j0, table=table, nrep=len(reps), scratch=scratch,
                  ctrl=self._ctrl[j0:j0 + len(reps)], stream=torch.cuda.Stream(device=self.device),
                  walkers=sum(self.n0[r] for r in reps))
        bk["sim"] = self._make_sim(bk, self.fixed_tpb or 0)
        return bk

    def _make_sim(self, bk, tpb):
        s = _capi.Sim()
        s.natoms = self.A
        s.weighting = _capi.DISCRETE
        s.noise_mode = self.noise_mode
        s.track_who = 1
        s.ld = self.ld
        s.n0 = 1
        s.dt = self.dt
        s.alpha = 1.0 / (2.0 * self.dt)
        for a in range(self.A):
            s.sigma[a] = float(np.sqrt(self.dt / self.masses[a]))
            s.inv_mass[a] = float(1.0 / self.masses[a])
        s.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        s.block_threads = int(tpb)
        s.pes = self.potential.pes_struct()
        if self.imp_samp is not None:
            s.trial = self.imp_samp.trial_struct()
        else:
            s.trial.kind, s.trial.natoms = _capi.TRIAL_NONE, self.A
        j0 = bk["j0"]
        h = self._hist
        row = lambda t: t[j0].data_ptr()  # noqa: E731  (replica-major rows, stride T)
        s.hist.vref, s.hist.pop = row(h["vref"]), row(h["pop"])
        if self.stats:
            s.hist.vmin, s.hist.vmax, s.hist.vmean = row(h["vmin"]), row(h["vmax"]), row(h["vmean"])
        s.hist.len = self.T
        return s

    def _walkers(self, b, with_idx):
        w = _capi.Walkers()
        w.x, w.v, w.who = b["x"].data_ptr(), b["v"].data_ptr(), b["who"].data_ptr()
        if "f" in b:
            w.f, w.psi, w.ke = b["f"].data_ptr(), b["psi"].data_ptr(), b["ke"].data_ptr()
        if with_idx:
            w.idx = b["idx"].data_ptr()
        return w

    # ------------------------------------------------------------ stepping
    def _step_bucket(self, bk, cur, lazy, stream):
        L = _capi.load()
        src = self._walkers(self._bufs[cur], lazy)
        dst = self._walkers(self._bufs[1 - cur], True)
        _capi.check(L.gbdmc_batch_step(C.byref(bk["sim"]), bk["table"], bk["nrep"], C.byref(src), C.byref(dst),
                                       C.c_void_p(bk["ctrl"].data_ptr()), C.c_void_p(bk["scratch"].data_ptr()),
                                       None, C.c_void_p(stream.cuda_stream)), "gbdmc_batch_step")

    def _step_all(self, cur, lazy, serial=False, events=None):
        """One step of every bucket, each on its own stream (one after the
        other when `serial`; `events[b]` = (start, end) recorded around bucket b)."""
        main = torch.cuda.current_stream()
        prev = main
        for b, bk in enumerate(self.buckets):
            bk["stream"].wait_stream(prev if serial else main)
            if events is not None:
                events[b][0].record(bk["stream"])
            self._step_bucket(bk, cur, lazy, bk["stream"])
            if events is not None:
                events[b][1].record(bk["stream"])
            prev = bk["stream"]
        for bk in self.buckets:
            main.wait_stream(bk["stream"])
        return 1 - cur, True

    def init(self):
        """Step-0 potential and vref of every replica."""
        L = _capi.load()
        w = self._walkers(self._bufs[self._cur], False)
        for bk in self.buckets:
            _capi.check(L.gbdmc_batch_init(C.byref(bk["sim"]), bk["table"], bk["nrep"], C.byref(w),
                                           C.c_void_p(bk["ctrl"].data_ptr()), C.c_void_p(bk["scratch"].data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)), "gbdmc_batch_init")
        self.step = 0

    def autotune(self, steps_per_candidate=20, graph_lengths=(8, 16, 32)):
        """Pick the tile width of each bucket and the steps per CUDA graph by
        timing real steps of the run: first every tile width on every bucket
        (buckets stepped one after the other, CUDA events around each,
        ``steps_per_candidate`` steps per width), then every graph length with
        the chosen widths (replays covering at least ``steps_per_candidate``
        steps, events around them).  Returns {bucket index: (tpb, microseconds
        per step, all timings)} and records the graph length under
        ``tuning['graph_steps']``."""
        if self.fixed_tpb:
            return {}
        if not self._lazy:
            self._cur, self._lazy = self._step_all(self._cur, self._lazy)
            self.step += 1
        timing = {b: {} for b in range(len(self.buckets))}
        for tpb in self.CANDIDATES:
            for bk in self.buckets:
                bk["sim"] = self._make_sim(bk, tpb)
            evs = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
                     for _ in self.buckets] for _ in range(steps_per_candidate)]
            for k in range(steps_per_candidate):
                self._cur, self._lazy = self._step_all(self._cur, True, serial=True, events=evs[k])
                self.step += 1
            torch.cuda.synchronize()
            for b in range(len(self.buckets)):
                timing[b][tpb] = sum(e[b][0].elapsed_time(e[b][1]) for e in evs) * 1e3 / steps_per_candidate
        for b, bk in enumerate(self.buckets):
            tpb = min(timing[b], key=timing[b].get)
            bk["sim"] = self._make_sim(bk, tpb)
            self.tuning[b] = (tpb, timing[b][tpb], dict(timing[b]))
        self._graphs.clear()
        gtime = {}
        s = torch.cuda.current_stream()
        for gl in graph_lengths:
            self.graph_steps = max(2, int(gl) // 2 * 2)
            self._graphs.clear()
            self._graph(self._cur).replay()  # capture + one warm replay
            self.step += self.graph_steps
            reps = max(1, -(-steps_per_candidate // self.graph_steps))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                self._graph(self._cur).replay()
            e1.record(s)
            torch.cuda.synchronize()
            self.step += reps * self.graph_steps
            gtime[self.graph_steps] = e0.elapsed_time(e1) * 1e3 / (reps * self.graph_steps)
        self.graph_steps = min(gtime, key=gtime.get)
        self._graphs.clear()
        self.tuning["graph_steps"] = (self.graph_steps, gtime[self.graph_steps], gtime)
        self.check()
        return dict(self.tuning)

    def _graph(self, cur):
        g = self._graphs.get(cur)
        if g is None:
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.graph(g, stream=side):
                c, lz = cur, True
                for _ in range(self.graph_steps):
                    c, lz = self._step_all(c, lz)
            torch.cuda.current_stream().wait_stream(side)
            self._graphs[cur] = g
        return g

    def run(self, nsteps, check=True):
        """Queue nsteps steps of every replica (CUDA graphs of graph_steps steps)."""
        done = 0
        if nsteps and not self._lazy:
            self._cur, self._lazy = self._step_all(self._cur, self._lazy)
            done = 1
        while nsteps - done >= self.graph_steps:
            self._graph(self._cur).replay()
            done += self.graph_steps
        while done < nsteps:
            self._cur, self._lazy = self._step_all(self._cur, True)
            done += 1
        self.step += nsteps
        if check:
            self.check()
        return self

    # ------------------------------------------------------------ results
    def ctrl(self):
        raw = self._ctrl.cpu().numpy()
        out = [None] * self.R
        for j, r in enumerate(self.order):
            out[r] = _capi.Ctrl.from_buffer_copy(raw[j].tobytes())
        return out

    def check(self):
        for r, c in enumerate(self.ctrl()):
            if c.status:
                raise ValueError(f"replica {r}: {_MASSIVE} (status {c.status}, step {c.err_step})")

    def vref_history(self):
        """(R, T) vref per replica (hartree), in replica order."""
        h = self._hist["vref"].cpu().numpy()
        out = np.zeros_like(h)
        for j, r in enumerate(self.order):
            out[r] = h[j]
        return out

    def pop_history(self):
        h = self._hist["pop"].cpu().numpy()
        out = np.zeros_like(h)
        for j, r in enumerate(self.order):
            out[r] = h[j]
        return out

    def zpe(self, start=None, stop=None, nblocks=20):
        """Per-replica ZPE (cm^-1) and its blocking error over steps [start, stop)."""
        v = Constants.convert(self.vref_history(), "wavenumbers", to_AU=False)
        stop = self.step if stop is None else stop
        start = stop // 4 if start is None else start
        res = [blocking_error(v[r, start:stop], nblocks) for r in range(self.R)]
        return np.array([m for m, _ in res]), np.array([e for _, e in res])

    def walker_steps(self, t0, t1):
        """Walkers moved in steps [t0, t1) summed over replicas."""
        p = self.pop_history()
        prev = np.concatenate([np.asarray(self.n0, dtype=float)[:, None], p[:, :-1]], axis=1)
        return float(prev[:, t0:t1].sum())

    def walkers(self, r):
        """Host copy of replica r's walkers (compacted on the device)."""
        c = self.ctrl()[r]
        n = int(c.n)
        L = _capi.load()
        if self._lazy:
            src = self._walkers(self._bufs[self._cur], True)
            dst = self._walkers(self._bufs[1 - self._cur], False)
            for bk in self.buckets:
                _capi.check(L.gbdmc_walkers_compact(C.byref(bk["sim"]), bk["table"], bk["nrep"], C.byref(src),
                                                    C.byref(dst), C.c_void_p(bk["ctrl"].data_ptr()),
                                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                            "gbdmc_walkers_compact")
            self._cur, self._lazy = 1 - self._cur, False
        x = self._bufs[self._cur]["x"][:, self.offs[r]:self.offs[r] + n]
        return from_soa(x, n, self.A)
