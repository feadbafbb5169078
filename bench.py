#!/usr/bin/env python
"""Walker-steps/s of the plain FP64 DMC step on one GB300.

Workload: H2O local-mode PES (O,H,H), 20000 walkers, dt = 10 a.u., discrete
birth/death with descendant weighting in 50-step windows, Philox4x32-10
noise.  A "step" is one pass of the walker step (move + PES + weights +
branching + vref) over the current population.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  A bench step is one 50-step descendant-
weighting window of the workload (gbdmc_desc_begin, 50 DMC steps in one
gbdmc_sim_run launch with the walkers resident in shared memory,
gbdmc_desc_weights).  ``value``: device-resident walker-steps/s, each window
timed with CUDA events on the launching stream, a 256 MiB buffer written
between windows so that every window starts with the walkers in HBM (L2
flushed).  ``e2e``: the same metric through the C ABI with the walkers in
page-locked host memory between calls: per window one gbdmc_sim_run_host
call, whose gbdmc_sim_run launch reads the walkers from the host arrays and
whose second kernel writes the control block, the branched walkers and the
window's history back into host memory, then one stream wait (three untimed
warm-up windows first; the timed region is the host's wall clock around the
calls).  The per-step
kernels (gbdmc_sim_step, L2 flushed every step) are reported under config.
``--impl reference`` times the CPU restatement of the reference's step loop
(oracle/) on the host cores.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-steps/s on 1 GB300, plain FP64 vs IS+NN-PES+batched at ZPE err ≤1 cm⁻¹"
UNIT = "walker-steps/s"
N_WALKERS = 20000
DT = 10.0
DESC_WINDOW = 50
WORKLOAD = "h2o_local_mode_plain_discrete_20k"
BYTES_MOVE_KERNEL = 2 * 9 * 8 + 8 + 4  # x read+write, V write, count write per walker (A=3, fp64)


def start_structures(n, seed):
    p = dict(re=1.81, theta_e=np.deg2rad(104.5))
    eq = np.array([[0.0, 0.0, 0.0], [p["re"], 0.0, 0.0],
                   [p["re"] * np.cos(p["theta_e"]), p["re"] * np.sin(p["theta_e"]), 0.0]])
    return eq[None] + 0.05 * np.random.default_rng(seed).standard_normal((n, 3, 3))


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# -------------------------------------------------------------- CPU sides
class _NumpyNoise:
    """NumPy's legacy RandomState deviates for the CPU baseline, drawn as the
    reference draws them (np.random.normal(0, sigmas, size) in move_randomly,
    np.random.random(N) in birth_or_death, pyvibdmc.py:544, :392)."""

    def __init__(self, seed):
        self.g = np.random.RandomState(seed)

    def normal(self, loc=0.0, scale=1.0, size=None):
        return self.g.normal(loc, scale, size)

    def random(self, size=None):
        return self.g.random_sample(size)


def _pool_pes(chunk):
    import oracle
    p, _ = oracle.h2o_config()
    return oracle.pes_h2o_lm(chunk, p)


def _pool_pes_dimer(chunk):
    import oracle
    p, _ = oracle.dimer_config()
    return oracle.pes_dimer(chunk, p)


def cpu_reference_rate(n_walkers, steps, cores, system="h2o", min_s=0.0, max_steps=100000):
    """Oracle port of DMC_Sim.propagate on the host: walker-steps/s of the
    local-mode water (system "h2o") or the water dimer ("dimer").  With
    cores > 1 the PES is sharded over a spawn pool the way
    potential_manager.Potential.getpot does (np.array_split, pool.map,
    np.concatenate).  Runs at least `steps` steps and at least `min_s`
    seconds (at most `max_steps` steps); returns (rate, seconds, steps)."""
    import oracle
    if system == "dimer":
        p, m = oracle.dimer_config()
        x0 = oracle.dimer_equilibrium()[None] + 0.02 * np.random.default_rng(5).standard_normal((n_walkers, 6, 3))
        pes1, poolf = (lambda c: oracle.pes_dimer(c, p)), _pool_pes_dimer
    else:
        p, m = oracle.h2o_config()
        x0 = start_structures(n_walkers, 5)
        pes1, poolf = (lambda c: oracle.pes_h2o_lm(c, p)), _pool_pes
    if cores > 1:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        pool = ctx.Pool(cores)
        pes = lambda c: np.concatenate(pool.map(poolf, np.array_split(c, cores)))  # noqa: E731
    else:
        pool = None
        pes = pes1
    try:
        sim = oracle.OracleDMC(x0, m, DT, pes, _NumpyNoise(1))
        sim.run(3)  # warm-up (step 0 potential + vref)
        pops = []
        t0 = time.perf_counter()
        while len(pops) < max_steps and (len(pops) < steps or time.perf_counter() - t0 < min_s):
            pops.append(len(sim.x))
            _single_step(sim)
        dt = time.perf_counter() - t0
    finally:
        if pool is not None:
            pool.close()
            pool.join()
    return float(np.sum(pops)) / dt, dt, len(pops)


def _single_step(sim):
    """One oracle step continuing an OracleDMC that has run (restates the
    loop body of pyvibdmc.py:772-848 for the plain discrete case)."""
    import oracle
    oracle.move_randomly(sim.x, sim.sigmas, sim.noise)
    sim.v = sim.pes(sim.x)
    u = sim.noise.random(size=len(sim.x))
    idx, counts, b, d = oracle.birth_or_death_discrete(sim.v, sim.vref, sim.dt, u, sim.pop_thresh[1])
    sim.x = sim.x[idx]
    sim.v = sim.v[idx]
    sim.vref = oracle.calc_vref(sim.v, sim.n0, sim.alpha)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    rate1, t1, k1 = cpu_reference_rate(N_WALKERS, max(args.steps // 10, 20), 1, min_s=10.0)
    best, kind_cores, sample = rate1, 1, f"{k1} steps in {t1:.1f} s"
    if cores > 1:
        try:
            ratep, tp, kp = cpu_reference_rate(N_WALKERS, max(args.steps // 20, 10), cores, min_s=10.0)
            if ratep > best:
                best, kind_cores, sample = ratep, cores, f"{kp} steps in {tp:.1f} s"
        except Exception:
            pass
    line = {"impl": "reference", "metric": METRIC, "value": best, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "walkers": N_WALKERS, "dt": DT},
            "cpu_baseline": {"value": best, "unit": UNIT, "cores": kind_cores, "kind": "port",
                             "sample": f"oracle restatement of DMC_Sim.propagate (plain, discrete), "
                                       f"{N_WALKERS} walkers, numpy; best of 1-process and "
                                       f"{cores}-process PES pool ({sample})"},
            "e2e": {"value": best, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- ours
def reduce_over_ranks(ms, walker_steps, dist, device):
    """Whole-job figures of N independent replicas: the slowest rank's time
    (max) and the walker-steps of all ranks (sum)."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ws = torch.tensor([walker_steps], dtype=torch.float64, device=device)
    dist.all_reduce(ws, op=dist.ReduceOp.SUM)
    return float(t.item()), float(ws.item())


def run_ours(args):
    import torch
    import pyvibdmc_gb300 as pg
    from pyvibdmc_gb300 import _capi

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = _capi.load()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    masses = [pg.Constants.mass("O"), pg.Constants.mass("H"), pg.Constants.mass("H")]
    K, W = args.steps, args.warmup
    # history length: warm-up, timed, back-to-back and e2e windows, the per-step leg and the host-resident leg
    T = (W + 3 * K + 10) * DESC_WINDOW + 6000
    sim = pg.DMC_Sim(sim_name="bench", num_walkers=N_WALKERS, num_timesteps=T, equil_steps=10 ** 9,
                     atoms=["O", "H", "H"], masses=masses, delta_t=DT, potential=pg.h2o_local_mode(),
                     start_structures=start_structures(N_WALKERS, 1 + rank), seed=1234 + rank, write_files=False,
                     fused_steps=DESC_WINDOW)
    sim._init_device()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ctrl_ptr = C.c_void_p(sim._ctrl.data_ptr())
    run_scratch = torch.zeros(L.gbdmc_sim_run_scratch_bytes(sim.capacity), dtype=torch.uint8, device=dev)
    desc = torch.zeros(int(sim.capacity), dtype=torch.float64, device=dev)
    evs = []

    def window(step_end, ev=None):
        """One descendant-weighting window of config 2: desc_begin, DESC_WINDOW
        steps in one gbdmc_sim_run launch (walkers resident in shared memory),
        desc_weights.  Three launches of this library."""
        b = sim._bufs[sim._cur]
        if ev is not None:
            ev[0].record(stream)
        _capi.check(L.gbdmc_desc_begin(C.c_void_p(b["who"].data_ptr()), ctrl_ptr, sp), "desc_begin")
        if ev is not None:
            ev[1].record(stream)
        src = sim._walker_struct(b, False)
        out = sim._bufs[1 - sim._cur]
        dst = sim._walker_struct(out, False)
        _capi.check(L.gbdmc_sim_run(C.byref(sim._sim), C.byref(src), C.byref(dst), ctrl_ptr,
                                    C.c_void_p(run_scratch.data_ptr()), step_end, DESC_WINDOW, sp), "sim_run")
        sim._cur = 1 - sim._cur
        if ev is not None:
            ev[2].record(stream)
        _capi.check(L.gbdmc_desc_weights(C.c_void_p(out["who"].data_ptr()), None, ctrl_ptr, int(sim.capacity),
                                         C.c_void_p(desc.data_ptr()), sp), "desc_weights")
        if ev is not None:
            ev[3].record(stream)

    sim._compact()
    s = int(sim._read_ctrl().step)
    for i in range(W):
        window(s + (i + 1) * DESC_WINDOW)
    torch.cuda.synchronize()
    step0 = int(sim._read_ctrl().step)
    # ---- timed: one event quadruple per window, L2 flushed between windows
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(K)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for i in range(K):
            flush.fill_(i & 0xFF)
            window(step0 + (i + 1) * DESC_WINDOW, evs[i])
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    gpu_launches = 3 * K
    ms = float(sum(e[0].elapsed_time(e[3]) for e in evs))
    run_ms = [e[1].elapsed_time(e[2]) for e in evs]
    c = sim._read_ctrl()
    if c.status:
        raise RuntimeError(f"device status {c.status} during the bench")
    step1 = int(c.step)
    pops = sim._hist["pop"][step0 - 1:step1 - 1].cpu().numpy()
    walker_steps = float(pops.sum())  # the population entering each timed step
    if dist is not None:
        ms, walker_steps = reduce_over_ranks(ms, walker_steps, dist, dev)
    value = walker_steps / (ms / 1e3)
    ms_per_step = ms / K

    # ---- the same windows back to back without flushing (information)
    e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s_before = int(sim._read_ctrl().step)
    e_a.record(stream)
    for i in range(K):
        window(s_before + (i + 1) * DESC_WINDOW)
    e_b.record(stream)
    torch.cuda.synchronize()
    s_after = int(sim._read_ctrl().step)
    popw = sim._hist["pop"][s_before - 1:s_after - 1].cpu().numpy()
    warm_rate = float(popw.sum()) / (e_a.elapsed_time(e_b) / 1e3)

    # ---- the per-step kernels (gbdmc_sim_step: k_move + k_branch per step), L2 flushed per step
    kp = min(max(K * DESC_WINDOW // 4, 100), 2000)
    ps_ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(kp)]
    s_before = int(sim._read_ctrl().step)
    _capi.check(L.gbdmc_prof_enable(1), "prof_enable")
    for i in range(kp):
        flush.fill_(i & 0xFF)
        ps_ev[i][0].record(stream)
        sim._cur, sim._lazy = sim._launch_step(sim._cur, sim._lazy)
        ps_ev[i][1].record(stream)
    mv_ms, mv_n, sc_ms, sc_n = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
    _capi.check(L.gbdmc_prof_read(C.byref(mv_ms), C.byref(mv_n), C.byref(sc_ms), C.byref(sc_n)), "prof_read")
    _capi.check(L.gbdmc_prof_enable(0), "prof_enable")
    s_after = int(sim._read_ctrl().step)
    popp = sim._hist["pop"][s_before - 1:s_after - 1].cpu().numpy()
    ps_ms = float(sum(a.elapsed_time(b) for a, b in ps_ev))
    per_step = {"walker_steps_per_s": float(popp.sum()) / (ps_ms / 1e3), "steps": kp,
                "us_per_step": ps_ms / kp * 1e3, "k_move_avg_us": mv_ms.value / max(mv_n.value, 1) * 1e3,
                "l2": "flushed between steps"}
    sim._compact()

    # ---- roofline of the dominant kernel, k_run (the gbdmc_sim_run launch)
    run_avg_s = float(np.mean(run_ms)) / 1e3
    ws_per_launch = walker_steps / K if dist is None else float(pops.sum()) / K
    achieved = BYTES_MOVE_KERNEL * ws_per_launch / run_avg_s / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "k_run_h2o_20k_traffic.json")
    if os.path.exists(tr_path):
        traffic = json.load(open(tr_path)).get("dram_bytes_per_launch")

    # ---- fp64 pipe probe (measured fp64 FMA rate)
    sink = torch.zeros(152 * 8, dtype=torch.float64, device=dev)
    flops = C.c_double()
    _capi.check(L.gbdmc_fp64_fma_probe(C.c_void_p(sink.data_ptr()), 64, 152 * 8, C.byref(flops), sp), "fp64")
    e_a.record(stream)
    _capi.check(L.gbdmc_fp64_fma_probe(C.c_void_p(sink.data_ptr()), 512, 152 * 8, C.byref(flops), sp), "fp64")
    e_b.record(stream)
    torch.cuda.synchronize()
    fp64_tflops = flops.value / (e_a.elapsed_time(e_b) / 1e3) / 1e12
    # the bound that binds: the FP64 FLOPs of a walker-step (ncu DADD/DMUL/DFMA counts) over the launch time
    fp64_roof = None
    fp_path = os.path.join(ROOT, "profiles", "k_run_h2o_20k_fp64.json")
    if os.path.exists(fp_path):
        fpw = json.load(open(fp_path))["fp64_flops_per_walker_step"]
        ach = fpw * ws_per_launch / run_avg_s / 1e12
        fp64_roof = {"bound": "fp64", "achieved": ach, "peak": fp64_tflops, "unit": "TFLOP/s",
                     "frac": ach / fp64_tflops, "peak_kind": "measured (gbdmc_fp64_fma_probe, this run)",
                     "flops_per_walker_step": fpw}

    # ---- e2e through the C ABI with host buffers
    e2e = run_e2e_windows(sim, L, dev, max(5, min(K, 100)), run_scratch)
    e2e["per_step_host_resident"] = run_e2e(sim, L, dev, max(50, min(K * 10, 500)))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded start geometries, Philox4x32-10 deviates)",
            "config": {"workload": WORKLOAD, "walkers_per_gpu": N_WALKERS, "dt": DT, "atoms": "O,H,H",
                       "weighting": "discrete", "desc_window": DESC_WINDOW, "noise": "philox32",
                       "step": f"one {DESC_WINDOW}-step descendant-weighting window: gbdmc_desc_begin, "
                               f"{DESC_WINDOW} DMC steps in one gbdmc_sim_run launch, gbdmc_desc_weights",
                       "dmc_steps_timed": step1 - step0,
                       "l2": "flushed between windows (256 MiB write); inside a window the walkers stay in "
                             "shared memory", "parallelism": f"replicas x{world}",
                       "windows_back_to_back_walker_steps_per_s": warm_rate,
                       "per_step_kernels": per_step, "wall_s_timed": wall},
            "gpu_launches": gpu_launches,
            "roofline": {"bound": "hbm", "kernel": "k_run (gbdmc_sim_run: 50 steps of move+PES+weights+"
                                                   "branching, walkers in shared memory)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": peak_kind, "traffic": traffic, "bytes_per_walker_step": BYTES_MOVE_KERNEL,
                         "kernel_avg_us": run_avg_s * 1e6, "fp64_fma_probe_tflops": fp64_tflops,
                         "fp64": fp64_roof},
            "e2e": e2e}
    if not args.no_extras and world == 1:
        try:
            line["extras"] = run_extras(max(64, min(K * DESC_WINDOW, 400)))
        except Exception as exc:  # the headline line must still print
            line["extras"] = {"error": repr(exc)[:300]}
    if rank == 0 and world == 1:
        rate, secs, ksteps = cpu_reference_rate(N_WALKERS, 20, 1, min_s=10.0)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"oracle restatement of DMC_Sim.propagate (plain, discrete), "
                                          f"{N_WALKERS} walkers x {ksteps} steps, numpy, {secs:.1f} s"}
    line["clocks"] = clk.summary()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_e2e_windows(sim, L, dev, windows, run_scratch):
    """The headline e2e: the reference-facing C-ABI call with host buffers,
    gbdmc_sim_run_host.  The walkers (coordinates, potentials, ancestor ids,
    lineage keys) live in page-locked host memory between calls, as the
    reference's NumPy walker arrays do; per window (one bench step) one call
    runs DESC_WINDOW steps in one gbdmc_sim_run launch that reads the N
    walkers from the host arrays over the host link, then a kernel writes the
    control block, the N' walkers and the window's vref / population history
    into host memory; one stream wait."""
    import torch
    from pyvibdmc_gb300 import _capi
    A3 = 3 * sim.natoms
    sim._compact()
    ld = int(sim._sim.ld)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    cb = C.sizeof(_capi.Ctrl)
    b0, b1 = sim._bufs[sim._cur], sim._bufs[1 - sim._cur]
    hx = torch.empty((A3, ld), dtype=torch.float64).pin_memory()
    hv = torch.empty(ld, dtype=torch.float64).pin_memory()
    hw = torch.empty(ld, dtype=torch.int32).pin_memory()
    hk = torch.empty(ld, dtype=torch.int64).pin_memory()
    hc = torch.empty(cb, dtype=torch.uint8).pin_memory()
    hh = torch.empty((2, DESC_WINDOW), dtype=torch.float64).pin_memory()
    n = int(sim._read_ctrl().n)
    hx[:, :n].copy_(b0["x"][:, :n])
    hw[:n].copy_(b0["who"][:n])
    hk[:n].copy_(b0["key"][:n])
    hc.copy_(sim._ctrl)
    torch.cuda.synchronize()
    ctrl_host = _capi.Ctrl.from_address(hc.data_ptr())
    host = _capi.HostWalkersC(x=hx.data_ptr(), v=hv.data_ptr(), who=hw.data_ptr(), key=hk.data_ptr(), ld=ld)
    w_src, w_dst = sim._walker_struct(b0, False), sim._walker_struct(b1, False)
    ctrl_ptr, scr, hist = C.c_void_p(sim._ctrl.data_ptr()), C.c_void_p(run_scratch.data_ptr()), C.c_void_p(hh.data_ptr())
    # the call's arguments are built once; the bookkeeping per window reads the
    # history through a NumPy view of the page-locked buffer
    head = (C.byref(sim._sim), C.byref(host), C.byref(w_src), C.byref(w_dst), ctrl_ptr, C.byref(ctrl_host), scr)
    pop = hh.numpy()[1]
    run_host = L.gbdmc_sim_run_host

    def call():
        step = ctrl_host.step
        rc = run_host(*head, step + DESC_WINDOW, DESC_WINDOW, hist, sp)
        if rc or ctrl_host.status:
            _capi.check(rc, "gbdmc_sim_run_host")
            raise RuntimeError(f"device status {ctrl_host.status} in the e2e leg")
        return step

    for _ in range(3):  # untimed warm-up windows
        call()
    h2d = d2h = 0
    total = 0.0
    t0 = time.perf_counter()
    for _ in range(windows):
        n = ctrl_host.n
        k = ctrl_host.step - call()
        total += n + float(pop[:k - 1].sum())  # the population entering each of the k steps
        h2d += (A3 * 8 + 4 + 8) * n
        d2h += cb + (A3 * 8 + 8 + 4 + 8) * ctrl_host.n + 16 * k
    secs = time.perf_counter() - t0
    sim._cur, sim._lazy = 1 - sim._cur, False  # the walkers are in the output buffer (and on the host)
    return {"value": total / secs, "unit": UNIT, "h2d_bytes_per_step": h2d // windows,
            "d2h_bytes_per_step": d2h // windows, "steps": windows,
            "path": f"walkers in page-locked host memory between calls; per bench step (one {DESC_WINDOW}-step "
                    "window) one gbdmc_sim_run_host call (C ABI): one gbdmc_sim_run launch reading the N walkers' "
                    "coordinates, ancestor ids and lineage keys from host memory, one kernel writing the control "
                    "block, the N' walkers (coordinates, potentials, ancestor ids, keys) and the window's vref and "
                    "population history to host memory; one stream wait per window"}


def _timed_graph_rate(run_steps, pop_of, steps):
    """walker-steps/s of `steps` queued steps (CUDA events around them)."""
    import torch
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = pop_of()
    e0.record(s)
    run_steps(steps)
    e1.record(s)
    torch.cuda.synchronize()
    return t0, e0.elapsed_time(e1) / 1e3


def run_extras(steps):
    """The other workloads of the metric, measured on the same GPU (walkers
    resident on the device, back-to-back graph-captured steps)."""
    import torch
    import pyvibdmc_gb300 as pg
    out = {}
    masses = [pg.Constants.mass("O"), pg.Constants.mass("H"), pg.Constants.mass("H")]
    # importance-sampled H2O, 50000 walkers
    sim = pg.DMC_Sim(num_walkers=50000, num_timesteps=steps + 64, equil_steps=10 ** 9, atoms=["O", "H", "H"],
                     masses=masses, delta_t=DT, potential=pg.h2o_local_mode(), imp_samp=pg.h2o_gaussian_trial(),
                     start_structures=start_structures(50000, 7), seed=11, write_files=False, graph_steps=16)
    sim._init_device()
    sim._run_steps(32)
    torch.cuda.synchronize()
    s0 = int(sim._read_ctrl().step)
    _, secs = _timed_graph_rate(sim._run_steps, lambda: 0, steps)
    pop = sim._hist["pop"][s0 - 1:s0 - 1 + steps].cpu().numpy()
    rej = sim._hist["rejected"][s0:s0 + steps].cpu().numpy()
    out["is_h2o_50k"] = {"walker_steps_per_s": float(pop.sum()) / secs, "us_per_step": secs / steps * 1e6,
                         "acceptance": float(1 - rej.sum() / pop.sum())}
    # variance-normalised efficiency of importance sampling: ZPE error bar per unit time, 20000 walkers each
    eff = {}
    for tag, trial in (("plain", None), ("is", pg.h2o_gaussian_trial())):
        T = 12000
        sm = pg.DMC_Sim(num_walkers=20000, num_timesteps=T, equil_steps=10 ** 9, atoms=["O", "H", "H"],
                        masses=masses, delta_t=DT, potential=pg.h2o_local_mode(), imp_samp=trial,
                        start_structures=start_structures(20000, 9), seed=21, write_files=False, graph_steps=32)
        sm._init_device()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sm._run_steps(T)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        vr = pg.Constants.convert(sm._hist["vref"].cpu().numpy()[T // 4:], "wavenumbers", to_AU=False)
        z, e = pg.blocking_error(vr, 30)
        eff[tag] = {"zpe_cm": z, "err_cm": e, "seconds": secs, "steps": T, "efficiency": 1.0 / (e * e * secs)}
    eff["is_gain_at_equal_error"] = eff["is"]["efficiency"] / eff["plain"]["efficiency"]
    out["is_vs_plain_h2o_20k"] = eff
    # importance sampling + batching: 64 IS replicas (N_r ~ U[1000, 65536]); the ensemble
    # estimate is the N0-weighted mean of the replicas' vref at each step
    ns = [int(v) for v in np.random.default_rng(0).integers(1000, 65537, size=64)]
    th = np.deg2rad(104.5)
    eq = np.array([[0.0, 0.0, 0.0], [1.81, 0.0, 0.0], [1.81 * np.cos(th), 1.81 * np.sin(th), 0.0]])
    Tb = 4000
    bi = pg.DMC_Batch(pg.h2o_local_mode(), ns, eq[None], masses, DT, Tb + 400, imp_samp=pg.h2o_gaussian_trial(),
                      seed=5, start_noise=0.05, graph_steps=16)
    bi.init()
    bi.autotune(steps_per_candidate=20)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    bi.run(Tb)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0 + 0.0
    s0 = bi.step - Tb
    w = np.asarray(ns, dtype=float)
    vr = pg.Constants.convert(bi.vref_history()[:, s0:bi.step], "wavenumbers", to_AU=False)
    ens = (w[:, None] * vr).sum(0) / w.sum()
    z, e = pg.blocking_error(ens[Tb // 4:], 30)
    ws = bi.walker_steps(s0, bi.step)
    isb = {"replicas": len(ns), "walkers_total": int(sum(ns)), "steps": Tb, "seconds": secs,
           "walker_steps_per_s": ws / secs, "zpe_cm": z, "err_cm": e, "efficiency": 1.0 / (e * e * secs)}
    isb["gain_vs_plain_h2o_20k_at_equal_error"] = isb["efficiency"] / eff["plain"]["efficiency"]
    out["is_batched_64_replicas_h2o"] = isb
    # continuous weighting (pyvibdmc.py:432-454), H2O, 20000 walkers: the per-step kernels with the
    # sequential argmax cloning of every walker below 1/N0
    sc = pg.DMC_Sim(num_walkers=20000, num_timesteps=1264, equil_steps=10 ** 9, atoms=["O", "H", "H"],
                    masses=masses, delta_t=DT, potential=pg.h2o_local_mode(), start_structures=start_structures(20000, 13),
                    seed=17, weighting="continuous", write_files=False, graph_steps=16)
    sc._init_device()
    sc._run_steps(64)
    torch.cuda.synchronize()
    _, secs = _timed_graph_rate(sc._run_steps, lambda: 0, 1000)
    kills = sc._hist["births"][64:1064].cpu().numpy()
    out["continuous_h2o_20k"] = {"walker_steps_per_s": 20000 * 1000 / secs, "us_per_step": secs / 1000 * 1e6,
                                 "clones_per_step": float(kills.mean())}
    del sc
    # batched ensemble (config 5): 64 plain FP64 replicas, N_r ~ U[1000, 65536] (seeded), tile widths and
    # graph length autotuned, 10000 steps; every replica's ZPE with its blocking error, and 16 of them
    # against the individually run plain path (DMC_Sim, another seed)
    out["batched_64_replicas"] = run_batched_replicas(masses)
    # surrogate dimer (200000 walkers) vs the analytic fp64 dimer
    dm = [pg.Constants.mass(a) for a in ("O", "H", "H", "O", "H", "H")]
    pot = pg.water_dimer()
    t_h = time.perf_counter()
    x, v, g, _ = pg.harvest_training_data(pot, 200000, 420, 20, pg.WATER_DIMER_EQ[None], dm, seed=1, equil=20)
    torch.cuda.synchronize()
    t_h = time.perf_counter() - t_h
    t_t = time.perf_counter()
    m = pg.MLPSurrogate(seed=0).fit(x, v, g, epochs=40, batch=8192, lr=2e-3)
    torch.cuda.synchronize()
    t_t = time.perf_counter() - t_t
    nd = pg.NNDMC(m, pot, 200000, pg.WATER_DIMER_EQ[None], dm, DT, steps + 64, seed=5, audit_every=100).init()
    nd.run(32)
    torch.cuda.synchronize()
    s0 = nd.step
    _, secs = _timed_graph_rate(nd.run, lambda: 0, steps)
    nn_ws = nd.walker_steps(s0, s0 + steps)
    fp = pg.DMC_Sim(num_walkers=200000, num_timesteps=steps + 64, equil_steps=10 ** 9, atoms=["O", "H", "H"] * 2,
                    masses=dm, delta_t=DT, potential=pot, start_structures=pg.WATER_DIMER_EQ[None], seed=5,
                    write_files=False)
    fp._init_device()
    fp._run_steps(32)
    torch.cuda.synchronize()
    f0 = int(fp._read_ctrl().step)
    _, fsecs = _timed_graph_rate(fp._run_steps, lambda: 0, steps)
    pf = fp._hist["pop"][f0 - 1:f0 - 1 + steps].cpu().numpy()
    out["surrogate_dimer_200k"] = {"walker_steps_per_s": nn_ws / secs, "us_per_step": secs / steps * 1e6,
                                   "fp64_analytic_walker_steps_per_s": float(pf.sum()) / fsecs,
                                   "fp64_analytic_us_per_step": fsecs / steps * 1e6,
                                   "harvest_s": t_h, "train_s": t_t, "train_samples": int(x.shape[1]),
                                   "train_rmse_cm": m.history[-1]["rmse_e_cm"], "audit": nd.audit()}
    del nd, fp
    # the dimer trial fitted to the harvested plain-run walkers (local-energy variance)
    sel = torch.randperm(x.shape[1], device=x.device)[:300000]
    xs = x[:, sel].contiguous()
    t_f = time.perf_counter()
    trial, s0, s1 = pg.fit_trial(pg.dimer_gaussian_trial(), pot, xs, xs.shape[1], dm)
    torch.cuda.synchronize()
    t_f = time.perf_counter() - t_f
    out["is_nn_batched_dimer"] = run_combined_dimer(m, pot, dm, trial, prep_s={"harvest": t_h, "train": t_t,
                                                                               "trial_fit": t_f})
    out["is_nn_batched_dimer"]["trial"]["sd_local_energy_cm"] = [s0 / pg.Constants.atomic_units["wavenumbers"],
                                                                 s1 / pg.Constants.atomic_units["wavenumbers"]]
    return out


DIMER_TAU = 60000.0  # imaginary time of every run of the dimer efficiency comparison (a.u.)
# dt and dt/2 of the extrapolation.  The walks' time-step errors are curved
# (plain FP64 dimer, 64 seeds each: E(2.5) - E(5) = 1.72 and E(1.25) - E(2.5)
# = 0.59 cm^-1), and a straight line keeps a bias of -12.5 b for the steps 5
# and 2.5 (b the dt^2 coefficient) but a quarter of it for 2.5 and 1.25:
# +0.72 and +0.18 cm^-1 for the plain walk.
DIMER_DTS = (2.5, 1.25)


def zpe_estimate(vref_series_cm):
    """The one error estimator of the dimer efficiency comparison: the mean of the
    production part (the last 3/4) of a vref series and its blocking error
    (30 block means).  For a batch of replicas the series is the N0-weighted
    mean of the replicas' vref at each step."""
    import pyvibdmc_gb300 as pg
    v = np.asarray(vref_series_cm, dtype=np.float64)
    return pg.blocking_error(v[len(v) // 4:], 30)


def extrapolate(res):
    """Time-step extrapolation of a method measured at dt and dt/2 (linear in
    dt, the leading error of the walk): E0 = 2 E(dt/2) - E(dt),
    sigma0^2 = 4 sigma(dt/2)^2 + sigma(dt)^2, cost = the seconds of both runs;
    efficiency at equal error = 1 / (sigma0^2 cost)."""
    a, b = res[f"dt{DIMER_DTS[0]:g}"], res[f"dt{DIMER_DTS[1]:g}"]
    e0 = 2 * b["zpe_cm"] - a["zpe_cm"]
    s0 = float(np.sqrt(4 * b["err_cm"] ** 2 + a["err_cm"] ** 2))
    cost = a["seconds"] + b["seconds"]
    return {"zpe_cm": e0, "err_cm": s0, "seconds": cost, "efficiency": 1.0 / (s0 * s0 * cost) if cost > 0 else None}


def run_batched_replicas(masses, T=10000, nsingle=16):
    """Config 5: 64 independent plain FP64 water replicas with N_r ~ U[1000,
    65536] (seeded) stepped together (DMC_Batch: buckets by walker count, tile
    width and graph length autotuned with 20 timed steps per candidate), for T
    production steps.  Every replica's ZPE (the last 3/4 of its vref series,
    blocking error of 30 blocks) and, for every fourth replica, the same
    system run alone through the plain path (DMC_Sim, another Philox seed):
    chi^2 of the differences over their combined errors."""
    import torch
    import pyvibdmc_gb300 as pg
    ns = [int(v) for v in np.random.default_rng(0).integers(1000, 65537, size=64)]
    th = np.deg2rad(104.5)
    eq = np.array([[0.0, 0.0, 0.0], [1.81, 0.0, 0.0], [1.81 * np.cos(th), 1.81 * np.sin(th), 0.0]])
    b = pg.DMC_Batch(pg.h2o_local_mode(), ns, eq[None], masses, DT, T + 600, seed=3, start_noise=0.05,
                     graph_steps=16)
    b.init()
    tune = b.autotune(steps_per_candidate=20)
    b.run(16)
    torch.cuda.synchronize()
    s0 = b.step
    _, secs = _timed_graph_rate(lambda k: b.run(k, check=False), lambda: 0, T)
    b.check()
    ws = b.walker_steps(s0, s0 + T)
    conv = lambda v: pg.Constants.convert(v, "wavenumbers", to_AU=False)  # noqa: E731
    vr = conv(b.vref_history()[:, s0:s0 + T])
    table = [[ns[r]] + list(zpe_estimate(vr[r])) for r in range(len(ns))]
    comp = []
    for r in range(0, len(ns), len(ns) // nsingle):
        sm = pg.DMC_Sim(num_walkers=ns[r], num_timesteps=T, equil_steps=10 ** 9, atoms=["O", "H", "H"], masses=masses,
                        delta_t=DT, potential=pg.h2o_local_mode(), start_structures=start_structures(ns[r], 500 + r),
                        seed=777, replica_id=r, write_files=False)
        sm._init_device()
        sm._run_steps(T)
        torch.cuda.synchronize()
        zs, es = zpe_estimate(conv(sm._hist["vref"].cpu().numpy()[:T]))
        comp.append([r, ns[r], table[r][1], table[r][2], zs, es])
        del sm
    chi2 = float(sum(((zb - zs) / np.hypot(eb, es)) ** 2 for _, _, zb, eb, zs, es in comp))
    return {"replicas": len(ns), "walkers_total": int(sum(ns)), "steps": T, "seconds": secs,
            "walker_steps_per_s": ws / secs, "us_per_step": secs / T * 1e6,
            "tile_width_per_bucket": {str(k): v[0] for k, v in tune.items() if k != "graph_steps"},
            "graph_steps": tune["graph_steps"][0],
            "zpe_per_replica_cm": {"columns": ["n0", "zpe_cm", "err_cm"], "rows": table},
            "vs_single_runs": {"columns": ["replica", "n0", "batch_zpe_cm", "batch_err_cm", "single_zpe_cm",
                                           "single_err_cm"], "rows": comp,
                               "chi2": chi2, "dof": len(comp), "chi2_per_dof": chi2 / len(comp)}}


def run_combined_dimer(m, pot, dm, trial, plain_seeds=(13, 14, 15, 16, 17, 18), prep_s=None):
    """The efficiency comparison on the water dimer: the engine with its three
    accelerations (importance sampling with the fitted dimer trial, the tcgen05
    surrogate PES, 64 batched replicas with N_r ~ U[1000, 65536]) against the
    plain FP64 GPU path (200000 walkers, one replica, several seeds), at equal
    ZPE error including the time-step error: every method runs at dt = 2.5 and
    1.25 for the same imaginary time, its ZPE is extrapolated to dt -> 0 and its
    efficiency is 1 / (sigma0^2 x seconds) (zpe_estimate, extrapolate).  The
    FP64 importance-sampled path with the same trial (100000 walkers) pins
    the surrogate's accuracy at each dt; profiles/dimer_fp64_oracle.json holds
    a long plain FP64 extrapolation of the same surface (dt = 5, 2.5, 1.25,
    the parabola through the three), the ZPE the three accelerations must
    reproduce within 1 cm^-1."""
    import torch
    import pyvibdmc_gb300 as pg
    conv = lambda v: pg.Constants.convert(v, "wavenumbers", to_AU=False)  # noqa: E731
    res = {"estimator": "mean of the last 3/4 of the vref series (N0-weighted over replicas), blocking error of "
                        "30 block means; dt -> 0 from dt = 2.5 and 1.25 (E0 = 2 E1.25 - E2.5)",
           "surrogate": "sorted-atom Coulomb descriptor (DistIt order); bias control on the audited errors, "
                        "weighted by descendants in forward-walking windows of 2000 a.u.",
           "trial": {"alpha": trial.alpha, "qe": trial.qe}}

    def fp64(n, imp, seed, dt):
        T = int(round(DIMER_TAU / dt))
        sm = pg.DMC_Sim(num_walkers=n, num_timesteps=T, equil_steps=10 ** 9, atoms=["O", "H", "H"] * 2, masses=dm,
                        delta_t=dt, potential=pot, imp_samp=imp, start_structures=pg.WATER_DIMER_EQ[None], seed=seed,
                        write_files=False, graph_steps=32)
        sm._init_device()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sm._run_steps(T)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        if sm._read_ctrl().status:
            raise RuntimeError(f"fp64 dimer run stopped (status {sm._read_ctrl().status})")
        vr = conv(sm._hist["vref"].cpu().numpy()[:T])
        ws = float(n + sm._hist["pop"].cpu().numpy()[:T - 1].sum())
        del sm
        return vr, secs, ws

    for tag, n, imp, seeds in (("plain_fp64_200k", 200000, None, plain_seeds),
                               ("is_fp64_100k", 100000, trial, (13,))):
        res[tag] = {"walkers": n, "seeds": list(seeds)}
        for dt in DIMER_DTS:
            zs, es, secs, ws = [], [], 0.0, 0.0
            for seed in seeds:
                vr, sc, w = fp64(n, imp, seed, dt)
                z, e = zpe_estimate(vr)
                zs.append(z)
                es.append(e)
                secs += sc
                ws += w
            res[tag][f"dt{dt:g}"] = {"zpe_cm": float(np.mean(zs)),
                                     "err_cm": float(np.sqrt(np.sum(np.square(es))) / len(es)),
                                     "seconds": secs, "walker_steps_per_s": ws / secs, "steps": int(DIMER_TAU / dt)}
        res[tag]["dt0"] = extrapolate(res[tag])
    ns = [int(v) for v in np.random.default_rng(0).integers(1000, 65537, size=64)]
    w = np.asarray(ns, dtype=float)
    tag = "is_nn_64_replicas"
    res[tag] = {"replicas": len(ns), "walkers": int(sum(ns))}
    for dt in DIMER_DTS:
        T = int(round(DIMER_TAU / dt))
        nd = pg.NNDMC(m, pot, ns, pg.WATER_DIMER_EQ[None], dm, dt, T + 16, seed=13, audit_every=100,
                      imp_samp=trial, graph_steps=16).init()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nd.run(T)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        v = conv(nd.vref_history()[:, :T])
        z, e = zpe_estimate((w[:, None] * v).sum(0) / w.sum())
        res[tag][f"dt{dt:g}"] = {"zpe_cm": z, "err_cm": e, "seconds": secs, "steps": T,
                                 "walker_steps_per_s": nd.walker_steps(0, T) / secs, "audit": nd.audit()}
        del nd
    res[tag]["dt0"] = extrapolate(res[tag])
    base = res["plain_fp64_200k"]["dt0"]["efficiency"]
    res["gain_vs_plain_fp64_at_equal_error"] = res[tag]["dt0"]["efficiency"] / base
    if prep_s:  # the same with the surrogate's preparation (harvest, training, trial fit) counted as run time
        prep = float(sum(prep_s.values()))
        d0 = res[tag]["dt0"]
        res["preparation_s"] = dict(prep_s, total=prep)
        res["gain_vs_plain_fp64_including_preparation"] = (1.0 / (d0["err_cm"] ** 2 * (d0["seconds"] + prep))) / base
    res["is_fp64_gain_vs_plain_fp64_at_equal_error"] = res["is_fp64_100k"]["dt0"]["efficiency"] / base
    for dt in DIMER_DTS:  # the same comparison at each fixed dt (statistical error only), for reference
        k = f"dt{dt:g}"
        e_of = lambda r: 1.0 / (r[k]["err_cm"] ** 2 * r[k]["seconds"])  # noqa: E731
        res[f"gain_at_fixed_{k}"] = e_of(res[tag]) / e_of(res["plain_fp64_200k"])
        d = res[tag][k]["zpe_cm"] - res["is_fp64_100k"][k]["zpe_cm"]
        res[f"zpe_minus_fp64_is_{k}_cm"] = [d, float(np.hypot(res[tag][k]["err_cm"],
                                                               res["is_fp64_100k"][k]["err_cm"]))]
    a, b = res[tag]["dt0"], res["plain_fp64_200k"]["dt0"]
    res["zpe_dt0_minus_plain_fp64_dt0_cm"] = [a["zpe_cm"] - b["zpe_cm"], float(np.hypot(a["err_cm"], b["err_cm"]))]
    orc = os.path.join(ROOT, "profiles", "dimer_fp64_oracle.json")
    if os.path.exists(orc):
        o = json.load(open(orc))
        res["fp64_oracle_dt0_cm"] = [o["zpe_dt0_cm"], o["err_dt0_cm"]]
        res["zpe_dt0_minus_fp64_oracle_cm"] = [a["zpe_cm"] - o["zpe_dt0_cm"],
                                               float(np.hypot(a["err_cm"], o["err_dt0_cm"]))]
    # the reference's CPU path on the same dimer (oracle port, plain discrete), a bounded sample: its
    # error per walker-step is the plain FP64 run's (same algorithm), so the gain at equal error scales
    # with the throughput ratio
    cores = os.cpu_count() or 1
    cpu, ccores = cpu_reference_rate(20000, 20, 1, "dimer")[0], 1
    if cores > 1:
        try:
            cp = cpu_reference_rate(20000, 10, cores, "dimer")[0]
            if cp > cpu:
                cpu, ccores = cp, cores
        except Exception:
            pass
    res["cpu_reference_dimer"] = {"walker_steps_per_s": cpu, "cores": ccores,
                                  "sample": "oracle restatement of DMC_Sim.propagate (plain, discrete), "
                                            "20000 dimer walkers, numpy; best of 1 process and a "
                                            f"{cores}-process PES pool"}
    plain_rate = res["plain_fp64_200k"][f"dt{DIMER_DTS[0]:g}"]["walker_steps_per_s"]
    res["gain_vs_cpu_reference_at_equal_error"] = res["gain_vs_plain_fp64_at_equal_error"] * plain_rate / cpu
    return res


def oracle_extrapolation(runs):
    """dt -> 0 of the plain FP64 dimer ZPEs in ``runs`` ({"dt<dt>": {zpe_cm,
    err_cm}}): the straight line through each pair of neighbouring steps
    (E0 = 2 E(h/2) - E(h)) and, with dt = 5, 2.5 and 1.25, the parabola
    through the three (Richardson: E0 = (E(5) - 6 E(2.5) + 8 E(1.25)) / 3,
    which removes the dt^2 term the straight lines keep).  The oracle value
    is the parabola when all three steps are present."""
    out = {}
    dts = sorted((float(k[2:]) for k in runs), reverse=True)
    for h, h2 in zip(dts, dts[1:]):
        if abs(h2 * 2 - h) < 1e-12:
            a, b = runs[f"dt{h:g}"], runs[f"dt{h2:g}"]
            out[f"linear_{h:g}_{h2:g}"] = [2 * b["zpe_cm"] - a["zpe_cm"],
                                           float(np.sqrt(4 * b["err_cm"] ** 2 + a["err_cm"] ** 2))]
    if all(f"dt{d:g}" in runs for d in (5.0, 2.5, 1.25)):
        e = [runs[f"dt{d:g}"] for d in (5.0, 2.5, 1.25)]
        out["quadratic_5_2.5_1.25"] = [(e[0]["zpe_cm"] - 6 * e[1]["zpe_cm"] + 8 * e[2]["zpe_cm"]) / 3,
                                        float(np.sqrt(e[0]["err_cm"] ** 2 + 36 * e[1]["err_cm"] ** 2 +
                                                      64 * e[2]["err_cm"] ** 2) / 3)]
        out["zpe_dt0_cm"], out["err_dt0_cm"] = out["quadratic_5_2.5_1.25"]
    else:
        k = next(iter(out))
        out["zpe_dt0_cm"], out["err_dt0_cm"] = out[k]
    return out


def dimer_oracle(dts, merge=None, plain_seeds=tuple(range(101, 165))):
    """A long plain FP64 extrapolation of the water dimer's ZPE (200000
    walkers, 64 seeds at each dt, 60000 a.u. of imaginary time per run): the
    value profiles/dimer_fp64_oracle.json keeps for the dimer efficiency
    comparison.  ``merge``: a JSON file of this function whose runs at other
    steps are kept."""
    import torch
    import pyvibdmc_gb300 as pg
    dm = [pg.Constants.mass(a) for a in ("O", "H", "H", "O", "H", "H")]
    pot = pg.water_dimer()
    res, secs = {}, 0.0
    if merge:
        old = json.load(open(merge))
        res, secs = dict(old["runs"]), float(old.get("seconds", 0.0))
    t_all = time.perf_counter()
    for dt in dts:
        T = int(round(DIMER_TAU / dt))
        zs, es = [], []
        for seed in plain_seeds:
            sm = pg.DMC_Sim(num_walkers=200000, num_timesteps=T, equil_steps=10 ** 9, atoms=["O", "H", "H"] * 2,
                            masses=dm, delta_t=dt, potential=pot, start_structures=pg.WATER_DIMER_EQ[None], seed=seed,
                            write_files=False, graph_steps=32)
            sm._init_device()
            sm._run_steps(T)
            torch.cuda.synchronize()
            if sm._read_ctrl().status:
                continue  # a run that tripped a population guard is left out (and counted)
            z, e = zpe_estimate(pg.Constants.convert(sm._hist["vref"].cpu().numpy()[:T], "wavenumbers", to_AU=False))
            zs.append(z)
            es.append(e)
            del sm
        res[f"dt{dt:g}"] = {"zpe_cm": float(np.mean(zs)), "err_cm": float(np.sqrt(np.sum(np.square(es))) / len(es)),
                            "scatter_err_cm": float(np.std(zs, ddof=1) / np.sqrt(len(zs))), "runs": len(zs),
                            "runs_left_out": len(plain_seeds) - len(zs)}
    out = dict(oracle_extrapolation(res), runs=res, walkers=200000, imaginary_time_au=DIMER_TAU,
               seeds=[plain_seeds[0], plain_seeds[-1]], seconds=secs + time.perf_counter() - t_all,
               command="python bench.py --dimer-oracle " + ",".join(f"{d:g}" for d in sorted(
                   (float(k[2:]) for k in res), reverse=True)))
    print(json.dumps(out), flush=True)


def run_e2e(sim, L, dev, steps):
    """The walkers in page-locked host memory, stepped through the public
    host-resident API (``pyvibdmc_gb300.HostWalkers`` ->
    ``gbdmc_sim_step_host``): every step the move kernel reads the walkers
    from host memory, and the branching kernel writes the branched
    population, its potentials, ancestor ids and the control block back to
    host memory.  The headline value queues the timed steps back to back
    (``HostWalkers.run``, one wait at the end; the kernels take N from the
    device control block); ``per_step_sync`` waits for every step and reads
    N' on the host (``HostWalkers.step``)."""
    import torch
    import pyvibdmc_gb300 as pg
    from pyvibdmc_gb300 import _capi
    A3 = 3 * sim.natoms
    cb = C.sizeof(_capi.Ctrl)
    hw = pg.HostWalkers(sim)
    n = hw.n
    for _ in range(3):
        n = hw.step()
    h2d = d2h = 0
    total = 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        h2d += (A3 * 8 + 4) * n  # coordinates and ancestor ids of the N walkers
        total += n
        n = hw.step()
        d2h += (A3 * 8 + 8 + 4) * n + cb
    secs = time.perf_counter() - t0
    sync = {"value": total / secs, "unit": UNIT, "h2d_bytes_per_step": h2d // steps,
            "d2h_bytes_per_step": d2h // steps, "steps": steps}
    # the same steps queued back to back; the populations come from the device history
    s0, n0 = int(hw.ctrl().step), hw.n
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hw.run(steps)
    secs = time.perf_counter() - t0
    after = sim._hist["pop"][s0:s0 + steps].cpu().numpy().astype(np.int64)
    before = np.concatenate([[n0], after[:-1]])
    hw.close()
    return {"value": float(before.sum()) / secs, "unit": UNIT,
            "h2d_bytes_per_step": int((A3 * 8 + 4) * before.sum()) // steps,
            "d2h_bytes_per_step": int((A3 * 8 + 8 + 4) * after.sum() + cb * steps) // steps, "steps": steps,
            "path": "walkers in page-locked host memory; per step one gbdmc_sim_step_host call (C ABI, "
                    "graph-replayed): the move kernel reads the N walkers from host memory, the branching kernel "
                    "writes the branched walkers, V, ancestor ids and the control block to host memory; the steps "
                    "are queued back to back (HostWalkers.run) with one host wait at the end",
            "per_step_sync": sync}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-extras", dest="no_extras", action="store_true",
                    help="skip the IS / batched / surrogate workloads reported under 'extras'")
    ap.add_argument("--dimer-oracle", dest="dimer_oracle", default=None, metavar="DT,...",
                    help="print the long plain FP64 dt -> 0 ZPE of the water dimer from runs at these time steps "
                         "(profiles/dimer_fp64_oracle.json: 5,2.5,1.25)")
    ap.add_argument("--merge", default=None, help="with --dimer-oracle: keep the runs of this oracle JSON")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.dimer_oracle:
        dimer_oracle([float(v) for v in args.dimer_oracle.split(",")], args.merge)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
