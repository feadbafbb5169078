"""Times the unmodified reference DMC_Sim against the oracle port on one host
core (the port is what `bench.py --impl reference` and the `cpu_baseline`
leg time, because the reference, a Python package, is not on the GPU host).

Both run plain discrete DMC on the local-mode water at 20000 walkers, dt = 10,
with the same numpy potential; the reference through its own Potential_Direct
and its own NumPy RandomState draws, the port through bench.cpu_reference_rate
(RandomState draws as well).  The reference's time includes its setup and
file handling, which its run loop does once.

    python tests/golden/time_reference_vs_port.py --reference <pyvibdmc source root> [--steps 150]

prints one JSON line; tests/golden/reference_vs_port_timing.json keeps the
last result.
"""
import argparse
import json
import os
import platform
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="root of the pyvibdmc source tree")
    ap.add_argument("--walkers", type=int, default=20000)
    ap.add_argument("--steps", type=int, default=150)
    a = ap.parse_args()
    import make_golden as mg
    import oracle
    import bench
    pv = mg._import_reference(a.reference)
    p, m = oracle.h2o_config()
    x0 = bench.start_structures(a.walkers, 5)
    with tempfile.TemporaryDirectory() as tmp:
        sim = pv.DMC_Sim(sim_name="t", output_folder=tmp, weighting="discrete", num_walkers=a.walkers,
                         num_timesteps=a.steps, equil_steps=10 ** 6, chkpt_every=10 ** 6, wfn_every=10 ** 6,
                         desc_wt_steps=10, atoms=["O", "H", "H"], masses=m, delta_t=10.0,
                         potential=pv.Potential_Direct(lambda c: oracle.pes_h2o_lm(c, p)),
                         start_structures=x0.copy(), log_every=10 ** 6)
        t0 = time.perf_counter()
        sim.run()
        tr = time.perf_counter() - t0
    ws = float(np.sum(sim._pop_vs_tau[:-1])) + a.walkers
    rate, secs, k = bench.cpu_reference_rate(a.walkers, a.steps, 1)
    print(json.dumps({"reference_walker_steps_per_s": ws / tr, "reference_seconds": tr, "reference_steps": a.steps,
                      "port_walker_steps_per_s": rate, "port_seconds": secs, "port_steps": k,
                      "walkers": a.walkers, "cores": 1, "machine": platform.machine(),
                      "processor": platform.processor() or platform.machine(),
                      "command": "python tests/golden/time_reference_vs_port.py --reference <pyvibdmc source root>"}))


if __name__ == "__main__":
    main()
