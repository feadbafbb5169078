"""Summaries of the reference's own sample runs on the Partridge-Schwenke PES
(pyvibdmc/sample_sim_data/tutorial_water_{0..4}_log.txt: the unmodified
reference engine with the Fortran PES, 8000 walkers, dt = 5, 5000 steps,
discrete weighting).  Each log prints, per step, the mean potential energy of
the ensemble after the move (cm^-1) and the population.  This script keeps,
per run, the average over steps 500-4999 of that mean and of the population.

    python tests/golden/make_ps_reference.py <reference checkout>   (or set GBDMC_REFERENCE)
"""
import json
import os
import re
import sys

import numpy as np


def main(ref):
    d = os.path.join(ref, "pyvibdmc", "sample_sim_data")
    runs = []
    for k in range(5):
        txt = open(os.path.join(d, f"tutorial_water_{k}_log.txt")).read()
        head = dict(walkers=int(re.search(r"Num Walkers: (\d+)", txt).group(1)),
                    steps=int(re.search(r"Num Time Steps: (\d+)", txt).group(1)),
                    dt=float(re.search(r"Delta Tau: ([\d.]+)", txt).group(1)),
                    masses=[float(v) for v in re.search(r"Masses of Each Atom: \[([^\]]+)\]", txt).group(1).split()])
        vbar = np.array([float(v) for v in re.findall(r"Average energy of ensemble: ([-\d.eE+]+) cm-1", txt)])
        pop = np.array([int(v) for v in re.findall(r"Number of Walkers: (\d+)", txt)])
        runs.append(dict(head, mean_v_cm=float(vbar[500:].mean()), mean_pop=float(pop[500:].mean()),
                         n_steps_logged=len(vbar)))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ps_tutorial_reference.json")
    json.dump(dict(source="pyvibdmc/sample_sim_data/tutorial_water_[0-4]_log.txt", first_step=500, runs=runs),
              open(out, "w"), indent=1)
    m = np.array([r["mean_v_cm"] for r in runs])
    print(out, m, m.mean(), m.std(ddof=1) / np.sqrt(len(m)))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBDMC_REFERENCE")
    if not ref:
        sys.exit("usage: %s <reference checkout>  (or set GBDMC_REFERENCE)" % sys.argv[0])
    main(ref)
