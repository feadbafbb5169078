"""Golden fixture for the sorted dimer descriptor, from the UNMODIFIED
reference's DistIt (tensorflow_descriptors/distance_descriptors.py):

    python tests/golden/make_distit_golden.py <reference checkout>   (or set GBDMC_REFERENCE)

Writes ``tests/golden/distit_dimer.npz``: 512 water-dimer geometries (the
dimer minimum with Gaussian displacements of 0.25 bohr, each copy with one of
the eight permutations of like atoms applied: the hydrogens of either water,
the two waters) and the upper triangle of their Coulomb matrix from
``DistIt(zs=[8,1,1,8,1,1], method='coulomb', sorted_atoms=[[0],[1,2],[3],[4,5]],
sorted_groups=[[0,1,2],[3,4,5]])``, plus the unsorted Coulomb descriptor.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import _import_reference, ROOT  # noqa: E402

EQ = np.array([[0.000000000000, 0.000000000000, 0.000000000000],
               [1.427477952458, -0.371496091643, 1.058267415716],
               [-0.475355230876, -1.624174243271, -0.657060123398],
               [-0.890893874743, 4.517468473284, -2.310760800984],
               [-2.231456348667, 5.100851802863, -1.249695023025],
               [-0.483907575038, 2.882598047543, -1.568314000679]])


def group_permutations():
    out = []
    for g in (False, True):
        for a in (False, True):
            for b in (False, True):
                w1 = [0, 2, 1] if a else [0, 1, 2]
                w2 = [3, 5, 4] if b else [3, 4, 5]
                out.append((w2 + w1) if g else (w1 + w2))
    return np.array(out)


def main(ref):
    _import_reference(ref)
    from pyvibdmc.simulation_utilities.tensorflow_descriptors.distance_descriptors import DistIt
    rng = np.random.default_rng(2024)
    n = 512
    x = EQ[None] + 0.25 * rng.standard_normal((n, 6, 3))
    perms = group_permutations()
    x = x[np.arange(n)[:, None], perms[np.arange(n) % 8]]
    zs = [8, 1, 1, 8, 1, 1]
    srt = DistIt(zs=zs, method="coulomb", sorted_atoms=[[0], [1, 2], [3], [4, 5]],
                 sorted_groups=[[0, 1, 2], [3, 4, 5]], force_numpy=True).run(x)
    uns = DistIt(zs=zs, method="coulomb", force_numpy=True).run(x)
    np.savez_compressed(os.path.join(HERE, "distit_dimer.npz"), x=x, sorted=np.asarray(srt), unsorted=np.asarray(uns))
    print("distit_dimer.npz:", x.shape, np.asarray(srt).shape)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBDMC_REFERENCE")
    if not ref:
        sys.exit("usage: %s <reference checkout>  (or set GBDMC_REFERENCE)" % sys.argv[0])
    main(ref)
