"""Output files with the reference's names and keys.

* ``save_h5`` writes ``keyz -> valz`` (SimArchivist.save_h5,
  simulation_utilities/sim_archive.py:12-23).  With h5py installed it writes
  HDF5; otherwise the same keys go to ``<fname>.npz`` next to the requested
  name (h5py is optional here).
* ``create_filesystem`` / ``delete_older_checkpoints`` /
  ``delete_future_checkpoints`` mirror FileManager
  (simulation_utilities/file_manager.py:7-54).
* The text log follows SimLogger's lines (simulation_utilities/sim_logger.py).
"""
import glob
import importlib
import os
import pickle

import numpy as np

from .constants import Constants

__all__ = ["save_h5", "load_h5", "create_filesystem", "delete_older_checkpoints", "delete_future_checkpoints",
           "checkpoint_step", "SimLogger", "load_checkpoint", "ReferenceCheckpoint"]

try:  # optional dependency
    import h5py as _h5py
except Exception:  # pragma: no cover - depends on the environment
    _h5py = None


def save_h5(fname, keyz, valz):
    if _h5py is not None:
        with _h5py.File(fname, "w") as hf:
            for k, v in zip(keyz, valz):
                hf.create_dataset(k, data=v)
        return fname
    path = fname + ".npz"
    np.savez(path, **{k: np.asarray(v) for k, v in zip(keyz, valz)})
    return path


def load_h5(fname):
    """Read a file written by save_h5: the HDF5 file when h5py is installed and
    it exists, else the ``.npz`` written in its place."""
    if _h5py is not None and os.path.exists(fname):
        with _h5py.File(fname, "r") as hf:
            return {k: hf[k][()] for k in hf.keys()}
    if os.path.exists(fname + ".npz"):
        with np.load(fname + ".npz") as z:
            return {k: z[k] for k in z.files}
    raise FileNotFoundError(fname)


class ReferenceCheckpoint:
    """The attributes of a checkpoint the reference wrote: SimArchivist.chkpt
    pickles a copy of the DMC_Sim object, potential and trial removed
    (sim_archive.py:25-32, pyvibdmc.py:934-947).  Unpickled without the
    reference installed: the object's attribute dict lands here."""

    def __setstate__(self, state):
        self.__dict__.update(state)


class _CheckpointUnpickler(pickle.Unpickler):
    """Loads this engine's checkpoints (a dict) and the reference's (a pickled
    DMC_Sim) with a fixed list of globals: the reference's DMC_Sim class
    (mapped to ReferenceCheckpoint) and NumPy's array and scalar
    reconstructors, whose module moved from numpy.core to numpy._core in
    NumPy 2 (either spelling loads with either NumPy)."""

    _NUMPY = {"_reconstruct", "scalar", "ndarray", "dtype", "_frombuffer"}

    def find_class(self, module, name):
        if (module, name) == ("pyvibdmc.pyvibdmc", "DMC_Sim"):
            return ReferenceCheckpoint
        if module in ("numpy", "numpy.core.multiarray", "numpy._core.multiarray", "numpy.core.numeric",
                      "numpy._core.numeric") and name in self._NUMPY | {"ndarray", "dtype"}:
            for m in (module, module.replace("numpy._core", "numpy.core"), module.replace("numpy.core", "numpy._core")):
                try:
                    return getattr(importlib.import_module(m), name)
                except (ImportError, AttributeError):
                    continue
        if module == "numpy" and name in ("dtype", "ndarray"):
            return getattr(np, name)
        if module.startswith("numpy.dtypes") or (module == "builtins" and name in ("set", "frozenset", "slice")):
            return super().find_class(module, name)
        raise pickle.UnpicklingError(f"checkpoint refers to {module}.{name}, which a DMC checkpoint does not hold")


def load_checkpoint(path):
    """A checkpoint of this engine (dict) or of the reference (ReferenceCheckpoint)."""
    with open(path, "rb") as fh:
        return _CheckpointUnpickler(fh).load()


def create_filesystem(output_folder):
    for sub in ("", "/chkpts", "/wfns"):
        os.makedirs(output_folder + sub, exist_ok=True)


def checkpoint_step(path):
    """Step number of a ``{sim_name}_{t}.pickle`` checkpoint (None if the name has none)."""
    try:
        return int(os.path.basename(path).split("_")[-1].split(".")[0])
    except ValueError:
        return None


def _wfn_step(path):
    try:  # {sim_name}_wfn_{t}ts.hdf5 (or .hdf5.npz)
        return int(os.path.basename(path).split("_")[-1].split("ts")[0])
    except ValueError:
        return None


def delete_older_checkpoints(sim_folder, sim_name, time_step):
    """Remove the checkpoints of steps before ``time_step`` (file_manager.py:29-38)."""
    for p in glob.glob(f"{sim_folder}/chkpts/{sim_name}_*.pickle"):
        t = checkpoint_step(p)
        if t is not None and t < time_step:
            os.remove(p)


def delete_future_checkpoints(sim_folder, sim_name, time_step):
    """Remove the checkpoints and wave-function files of steps after
    ``time_step`` (file_manager.py:11-26), before a restart from it."""
    for p in glob.glob(f"{sim_folder}/chkpts/{sim_name}_*.pickle"):
        t = checkpoint_step(p)
        if t is not None and t > time_step:
            os.remove(p)
    for p in glob.glob(f"{sim_folder}/wfns/{sim_name}_*.hdf5*"):
        t = _wfn_step(p)
        if t is not None and t > time_step:
            os.remove(p)


class SimLogger:
    """Text log with the reference's wording (sim_logger.py:6-93)."""

    def __init__(self, fname, overwrite=False):
        self.fl = open(fname, "w" if overwrite else "a")

    def close(self):
        self.fl.close()

    def write(self, s):
        self.fl.write(s)

    def beginning(self, sim):
        w = self.fl.write
        w(f"Simulation {sim.sim_name} starting at step {sim.cur_timestep}\n")
        w("Potential attributes: \n")
        for k, v in sim.potential_info.items():
            if not k.startswith("_"):
                w(f"\t{k}: {v}\n")
        w(f"Num Walkers: {sim.num_walkers}\n")
        w(f"Num Time Steps: {sim.num_timesteps}\n")
        w(f"Weighting Type: {sim.weighting}\n")
        w(f"Branch every {sim.branch_every} Time Step(s)\n")
        w(f"Delta Tau: {sim.delta_t} a.u.\n")
        w(f"Masses of Each Atom: {sim.masses}\n")
        w(f"Equilibration Steps Before Collecting Wave Functions: {sim.equil_steps}\n")
        w(f"Checkpoint Every {sim.chkpt_every} time steps\n")
        w(f"Collect Wave Functions Every {sim.wfn_every} Time Steps After Equilibration\n\n")

    def step_block(self, t, weighting, h, gpu_time=None):
        """Per-step lines for step t from the device history h (dict of arrays)."""
        cv = lambda e: Constants.convert(e, "wavenumbers", to_AU=False)  # noqa: E731
        w = self.fl.write
        w(f"Time step {t}\n")
        if "pop_before" in h:  # importance sampling: Metropolis rejections of the step's proposals
            tot = h["pop_before"][t]
            w(f"Metropolis rejected {h['rejected'][t]} of {tot} walkers "
              f"({(h['rejected'][t] / max(tot, 1)) * 100:0.2f} %)\n")
        w(f"Potential call time at time step {t}:\n")
        w(f"\t{gpu_time if gpu_time is not None else 'fused'} seconds\n")
        w(f"\tAverage energy of ensemble: {cv(h['vmean'][t])} cm-1 (without vref correction)\n")
        w(f"\tHighest energy walker: {cv(h['vmax'][t])} cm-1\n")
        w(f"\tLowest energy walker: {cv(h['vmin'][t])} cm-1\n")
        if weighting == "discrete":
            w(f"Birth/Death at time step {t}:\n")
            w(f"\tWalker Births: {h['births'][t]}\n")
            w(f"\tWalker Deaths: {h['deaths'][t]}\n")
            w(f"\tNumber of Walkers: {int(h['pop'][t])}\n")
        else:
            w(f"Branching at time step {t}:\n")
            w(f"\tWalkers Branched: {h['births'][t]}:\n")

    def finish(self, seconds):
        self.fl.write("Simulation has finished.\n\n")
        self.fl.write(f"Simulation took {seconds} seconds.\n\n")
        self.fl.close()
