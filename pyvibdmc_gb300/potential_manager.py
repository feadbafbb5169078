"""Potential managers for energy functions written in Python, with the
reference's names and arguments (pyvibdmc/simulation_utilities/
potential_manager.py:12-253).

Each manager wraps a user function ``f(cds[, pot_kwargs]) -> (N,) hartree``
behind ``getpot(cds, timeit=False)``, so the object can be handed to
:class:`pyvibdmc_gb300.DMC_Sim` (which moves and branches the walkers on the
GPU and calls ``getpot`` on the moved walkers every step) as well as to the
reference engine.

* ``Potential``: the function is imported from ``python_file`` in
  ``potential_directory`` and evaluated by a pool of ``num_cores`` worker
  processes on ``np.array_split`` chunks of the walkers
  (potential_manager.py:12-103).  The workers are started with the 'spawn'
  method -- a process forked after CUDA initialised in the parent cannot use
  it -- and each imports the function itself.
* ``Potential_NoMP``: the same function called in this process (:106-174);
  ``ch_dir`` runs each call inside ``potential_directory``.
* ``NN_Potential``: ``Potential_NoMP`` whose function also receives ``model``
  (:177-214).
* ``Potential_Direct``: a function object passed in directly (:237-253).

``pot_kwargs`` (a dict) is passed as the second positional argument when
given; ``pass_timestep`` adds ``pot_kwargs['timestep']``, counting the calls
from 0 (:41-46, :92-93).
"""
import contextlib
import importlib.util
import multiprocessing as mp
import os
import sys
import time

import numpy as np

__all__ = ["Potential", "Potential_NoMP", "NN_Potential", "Potential_Direct"]


@contextlib.contextmanager
def _inside(directory):
    old = os.getcwd()
    os.chdir(directory)
    try:
        yield
    finally:
        os.chdir(old)


def _load_function(directory, python_file, name):
    """Import ``name`` from ``python_file`` in ``directory``.  The module is
    executed with ``directory`` as working directory and on ``sys.path``, so
    it can load its own data files and compiled extensions by relative path."""
    directory = os.path.abspath(directory)
    modname = os.path.splitext(os.path.basename(python_file))[0]
    if directory not in sys.path:
        sys.path.insert(0, directory)
    with _inside(directory):
        mod = sys.modules.get(modname)
        if mod is None or os.path.dirname(os.path.abspath(getattr(mod, "__file__", "") or "")) != directory:
            spec = importlib.util.spec_from_file_location(modname, os.path.join(directory, python_file))
            mod = importlib.util.module_from_spec(spec)
            sys.modules[modname] = mod
            spec.loader.exec_module(mod)
    return getattr(mod, name)


def _timed(fn, cds, timeit):
    if not timeit:
        return fn(cds)
    t0 = time.time()
    v = fn(cds)
    return v, time.time() - t0


class _KwargsMixin:
    def _init_kwargs(self, pot_kwargs, pass_timestep):
        self.pass_timestep = pass_timestep
        self.pot_kwargs = pot_kwargs
        if pass_timestep:
            self.pot_kwargs = {} if pot_kwargs is None else pot_kwargs
            self.pot_kwargs["timestep"] = 0

    def _after_call(self):
        if self.pass_timestep:
            self.pot_kwargs["timestep"] += 1


# worker side of Potential's pool
_WORKER_FN = None


def _worker_init(directory, python_file, name):
    global _WORKER_FN
    _WORKER_FN = _load_function(directory, python_file, name)


def _worker_call(cds, *kwargs):
    return _WORKER_FN(cds, *kwargs)


class Potential(_KwargsMixin):
    """A Python potential evaluated by ``num_cores`` worker processes
    (potential_manager.py:12-103).

    :param potential_function: name of the function ``f(cds[, pot_kwargs])``
    :param potential_directory: directory holding ``python_file``
    :param python_file: the module file defining the function
    :param num_cores: worker processes (the walkers are split into this many chunks)
    """

    def __init__(self, potential_function, potential_directory, python_file, num_cores=1, pass_timestep=False,
                 pot_kwargs=None):
        self.potential_function = potential_function
        self.potential_directory = os.path.abspath(potential_directory)
        self.python_file = python_file
        if num_cores <= 0:
            print("Weird number of cores specified. Defaulting to 1...")
            num_cores = 1
        self.num_cores = int(num_cores)
        self._init_kwargs(pot_kwargs, pass_timestep)
        self._potPool = mp.get_context("spawn").Pool(
            self.num_cores, initializer=_worker_init,
            initargs=(self.potential_directory, self.python_file, self.potential_function))

    @property
    def pool(self):
        """The worker pool (the reference exposes it for importance sampling)."""
        return self._potPool

    def getpot(self, cds, timeit=False):
        def call(c):
            chunks = np.array_split(c, self.num_cores)
            if self.pot_kwargs is not None:
                res = self._potPool.starmap(_worker_call, [(ch, self.pot_kwargs) for ch in chunks])
            else:
                res = self._potPool.map(_worker_call, chunks)
            return np.concatenate(res)

        out = _timed(call, cds, timeit)
        self._after_call()
        return out

    def mp_close(self):
        if self._potPool is not None:
            self._potPool.close()
            self._potPool.join()
            self._potPool = None

    def __getstate__(self):  # the pool does not travel (checkpoints, deep copies)
        d = dict(self.__dict__)
        d["_potPool"] = None
        return d


class Potential_NoMP(_KwargsMixin):
    """A Python potential called in this process (potential_manager.py:106-174)."""

    def __init__(self, potential_function, potential_directory, python_file, pass_timestep=False, ch_dir=False,
                 pot_kwargs=None):
        self.potential_function = potential_function
        self.potential_directory = os.path.abspath(potential_directory)
        self.python_file = python_file
        self.ch_dir = ch_dir
        self._init_kwargs(pot_kwargs, pass_timestep)
        self._pot = _load_function(self.potential_directory, python_file, potential_function)

    def _args(self):
        return () if self.pot_kwargs is None else (self.pot_kwargs,)

    def getpot(self, cds, timeit=False):
        def call(c):
            if self.ch_dir:
                with _inside(self.potential_directory):
                    return self._pot(c, *self._args())
            return self._pot(c, *self._args())

        out = _timed(call, cds, timeit)
        self._after_call()
        return out


class NN_Potential(Potential_NoMP):
    """``Potential_NoMP`` whose function is called as ``f(cds, model[, pot_kwargs])``
    (potential_manager.py:177-214)."""

    def __init__(self, potential_function, potential_directory, python_file, model, ch_dir=False, pot_kwargs=None,
                 pass_timestep=False):
        super().__init__(potential_function, potential_directory, python_file, pass_timestep, ch_dir, pot_kwargs)
        self.model = model

    def getpot(self, cds, timeit=False):
        out = _timed(lambda c: self._pot(c, self.model, *self._args()), cds, timeit)
        self._after_call()
        return out


class Potential_Direct(_KwargsMixin):
    """A function object used as the potential (potential_manager.py:237-253)."""

    def __init__(self, potential_function, pot_kwargs=None, pass_timestep=False):
        self.potential_function = potential_function
        self._init_kwargs(pot_kwargs, pass_timestep)

    def getpot(self, cds, timeit=False):
        args = () if self.pot_kwargs is None else (self.pot_kwargs,)
        out = _timed(lambda c: self.potential_function(c, *args), cds, timeit)
        self._after_call()
        return out
