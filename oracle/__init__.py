"""CPU oracle for the DMC walker step loop.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``pyvibdmc_gb300`` package imports,
links or executes this package.  Only ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it,
and only as the checker or as the timed CPU baseline.
"""
from .dmc_oracle import *  # noqa: F401,F403
from . import mlp_oracle  # noqa: F401,E402
