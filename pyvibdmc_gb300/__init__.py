"""pyvibdmc_gb300 -- GB300-native diffusion Monte Carlo walker engine.

Drop-in for PyVibDMC's walker step loop: ``DMC_Sim`` / ``dmc_restart`` with the
reference's keywords, GPU potential plug-ins with the ``getpot`` contract and
GPU importance-sampling managers with ``call_trial`` / ``call_derivs``.  The
per-step work runs in hand-written sm_103a CUDA kernels (libgbdmc.so) behind
the C ABI of ``include/gbdmc.h``.
"""
from .constants import Constants, get_atomic_num, get_atomic_string
from .potentials import (Potential_GPU, PESFunction, harmonic_oscillator, h2o_local_mode, water_dimer,
                         partridge_schwenke,
                         WATER_DIMER_EQ, to_soa, from_soa)
from .imp_samp import ImpSampManager_GPU, TrialFunction, h2o_gaussian_trial, ho_gaussian_trial, \
    dimer_gaussian_trial, local_energy, fit_trial
from .potential_manager import Potential, Potential_NoMP, NN_Potential, Potential_Direct
from .engine import DMC_Sim, HostWalkers, dmc_restart
from .initial import HarmonicAnalysis, InitialConditioner
from .batch import DMC_Batch, blocking_error
from .surrogate import MLPSurrogate, NN_Potential_GPU, NNDMC, harvest_training_data
from . import _capi

__all__ = ["HostWalkers", "HarmonicAnalysis", "InitialConditioner", "Constants", "get_atomic_num", "get_atomic_string", "Potential_GPU", "PESFunction",
           "harmonic_oscillator", "h2o_local_mode", "water_dimer", "partridge_schwenke", "ImpSampManager_GPU", "TrialFunction",
           "h2o_gaussian_trial", "ho_gaussian_trial", "dimer_gaussian_trial", "local_energy", "fit_trial", "DMC_Sim", "dmc_restart", "DMC_Batch", "blocking_error",
           "MLPSurrogate", "NN_Potential_GPU", "NNDMC", "harvest_training_data", "WATER_DIMER_EQ",
           "to_soa", "from_soa", "Potential", "Potential_NoMP", "NN_Potential", "Potential_Direct"]

__version__ = "0.1.0"


def library():
    """Load (building when absent) and return the ctypes handle of libgbdmc.so."""
    return _capi.load()
