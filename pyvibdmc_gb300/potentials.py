"""GPU potential-energy plug-ins with the reference's ``getpot`` contract.

``Potential_GPU.getpot(cds, timeit=False)`` takes an (N, A, 3) array in bohr
and returns the (N,) energies in hartree -- or ``(v, seconds)`` with
``timeit`` -- exactly like ``Potential*.getpot`` in
pyvibdmc/simulation_utilities/potential_manager.py:71-99, 144-174, 237-253,
so the same object can be handed to the reference engine or to
:class:`pyvibdmc_gb300.DMC_Sim`.  The latter fuses the PES into its step
kernel instead of calling ``getpot``.

The energy is evaluated by ``gbdmc_pes_eval`` (CUDA, sm_103a); the gradient
comes from the hand-written adjoint in the same kernel and is exposed to
PyTorch through :class:`PESFunction`.
"""
import ctypes as C
import time

import numpy as np
import torch

from . import _capi
from .constants import Constants

__all__ = ["Potential_GPU", "PESFunction", "harmonic_oscillator", "h2o_local_mode", "water_dimer",
           "partridge_schwenke", "WATER_DIMER_EQ",
           "to_soa", "from_soa", "default_device"]


def default_device():
    if not torch.cuda.is_available():
        raise RuntimeError("pyvibdmc_gb300 needs a CUDA device (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def to_soa(cds, device, dtype=torch.float64):
    """(N, A, 3) host or device array -> contiguous (3A, N) device tensor."""
    t = torch.as_tensor(np.asarray(cds) if not torch.is_tensor(cds) else cds, dtype=dtype)
    n, m = t.shape[0], int(np.prod(t.shape[1:]))  # explicit width: N may be 0
    return t.reshape(n, m).t().contiguous().to(device)


def from_soa(x, n, natoms):
    """(3A, >=n) device tensor -> (n, A, 3) host numpy array."""
    return x[:, :n].t().reshape(n, natoms, 3).cpu().numpy()


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Potential_GPU:
    """Built-in analytic PES evaluated on the GPU.

    :param kind: 'harmonic_oscillator' | 'h2o_local_mode' | 'water_dimer' |
        'partridge_schwenke'
    :param params: dict of the PES parameters (see the factory functions)
    :param natoms: number of atoms (fixed for the water PESs)
    """

    KINDS = {"harmonic_oscillator": _capi.PES_HO, "h2o_local_mode": _capi.PES_H2O_LM,
             "water_dimer": _capi.PES_DIMER, "partridge_schwenke": _capi.PES_H2O_PS}
    ORDER = {"harmonic_oscillator": ["k"],
             "h2o_local_mode": ["De", "a", "re", "ktheta", "theta_e", "krr"],
             "water_dimer": ["De", "a", "re", "ktheta", "theta_e", "krr", "eps", "sigma", "qH", "qO"],
             "partridge_schwenke": ["hho"]}

    def __init__(self, kind, params, natoms=None, device=None):
        if kind not in self.KINDS:
            raise ValueError(f"unknown PES kind {kind!r}; choose one of {sorted(self.KINDS)}")
        self.kind = kind
        self.params = dict(params)
        fixed = {"h2o_local_mode": 3, "water_dimer": 6, "partridge_schwenke": 3}
        self.natoms = fixed.get(kind, natoms if natoms is not None else 1)
        if natoms is not None and natoms != self.natoms:
            raise ValueError(f"{kind} has {self.natoms} atoms, got natoms={natoms}")
        missing = [k for k in self.ORDER[kind] if k not in self.params]
        if missing:
            raise ValueError(f"missing PES parameters {missing}")
        self.device = device

    def pes_struct(self):
        s = _capi.PES()
        s.kind = self.KINDS[self.kind]
        s.natoms = self.natoms
        for i, k in enumerate(self.ORDER[self.kind]):
            s.p[i] = float(self.params[k])
        return s

    def _dev(self):
        return torch.device(self.device) if self.device is not None else default_device()

    def eval_soa(self, x, n, ld=None, grad=False):
        """V (and dV/dx in SoA when grad) for the first n walkers of a (3A, ld) device tensor."""
        L = _capi.load()
        ld = x.shape[1] if ld is None else ld
        v = torch.empty(max(n, 1), dtype=torch.float64, device=x.device)
        g = torch.empty_like(x) if grad else None
        _capi.check(L.gbdmc_pes_eval(C.byref(self.pes_struct()), _ptr(x), n, ld, _ptr(v), _ptr(g), _stream()),
                    "gbdmc_pes_eval")
        return (v[:n], g) if grad else v[:n]

    def getpot(self, cds, timeit=False):
        """(N, A, 3) bohr -> (N,) hartree, the contract of potential_manager.py:71-99."""
        if timeit:
            start = time.time()
        cds = np.asarray(cds, dtype=np.float64)
        if cds.ndim != 3 or cds.shape[1] != self.natoms or cds.shape[2] != 3:
            raise ValueError(f"cds must be (N, {self.natoms}, 3), got {cds.shape}")
        x = to_soa(cds, self._dev())
        v = self.eval_soa(x, cds.shape[0]).cpu().numpy()
        if timeit:
            return v, time.time() - start
        return v

    def getgrad(self, cds):
        """(V, dV/dx) from the adjoint kernel, host arrays."""
        cds = np.asarray(cds, dtype=np.float64)
        n = cds.shape[0]
        x = to_soa(cds, self._dev())
        v, g = self.eval_soa(x, n, grad=True)
        return v.cpu().numpy(), from_soa(g, n, self.natoms)


class PESFunction(torch.autograd.Function):
    """V(x) for x of shape (N, A, 3) float64 on the GPU, with the hand-written
    adjoint kernel as its backward: dL/dx = dL/dV * dV/dx."""

    @staticmethod
    def forward(ctx, x, potential):
        n, A, _ = x.shape
        xs = x.detach().reshape(n, 3 * A).t().contiguous()
        v, g = potential.eval_soa(xs, n, grad=True)
        ctx.save_for_backward(g.t().reshape(n, A, 3))
        return v.clone()

    @staticmethod
    def backward(ctx, gv):
        (g,) = ctx.saved_tensors
        return gv[:, None, None] * g, None


# ----------------------------------------------------------- factories
def harmonic_oscillator(omega_wavenumbers=3000.0, mass_amu=1.00782505, natoms=1, device=None):
    """Isotropic 3D harmonic well V = 1/2 k |x|^2 with k = m omega^2."""
    m = mass_amu * Constants.atomic_units["amu"]
    w = Constants.convert(omega_wavenumbers, "wavenumbers")
    return Potential_GPU("harmonic_oscillator", {"k": m * w * w}, natoms=natoms, device=device)


def partridge_schwenke(atom_order="OHH", device=None):
    """The Partridge-Schwenke water PES (J. Chem. Phys. 106, 4618 (1997)) that
    the reference ships as its Fortran sample potential
    (sample_potentials/FortPots/Partridge_Schwenke_H2O), as a GPU kernel.
    ``atom_order`` 'HHO' takes the reference's calc_hoh_pot coordinate order
    (H, H, O); 'OHH' the order of the other water PESs here."""
    if atom_order not in ("OHH", "HHO"):
        raise ValueError("atom_order must be 'OHH' or 'HHO'")
    return Potential_GPU("partridge_schwenke", {"hho": 1.0 if atom_order == "HHO" else 0.0}, device=device)


def h2o_local_mode(De=0.1869, a=1.2, re=1.81, ktheta=0.16, theta_e_deg=104.5, krr=0.01, device=None):
    """Local-mode H2O, atoms O,H,H: Morse OH stretches, harmonic bend
    1/2 k_theta (theta - theta_e)^2 and a k_rr (r1-re)(r2-re) coupling."""
    return Potential_GPU("h2o_local_mode", dict(De=De, a=a, re=re, ktheta=ktheta,
                                                theta_e=np.deg2rad(theta_e_deg), krr=krr), device=device)


# Minimum of the default water_dimer surface (O,H,H,O,H,H; bohr; E = -0.0108784 Eh).
WATER_DIMER_EQ = np.array([
    [0.000000000000, 0.000000000000, 0.000000000000],
    [1.427477952458, -0.371496091643, 1.058267415716],
    [-0.475355230876, -1.624174243271, -0.657060123398],
    [-0.890893874743, 4.517468473284, -2.310760800984],
    [-2.231456348667, 5.100851802863, -1.249695023025],
    [-0.483907575038, 2.882598047543, -1.568314000679]])


def water_dimer(eps=2.4e-4, sigma=5.95, qH=0.417, qO=-0.834, device=None, **monomer):
    """Water dimer O,H,H,O,H,H: two local-mode monomers + O-O Lennard-Jones +
    intermolecular point charges."""
    mono = h2o_local_mode(**monomer).params
    return Potential_GPU("water_dimer", dict(mono, eps=eps, sigma=sigma, qH=qH, qO=qO), device=device)
