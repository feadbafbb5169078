"""GPU importance-sampling plug-ins with the reference's manager contract.

``ImpSampManager_GPU`` exposes ``call_trial(cds) -> (N,)`` and
``call_derivs(cds) -> (dpsi/dx / psi, d2psi/dx2 / psi)`` (each (N, A, 3),
already divided by psi), the interface of ImpSampManager /
ImpSampManager_NoMP (pyvibdmc/simulation_utilities/imp_samp_manager.py:92-139,
197-224) that ``ImpSamp.drift`` (imp_samp.py:21-26) consumes.  The
derivatives are the analytic chain rule of the internal-coordinate trial
(the ChainRuleHelper formulas of imp_samp_helper.py), evaluated by
``gbdmc_trial_eval`` -- no finite differences.  Inside
:class:`pyvibdmc_gb300.DMC_Sim` the same device function runs fused in the
importance-sampled step kernel.
"""
import ctypes as C

import numpy as np
import torch

from . import _capi
from .constants import Constants
from .potentials import to_soa, from_soa, default_device, _ptr, _stream

__all__ = ["ImpSampManager_GPU", "TrialFunction", "h2o_gaussian_trial", "ho_gaussian_trial",
           "dimer_gaussian_trial", "local_energy", "fit_trial"]


class ImpSampManager_GPU:
    """Trial wave function evaluated on the GPU.

    :param kind: 'h2o_gauss' (product of Gaussians in r1, r2, theta of an
        O,H,H water), 'dimer_gauss' (the h2o_gauss trial of both monomers of an
        O,H,H,O,H,H dimer times a Gaussian in the O-O distance) or 'ho_gauss'
        (separable Cartesian Gaussian)
    :param alpha: Gaussian exponents (3 for h2o_gauss, 4 for dimer_gauss --
        the monomer's three and alpha_R -- one per atom for ho_gauss)
    :param qe: centres (r1e, r2e, theta_e) for h2o_gauss, plus R_e for dimer_gauss
    """

    def __init__(self, kind, alpha, qe=None, natoms=None, device=None):
        if kind not in ("h2o_gauss", "dimer_gauss", "ho_gauss"):
            raise ValueError(f"unknown trial kind {kind!r}")
        self.kind = kind
        self.alpha = [float(a) for a in alpha]
        self.qe = None if qe is None else [float(q) for q in qe]
        self.natoms = {"h2o_gauss": 3, "dimer_gauss": 6}.get(kind) or natoms or len(self.alpha)
        if kind == "h2o_gauss" and (len(self.alpha) != 3 or self.qe is None or len(self.qe) != 3):
            raise ValueError("h2o_gauss needs 3 alphas and 3 centres")
        if kind == "dimer_gauss" and (len(self.alpha) != 4 or self.qe is None or len(self.qe) != 4):
            raise ValueError("dimer_gauss needs 4 alphas and 4 centres")
        if kind == "ho_gauss" and len(self.alpha) != self.natoms:
            raise ValueError("ho_gauss needs one alpha per atom")
        self.device = device

    def trial_struct(self):
        t = _capi.Trial()
        t.natoms = self.natoms
        if self.kind == "h2o_gauss":
            t.kind = _capi.TRIAL_H2O_GAUSS
            for i, v in enumerate(self.alpha + self.qe):
                t.p[i] = v
        elif self.kind == "dimer_gauss":
            t.kind = _capi.TRIAL_DIMER_GAUSS
            for i, v in enumerate(self.alpha[:3] + self.qe[:3] + [self.alpha[3], self.qe[3]]):
                t.p[i] = v
        else:
            t.kind = _capi.TRIAL_HO_GAUSS
            for i, v in enumerate(self.alpha):
                t.p[i] = v
        return t

    def _dev(self):
        return torch.device(self.device) if self.device is not None else default_device()

    def eval_soa(self, x, n, ld=None):
        L = _capi.load()
        ld = x.shape[1] if ld is None else ld
        psi = torch.empty(max(n, 1), dtype=torch.float64, device=x.device)
        d1 = torch.empty_like(x)
        d2 = torch.empty_like(x)
        _capi.check(L.gbdmc_trial_eval(C.byref(self.trial_struct()), _ptr(x), n, ld, _ptr(psi), _ptr(d1),
                                       _ptr(d2), _stream()), "gbdmc_trial_eval")
        return psi[:n], d1, d2

    def call_trial(self, cds):
        cds = np.asarray(cds, dtype=np.float64)
        psi, _, _ = self.eval_soa(to_soa(cds, self._dev()), len(cds))
        return psi.cpu().numpy()

    def call_derivs(self, cds):
        cds = np.asarray(cds, dtype=np.float64)
        n = len(cds)
        _, d1, d2 = self.eval_soa(to_soa(cds, self._dev()), n)
        return from_soa(d1, n, self.natoms), from_soa(d2, n, self.natoms)


class TrialFunction(torch.autograd.Function):
    """psi_T(x) for x (N, A, 3) float64 on the GPU; backward uses the
    hand-written adjoint: dpsi/dx = psi * (dpsi/dx / psi)."""

    @staticmethod
    def forward(ctx, x, manager):
        n, A, _ = x.shape
        xs = x.detach().reshape(n, 3 * A).t().contiguous()
        psi, d1, _ = manager.eval_soa(xs, n)
        ctx.save_for_backward(psi, d1.t().reshape(n, A, 3))
        return psi.clone()

    @staticmethod
    def backward(ctx, gp):
        psi, d1 = ctx.saved_tensors
        return (gp * psi)[:, None, None] * d1, None


def h2o_gaussian_trial(omega_r=3800.0, omega_theta=1600.0, re=1.81, theta_e_deg=104.5, device=None):
    """Gaussians in (r1, r2, theta): alpha_r = mu_OH omega_r and
    alpha_theta = omega_theta / G_thetatheta at the equilibrium geometry
    (the bend G-matrix element of call_trl_h2o.py:38-46)."""
    mo, mh = Constants.mass("O"), Constants.mass("H")
    mu = mo * mh / (mo + mh)
    th = np.deg2rad(theta_e_deg)
    g = 1 / (mh * re ** 2) + 1 / (mh * re ** 2) + (1 / mo) * (2 / re ** 2 - 2 * np.cos(th) / (re * re))
    w = Constants.atomic_units["wavenumbers"]
    alpha = [mu * omega_r * w, mu * omega_r * w, omega_theta * w / g]
    return ImpSampManager_GPU("h2o_gauss", alpha, [re, re, th], device=device)


def dimer_gaussian_trial(omega_r=3800.0, omega_theta=1600.0, re=1.81, theta_e_deg=104.5, omega_R=180.0,
                         R_e=5.152, device=None):
    """The water trial of each monomer (as :func:`h2o_gaussian_trial`) times
    exp(-1/2 alpha_R (R_OO - R_e)^2) with alpha_R = mu omega_R, mu the reduced
    mass of the two waters; R_e = 5.152 bohr is the O-O distance at the
    minimum of the dimer PES."""
    mono = h2o_gaussian_trial(omega_r, omega_theta, re, theta_e_deg)
    mw = Constants.mass("O") + 2 * Constants.mass("H")
    aR = 0.5 * mw * omega_R * Constants.atomic_units["wavenumbers"]
    return ImpSampManager_GPU("dimer_gauss", mono.alpha + [aR], mono.qe + [R_e], device=device)


def ho_gaussian_trial(masses, omega_wavenumbers, device=None):
    """Separable Gaussian with alpha_a = m_a omega per atom."""
    w = Constants.convert(omega_wavenumbers, "wavenumbers")
    return ImpSampManager_GPU("ho_gauss", [m * w for m in masses], natoms=len(masses), device=device)


def local_energy(manager, potential, x, n, masses):
    """E_L = V + local kinetic energy (imp_samp.py:49-53, pyvibdmc.py:807-809) of
    the first n walkers of the SoA device array x (3A, ld): V from the GPU
    potential, the kinetic part -1/2 sum_k (1/m) (d2 psi/dx_k^2)/psi from the
    trial's adjoint kernel.  Returns a float64 device tensor."""
    v = potential.eval_soa(x, n)
    _, _, d2 = manager.eval_soa(x, n)
    inv_m = torch.as_tensor(np.repeat(1.0 / np.asarray(masses, dtype=np.float64), 3), device=x.device)
    return v - 0.5 * (inv_m[:, None] * d2[:, :n]).sum(0)


def fit_trial(manager, potential, x, n, masses, maxiter=600, fit_oo=False, verbose=False):
    """Variance minimisation of the local energy over a sample of walkers.

    The trial's parameters are set to minimise Var(E_L) over the n walkers of
    x (for example the walkers of a plain DMC run, which sample the ground
    state): E_L is the same constant everywhere for the exact ground state, so
    a smaller spread means a trial closer to it, a smaller time-step error of
    the importance-sampled walk and a smaller variance of its energy.  The
    symmetric parameters are fitted together: for 'h2o_gauss' the stretch
    exponent and centre (shared by r1 and r2), the bend exponent and centre;
    for 'dimer_gauss' the monomers' four and, with ``fit_oo``, the O-O
    exponent and centre (the O-O factor barely moves the time-step error of
    the walk, and over a ground-state sample its fit can drift to an
    unphysical centre, so by default it is kept).  Exponents are fitted on a
    log scale (Nelder-Mead).  Returns a new ImpSampManager_GPU and the
    standard deviations of E_L (hartree) before and after."""
    from scipy.optimize import minimize
    if manager.kind not in ("h2o_gauss", "dimer_gauss"):
        raise ValueError("fit_trial fits the h2o_gauss and dimer_gauss trials")
    dimer = manager.kind == "dimer_gauss"
    a0, q0 = list(manager.alpha), list(manager.qe)
    p0 = [np.log(a0[0]), np.log(a0[2]), q0[0], q0[2]] + ([np.log(a0[3]), q0[3]] if dimer and fit_oo else [])
    v = potential.eval_soa(x, n)
    inv_m = torch.as_tensor(np.repeat(1.0 / np.asarray(masses, dtype=np.float64), 3), device=x.device)

    def make(p):
        al = [np.exp(p[0]), np.exp(p[0]), np.exp(p[1])]
        qe = [p[2], p[2], p[3]]
        if dimer:
            al.append(np.exp(p[4]) if fit_oo else a0[3])
            qe.append(p[5] if fit_oo else q0[3])
        return ImpSampManager_GPU(manager.kind, al, qe, natoms=manager.natoms, device=manager.device)

    def spread(p):
        _, _, d2 = make(p).eval_soa(x, n)
        el = v - 0.5 * (inv_m[:, None] * d2[:, :n]).sum(0)
        s = float(el.std())
        return s if np.isfinite(s) else 1e30

    s0 = spread(p0)
    res = minimize(spread, p0, method="Nelder-Mead",
                   options=dict(maxiter=maxiter, xatol=1e-4, fatol=s0 * 1e-6, adaptive=True))
    if verbose:
        print(f"fit_trial: sd(E_L) {s0:.6g} -> {res.fun:.6g} Eh in {res.nit} iterations")
    return make(res.x), s0, float(res.fun)
