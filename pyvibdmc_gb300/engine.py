"""``DMC_Sim`` -- the GPU diffusion Monte Carlo engine with PyVibDMC's API.

Constructor keywords, properties, output files and error behaviour follow
``DMC_Sim`` of pyvibdmc/pyvibdmc.py:67-130 (keywords), :132-297 (set-up),
:358-370 (properties), :701-876 (``propagate``) and :878-932 (``run``).
The per-step work runs in libgbdmc (sm_103a) on walkers that stay resident in
HBM; the host only orders steps, handles the event schedule (checkpoints,
descendant-weighting windows, logs) and reads a 128-byte control block once
per batch of steps.  Batches of steps are captured into CUDA graphs.

Extra keywords (after ``*``): ``seed`` (Philox key), ``rng`` ('philox32',
'philox64', or an object with ``standard_normal(shape)`` / ``uniform(n)``
that supplies the deviates on the host in the reference's call order),
``capacity`` (walker buffer size, default ``floor(1.5 N0) + 1`` rounded up to
256), ``graph_steps`` (steps per captured CUDA graph), ``device``,
``write_files``, ``training_sink`` (callable receiving device walkers at the
``DEBUG_save_training_every`` steps), ``replica_id`` (Philox stream),
``block_threads`` (tile width; 0 = chosen from the population) and
``fused_steps`` (plain discrete Philox runs: up to this many steps per launch
of the multi-step kernel, walkers resident in shared memory; its walkers draw
from the Philox streams of their lineage keys, which travel with them from
launch to launch and into checkpoints; 0 = one launch pair per step with the
index-keyed streams, which ``block_threads`` also selects).
"""
import contextlib
import ctypes as C
import pickle
import time

import numpy as np
import torch

from . import _capi
from . import archive
from .constants import Constants, get_atomic_num
from .potentials import Potential_GPU, default_device, to_soa, from_soa

try:  # NVTX ranges around the host's phases (step batches, events), seen by nsys / ncu --nvtx
    from torch.cuda import nvtx as _nvtx
    _nvtx.range_push("gbdmc")
    _nvtx.range_pop()
except Exception:  # a torch without NVTX: the ranges are skipped
    _nvtx = None


@contextlib.contextmanager
def nvtx_range(name):
    if _nvtx is None:
        yield
        return
    _nvtx.range_push(name)
    try:
        yield
    finally:
        _nvtx.range_pop()

__all__ = ["DMC_Sim", "HostWalkers", "dmc_restart"]

_MASSIVE = "Massive walker birth or death event!!!!!!! Dying..."


class DMC_Sim:
    def __init__(self, sim_name="DMC_Sim", output_folder="exSimResults", weighting="discrete", num_walkers=10000,
                 num_timesteps=20000, equil_steps=2000, chkpt_every=1000, wfn_every=1000, desc_wt_steps=100,
                 atoms=[], delta_t=1, potential=None, masses=None, start_structures=None, start_cont_wts=None,
                 branch_every=1, log_every=1, cur_timestep=0, cont_wt_thresh=None, imp_samp=None,
                 imp_samp_oned=False, second_impsamp_displacement=False, excited_state_imp_samp=False,
                 adiabatic_dmc=None, fixed_node=None, DEBUG_alpha=None, DEBUG_save_desc_wt_tracker=None,
                 DEBUG_save_training_every=None, DEBUG_save_before_bod=False, DEBUG_mass_change=None,
                 *, seed=0, rng="philox32", capacity=None, graph_steps=32, device=None, write_files=True,
                 training_sink=None, replica_id=0, block_threads=0, fused_steps=64):
        unsupported = {"imp_samp_oned": imp_samp_oned, "second_impsamp_displacement": second_impsamp_displacement,
                       "excited_state_imp_samp": excited_state_imp_samp, "adiabatic_dmc": adiabatic_dmc,
                       "fixed_node": fixed_node, "DEBUG_mass_change": DEBUG_mass_change,
                       "DEBUG_save_desc_wt_tracker": DEBUG_save_desc_wt_tracker,
                       "DEBUG_save_before_bod": DEBUG_save_before_bod}
        bad = [k for k, v in unsupported.items() if v not in (None, False)]
        if bad:
            raise NotImplementedError(f"DMC_Sim options not provided by the GPU engine: {bad}")
        if int(branch_every) < 1:
            raise ValueError("branch_every must be >= 1")
        if int(branch_every) != 1 and imp_samp is not None and weighting.lower() == "discrete":
            raise NotImplementedError("branch_every > 1 with importance-sampled discrete weighting")
        # a built-in GPU surface is fused into the step kernel; any other object with
        # the reference's getpot(cds) contract (potential_manager.py:71-253) is called on
        # the moved walkers between the move and branching kernels
        from .surrogate import NN_Potential_GPU
        self._nn_route = isinstance(potential, NN_Potential_GPU) and potential.fallback is not None
        self._external = not isinstance(potential, Potential_GPU) and not self._nn_route
        if self._external and not callable(getattr(potential, "getpot", None)):
            raise TypeError("potential must have a getpot(cds, timeit=False) method returning (N,) hartree")
        if self._nn_route and (weighting.lower() != "discrete" or not isinstance(rng, str) or int(cur_timestep) or
                               int(branch_every) != 1 or
                               (imp_samp is not None and getattr(imp_samp, "kind", None) != "dimer_gauss")):
            raise NotImplementedError("the fused surrogate step runs fresh discrete-weighting runs with Philox "
                                      "deviates (and the dimer trial for importance sampling)")
        if self._external and imp_samp is not None:
            raise NotImplementedError("importance sampling runs with the built-in GPU potentials "
                                      "(pyvibdmc_gb300.potentials) and trial functions")
        self.atoms = atoms if isinstance(atoms, list) else [atoms]
        self.sim_name = sim_name
        self.output_folder = output_folder
        self.num_walkers = int(num_walkers)
        self.num_timesteps = int(num_timesteps)
        self.potential_info = {k: v for k, v in vars(potential).items()} if hasattr(potential, "__dict__") else {}
        self.potential = potential
        self.weighting = weighting.lower()
        self.desc_wt_time_steps = desc_wt_steps
        self.branch_every = int(branch_every)
        self.delta_t = delta_t
        self.start_structures = start_structures
        self.start_cont_wts = start_cont_wts
        self.equil_steps = equil_steps
        self.chkpt_every = chkpt_every
        self.wfn_every = wfn_every
        self.log_every = log_every
        self.cur_timestep = int(cur_timestep)
        self.cont_wt_thresh = cont_wt_thresh
        self.impsamp_manager = imp_samp
        self._deb_training_every = DEBUG_save_training_every
        self._deb_alpha = DEBUG_alpha
        self.seed = int(seed)
        self.rng = rng
        self.graph_steps = max(2, int(graph_steps) // 2 * 2)
        self.write_files = write_files
        self.training_sink = training_sink
        self.replica_id = int(replica_id)
        self.block_threads = int(block_threads)
        self.fused_steps = int(fused_steps)
        self.device = torch.device(device) if device is not None else default_device()
        self.masses = masses
        self._initialize(capacity)

    # ------------------------------------------------------------ set-up
    def _initialize(self, capacity):
        """pyvibdmc.py:132-297 (schedules, walkers, masses, weighting, guards)."""
        T = self.num_timesteps
        self._chkpt_step = set(range(self.chkpt_every, T + self.chkpt_every, self.chkpt_every))
        wfn = np.arange(self.equil_steps, T + self.wfn_every, self.wfn_every)
        self._wfn_save_step = set(int(v) for v in wfn)
        self._desc_wt_save_step = set(int(v) for v in wfn + self.desc_wt_time_steps)
        if self._deb_training_every is not None:
            self._train_step = set(range(0, T + self._deb_training_every, self._deb_training_every))
        else:
            self._train_step = set()
        self._log_steps = set(range(0, T, self.log_every))
        if self.start_structures is None:
            raise Exception("Please supply a starting structure for your chemical system.")
        ss = np.asarray(self.start_structures, dtype=np.float64)
        if ss.ndim != 3:
            raise Exception("Start structure must have format (n,m,d), where n = 1 or num_walkers, m = num atoms, "
                            "d = dimensions (usually 3)")
        if ss.shape[0] == 1:
            coords = np.repeat(ss, self.num_walkers, axis=0)
        else:
            if ss.shape[0] != self.num_walkers:
                print("WARNING: NUMBER OF STARTING GEOMETRIES DOES NOT EQUAL NUM_WALKERS VARIABLE. MAKE SURE THIS IS"
                      "INTENTIONAL.")
            coords = ss
        if self.masses is None:
            if "-" in self.atoms[0]:
                self.masses = np.array([Constants.reduced_mass(self.atoms[0])])
                self._atm_nums = get_atomic_num(self.atoms[0].split("-"))
            else:
                self.masses = np.array([Constants.mass(a) for a in self.atoms])
                self._atm_nums = get_atomic_num(self.atoms)
        elif isinstance(self.masses, (int, float)):
            self.masses = np.array([self.masses])
            self._atm_nums = [-1]
        else:
            self.masses = np.array(self.masses, dtype=np.float64)
            self._atm_nums = get_atomic_num(self.atoms[0].split("-") if "-" in self.atoms[0] else self.atoms)
        if len(self.masses) != len(self.atoms):
            raise Exception("Your number of atoms list does not match your number of masses you provided.")
        if coords.shape[1] != len(self.atoms):
            raise Exception("Your number of atoms list does not match the shape of your walkers.")
        self.natoms = coords.shape[1]
        self.dims = coords.shape[2]
        if self.natoms > _capi.MAX_ATOMS:
            raise ValueError(f"at most {_capi.MAX_ATOMS} atoms")
        if self._external:
            if self.dims not in (1, 2, 3):
                raise ValueError("walkers must have 1, 2 or 3 dimensions per atom")
        else:
            if self.dims != 3:
                raise NotImplementedError("the built-in GPU potentials take 3D Cartesian walkers; pass a "
                                          "getpot potential for 1D or 2D walkers")
            pot_atoms = self.potential.fallback.natoms if self._nn_route else self.potential.natoms
            if self.natoms != pot_atoms:
                raise ValueError(f"potential has {pot_atoms} atoms, walkers have {self.natoms}")
        # walker rows on the device: 3 per storage atom (the caller's nc = natoms*dims coordinates, padded)
        self._ncoord = self.natoms * self.dims
        self._store_atoms = (self._ncoord + 2) // 3
        self._sigmas = np.sqrt(self.delta_t / self.masses)
        self._alpha = 1.0 / (2.0 * self.delta_t) if self._deb_alpha is None else self._deb_alpha
        self._pop_thresh = [self.num_walkers - self.num_walkers * 0.5, self.num_walkers + self.num_walkers * 0.5]
        n = coords.shape[0]
        if n < self._pop_thresh[0] or n > self._pop_thresh[1]:
            if self.weighting == "discrete":
                raise ValueError(_MASSIVE)
        self._thresh_lower, self._thresh_upper = None, None
        if self.weighting == "continuous":
            t = self.cont_wt_thresh
            if t is None:
                self._thresh_lower = 1 / self.num_walkers
            elif isinstance(t, (int, float)):
                self._thresh_lower = t
            elif isinstance(t, list) and len(t) in (1, 2):
                self._thresh_lower = t[0]
                self._thresh_upper = t[1] if len(t) == 2 else None
            else:
                raise ValueError("Invalid input for continuous weight threshold")
        elif self.weighting != "discrete":
            raise ValueError(f"weighting must be 'discrete' or 'continuous', got {self.weighting!r}")
        if self.impsamp_manager is not None and not self._nn_route:
            if getattr(self.impsamp_manager, "natoms", None) != self.natoms or \
                    not hasattr(self.impsamp_manager, "trial_struct"):
                raise TypeError("imp_samp must be a pyvibdmc_gb300.ImpSampManager_GPU for these atoms")
            if self.delta_t != 1:
                print("WARNING! Using DT>1 for Imp Samp. Make sure this is not a mistake!!!!")
        if isinstance(self.rng, str):
            if self.rng not in ("philox32", "philox64"):
                raise ValueError("rng must be 'philox32', 'philox64' or a deviate source object")
            self._noise_mode = _capi.NOISE_PHILOX32 if self.rng == "philox32" else _capi.NOISE_PHILOX64
        else:
            self._noise_mode = _capi.NOISE_INJECTED
        min_cap = int(np.floor(self._pop_thresh[1])) + 1
        cap = max(min_cap, n) if capacity is None else int(capacity)
        if cap < max(min_cap, n):
            raise ValueError(f"capacity must be >= {max(min_cap, n)}")
        self.capacity = (cap + 255) // 256 * 256
        if self._nn_route:
            self._nn_setup(coords)
            return
        self._alloc(coords)
        self._vref_vs_tau = np.zeros(self.num_timesteps)
        self._pop_vs_tau = np.zeros(self.num_timesteps)
        self._eff_ts = np.zeros(self.num_timesteps)
        self._desc_open = None
        self._graphs = {}
        self._host_vstats = {}
        # the multi-step kernel: plain DMC, discrete weighting, Philox deviates, built-in surface
        self._multi = (self.fused_steps > 0 and not self._external and self.weighting == "discrete" and
                       self.impsamp_manager is None and self._noise_mode != _capi.NOISE_INJECTED and
                       self.block_threads == 0 and self.branch_every == 1)
        self._multi_used = False
        self._multi_launches = 0
        if self.write_files:
            archive.create_filesystem(self.output_folder)

    def _nn_setup(self, coords):
        """The fused surrogate step (NNDMC) in place of the FP64 buffers."""
        from .surrogate import NNDMC
        pot = self.potential
        self._nnd = NNDMC(pot.model, pot.fallback, self.num_walkers, coords, self.masses, self.delta_t,
                          max(self.num_timesteps, 1), seed=self.seed, audit_every=pot.audit_every, rng=self.rng,
                          graph_steps=min(self.graph_steps, 16), replica_id=self.replica_id,
                          bias_control=pot.bias_control, imp_samp=self.impsamp_manager)
        self._vref_vs_tau = np.zeros(self.num_timesteps)
        self._pop_vs_tau = np.zeros(self.num_timesteps)
        self._eff_ts = np.zeros(self.num_timesteps)
        self._desc_open = None
        self._multi = self._multi_used = self._external = False
        self._host_vstats = {}
        if self.write_files:
            archive.create_filesystem(self.output_folder)

    def _propagate_nn(self):
        """propagate (pyvibdmc.py:701-876) on the fused surrogate step: the steps
        between events run as NNDMC batches (CUDA graphs); checkpoints,
        descendant-weighting windows and histories as in the FP64 path."""
        L = _capi.load()
        nd = self._nnd
        T = self.num_timesteps
        nd.init()
        t = 0
        bounds = [b for b in self._boundaries() if b > 0] + [T]
        ctrl_ptr = C.c_void_p(nd._ctrl.data_ptr())
        while t < T:
            self.cur_timestep = self._next_step = t
            if t in self._chkpt_step and self.write_files:
                archive.delete_older_checkpoints(self.output_folder, self.sim_name, t)
                self._chkpt(t)
            if t in self._wfn_save_step:
                self._parent = nd.walkers(0).astype(np.float64)
                self._parent_wts = None
                _capi.check(L.gbdmc_desc_begin(C.c_void_p(nd._bufs[nd._cur]["who"].data_ptr()), ctrl_ptr,
                                               self._stream()), "gbdmc_desc_begin")
                self._desc_open = t
            t_end = min(min(b for b in bounds if b > t), T)
            try:
                nd.run(t_end - t)
            finally:
                k = min(nd.step, T)
                self._vref_vs_tau[t:k] = nd._hist["vref"][0, t:k].cpu().numpy()
                self._pop_vs_tau[t:k] = nd._hist["pop"][0, t:k].cpu().numpy()
            last = t_end - 1
            if t_end in self._desc_wt_save_step and self._desc_open is not None:
                nd.walkers(0)  # compact
                npar = len(self._parent)
                desc = torch.zeros(max(npar, 1), dtype=torch.float64, device=self.device)
                _capi.check(L.gbdmc_desc_weights(C.c_void_p(nd._bufs[nd._cur]["who"].data_ptr()), None, ctrl_ptr,
                                                 npar, C.c_void_p(desc.data_ptr()), self._stream()),
                            "gbdmc_desc_weights")
                self._desc_wts = desc[:npar].cpu().numpy()
                rec = dict(start=last + 1 - self.desc_wt_time_steps, coords=self._parent, desc_wts=self._desc_wts,
                           parent_wts=None)
                self.wfns = getattr(self, "wfns", []) + [rec]
                if self.write_files:
                    archive.save_h5(f"{self.output_folder}/wfns/{self.sim_name}_wfn_{rec['start']}ts.hdf5",
                                    ["coords", "desc_wts"], [self._parent, self._desc_wts])
                self._desc_open = None
            t = t_end
        self.cur_timestep = T - 1
        self._next_step = T

    def _alloc(self, coords):
        dev, ld, A = self.device, self.capacity, self._store_atoms
        f64 = dict(dtype=torch.float64, device=dev)
        IS = self.impsamp_manager is not None
        cont = self.weighting == "continuous"
        self._bufs = []
        for _ in range(2):
            b = dict(x=torch.zeros(3 * A, ld, **f64), v=torch.zeros(ld, **f64),
                     who=torch.zeros(ld, dtype=torch.int32, device=dev),
                     key=torch.zeros(ld, dtype=torch.int64, device=dev))  # the multi-step kernel's lineage keys
            if IS:
                b.update(f=torch.zeros(3 * A, ld, **f64), psi=torch.zeros(ld, **f64), ke=torch.zeros(ld, **f64))
            if cont:
                b["w"] = torch.zeros(ld, **f64)
            else:
                b["idx"] = torch.zeros(ld, dtype=torch.int32, device=dev)
            self._bufs.append(b)
        if cont:
            w0 = np.ones(len(coords)) if self.start_cont_wts is None else np.asarray(self.start_cont_wts, float)
            self._bufs[0]["w"][:len(coords)] = torch.as_tensor(w0, **f64)
        self._bufs[0]["x"][:self._ncoord, :len(coords)] = to_soa(coords, dev)
        self._bufs[0]["key"][:len(coords)] = torch.arange(len(coords), dtype=torch.int64, device=dev)
        self._cur = 0
        self._lazy = False  # current buffer holds its walkers through a gather index
        self._ctrl = torch.zeros(C.sizeof(_capi.Ctrl), dtype=torch.uint8, device=dev)
        L = _capi.load()
        self._scratch = torch.zeros(L.gbdmc_scratch_bytes(ld), dtype=torch.uint8, device=dev)
        T = max(self.num_timesteps, 1)
        self._hist = dict(vref=torch.zeros(T, **f64), pop=torch.zeros(T, **f64),
                          births=torch.zeros(T, dtype=torch.int32, device=dev),
                          deaths=torch.zeros(T, dtype=torch.int32, device=dev),
                          rejected=torch.zeros(T, dtype=torch.int32, device=dev),
                          vmin=torch.zeros(T, **f64), vmax=torch.zeros(T, **f64), vmean=torch.zeros(T, **f64),
                          eff_ts=torch.zeros(T, **f64))
        self._n_start = len(coords)
        self._sim = self._make_sim()

    def _make_sim(self):
        s = _capi.Sim()
        s.natoms = self._store_atoms
        s.weighting = _capi.DISCRETE if self.weighting == "discrete" else _capi.CONTINUOUS
        s.noise_mode = self._noise_mode
        s.track_who = 1
        s.ld = self.capacity
        s.n0 = self.num_walkers
        s.dt = float(self.delta_t)
        s.alpha = float(self._alpha)
        for a in range(self.natoms):
            s.sigma[a] = float(self._sigmas[a])
            s.inv_mass[a] = float(1.0 / self.masses[a])
        s.thresh_lower = float(self._thresh_lower) if self._thresh_lower is not None else 0.0
        s.thresh_upper = float(self._thresh_upper) if self._thresh_upper is not None else -1.0
        s.seed = self.seed & 0xFFFFFFFFFFFFFFFF
        s.block_threads = self.block_threads
        s.replica_id = self.replica_id
        if self._external:
            s.pes.kind, s.pes.natoms = _capi.PES_EXTERNAL, self._store_atoms
            s.pes.p[0], s.pes.p[1] = float(self._ncoord), float(self.dims)
        else:
            s.pes = self.potential.pes_struct()
        if self.impsamp_manager is not None:
            s.trial = self.impsamp_manager.trial_struct()
        else:
            s.trial.kind = _capi.TRIAL_NONE
            s.trial.natoms = self._store_atoms
        h = self._hist
        s.hist.vref, s.hist.pop = h["vref"].data_ptr(), h["pop"].data_ptr()
        s.hist.births, s.hist.deaths = h["births"].data_ptr(), h["deaths"].data_ptr()
        s.hist.rejected = h["rejected"].data_ptr()
        s.hist.vmin, s.hist.vmax, s.hist.vmean = h["vmin"].data_ptr(), h["vmax"].data_ptr(), h["vmean"].data_ptr()
        s.hist.eff_ts = h["eff_ts"].data_ptr()
        s.hist.len = self.num_timesteps
        return s

    def _walker_struct(self, b, with_idx):
        w = _capi.Walkers()
        w.x, w.v, w.who = b["x"].data_ptr(), b["v"].data_ptr(), b["who"].data_ptr()
        if "f" in b:
            w.f, w.psi, w.ke = b["f"].data_ptr(), b["psi"].data_ptr(), b["ke"].data_ptr()
        if "w" in b:
            w.w = b["w"].data_ptr()
        if with_idx and "idx" in b:
            w.idx = b["idx"].data_ptr()
        if "key" in b:
            w.key = b["key"].data_ptr()
        return w

    # ------------------------------------------------------- device calls
    @staticmethod
    def _stream():
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _read_ctrl(self):
        if self._nn_route:
            return self._nnd.ctrl(0)
        return _capi.Ctrl.from_buffer_copy(self._ctrl.cpu().numpy().tobytes())

    def _write_ctrl(self, ctrl):
        self._ctrl.copy_(torch.frombuffer(bytearray(bytes(ctrl)), dtype=torch.uint8))

    def _init_device(self):
        """Step-0 potential / local energy and vref (pyvibdmc.py:760-769)."""
        self._compact()
        c = _capi.Ctrl()
        c.n = self._n_start if self.cur_timestep == 0 or not hasattr(self, "_n_now") else self._n_now
        c.step = self.cur_timestep
        c.eff_ts = self._eff_ts[self.cur_timestep - 1] if self.cur_timestep > 0 else 0.0
        self._write_ctrl(c)
        if self._external:  # step-0 potential (pyvibdmc.py:760-761) from the caller's getpot
            b = self._bufs[self._cur]
            b["v"][:c.n] = self._call_potential(b["x"], c.n)
        L = _capi.load()
        _capi.check(L.gbdmc_sim_init(C.byref(self._sim), C.byref(self._walker_struct(self._bufs[self._cur], False)),
                                     C.c_void_p(self._ctrl.data_ptr()), C.c_void_p(self._scratch.data_ptr()),
                                     self._stream()), "gbdmc_sim_init")

    def _step_sim(self, step):
        """The system description for step `step`.  Off the branching schedule
        (steps t % branch_every != 0, pyvibdmc.py:139, :828-837) discrete walkers
        are not weighted -- the branching dt is 0, so every weight is 1, every
        count 1 and vref the plain mean (calc_vref, :651-661) -- and continuous
        weights are updated without replacements (both thresholds off)."""
        if self.branch_every == 1 or step % self.branch_every == 0:
            return self._sim
        s = _capi.Sim.from_buffer_copy(self._sim)
        if self.weighting == "discrete":
            s.dt = 0.0
        else:
            s.thresh_lower, s.thresh_upper = -1.0, 0.0
        return s

    def _launch_step(self, cur, lazy, noise=None, sim=None):
        """Queue one step reading buffer `cur` (through its gather index when
        `lazy`) and writing the other buffer; returns the new (cur, lazy)."""
        L = _capi.load()
        src = self._walker_struct(self._bufs[cur], lazy)
        dst = self._walker_struct(self._bufs[1 - cur], True)
        rc = L.gbdmc_sim_step(C.byref(self._sim if sim is None else sim), C.byref(src), C.byref(dst),
                              C.c_void_p(self._ctrl.data_ptr()), C.c_void_p(self._scratch.data_ptr()),
                              C.byref(noise) if noise is not None else None, self._stream())
        _capi.check(rc, "gbdmc_sim_step")
        return 1 - cur, self.weighting == "discrete"

    def _compact(self):
        """Materialise the current walkers contiguously (gbdmc_walkers_compact)."""
        if not self._lazy:
            return
        L = _capi.load()
        src = self._walker_struct(self._bufs[self._cur], True)
        dst = self._walker_struct(self._bufs[1 - self._cur], False)
        _capi.check(L.gbdmc_walkers_compact(C.byref(self._sim), None, 0, C.byref(src), C.byref(dst),
                                            C.c_void_p(self._ctrl.data_ptr()), self._stream()),
                    "gbdmc_walkers_compact")
        self._cur, self._lazy = 1 - self._cur, False

    def _graph_for(self, cur, lazy):
        key = (cur, lazy)
        g = self._graphs.get(key)
        if g is None:
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=self.device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.graph(g, stream=side):
                c, lz = cur, lazy
                for _ in range(self.graph_steps):
                    c, lz = self._launch_step(c, lz)
            torch.cuda.current_stream().wait_stream(side)
            self._graphs[key] = g
        return g

    def _injected_noise(self, n, branch=True):
        """Host-supplied deviates in the reference's draw order (pyvibdmc.py:544, :556, :601, :392):
        normal (n, dims, natoms) transposed to (n, natoms, dims), then the uniforms (the
        branching ones only on a branching step)."""
        A, D = self.natoms, self.dims
        z = np.asarray(self.rng.standard_normal((n, D, A)), dtype=np.float64)
        zs = torch.as_tensor(np.ascontiguousarray(z.transpose(2, 1, 0).reshape(D * A, n)), device=self.device)
        ua = None
        if self.impsamp_manager is not None:
            ua = torch.as_tensor(np.asarray(self.rng.uniform(n), dtype=np.float64), device=self.device)
        ub = torch.as_tensor(np.asarray(self.rng.uniform(n), dtype=np.float64), device=self.device) \
            if self.weighting == "discrete" and branch else \
            torch.zeros(max(n, 1), dtype=torch.float64, device=self.device)
        nz = _capi.Noise()
        nz.normal, nz.u_branch = zs.data_ptr(), ub.data_ptr()
        nz.u_accept = ua.data_ptr() if ua is not None else None
        nz.ld_noise = max(n, 1)
        self._keep = (zs, ub, ua)
        return nz

    def _injected_step(self, n):
        nz = self._injected_noise(n)
        self._cur, self._lazy = self._launch_step(self._cur, self._lazy, nz)

    def _call_potential(self, x, n, timeit=False):
        """V of the first n walkers of the SoA device array x from the caller's
        potential: ``getpot_device`` on a CUDA tensor when the object has one,
        else ``getpot`` on an (n, natoms, dims) NumPy array (the reference's call,
        pyvibdmc.py:785-793).  Returns a float64 device tensor of length n."""
        dev_fn = getattr(self.potential, "getpot_device", None)
        xs = x[:self._ncoord, :n].t().reshape(n, self.natoms, self.dims)
        t0 = time.perf_counter()
        if dev_fn is not None:
            v = dev_fn(xs.contiguous())
            v = torch.as_tensor(v, dtype=torch.float64, device=self.device).reshape(-1)
        else:
            out = self.potential.getpot(np.ascontiguousarray(xs.cpu().numpy()))
            v = torch.as_tensor(np.asarray(out, dtype=np.float64).reshape(-1), device=self.device)
        self._pot_secs = time.perf_counter() - t0
        if v.numel() != n:
            raise ValueError(f"getpot returned {v.numel()} energies for {n} walkers")
        return v

    def _external_step(self, noise=None, sim=None):
        """One step around the caller's potential: gbdmc_sim_move, getpot on the
        moved walkers, gbdmc_sim_branch (pyvibdmc.py:540-547, 785-793, 380-454,
        651-682).  Returns False when a guard stopped the run."""
        L = _capi.load()
        n = self._n_now
        src = self._walker_struct(self._bufs[self._cur], self._lazy)
        b = self._bufs[1 - self._cur]
        dst = self._walker_struct(b, True)
        nz = C.byref(noise) if noise is not None else None
        _capi.check(L.gbdmc_sim_move(C.byref(self._sim), C.byref(src), C.byref(dst), C.c_void_p(self._ctrl.data_ptr()),
                                     C.c_void_p(self._scratch.data_ptr()), nz, self._stream()), "gbdmc_sim_move")
        v = self._call_potential(b["x"], n)
        b["v"][:n] = v
        step = int(self._step_device)
        vn = v.cpu().numpy() if n else np.zeros(1)
        self._host_vstats[step] = (float(vn.min()), float(vn.max()), float(vn.mean()))
        _capi.check(L.gbdmc_sim_branch(C.byref(self._sim if sim is None else sim), C.byref(dst),
                                       C.c_void_p(self._ctrl.data_ptr()),
                                       C.c_void_p(self._scratch.data_ptr()), nz, self._stream()), "gbdmc_sim_branch")
        c = self._read_ctrl()
        # a step whose guards tripped leaves its moved walkers in dst, unbranched
        self._cur, self._lazy = 1 - self._cur, self.weighting == "discrete" and not c.status
        self._n_now = int(c.n)
        self._step_device = int(c.step)
        return not c.status

    def _run_multi(self, nsteps):
        """nsteps steps through gbdmc_sim_run: launches of up to fused_steps steps,
        alternating the two walker buffers.  Returns False when the multi-step
        kernel does not take this system (the per-block buffers do not fit)."""
        L = _capi.load()
        if not hasattr(self, "_run_scratch"):
            self._run_scratch = torch.zeros(L.gbdmc_sim_run_scratch_bytes(self.capacity), dtype=torch.uint8, device=self.device)
        self._compact()
        c = self._read_ctrl()
        end = int(c.step) + nsteps
        K = self.fused_steps
        while True:
            for _ in range((end - int(c.step) + K - 1) // K):
                src = self._walker_struct(self._bufs[self._cur], False)
                dst = self._walker_struct(self._bufs[1 - self._cur], False)
                rc = L.gbdmc_sim_run(C.byref(self._sim), C.byref(src), C.byref(dst), C.c_void_p(self._ctrl.data_ptr()),
                                     C.c_void_p(self._run_scratch.data_ptr()), end, K, self._stream())
                if rc == _capi.ERR_CAPACITY and not self._multi_used:
                    self._multi = False
                    return False
                _capi.check(rc, "gbdmc_sim_run")
                self._multi_used = True
                self._multi_launches += 1
                self._cur, self._lazy = 1 - self._cur, False
            c = self._read_ctrl()
            if c.status or int(c.step) >= end:
                return True

    def _run_steps_schedule(self, nsteps):
        """nsteps steps with branching every branch_every steps: one launch per
        step with that step's system description (_step_sim)."""
        c = self._read_ctrl()
        step, self._n_now, self._step_device = int(c.step), int(c.n), int(c.step)
        sync = self._external or self._noise_mode == _capi.NOISE_INJECTED
        for k in range(nsteps):
            if sync:
                c = self._read_ctrl()
                if c.status:
                    return
                self._n_now = int(c.n)
            sim = self._step_sim(step + k)
            br = (step + k) % self.branch_every == 0
            nz = self._injected_noise(self._n_now, br) if self._noise_mode == _capi.NOISE_INJECTED else None
            if self._external:
                if not self._external_step(nz, sim):
                    return
            else:
                self._cur, self._lazy = self._launch_step(self._cur, self._lazy, nz, sim)

    def _run_steps(self, nsteps):
        """Queue nsteps steps (no host sync in the Philox modes)."""
        if self.branch_every != 1:
            return self._run_steps_schedule(nsteps)
        if self._multi and nsteps > 0 and self._run_multi(nsteps):
            return
        if self._external:
            c = self._read_ctrl()
            self._n_now, self._step_device = int(c.n), int(c.step)
            for _ in range(nsteps):
                if self._noise_mode == _capi.NOISE_INJECTED:
                    nz = self._injected_noise(self._n_now)
                else:
                    nz = None
                if not self._external_step(nz):
                    return
            return
        if self._noise_mode == _capi.NOISE_INJECTED:
            for _ in range(nsteps):
                c = self._read_ctrl()
                if c.status:
                    return
                self._injected_step(c.n)
            return
        done = 0
        if nsteps and self.weighting == "discrete" and not self._lazy:
            self._cur, self._lazy = self._launch_step(self._cur, self._lazy)
            done = 1
        while nsteps - done >= self.graph_steps:
            self._graph_for(self._cur, self._lazy).replay()
            done += self.graph_steps
        while done < nsteps:
            self._cur, self._lazy = self._launch_step(self._cur, self._lazy)
            done += 1

    # ------------------------------------------------------------ events
    def _boundaries(self):
        pts = set(self._chkpt_step) | set(self._wfn_save_step) | set(self._desc_wt_save_step)
        pts |= {s + 1 for s in self._train_step}
        return sorted(p for p in pts if p > 0)

    def _n_device(self):
        return int(self._read_ctrl().n)

    def _coords_host(self, n=None):
        if self._nn_route:
            return self._nnd.walkers(0).astype(np.float64)
        self._compact()
        n = self._n_device() if n is None else n
        x = self._bufs[self._cur]["x"]
        return x[:self._ncoord, :n].t().reshape(n, self.natoms, self.dims).cpu().numpy()

    def _begin_desc(self, t):
        """pyvibdmc.py:739-747."""
        L = _capi.load()
        self._compact()
        n = self._n_device()
        self._parent = self._coords_host(n)
        self._parent_wts = None if "w" not in self._bufs[0] else self._bufs[self._cur]["w"][:n].cpu().numpy().copy()
        _capi.check(L.gbdmc_desc_begin(C.c_void_p(self._bufs[self._cur]["who"].data_ptr()),
                                       C.c_void_p(self._ctrl.data_ptr()), self._stream()), "gbdmc_desc_begin")
        self._desc_open = t

    def _end_desc(self, t):
        """pyvibdmc.py:856-872."""
        L = _capi.load()
        self._compact()
        npar = len(self._parent)
        desc = torch.zeros(max(npar, 1), dtype=torch.float64, device=self.device)
        wb = self._bufs[self._cur].get("w")
        wptr = C.c_void_p(wb.data_ptr()) if wb is not None else None
        _capi.check(L.gbdmc_desc_weights(C.c_void_p(self._bufs[self._cur]["who"].data_ptr()), wptr,
                                         C.c_void_p(self._ctrl.data_ptr()), npar, C.c_void_p(desc.data_ptr()),
                                         self._stream()), "gbdmc_desc_weights")
        self._desc_wts = desc[:npar].cpu().numpy()
        start = t + 1 - self.desc_wt_time_steps
        self.wfns = getattr(self, "wfns", [])
        rec = dict(start=start, coords=self._parent, desc_wts=self._desc_wts, parent_wts=self._parent_wts)
        self.wfns.append(rec)
        if self.write_files:
            fname = f"{self.output_folder}/wfns/{self.sim_name}_wfn_{start}ts.hdf5"
            if self.weighting == "continuous":
                archive.save_h5(fname, ["coords", "desc_wts", "parent_wts"],
                                [self._parent, self._desc_wts, self._parent_wts])
            else:
                archive.save_h5(fname, ["coords", "desc_wts"], [self._parent, self._desc_wts])
        self._desc_open = None

    def _harvest(self, t):
        self._compact()
        n = self._n_device()
        b = self._bufs[self._cur]
        if self.training_sink is not None:
            self.training_sink(t, b["x"], b["v"], n)
        if self.write_files and self._deb_training_every is not None:
            archive.save_h5(f"{self.output_folder}/{self.sim_name}_training_{t}ts.hdf5", ["coords", "pots"],
                            [self._coords_host(n), b["v"][:n].cpu().numpy()])

    def _sync_history(self, t0, t1):
        h = {k: v[t0:t1].cpu().numpy() for k, v in self._hist.items()}
        if self._external:  # the potential's statistics come from the host-side energies
            for t in range(t0, t1):
                s = self._host_vstats.pop(t, None)
                if s is not None:
                    h["vmin"][t - t0], h["vmax"][t - t0], h["vmean"][t - t0] = s
        self._vref_vs_tau[t0:t1] = h["vref"]
        self._pop_vs_tau[t0:t1] = h["pop"]
        self._eff_ts[t0:t1] = h["eff_ts"]
        return h

    def _log(self, t0, t1, h, secs):
        if not self.write_files or self._logger is None:
            return
        full = {k: np.zeros(self.num_timesteps, dtype=v.dtype) for k, v in h.items()}
        for k, v in h.items():
            full[k][t0:t1] = v
        if self.impsamp_manager is not None:
            prev = np.concatenate([[self._pop_before], self._pop_vs_tau[t0:t1 - 1]]) if t1 > t0 else []
            full["pop_before"] = np.zeros(self.num_timesteps, dtype=np.int64)
            full["pop_before"][t0:t1] = np.asarray(prev, dtype=np.int64)
        for t in range(t0, t1):
            if t in self._log_steps:
                self._logger.step_block(t, self.weighting, full, gpu_time=secs / max(t1 - t0, 1))
        self._logger.fl.flush()

    # ------------------------------------------------------------ run
    def propagate(self):
        """The main loop (pyvibdmc.py:701-876), batched between events."""
        T = self.num_timesteps
        t = self.cur_timestep
        if self.write_files:
            self._logger.beginning(self)
        if self._nn_route:
            return self._propagate_nn()
        self._init_device()
        bounds = [b for b in self._boundaries() if b > t] + [T]
        while t < T:
            # as pyvibdmc.py:710-711: a checkpoint at step t holds the walkers before step t
            self.cur_timestep = self._next_step = t
            if t in self._chkpt_step and self.write_files:
                with nvtx_range("gbdmc.checkpoint"):
                    archive.delete_older_checkpoints(self.output_folder, self.sim_name, t)
                    self._chkpt(t)
            if t in self._wfn_save_step:
                with nvtx_range("gbdmc.desc_begin"):
                    self._begin_desc(t)
            t_end = min(b for b in bounds if b > t)
            t_end = min(t_end, T)
            self._pop_before = self._n_device() if self.impsamp_manager is not None else 0
            cur0 = self._cur
            if self.weighting == "discrete" and not self._lazy and self._noise_mode != _capi.NOISE_INJECTED:
                cur0 = self._cur  # the first step of the batch is a direct launch from this buffer
            t_start = time.perf_counter()
            with nvtx_range(f"gbdmc.steps {t}-{t_end}"):
                self._run_steps(t_end - t)
                c = self._read_ctrl()
            secs = time.perf_counter() - t_start
            if c.status:
                done = int(c.err_step) - t
                # the failing step moved its walkers into its dst buffer and did not branch
                # (the multi-step launches pass them on to the last launch's output)
                if not self._multi_used and not self._external:
                    self._cur, self._lazy = cur0 ^ (done & 1) ^ 1, False
                h = self._sync_history(t, int(c.err_step))
                self.cur_timestep = self._next_step = int(c.err_step)
                self._n_now = int(c.n)
                raise ValueError(_MASSIVE)
            self._n_now = int(c.n)
            h = self._sync_history(t, t_end)
            self._log(t, t_end, h, secs)
            self.cur_timestep = t_end - 1
            last = t_end - 1
            if t_end in self._desc_wt_save_step and self._desc_open is not None:
                with nvtx_range("gbdmc.desc_end"):
                    self._end_desc(last)
            if last in self._train_step:
                self._harvest(last)
            t = t_end
        self.cur_timestep = T - 1
        self._next_step = T  # the final checkpoint continues with step T

    def run(self):
        """pyvibdmc.py:878-932: propagate, final checkpoint, ZPE, sim_info."""
        print("Starting Simulation...")
        start = time.time()
        self._logger = archive.SimLogger(f"{self.output_folder}/{self.sim_name}_log.txt",
                                         overwrite=self.cur_timestep == 0) if self.write_files else None
        err = None
        try:
            self.propagate()
            if self.write_files:
                archive.delete_older_checkpoints(self.output_folder, self.sim_name, self.cur_timestep)
        except Exception as e:  # the reference dumps a checkpoint and re-raises
            import traceback
            print("ERROR! An error occurred while running the DMC simulation. Dumping a final checkpoint...")
            print("Ignore Approximate ZPE!!!")
            traceback.print_exc()
            err = e
        finally:
            if self.write_files:
                self._logger.write("\nFinal checkpoint is written to chkpts folder.\n\n")
                self._chkpt(self.cur_timestep)
            vref_wvn = Constants.convert(self._vref_vs_tau, "wavenumbers", to_AU=False)
            print("Simulation Complete")
            print("Approximate ZPE", np.average(vref_wvn[len(vref_wvn) // 4:]))
            ts = self._eff_ts if self.impsamp_manager is not None else np.arange(len(vref_wvn)) * self.delta_t
            if self.write_files:
                archive.save_h5(f"{self.output_folder}/{self.sim_name}_sim_info.hdf5",
                                ["vref_vs_tau", "pop_vs_tau", "atomic_nums", "atomic_masses"],
                                [np.column_stack((ts, self._vref_vs_tau)), np.column_stack((ts, self._pop_vs_tau)),
                                 self._atm_nums, self.masses])
            self.elapsed = time.time() - start
        if self.write_files:
            self._logger.finish(self.elapsed)
        self._logger = None
        if err is not None:
            raise err

    # ---------------------------------------------------- checkpointing
    def _state(self):
        n = self._n_device()
        st = {k: v for k, v in self.__dict__.items() if not k.startswith("_") and k not in (
            "potential", "impsamp_manager", "potential_info", "training_sink", "device", "rng")}
        st.update(_coords=self._coords_host(n), _vref_vs_tau=self._vref_vs_tau.copy(),
                  _keys=None if self._nn_route else self._bufs[self._cur]["key"][:n].cpu().numpy().copy(),
                  _pop_vs_tau=self._pop_vs_tau.copy(), _eff_ts=self._eff_ts.copy(),
                  _cont_wts=None if self._nn_route or "w" not in self._bufs[0] else
                  self._bufs[self._cur]["w"][:n].cpu().numpy(),
                  _masses=np.asarray(self.masses), _atm_nums=self._atm_nums,
                  _rng=self.rng if isinstance(self.rng, str) else "philox32",
                  _vref=float(self._read_ctrl().vref),
                  _next_step=getattr(self, "_next_step", self.cur_timestep))
        return st

    def _chkpt(self, t):
        with open(f"{self.output_folder}/chkpts/{self.sim_name}_{t}.pickle", "wb") as fh:
            pickle.dump(self._state(), fh, protocol=4)

    # ------------------------------------------------------ properties
    @property
    def vref_vs_tau(self):
        v = self._vref_vs_tau[:self.cur_timestep]
        return np.column_stack((np.arange(len(v)), v))

    @property
    def walkers(self):
        x = self._coords_host()
        if self.weighting == "continuous":
            return x, self._bufs[self._cur]["w"][:len(x)].cpu().numpy()
        return x

    def zpe(self, onwards=None, ret_cm=True):
        """Mean vref from step ``onwards`` (default: last 3/4 of the run), cm^-1."""
        v = self._vref_vs_tau
        o = len(v) // 4 if onwards is None else onwards
        z = np.average(v[o:])
        return Constants.convert(z, "wavenumbers", to_AU=False) if ret_cm else z


class HostWalkers:
    """The walkers of a :class:`DMC_Sim` held in page-locked host memory and
    stepped there with ``gbdmc_sim_step_host``.

    The kernels read the walkers from host memory and write the branched
    population back over the host link, so every step starts and ends with
    the walkers on the host -- the way the reference's ``propagate`` loop
    holds them in NumPy arrays (``pyvibdmc.py:710-848``).  ``step()`` queues
    one step, waits for it and returns the new population; ``run(k)`` queues
    k steps and waits once; ``x``, ``v`` (and
    ``who``, IS and continuous-weight arrays) are the pinned SoA arrays
    ``[3A][ld]`` whose first ``n`` columns are valid.  Philox noise only.
    With ``graph`` the step's launches are captured once into a CUDA graph
    and replayed.  While in use, the simulation is stepped only through this
    object; ``close()`` puts the walkers back into the simulation's device
    buffers.
    """

    def __init__(self, sim, graph=True):
        self.graph = bool(graph)
        self._graph = None
        if sim._noise_mode == _capi.NOISE_INJECTED:
            raise ValueError("HostWalkers steps with Philox deviates (rng='philox32' or 'philox64')")
        if sim._external:
            raise ValueError("HostWalkers steps the built-in GPU potentials; a getpot potential is stepped by "
                             "DMC_Sim.run")
        if sim.branch_every != 1:
            raise ValueError("HostWalkers branches every step; a branch_every schedule is stepped by DMC_Sim.run")
        sim._compact()
        torch.cuda.synchronize()
        self.sim = sim
        b = sim._bufs[sim._cur]
        self.host = {k: torch.empty(t.shape, dtype=t.dtype).pin_memory() for k, t in b.items() if k != "idx"}
        for k, t in self.host.items():
            t.copy_(b[k])
        self.work = sim._bufs[1 - sim._cur]
        self.ctrl_host = torch.zeros(C.sizeof(_capi.Ctrl), dtype=torch.uint8).pin_memory()
        self._h = sim._walker_struct(self.host, False)
        self._w = sim._walker_struct(self.work, True)
        self.n = int(sim._read_ctrl().n)
        torch.cuda.synchronize()

    def __getattr__(self, name):
        host = self.__dict__.get("host", {})
        if name in host:
            return host[name]
        raise AttributeError(name)

    def ctrl(self):
        return _capi.Ctrl.from_address(self.ctrl_host.data_ptr())

    def _queue(self):
        sim = self.sim
        rc = _capi.load().gbdmc_sim_step_host(
            C.byref(sim._sim), C.byref(self._h), C.byref(self._w), C.c_void_p(sim._ctrl.data_ptr()),
            C.c_void_p(self.ctrl_host.data_ptr()), C.c_void_p(sim._scratch.data_ptr()), None, sim._stream())
        _capi.check(rc, "gbdmc_sim_step_host")

    def _launch(self):
        if not self.graph:
            self._queue()
            return
        # the step's launches and copies are captured once and replayed: the walker
        # arrays and the control block never move, and every launch reads N from
        # the device control block
        if self._graph is None:
            g = torch.cuda.CUDAGraph()
            side = torch.cuda.Stream(device=self.sim.device)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.graph(g, stream=side):
                self._queue()
            torch.cuda.current_stream().wait_stream(side)
            self._graph = g
        self._graph.replay()

    def run(self, nsteps):
        """Queue ``nsteps`` host-resident steps back to back and wait once.
        Every step still reads the walkers from, and writes the branched
        population, V and the control block to, page-locked host memory; the
        kernels take N from the device control block, so the host needs no
        value between steps.  A step whose guard trips stops the steps after
        it on the device (the host walkers keep the last good population) and
        raises the reference's ValueError here.  Returns the population."""
        for _ in range(int(nsteps)):
            self._launch()
        torch.cuda.current_stream().synchronize()
        c = self.ctrl()
        if c.status:
            raise ValueError(f"Massive walker birth or death event!!!!!!! Dying... (status {c.status})")
        self.n = int(c.n)
        return self.n

    def step(self):
        """One host-resident step; waits for it and returns the new population."""
        return self.run(1)

    def close(self):
        """Copy the walkers back into the simulation's device buffers."""
        sim = self.sim
        b = sim._bufs[sim._cur]
        for k, t in self.host.items():
            b[k].copy_(t)
        sim._lazy = False
        sim.cur_timestep = int(sim._read_ctrl().step)
        torch.cuda.synchronize()


def dmc_restart(potential, chkpt_folder, sim_name, additional_timesteps=0, impsamp=None, **kw):
    """Reload the checkpoint of ``sim_name`` and extend the run by
    ``additional_timesteps`` (pyvibdmc.py:949-965).  A run keeps one
    checkpoint (older ones are deleted as it goes); if there are several, the
    latest step is taken.  The run continues with the step after the saved
    walkers: step t for the checkpoint written before step t, step T for the
    final checkpoint of a T-step run.  Checkpoints and wave functions of later
    steps are deleted first, as FileManager.delete_future_checkpoints does.
    A checkpoint taken inside a descendant-weighting window restarts without
    that window's parents, so its wave function is not written.
    The Philox streams are keyed by step index, so a restarted run continues
    the trajectory of the uninterrupted one."""
    import glob
    files = [p for p in glob.glob(f"{chkpt_folder}/chkpts/{sim_name}_*.pickle")
             if archive.checkpoint_step(p) is not None]
    if not files:
        raise FileNotFoundError(f"no checkpoint for {sim_name} in {chkpt_folder}/chkpts")
    st = archive.load_checkpoint(max(files, key=archive.checkpoint_step))
    if isinstance(st, archive.ReferenceCheckpoint):
        return _restart_from_reference(st, potential, chkpt_folder, sim_name, additional_timesteps, impsamp, **kw)
    nxt = int(st.get("_next_step", st["cur_timestep"]))
    archive.delete_future_checkpoints(chkpt_folder, sim_name, nxt)
    T = st["num_timesteps"] + additional_timesteps
    for k in ("replica_id", "block_threads", "branch_every"):  # the Philox stream, the reduction order
        if k in st:                                             # and the branching schedule of the saved run
            kw.setdefault(k, st[k])
    sim = DMC_Sim(sim_name=st["sim_name"], output_folder=st["output_folder"], weighting=st["weighting"],
                  num_walkers=st["num_walkers"], num_timesteps=T, equil_steps=st["equil_steps"],
                  chkpt_every=st["chkpt_every"], wfn_every=st["wfn_every"], desc_wt_steps=st["desc_wt_time_steps"],
                  atoms=st["atoms"], delta_t=st["delta_t"], potential=potential, masses=list(st["_masses"]),
                  start_structures=st["_coords"], start_cont_wts=st["_cont_wts"], log_every=st["log_every"],
                  cur_timestep=nxt, cont_wt_thresh=st["cont_wt_thresh"], imp_samp=impsamp,
                  seed=st["seed"], rng=st["_rng"], **kw)
    n = len(st["_vref_vs_tau"])
    sim._vref_vs_tau[:n] = st["_vref_vs_tau"]
    sim._pop_vs_tau[:n] = st["_pop_vs_tau"]
    sim._eff_ts[:n] = st["_eff_ts"]
    if st.get("_keys") is not None and not sim._nn_route:  # the multi-step kernel's walk goes on unchanged
        k = torch.as_tensor(np.asarray(st["_keys"]), dtype=torch.int64, device=sim.device)
        sim._bufs[sim._cur]["key"][:len(k)] = k
    return sim


def _restart_from_reference(st, potential, chkpt_folder, sim_name, additional_timesteps, impsamp, **kw):
    """dmc_restart from a checkpoint the reference wrote (its pickled DMC_Sim,
    sim_archive.py:25-43).  As the reference's dmc_restart / _init_restart
    (pyvibdmc.py:299-338, 949-965) does, the run continues with step
    ``cur_timestep`` of the checkpoint, the schedules are extended by
    ``additional_timesteps``, the step-0 potential and vref are taken afresh
    from the saved walkers, and an open descendant-weighting window keeps its
    parents, parent weights and ancestor indices."""
    d = st.__dict__
    nxt = int(d["cur_timestep"])
    archive.delete_future_checkpoints(chkpt_folder, sim_name, nxt)
    T = int(d["num_timesteps"]) + int(additional_timesteps)
    masses = np.asarray(d["masses"], dtype=np.float64)
    scalar_mass = list(d.get("_atm_nums", [])) == [-1] and masses.size == 1
    coords = np.asarray(d["_walker_coords"], dtype=np.float64)
    cont = d["weighting"] == "continuous"
    kw.setdefault("seed", 0)
    sim = DMC_Sim(sim_name=d["sim_name"], output_folder=d["output_folder"], weighting=d["weighting"],
                  num_walkers=int(d["num_walkers"]), num_timesteps=T, equil_steps=int(d["equil_steps"]),
                  chkpt_every=int(d["chkpt_every"]), wfn_every=int(d["wfn_every"]),
                  desc_wt_steps=int(d["desc_wt_time_steps"]), atoms=list(d["atoms"]), delta_t=d["delta_t"],
                  potential=potential, masses=float(masses[0]) if scalar_mass else list(masses),
                  start_structures=coords, start_cont_wts=np.asarray(d["_cont_wts"]) if cont else None,
                  branch_every=int(d.get("branch_every", 1)), log_every=int(d["log_every"]), cur_timestep=nxt,
                  cont_wt_thresh=d.get("cont_wt_thresh"), imp_samp=impsamp, DEBUG_alpha=d.get("_deb_alpha"),
                  DEBUG_save_training_every=d.get("_deb_training_every"), **kw)
    n = min(len(d["_vref_vs_tau"]), T)
    sim._vref_vs_tau[:n] = np.asarray(d["_vref_vs_tau"])[:n]
    sim._pop_vs_tau[:n] = np.asarray(d["_pop_vs_tau"])[:n]
    if impsamp is not None and d.get("eff_ts") is not None:
        m = min(len(d["eff_ts"]), T)
        sim._eff_ts[:m] = np.asarray(d["eff_ts"])[:m]
    if d.get("_desc_wt"):  # inside a descendant-weighting window (pyvibdmc.py:739-747)
        starts = [int(s) for s in np.asarray(d["_wfn_save_step"]) if s <= nxt]
        sim._parent = np.asarray(d["_parent"], dtype=np.float64)
        sim._parent_wts = np.asarray(d["_parent_wts"], dtype=np.float64) if cont else None
        who = np.asarray(d["_who_from"], dtype=np.int32)
        sim._bufs[sim._cur]["who"][:len(who)] = torch.as_tensor(who, device=sim.device)
        sim._desc_open = max(starts) if starts else nxt
    return sim
