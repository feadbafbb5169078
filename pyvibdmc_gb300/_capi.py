"""ctypes binding of libgbdmc.so (the C ABI declared in include/gbdmc.h).

The structs here mirror the header field by field; ``check_abi()`` compares
their sizes against ``gbdmc_struct_size`` of the loaded library.  Loading
fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

from . import _build

MAX_ATOMS = 8

OK, ERR_ARG, ERR_CUDA, ERR_CAPACITY = 0, 1, 2, 3
ST_NONFINITE_WEIGHT, ST_HUGE_WEIGHT, ST_POP_LOW, ST_POP_HIGH, ST_OVERFLOW, ST_TIMEOUT = 1, 2, 4, 8, 16, 32
PES_HO, PES_H2O_LM, PES_DIMER, PES_H2O_PS, PES_EXTERNAL = 1, 2, 3, 4, 5
TRIAL_NONE, TRIAL_HO_GAUSS, TRIAL_H2O_GAUSS, TRIAL_DIMER_GAUSS = 0, 1, 2, 3
NOISE_PHILOX32, NOISE_PHILOX64, NOISE_INJECTED = 0, 1, 2
DISCRETE, CONTINUOUS = 0, 1


class PES(C.Structure):
    _fields_ = [("kind", C.c_int32), ("natoms", C.c_int32), ("p", C.c_double * 16)]


class Trial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("natoms", C.c_int32), ("p", C.c_double * 16)]


class Walkers(C.Structure):
    _fields_ = [("x", C.c_void_p), ("v", C.c_void_p), ("who", C.c_void_p), ("f", C.c_void_p),
                ("psi", C.c_void_p), ("ke", C.c_void_p), ("w", C.c_void_p), ("idx", C.c_void_p),
                ("key", C.c_void_p)]


class Ctrl(C.Structure):
    _fields_ = [("n", C.c_int64), ("n_prev", C.c_int64), ("step", C.c_int64), ("vref", C.c_double),
                ("dt_eff", C.c_double), ("eff_ts", C.c_double), ("status", C.c_int32),
                ("err_step", C.c_int32), ("ticket", C.c_uint32), ("flags", C.c_int32),
                ("n_acc", C.c_int64), ("reserved", C.c_int64 * 6)]


class History(C.Structure):
    _fields_ = [("vref", C.c_void_p), ("pop", C.c_void_p), ("births", C.c_void_p), ("deaths", C.c_void_p),
                ("rejected", C.c_void_p), ("vmin", C.c_void_p), ("vmax", C.c_void_p), ("vmean", C.c_void_p),
                ("eff_ts", C.c_void_p), ("len", C.c_int64)]


class Sim(C.Structure):
    _fields_ = [("natoms", C.c_int32), ("weighting", C.c_int32), ("noise_mode", C.c_int32),
                ("track_who", C.c_int32), ("ld", C.c_int64), ("n0", C.c_int64), ("dt", C.c_double),
                ("alpha", C.c_double), ("sigma", C.c_double * MAX_ATOMS), ("inv_mass", C.c_double * MAX_ATOMS),
                ("thresh_lower", C.c_double), ("thresh_upper", C.c_double), ("seed", C.c_uint64),
                ("block_threads", C.c_int32), ("replica_id", C.c_uint32),
                ("pes", PES), ("trial", Trial), ("hist", History)]


MAX_REPLICAS = 64
FW_BLOCKS = 512  # GBDMC_FW_BLOCKS


class Replica(C.Structure):
    _fields_ = [("off", C.c_int64), ("cap", C.c_int64), ("n0", C.c_int64), ("stream", C.c_uint32),
                ("reserved", C.c_int32)]


class Noise(C.Structure):
    _fields_ = [("normal", C.c_void_p), ("u_branch", C.c_void_p), ("u_accept", C.c_void_p),
                ("ld_noise", C.c_int64)]


class MLP(C.Structure):
    _fields_ = [("w1t", C.c_void_p), ("w2t", C.c_void_p), ("w3t", C.c_void_p), ("b1", C.c_void_p),
                ("b2", C.c_void_p), ("b3", C.c_void_p), ("w4", C.c_void_p), ("b4", C.c_float),
                ("e_mean", C.c_float), ("e_scale", C.c_float), ("hull_margin", C.c_float),
                ("feat_mu", C.c_float * 16), ("feat_inv_sd", C.c_float * 16), ("feat_lo", C.c_float * 16),
                ("feat_hi", C.c_float * 16), ("audit_every", C.c_int32), ("engine", C.c_int32),
                ("bias_beta", C.c_float), ("sort_atoms", C.c_int32)]


class WalkersF32(C.Structure):
    _fields_ = [("x", C.c_void_p), ("v", C.c_void_p), ("who", C.c_void_p), ("idx", C.c_void_p),
                ("f", C.c_void_p), ("lnpsi", C.c_void_p), ("ke", C.c_void_p)]


class AdamParam(C.Structure):
    _fields_ = [("p", C.c_void_p), ("g", C.c_void_p), ("m", C.c_void_p), ("v", C.c_void_p), ("wt", C.c_void_p),
                ("wn", C.c_void_p), ("n", C.c_int64), ("k", C.c_int32), ("pad", C.c_int32)]


class HostWalkersC(C.Structure):
    _fields_ = [("x", C.c_void_p), ("v", C.c_void_p), ("who", C.c_void_p), ("key", C.c_void_p), ("ld", C.c_int64)]


_STRUCTS = [Sim, Walkers, Ctrl, Noise, PES, Trial, History, Replica, MLP, WalkersF32, AdamParam, HostWalkersC]

_lib = None


def lib_path():
    """libgbdmc.so, or its bounds-checked build libgbdmc_bc.so when the
    environment sets GBDMC_BOUNDS_CHECK=1 (read at the first load)."""
    return _build.LIB_BC if os.environ.get("GBDMC_BOUNDS_CHECK") == "1" else _build.LIB


def load():
    """Load libgbdmc.so (building it first when absent); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        _build.build(variants=("bc",) if path == _build.LIB_BC else ("",))
    L = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "gbdmc_abi_version": ([], C.c_int),
        "gbdmc_last_error": ([], C.c_char_p),
        "gbdmc_scratch_bytes": ([C.c_int64], C.c_size_t),
        "gbdmc_struct_size": ([C.c_int32], C.c_size_t),
        "gbdmc_pes_eval": ([C.POINTER(PES), P, C.c_int64, C.c_int64, P, P, P], C.c_int),
        "gbdmc_trial_eval": ([C.POINTER(Trial), P, C.c_int64, C.c_int64, P, P, P, P], C.c_int),
        "gbdmc_sim_init": ([C.POINTER(Sim), C.POINTER(Walkers), P, P, P], C.c_int),
        "gbdmc_sim_step": ([C.POINTER(Sim), C.POINTER(Walkers), C.POINTER(Walkers), P, P,
                            C.POINTER(Noise), P], C.c_int),
        "gbdmc_sim_run_scratch_bytes": ([C.c_int64], C.c_size_t),
        "gbdmc_lineage_noise": ([C.POINTER(Sim), P, C.c_int64, C.c_int64, P, C.c_int64, P, P], C.c_int),
        "gbdmc_sim_run": ([C.POINTER(Sim), C.POINTER(Walkers), C.POINTER(Walkers), P, P, C.c_int64, C.c_int32, P],
                          C.c_int),
        "gbdmc_sim_run_host": ([C.POINTER(Sim), C.POINTER(HostWalkersC), C.POINTER(Walkers), C.POINTER(Walkers), P,
                                C.POINTER(Ctrl), P, C.c_int64, C.c_int32, P, P], C.c_int),
        "gbdmc_sim_move": ([C.POINTER(Sim), C.POINTER(Walkers), C.POINTER(Walkers), P, P, C.POINTER(Noise), P],
                           C.c_int),
        "gbdmc_sim_branch": ([C.POINTER(Sim), C.POINTER(Walkers), P, P, C.POINTER(Noise), P], C.c_int),
        "gbdmc_sim_step_host": ([C.POINTER(Sim), C.POINTER(Walkers), C.POINTER(Walkers), P, P, P,
                                 C.POINTER(Noise), P], C.c_int),
        "gbdmc_desc_weights": ([P, P, P, C.c_int64, P, P], C.c_int),
        "gbdmc_desc_begin": ([P, P, P], C.c_int),
        "gbdmc_argpartition": ([P, C.c_int64, C.c_int64, P, P, P, P], C.c_int),
        "gbdmc_batch_init": ([C.POINTER(Sim), C.POINTER(Replica), C.c_int32, C.POINTER(Walkers), P, P, P],
                             C.c_int),
        "gbdmc_batch_step": ([C.POINTER(Sim), C.POINTER(Replica), C.c_int32, C.POINTER(Walkers),
                              C.POINTER(Walkers), P, P, C.POINTER(Noise), P], C.c_int),
        "gbdmc_batch_scratch_bytes": ([C.POINTER(Replica), C.c_int32], C.c_size_t),
        "gbdmc_walkers_compact": ([C.POINTER(Sim), C.POINTER(Replica), C.c_int32, C.POINTER(Walkers),
                                   C.POINTER(Walkers), P, P], C.c_int),
        "gbdmc_mlp_gemm": ([P, C.c_int64, C.c_int32, P, P, P, P], C.c_int),
        "gbdmc_mlp_gemm_tn": ([P, P, C.c_int64, C.c_int32, P, P], C.c_int),
        "gbdmc_mlp_silu_fwd": ([P, P, P, P, C.c_int64, P], C.c_int),
        "gbdmc_mlp_silu_bwd": ([P, P, P, P, P, P, C.c_int64, P, P], C.c_int),
        "gbdmc_mlp_head": ([P, P, P, C.c_float, P, P, P, C.c_int64, C.c_float, C.c_float, P, P, P, P, P, P],
                           C.c_int),
        "gbdmc_mlp_gemm_status": ([C.c_int32], C.c_int),
        "gbdmc_mlp_gemm_tc": ([P, C.c_int64, C.c_int32, P, P, P, P], C.c_int),
        "gbdmc_mlp_gemm_tn_tc": ([P, P, C.c_int64, C.c_int32, P, P], C.c_int),
        "gbdmc_mlp_gemm_pair": ([P, P, C.c_int64, C.c_int32, P, P, P, P, P, C.c_int32, P], C.c_int),
        "gbdmc_mlp_gemm_tn_pair": ([P, P, P, P, C.c_int64, C.c_int32, P, C.c_int32, P], C.c_int),
        "gbdmc_mlp_train_inputs": ([P, P, P, C.c_int64, C.c_int64, P, C.c_uint64, P, P, C.c_float, C.c_float, P,
                                    C.c_int32, P, P, P, P, P], C.c_int),
        "gbdmc_mlp_adam_all": ([P, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int64,
                                C.c_int64, C.c_int64, P, P, P], C.c_int),
        "gbdmc_mlp_adam": ([P, P, P, P, C.c_int64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int32, P, P,
                            C.c_int32, P], C.c_int),
        "gbdmc_dimer_features": ([P, C.c_int64, C.c_int64, P, P, P, P, C.c_float, P, P, P, C.c_int32, P], C.c_int),
        "gbdmc_mlp_energy": ([C.POINTER(MLP), P, C.c_int64, C.c_int64, P, P, P, P], C.c_int),
        "gbdmc_mlp_sim_init": ([C.POINTER(Sim), C.POINTER(MLP), C.POINTER(WalkersF32), P, P, P], C.c_int),
        "gbdmc_mlp_sim_step": ([C.POINTER(Sim), C.POINTER(MLP), C.POINTER(WalkersF32), C.POINTER(WalkersF32), P, P,
                                P, C.POINTER(Noise), P], C.c_int),
        "gbdmc_mlp_compact": ([C.POINTER(Sim), C.POINTER(WalkersF32), C.POINTER(WalkersF32), P, P], C.c_int),
        "gbdmc_mlp_batch_init": ([C.POINTER(Sim), C.POINTER(MLP), P, C.c_int32, C.POINTER(WalkersF32), P, P, P],
                                 C.c_int),
        "gbdmc_mlp_batch_step": ([C.POINTER(Sim), C.POINTER(MLP), P, C.c_int32, C.POINTER(WalkersF32),
                                  C.POINTER(WalkersF32), P, P, P, C.POINTER(Noise), P], C.c_int),
        "gbdmc_mlp_batch_compact": ([C.POINTER(Sim), P, C.c_int32, C.POINTER(WalkersF32), C.POINTER(WalkersF32),
                                     P, P], C.c_int),
        "gbdmc_mlp_fw_begin": ([C.POINTER(Sim), P, C.c_int32, C.POINTER(WalkersF32), P, P, P, P, P, P], C.c_int),
        "gbdmc_mlp_fw_end": ([C.POINTER(Sim), P, C.c_int32, C.POINTER(WalkersF32), P, P, P, P], C.c_int),
        "gbdmc_sim_step_static": ([C.POINTER(Sim), C.POINTER(Walkers), C.POINTER(Walkers), P, C.POINTER(Noise), P],
                                  C.c_int),
        "gbdmc_sim_step_static_max_ld": ([], C.c_size_t),
        "gbdmc_prof_enable": ([C.c_int32], C.c_int),
        "gbdmc_prof_read": ([C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_double),
                             C.POINTER(C.c_int64)], C.c_int),
        "gbdmc_fp64_fma_probe": ([P, C.c_int64, C.c_int32, C.POINTER(C.c_double), P], C.c_int),
        "gbdmc_bounds_check_enabled": ([], C.c_int),
        "gbdmc_bounds_errors": ([C.c_int32], C.c_uint32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    check_abi()
    return L


def check_abi():
    L = _lib
    if L.gbdmc_abi_version() != 1:
        raise RuntimeError("libgbdmc ABI version mismatch")
    for i, s in enumerate(_STRUCTS):
        n = L.gbdmc_struct_size(i)
        if n != C.sizeof(s):
            raise RuntimeError(f"ABI struct {s.__name__}: C sizeof {n} != ctypes {C.sizeof(s)}")


def check(rc, what="gbdmc"):
    if rc != OK:
        msg = _lib.gbdmc_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed (code {rc}): {msg}")
