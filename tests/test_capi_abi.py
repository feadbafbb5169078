"""libgbdmc.so loads on a machine without a GPU and exports every entry point
declared in include/gbdmc.h; the ctypes structs match the C layout."""
import ctypes
import os
import re


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(gbdmc_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("gbdmc_pes_eval", "gbdmc_trial_eval", "gbdmc_sim_init", "gbdmc_sim_step", "gbdmc_desc_weights"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from pyvibdmc_gb300 import _capi
    lib = _capi.load()
    raw = ctypes.CDLL(_capi.lib_path())
    for name in declared_symbols():
        assert hasattr(raw, name), f"{name} declared in include/ but not exported"


def test_bounds_checked_build_exports_the_same_symbols():
    from pyvibdmc_gb300 import _build, _capi
    if not os.path.exists(_build.LIB_BC):
        _build.build(variants=("bc",))
    bc = ctypes.CDLL(_build.LIB_BC)
    for name in declared_symbols():
        assert hasattr(bc, name), f"{name} not exported by the bounds-checked build"
    assert bc.gbdmc_bounds_check_enabled() == 1
    assert _capi.load().gbdmc_bounds_check_enabled() == 0


def test_struct_layout_matches():
    from pyvibdmc_gb300 import _capi
    _capi.load()
    _capi.check_abi()


def test_scratch_bytes_scales():
    from pyvibdmc_gb300 import _capi
    L = _capi.load()
    assert L.gbdmc_scratch_bytes(0) == 0
    a, b = L.gbdmc_scratch_bytes(1000), L.gbdmc_scratch_bytes(100000)
    assert 0 < a < b


def test_error_reporting_without_gpu():
    from pyvibdmc_gb300 import _capi
    L = _capi.load()
    rc = L.gbdmc_pes_eval(None, None, 1, 1, None, None, None)
    assert rc == _capi.ERR_ARG
    assert b"invalid" in L.gbdmc_last_error()
    # no walkers: nothing to read, so no buffers are needed and no kernel runs
    pes = _capi.PES(kind=_capi.PES_H2O_LM, natoms=3)
    assert L.gbdmc_pes_eval(ctypes.byref(pes), None, 0, 0, None, None, None) == _capi.OK
    assert L.gbdmc_pes_eval(ctypes.byref(pes), None, 2, 1, None, None, None) == _capi.ERR_ARG  # ld < n


def test_gemm_pairs_refuse_bad_arguments_without_gpu():
    """The pair GEMMs check their arguments before any CUDA call: a null
    operand, K other than 16 or 128, an engine other than 0 or 1 and m < 0 are
    refused, and m = 0 returns at once (the pointer is never dereferenced)."""
    from pyvibdmc_gb300 import _capi
    L = _capi.load()
    p = ctypes.c_void_p(256)
    xw = lambda x0, m, k, e: L.gbdmc_mlp_gemm_pair(x0, p, m, k, p, None, None, p, p, e, None)  # noqa: E731
    tn = lambda x0, m, k, e: L.gbdmc_mlp_gemm_tn_pair(x0, p, p, p, m, k, p, e, None)  # noqa: E731
    for f in (xw, tn):
        assert f(None, 8, 16, 0) == _capi.ERR_ARG
        assert f(p, 8, 5, 0) == _capi.ERR_ARG
        assert f(p, 8, 16, 2) == _capi.ERR_ARG
        assert f(p, -1, 128, 1) == _capi.ERR_ARG
        assert f(p, 0, 128, 1) == _capi.OK
    assert b"engine 0 or 1" in L.gbdmc_last_error()  # the last refusal's message


def test_replica_table_is_checked_before_any_launch():
    """Bad replica tables are refused on the host (no pointer is touched)."""
    from pyvibdmc_gb300 import _capi
    L = _capi.load()
    s = _capi.Sim(natoms=3, weighting=_capi.DISCRETE, ld=1000, n0=100, block_threads=64)
    s.pes.kind, s.pes.natoms = _capi.PES_H2O_LM, 3
    s.trial.kind, s.trial.natoms = _capi.TRIAL_NONE, 3
    w = _capi.Walkers(x=16, v=16, idx=16)
    fake = ctypes.c_void_p(16)

    def init(pairs):
        reps = (_capi.Replica * len(pairs))()
        for k, (off, cap) in enumerate(pairs):
            reps[k].off, reps[k].cap, reps[k].n0 = off, cap, 50
        return L.gbdmc_batch_init(ctypes.byref(s), reps, len(pairs), ctypes.byref(w), fake, fake, None)

    assert init([(0, 400), (300, 400)]) == _capi.ERR_ARG
    assert b"overlap" in L.gbdmc_last_error()
    assert init([(0, 400), (600, 500)]) == _capi.ERR_ARG  # past ld
    assert b"bad off/cap" in L.gbdmc_last_error()
    assert init([(0, 10)] * 65) == _capi.ERR_CAPACITY  # more than 64 replicas


def _prototypes():
    """name -> list of parameter declarations, from every header in include/."""
    out = {}
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        for m in re.finditer(r"\b(gbdmc_\w+)\s*\(([^;{]*?)\)\s*;", text):
            params = [p.strip() for p in m.group(2).split(",")]
            out[m.group(1)] = [] if params == ["void"] else params
    return out


def test_ctypes_signatures_match_the_header():
    """Every function the Python host binds has the header's parameter count,
    and pointers where the header has pointers."""
    from pyvibdmc_gb300 import _capi
    L = _capi.load()
    protos = _prototypes()
    scalars = (ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_double, ctypes.c_uint32, ctypes.c_size_t,
               ctypes.c_int)
    checked = 0
    for name, params in protos.items():
        fn = getattr(L, name)
        if fn.argtypes is None:
            continue
        assert len(fn.argtypes) == len(params), f"{name}: ctypes {len(fn.argtypes)} args, header {len(params)}"
        for decl, ct in zip(params, fn.argtypes):
            if "*" in decl:
                assert ct not in scalars, f"{name}: '{decl}' bound as {ct.__name__}"
            else:
                assert ct in scalars, f"{name}: '{decl}' bound as {ct.__name__}"
        checked += 1
    assert checked >= 30
