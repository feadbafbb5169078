"""Build recipe for libgbdmc.so (sm_103a) -- nvcc, one object per .cu, in parallel.

Usage: ``python -m pyvibdmc_gb300._build [-v] [-f]`` or ``pyvibdmc_gb300._build.build()``.
The libraries land in ``pyvibdmc_gb300/_lib/`` (in-tree, git-ignored):
libgbdmc.so and libgbdmc_bc.so, the same sources compiled with
-DGBDMC_BOUNDS_CHECK (index checks that record an error bit instead of
trapping; loaded when GBDMC_BOUNDS_CHECK=1).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libgbdmc.so")
LIB_BC = os.path.join(OUT_DIR, "libgbdmc_bc.so")
VARIANTS = {"": (OBJ_DIR, LIB, []), "bc": (os.path.join(OUT_DIR, "obj_bc"), LIB_BC, ["-DGBDMC_BOUNDS_CHECK"])}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(cuda, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, variants=("", "bc")):
    """Compile every CUDA source for sm_103a and link the libraries of
    `variants` ("" libgbdmc.so, "bc" libgbdmc_bc.so), all objects in one
    parallel pool; returns the path of libgbdmc.so."""
    nvcc = _nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    jobs = []
    for v in variants:
        obj_dir, _, extra = VARIANTS[v]
        os.makedirs(obj_dir, exist_ok=True)
        for src in _sources():
            obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
            if force or _stale(obj, [src] + headers):
                jobs.append((src, obj, extra))

    def _compile(job):
        src, obj, extra = job
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(_compile, jobs))
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for v in variants:
        obj_dir, lib, _ = VARIANTS[v]
        objs = [os.path.join(obj_dir, os.path.basename(s)[:-3] + ".o") for s in _sources()]
        if force or _stale(lib, objs):
            cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", lib + ".tmp"] + objs + \
                  ["-Xlinker", f"-rpath,{os.path.join(cuda, 'lib64')}"]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
            os.replace(lib + ".tmp", lib)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
