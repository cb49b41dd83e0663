"""In-tree build of libgfcuda.so for sm_103a (nvcc, translation units compiled in parallel).

    python geophysicalflows.jl_gb300/gfcuda/build.py [--force]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libgfcuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++20", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", f"-I{INCLUDE}", f"-I{CSRC}"]


def units():
    """Translation units: the ABI, the dispatch layer and one unit per (precision, FFT length)."""
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "gfcuda.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=True, defines=(), lib=None):
    lib = lib or LIB
    if not force and lib == LIB and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_unit(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *FLAGS, *[f"-D{d}" for d in defines], "-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        return obj

    us = units()
    # largest kernels first so the slowest units start early
    us.sort(key=lambda u: (("df64" not in u) + ("f64" not in u), -int(u.rsplit("_", 1)[-1][:-3]) if u.startswith("gf_k_") else 0))
    with cf.ThreadPoolExecutor(max_workers=max(1, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_unit, us))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    # python build.py [--force] [-DNAME=VALUE ...] [--out PATH]
    defs = [a[2:] for a in sys.argv[1:] if a.startswith("-D")]
    out = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else None
    build(force="--force" in sys.argv or bool(defs) or out is not None, defines=defs, lib=out)
