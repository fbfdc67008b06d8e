"""In-tree build of the CUDA library (liblsm_gb300.so) for sm_103a.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library with a plain C ABI (include/lsm_c.h); PyTorch is not linked.
The FP64 translation units that restate the reference arithmetic are built
with --fmad=false so every multiply and add is rounded separately (and the
geometric reinitialisation's host-side Newton solve with the host compiler's
-ffp-contract=off, which matters on Arm hosts, where contraction is the
default).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)                 # ns-lsm-single-phase_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_NAME = "liblsm_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]

# translation unit -> extra flags
UNITS = {
    "lsm_runtime.cu": ["-Xcompiler", "-fvisibility=default"],
    "lsm_fp64.cu": ["--fmad=false"],
    "lsm_volume.cu": ["--fmad=false"],
    "lsm_sussman.cu": ["--fmad=false"],
    "lsm_geometric.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "lsm_capi.cu": ["-Xcompiler", "-fvisibility=default"],
    "lsm_batch.cu": ["--fmad=true"],
    "lsm_batch_capi.cu": ["-Xcompiler", "-fvisibility=default"],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblsm_gb300.so")
    return exe


def _sources():
    return [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link liblsm_gb300.so (skipped when up to date); return its path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    exe = nvcc()

    def compile_one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(obj_dir, unit.replace(".cu", ".o"))
        cmd = [exe] + ARCH + COMMON + UNITS[unit] + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, r.stdout + r.stderr

    units = _sources()
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(compile_one, units))
    if verbose or ptxas_info:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    tmp = LIB_PATH + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
        "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
