"""Builds the in-tree CUDA library pdds_gb300/_build/libpdds_gb300.so for sm_103a.

Each translation unit is compiled in parallel with nvcc (one -gencode,
compute_103a/sm_103a); the replay kernels are compiled with -fmad=false so
their FP64 arithmetic rounds exactly like the host restatement.  Host C++
(layout) is compiled by nvcc's host compiler with FMA contraction off.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpdds_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
            "-ffp-contract=off", "--expt-relaxed-constexpr"]
UNITS = {
    "capi.cu": [],
    "k_mixed.cu": [],
    "k_fp64.cu": [],
    "k_replay.cu": ["-fmad=false"],
    "k_rbf.cu": [],
    "k_misc.cu": ["-fmad=false"],
    "k_solve.cu": [],
    "k_gmres_cluster.cu": [],
    "batch.cu": [],
    "k_subdomain.cu": [],
    "layout.cpp": ["-x", "cu"],
    "layout_circle.cpp": ["-x", "cu"],
    "noalloc.cu": [],
    "selfcheck.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


OUT_DIR_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(OUT_DIR_CHECKED, "libpdds_gb300.so")


def build(force: bool = False, verbose: bool = False, extra=None, checked: bool = False) -> str:
    """Compiles the library (pdds_gb300/_build) and returns its path.
    checked=True builds the index-checked library instead
    (pdds_gb300/_build_checked, -DPDDS_CHECKED): every checked device index
    that falls outside its array sets an error flag, the access is skipped
    and the call returns PDDS_ERR_BOUNDS; for debugging and tests, slower."""
    out_dir, lib = (OUT_DIR_CHECKED, LIB_CHECKED) if checked else (OUT_DIR, LIB)
    if checked:
        extra = list(extra or []) + ["-DPDDS_CHECKED"]
    os.makedirs(out_dir, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "pdds.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = os.path.join(SRC, unit)
        obj = os.path.join(out_dir, unit + ".o")
        objs.append(obj)
        if not force and _newer(obj, [src] + headers):
            continue
        cmd = [cc] + ARCH + CU_FLAGS + flags + (extra or []) + ["-c", src, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, os.cpu_count() or 1))) as ex:
        for cmd, res in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
            if verbose or res.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + res.stdout + res.stderr)
            if res.returncode != 0:
                raise RuntimeError("nvcc failed for " + cmd[-3])
    if force or jobs or not _newer(lib, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
            raise RuntimeError("link failed")
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
