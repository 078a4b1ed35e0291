"""Builds libolcao_gb300.so (sm_103a) in-tree with nvcc.

Every translation unit is compiled in parallel into olcao_gb300/_build/ and
linked against cuBLAS/cuSOLVER into olcao_gb300/libolcao_gb300.so.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from typing import List

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libolcao_gb300.so")
SOURCES = ["olc_capi.cpp", "olc_setup.cpp", "olc_integrals.cu", "olc_integrals_f_overlap.cu",
           "olc_integrals_f_kinetic.cu", "olc_integrals_f_massvel.cu", "olc_integrals_f_nuclear.cu", "olc_integrals_f_nuclear_batch.cu",
           "olc_integrals_f_elecpot.cu", "olc_linalg.cu",
           "olc_eigen_small.cu", "olc_noalloc.cu", "olc_mixed.cu", "olc_tridiag.cu",
           "olc_ozaki.cu", "olc_tcgemm.cu", "olc_layout.cu", "olc_density.cu", "olc_populate.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build")
    return cand


def _flags() -> List[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                   "-I", CSRC]


def _stale(obj: str, deps: List[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra: List[str] = ()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "olcao_gpu.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if _stale(obj, [path] + headers):
            cmd = [cc] + _flags() + list(extra) + ["-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [cc, "-x", "cu"] + cmd[1:]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(16, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcublas", "-lcusolver"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link of libolcao_gb300.so failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
