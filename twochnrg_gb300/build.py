"""In-tree build of the GB300 engine library (sm_103a only).

Compiles every translation unit of ``csrc/`` in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` and links
``twochnrg_gb300/_build/libtwochnrg_gb300.so``.  No cmake, no setuptools.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtwochnrg_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["engine.cu", "k_assemble.cu", "k_tridiag.cu", "k_tdeig.cu", "k_cut.cu", "k_update.cu",
              "k_dm.cu", "k_ozaki.cu", "k_panel.cu", "k_tangent.cu", "noalloc.cu"]
CXX_SOURCES = ["nrg_model.cpp", "binfile.cpp", "thermofile.cpp", "chain.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "twochnrg_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES + CXX_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if not force and not _newer(obj, [path] + headers):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-c", path, "-o", obj]
        else:
            cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "c++", "-c", path, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
        if verbose and (p.stdout or p.stderr):
            sys.stderr.write(p.stdout + p.stderr)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _newer(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
