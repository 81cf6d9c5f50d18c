"""Build the native CUDA library ``libskfem_gb300.so`` for sm_103a (GB300).

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, then
linked into one shared library inside the Python package
(``skfemntv_gb300/_lib``), where ``skfemntv_gb300._native`` loads it.

    python scikit-fem-native_gb300/build_native.py [-v]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "skfemntv_gb300", "_lib")
LIB = os.path.join(LIBDIR, "libskfem_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# Translation units that must reproduce the reference's rounding exactly.
NO_CONTRACT = {"skg_geometry.cu": ["-fmad=false"]}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE)]
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(OBJ, src[:-3] + ".o")
        objs.append(obj)
        path = os.path.join(CSRC, src)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc(), *ARCH, *COMMON, *NO_CONTRACT.get(src, []), "-c", path, "-o", obj]
            jobs.append((src, cmd))

    def run(job):
        src, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        out = subprocess.run(cmd, capture_output=True, text=True)
        return src, out

    failures = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for src, out in ex.map(run, jobs):
                if out.returncode != 0:
                    failures.append(f"--- {src}\n{out.stdout}{out.stderr}")
                elif verbose and (out.stdout or out.stderr):
                    print(out.stdout + out.stderr)
    if failures:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failures))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed:\n" + out.stdout + out.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
