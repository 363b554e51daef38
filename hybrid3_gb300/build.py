"""Build libhybrid3_gb300.so in-tree: every CUDA source for sm_103a (one
-gencode, so the tcgen05/TMA forms are available), host C sources with gcc,
compiled in parallel and linked into one shared library whose exported
symbols are the C ABI declared in include/.

    python -m hybrid3_gb300.build          # or hybrid3_gb300.build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libhybrid3_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr",
                     "-I", INCLUDE, "-I", CSRC]
CC_FLAGS = ["-O2", "-fPIC", "-std=c11", "-fvisibility=default", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    return cu, c


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    cu, c = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers) or ptxas_info:
            flags = NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else [])
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    for f in c:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if jobs or not os.path.exists(LIB):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"])
    text = "".join(logs)
    if verbose and text:
        print(text)
    return text


if __name__ == "__main__":
    out = build(verbose=True, ptxas_info="-v" in sys.argv)
    print("built", LIB)
