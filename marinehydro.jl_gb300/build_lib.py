"""Build libmarinehydro_cuda.so in-tree for sm_103a (GB300).

Each CUDA translation unit under ``csrc/`` is compiled by its own ``nvcc`` process
(in parallel) with ``-gencode arch=compute_103a,code=sm_103a``, then linked into
``_build/libmarinehydro_cuda.so``.  Object files are reused when their source
and headers are older than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libmarinehydro_cuda.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)
HEADER = os.path.join(REPO_DIR, "include", "marinehydro_gb300.h")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmarinehydro_cuda.so")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [HEADER]


def _compile(nvcc: str, src: str, obj: str, verbose_ptxas: bool) -> tuple[str, str]:
    cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return src, r.stderr


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compile every csrc/*.cu for sm_103a and link the shared library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    newest_header = max(os.path.getmtime(h) for h in _headers())
    todo = []
    objs = []
    for s in srcs:
        obj = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(s), newest_header):
            todo.append((s, obj))
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for src, log in ex.map(lambda t: _compile(nvcc, t[0], t[1], verbose_ptxas), todo):
                logs[src] = log
    if todo or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    if verbose_ptxas:
        for src, log in logs.items():
            print(f"== {os.path.basename(src)}\n{log}")
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
