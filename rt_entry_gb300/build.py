"""Build librtentry.so in-tree (rt_entry_gb300/_build/) for sm_103a.

Every .cu file is compiled by nvcc for ``-gencode arch=compute_103a,code=sm_103a``
and every .cpp by g++ with ``-ffp-contract=off`` (the kd-tree's float
arithmetic must round exactly as the reference's x86-64 host build does),
in parallel; the library links the CUDA runtime statically so that it does
not depend on which libcudart the host process already loaded.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librtentry.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc") if os.path.exists(os.path.join(CUDA, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler",
                     "-fPIC,-fopenmp,-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}",
                     f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
             f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}", f"-I{os.path.join(CUDA, 'include')}"]


def _headers():
    return [p for ext in ("*.h", "*.cuh", "*.inc") for p in glob.glob(os.path.join(CSRC, ext))] + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _stale(obj, src, hdr_mtime):
    if not os.path.exists(obj):
        return True
    m = os.path.getmtime(obj)
    return os.path.getmtime(src) > m or hdr_mtime > m


def _compile(job):
    cmd, src = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {os.path.basename(src)}\n{r.stdout}\n{r.stderr}")
    return src


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu"))) + sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    objs, todo = [], []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, s, hdr_mtime):
            if s.endswith(".cu"):
                cmd = [NVCC] + NVCC_FLAGS + ["-c", s, "-o", o]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-c", s, "-o", o]
            todo.append((cmd, s))
    # largest instantiation files first so the pool stays busy
    todo.sort(key=lambda j: -os.path.getsize(j[1]) if "search_c" not in j[1] else -10**9)
    if todo:
        n = jobs or min(len(todo), max(2, os.cpu_count() or 2))
        with ThreadPoolExecutor(n) as ex:
            for src in ex.map(_compile, todo):
                if verbose:
                    print("compiled", os.path.basename(src), flush=True)
    if todo or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = ["g++", "-shared", "-o", tmp] + objs + [
            f"-L{os.path.join(CUDA, 'lib64')}", "-lcudart_static", "-ldl", "-lrt", "-lpthread",
            "-fopenmp", "-Wl,--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        shutil.move(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
    sys.exit(0)
