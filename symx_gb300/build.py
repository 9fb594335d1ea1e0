"""Build symx_gb300/_build/libsymxg.so from csrc/ (in-tree, incremental, parallel).

C++ host sources are compiled with g++, CUDA sources with nvcc for sm_103a only; the
shared library links the CUDA runtime statically and NVRTC dynamically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsymxg.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _sources():
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    return cpp, cu


def _headers_mtime() -> float:
    m = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")) or f == "symx":
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + CSRC, "-I" + INCLUDE]
    os.makedirs(BUILD, exist_ok=True)
    cpp, cu = _sources()
    hdr = _headers_mtime()
    jobs_list = []
    objs = []
    for f in cpp + cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        stale = force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr)
        if not stale:
            continue
        if f.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *inc, "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function", *inc, "-c", src, "-o", obj]
        jobs_list.append(cmd)
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs_list):
                if verbose and out.strip():
                    print(out)
    if force or jobs_list or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        lib64 = os.path.join(cuda, "lib64")
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-L" + lib64, "-lnvrtc", "-Xlinker", "-rpath=" + lib64,
              "-Xlinker", "--no-undefined"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
