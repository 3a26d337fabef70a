"""In-tree build of the pricer's native code (no cmake, no setuptools).

Outputs, all under diku.optionspricing_gb300/_build/:
  libhwtree.so   C-ABI shared library (include/hwtree.h), sm_103a kernels
  hwt-price      CLI with the reference's flags (-o -y -v -b -s -r -d -t)
  hwt-compare    Compare harness: two [..] arrays on stdin

Each CUDA translation unit is compiled in parallel with one -gencode
(compute_103a -> sm_103a) and -lineinfo; the host tools link the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC]
CU_SOURCES = ["hwt_batched.cu", "hwt_plain.cu", "hwt_api.cu", "hwt_noalloc.cu", "hwt_surrogate.cu"]
HOST_SOURCES = ["hwt_io.cpp"]  # host-only code of the library (g++)
TOOLS = {"hwt-price": "tools/price_main.cpp", "hwt-compare": "tools/compare_main.cpp"}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build the pricer")
    return path


def _run(cmd):
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    return proc.stdout + proc.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Builds libhwtree.so and the CLI tools; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "hwtree.h"))
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([cc] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cpp", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    lib = os.path.join(OUT, "libhwtree.so")
    if jobs or not os.path.exists(lib):
        _run([cc] + ARCH + ["-shared", "-o", lib] + objs + ["-Xcompiler", "-pthread"])
    tool_jobs = []
    for name, src in TOOLS.items():
        s = os.path.join(CSRC, src)
        exe = os.path.join(OUT, name)
        if _stale(exe, [s, lib, os.path.join(INCLUDE, "hwtree.hpp"), os.path.join(INCLUDE, "hwtree.h")]):
            tool_jobs.append(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, s, "-o", exe, "-L" + OUT,
                              "-lhwtree", "-Wl,-rpath,$ORIGIN"])
    for j in tool_jobs:
        _run(j)
    if verbose or ptxas_info:
        for log in logs:
            sys.stdout.write(log)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
