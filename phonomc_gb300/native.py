"""Build and load libphonomc_gb300.so (CUDA kernels for sm_103a + C ABI).

`build()` compiles the translation units in csrc/ in parallel (host C++ with
g++, CUDA with nvcc -gencode arch=compute_103a,code=sm_103a), links them with
the static CUDA runtime and writes phonomc_gb300/_build/libphonomc_gb300.so.
`lib()` loads that file; there is no fallback when it is absent.
"""

from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(BUILD, "libphonomc_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXX_SOURCES = ["phmc_host.cpp", "phmc_mesh.cpp", "phmc_output.cpp", "phmc_hdf5.cpp", "phmc_amm.cpp"]
CU_SOURCES = ["phmc_transport.cu", "phmc_cells.cu", "phmc_solver.cu", "phmc_capi.cu", "phmc_noalloc.cu", "phmc_sort.cu", "phmc_rough.cu"]
HEADERS = ["phmc_host.h", "phmc_pod.h", "phmc_rng.h", "phmc_device.cuh", "phmc_solver.h", "phmc_kernels.cuh", "phmc_tuning.h", "phmc_sort.cuh", "phmc_hdf5.h"]

_lock = threading.Lock()
_lib = None


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libphonomc_gb300.so")


def _deps():
    return ([os.path.join(CSRC, f) for f in CXX_SOURCES + CU_SOURCES + HEADERS] +
            [os.path.join(ROOT, "include", "phonomc_gb300.h")])


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in _deps())


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    with _lock:
        if not (force or _stale()):
            return OUT
        os.makedirs(BUILD, exist_ok=True)
        inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
        jobs = []
        objs = []
        for src in CXX_SOURCES:
            obj = os.path.join(BUILD, src + ".o")
            objs.append(obj)
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wno-unknown-pragmas", *inc, "-c",
                         os.path.join(CSRC, src), "-o", obj])
        for src in CU_SOURCES:
            obj = os.path.join(BUILD, src + ".o")
            objs.append(obj)
            jobs.append([nvcc(), ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--use_fast_math",
                         "-fmad=true", "-Xptxas", "-v" if verbose else "-O3", *inc, "-c",
                         os.path.join(CSRC, src), "-o", obj])
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            logs = list(ex.map(_compile, jobs))
        if verbose:
            for log in logs:
                print(log)
        tmp = OUT + f".{os.getpid()}.tmp"
        subprocess.run([nvcc(), ARCH, "-shared", "-cudart", "static", *objs, "-Xcompiler", "-fopenmp", "-o", tmp],
                       check=True)
        os.replace(tmp, OUT)
        return OUT


def lib() -> C.CDLL:
    """Load the CUDA library (building it first if sources are newer)."""
    global _lib
    if _lib is None:
        path = build()
        from . import abi
        L = C.CDLL(path)
        abi.bind(L, "phmc_", abi.SOLVER_PROTOS)
        abi.bind(L, "phmc_", abi.DEVICE_PROTOS)
        abi.bind(L, "phmc_", abi.DOMAIN_PROTOS)
        _lib = L
    return _lib
