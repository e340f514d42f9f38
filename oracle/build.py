"""Build oracle/_build/liboracle.so with g++ (OpenMP, -O3) -- test infrastructure only."""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build", "liboracle.so")
SOURCES = [os.path.join(HERE, "phmc_oracle.cpp"),
           os.path.join(ROOT, "phonomc_gb300", "csrc", "phmc_host.cpp"),
           os.path.join(ROOT, "phonomc_gb300", "csrc", "phmc_mesh.cpp"),
           os.path.join(ROOT, "phonomc_gb300", "csrc", "phmc_amm.cpp")]
DEPS = SOURCES + [os.path.join(ROOT, "phonomc_gb300", "csrc", f)
                  for f in ("phmc_host.h", "phmc_pod.h", "phmc_rng.h", "phmc_tuning.h")] + [
    os.path.join(ROOT, "include", "phonomc_gb300.h")]
_lock = threading.Lock()
_lib = None


def _stale() -> bool:
    if not os.path.exists(OUT):
        return True
    t = os.path.getmtime(OUT)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force: bool = False) -> str:
    if force or _stale():
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        tmp = OUT + f".{os.getpid()}.tmp"
        subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wno-unknown-pragmas",
                        *SOURCES, "-o", tmp], check=True)
        os.replace(tmp, OUT)
    return OUT


def load():
    global _lib
    with _lock:
        if _lib is None:
            from phonomc_gb300 import abi
            lib = C.CDLL(build())
            abi.bind(lib, "orc_", abi.SOLVER_PROTOS)
            abi.bind(lib, "orc_", abi.SUBSTEP_PROTOS)
            abi.bind(lib, "orc_", abi.ORACLE_EXTRA_PROTOS)
            _lib = lib
    return _lib
