"""The C-ABI library builds for sm_103a, loads without a GPU and exports
every entry point that include/phonomc_gb300.h declares."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "phonomc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(phmc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header():
    from phonomc_gb300 import native
    path = native.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_error_without_device_is_loud():
    """On a machine without a GPU the solver refuses to run instead of falling back."""
    import phonomc_gb300
    from phonomc_gb300 import abi, synthetic, workloads
    lib = phonomc_gb300.lib()
    n = ctypes.c_int32()
    assert lib.phmc_device_count(ctypes.byref(n)) == 0
    if n.value > 0:
        return
    m = abi.Material(lib, "phmc_", synthetic.make_material(mesh=8), 0.1, False, False)
    try:
        abi.Solver(lib, "phmc_", workloads.scaled(workloads.cross_plane_film(), 1000), [m])
    except abi.LibError as e:
        assert "CUDA device" in str(e)
    else:
        raise AssertionError("solver creation must fail without a CUDA device")
