"""phmc_dev_trace_box_noalloc against phmc_dev_trace_box (GPU).

The file name keeps this module last in collection order, so it also runs
after every other test in the same process; each test below passes alone as
well. Two calls in a row check that the static scratch (rays and the miss
counter) carries nothing from one call into the next."""

import ctypes as C

import numpy as np
import pytest

from phonomc_gb300 import abi

pytestmark = pytest.mark.gpu

MAX_RAYS = 65536


@pytest.fixture(scope="module")
def gpu():
    import phonomc_gb300
    lib = phonomc_gb300.lib()
    n = C.c_int32()
    assert lib.phmc_device_count(C.byref(n)) == 0 and n.value > 0, "no CUDA device"
    return lib


def _rays(n, seed, lo, hi, miss_fraction):
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    p = lo + rng.random((n, 3)) * (hi - lo)
    v = rng.normal(size=(n, 3)) * 5.0
    # some rays start outside the box moving away from it: no facet
    k = int(miss_fraction * n)
    p[:k, 0] = hi[0] + 10.0 + rng.random(k)
    v[:k, 0] = np.abs(v[:k, 0]) + 1.0
    return np.ascontiguousarray(p), np.ascontiguousarray(v)


def _reference_call(gpu, lo, hi, p, v):
    n = p.shape[0]
    hit, t, f = np.zeros((n, 3)), np.zeros(n), np.zeros(n, np.int32)
    D = abi.dptr
    assert gpu.phmc_dev_trace_box(D(np.asarray(lo, float)), D(np.asarray(hi, float)), n, D(p), D(v), D(hit), D(t),
                                  f.ctypes.data_as(abi.c_int32_p)) == 0, gpu.phmc_last_error()
    return hit, t, f


def _noalloc_call(gpu, lo, hi, p, v):
    n = p.shape[0]
    hit, t, f = np.zeros((n, 3)), np.zeros(n), np.zeros(n, np.int32)
    misses = C.c_int64(-1)
    D = abi.dptr
    rc = gpu.phmc_dev_trace_box_noalloc(D(np.asarray(lo, float)), D(np.asarray(hi, float)), n, D(p), D(v), D(hit),
                                        D(t), f.ctypes.data_as(abi.c_int32_p), C.byref(misses))
    assert rc == 0, gpu.phmc_last_error()
    return hit, t, f, misses.value


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    cases = [((0.0, 0.0, 0.0), (1000.0, 800.0, 600.0), 40000, 11, 0.05),
             ((-50.0, 10.0, 0.0), (250.0, 90.0, 1200.0), MAX_RAYS, 12, 0.0)]
    for lo, hi, n, seed, miss in cases:
        p, v = _rays(n, seed, lo, hi, miss)
        h0, t0, f0 = _reference_call(gpu, lo, hi, p, v)
        h1, t1, f1, m1 = _noalloc_call(gpu, lo, hi, p, v)
        assert np.array_equal(f0, f1)
        assert np.array_equal(h0, h1)
        assert np.array_equal(t0, t1, equal_nan=True)
        assert m1 == int(np.count_nonzero(f0 < 0))
        if miss:
            assert m1 >= int(miss * n)


def test_noalloc_rejects_oversized_and_sets_up_with_zero(gpu):
    lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    misses = C.c_int64(-1)
    D = abi.dptr
    assert gpu.phmc_dev_trace_box_noalloc(D(np.asarray(lo)), D(np.asarray(hi)), 0, None, None, None, None, None,
                                          C.byref(misses)) == 0
    assert misses.value == 0
    big = MAX_RAYS + 1
    p = np.zeros((big, 3))
    out = np.zeros((big, 3))
    t = np.zeros(big)
    f = np.zeros(big, np.int32)
    rc = gpu.phmc_dev_trace_box_noalloc(D(np.asarray(lo)), D(np.asarray(hi)), big, D(p), D(p), D(out), D(t),
                                        f.ctypes.data_as(abi.c_int32_p), C.byref(misses))
    assert rc == 1
    assert b"outside" in gpu.phmc_last_error()
    # the entry point still works after a rejection
    p1, v1 = _rays(1000, 3, lo, hi, 0.1)
    h0, t0, f0 = _reference_call(gpu, lo, hi, p1, v1)
    h1, t1, f1, m1 = _noalloc_call(gpu, lo, hi, p1, v1)
    assert np.array_equal(f0, f1) and np.array_equal(h0, h1)
    assert m1 == int(np.count_nonzero(f0 < 0))


def test_noalloc_full_call_takes_no_device_memory(gpu):
    """After the setup call, a full 65,536-ray call leaves the device's free
    memory unchanged (cudaMemGetInfo through torch); a first full call may
    still see the driver size the kernel's launch resources, so the memory is
    read around a second one."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    lo, hi = (0.0, 0.0, 0.0), (500.0, 400.0, 300.0)
    D = abi.dptr
    misses = C.c_int64(-1)
    assert gpu.phmc_dev_trace_box_noalloc(D(np.asarray(lo)), D(np.asarray(hi)), 0, None, None, None, None, None,
                                          C.byref(misses)) == 0
    p, v = _rays(MAX_RAYS, 21, lo, hi, 0.01)
    _noalloc_call(gpu, lo, hi, p, v)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _noalloc_call(gpu, lo, hi, p, v)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
