"""Arithmetic that the device kernels rely on, restated on the CPU.

* The two-level diffuse search of a rough table (rough_sample_dev,
  phonomc_gb300/csrc/phmc_device.cuh): a binary search over every 64th entry
  of the residual prefix narrows the window to one block before the search
  within it. For a non-decreasing prefix it must return the one-level upper
  bound over prefix[b+1 .. e] for every window and target, including targets
  on repeated values and windows shorter than a block.
* The third-order expansion of a Bose occupation in 1/T that the fused RTA
  cell update (rta_model_n, phonomc_gb300/csrc/phmc_cells.cu) uses for points
  within 1e-5 T0 of its last full evaluation: it must agree with
  1 / (exp(x) - 1) to about 1e-16 relative there, well inside the 1e-13
  stopping test of the pseudo-temperature iteration.
"""
import bisect

import numpy as np
import pytest


def two_level_upper_bound(prefix, coarse, b, e, target):
    """The device's search, integer arithmetic as written in the kernel."""
    lo, hi = b + 1, e + 1
    klo, khi = (lo + 63) >> 6, (hi - 1) >> 6
    a, z = klo, khi + 1
    while a < z:
        mid = (a + z) >> 1
        if coarse[mid] <= target:
            a = mid + 1
        else:
            z = mid
    if a > klo:
        lo = max(lo, ((a - 1) << 6) + 1)
    if a <= khi:
        hi = min(hi, a << 6)
    while lo < hi:
        mid = (lo + hi) >> 1
        if prefix[mid] <= target:
            lo = mid + 1
        else:
            hi = mid
    return lo


def test_two_level_search_equals_upper_bound():
    rng = np.random.default_rng(11)
    for trial in range(300):
        n = int(rng.integers(1, 3000))
        steps = rng.exponential(1.0, n)
        steps[rng.random(n) < 0.3] = 0.0  # repeated values
        prefix = np.concatenate([[0.0], np.cumsum(steps)])
        coarse = prefix[::64]
        for _ in range(20):
            b = int(rng.integers(0, n))
            e = int(rng.integers(b + 1, n + 1))
            fb, fe = prefix[b], prefix[e]
            u = rng.random() if rng.random() < 0.8 else float(rng.choice([0.0, 0.99999999999999989]))
            target = fb + u * (fe - fb)
            if rng.random() < 0.1:
                target = prefix[int(rng.integers(b, e + 1))]  # exactly on an entry
            want = bisect.bisect_right(prefix, target, b + 1, e + 1)
            assert two_level_upper_bound(prefix, coarse, b, e, target) == want


def test_bose_expansion_in_inverse_temperature():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    kb = 8.617333262145e-5
    for x0 in (1e-3, 0.03, 0.3, 1.0, 3.0, 10.0, 30.0, 40.0):
        T0 = 300.0
        hw = x0 * kb * T0
        p0 = 1.0 / (np.exp(x0) - 1.0)
        q = p0 * (p0 + 1.0)
        r2, r3 = q * (2.0 * p0 + 1.0), q * (6.0 * q + 1.0)
        for d in (1e-5, -1e-5, 3e-6, -1e-7):
            T = T0 * (1.0 + d)
            du = (T0 - T) / (T * T0 * kb)
            y = hw * du
            p = p0 + y * (-q + y * (0.5 * r2 - y * (r3 * (1.0 / 6.0))))
            # against the same formula's value at T0 moved exactly to T: the
            # expansion's own error, apart from the rounding p0 carries
            exact = p0 * mpmath.mpf(1) / (mpmath.e ** (mpmath.mpf(x0) * (T0 / mpmath.mpf(T) - 1)) * (1 + p0) - p0)
            assert abs(float((mpmath.mpf(p) - exact) / exact)) < 2e-15, (x0, d)
