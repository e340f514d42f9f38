"""GB300-native PhonoMC carrier loop: CUDA kernels behind a C ABI.

The compute path is libphonomc_gb300.so (phonomc_gb300/csrc, built by
`phonomc_gb300.native.build()`); `phonomc_gb300.lib()` loads it and fails
loudly when it is missing. `synthetic` makes the seeded phonon tables and
`workloads` the named configurations.
"""
from .native import lib, build  # noqa: F401
