"""CPU oracle of the carrier loop -- test infrastructure only.

`load()` builds (if needed) and loads oracle/_build/liboracle.so, the serial
FP64 restatement of the reference algorithm in phmc_oracle.cpp. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it.
"""
from .build import load, build  # noqa: F401
