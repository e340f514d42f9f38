"""CPU oracle of the carrier loop -- test infrastructure only.

`load()` builds (if needed) and loads oracle/_build/liboracle.so, the serial
FP64 restatement of the reference algorithm in phmc_oracle.cpp. Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it.
"""
from .build import load, build  # noqa: F401


def reference_root():
    """The reference checkout the tests compare with: $PHONOMC_REFERENCE, else
    the one oracle/_ref was last built from (recorded by the build), else None."""
    import os
    env = os.environ.get("PHONOMC_REFERENCE")
    if env:
        return env
    rec = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "REFERENCE")
    if os.path.exists(rec):
        with open(rec) as f:
            path = f.read().strip()
        return path or None
    return None
