"""Regenerate the golden fixtures in this folder from the reference solver.

Run in a container that has the reference sources (it builds them first):

    python tests/golden/make_golden.py [--ref /root/reference]

Steps: build ``oracle/_ref`` with ``oracle/ref/Makefile`` (the reference's own
C++ compiled unchanged, HDF5 readers stubbed), write the seeded synthetic
material tables (8^3 q mesh; the full-size workloads use 16^3) and run
``oracle/_ref/ref_harness`` for every deterministic sub-step. Outputs are
gzipped JSON; each records its inputs beside the reference's outputs.
"""

from __future__ import annotations

import argparse
import gzip
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from phonomc_gb300 import synthetic  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# name -> harness arguments ("{m}" = plain 8^3 table, "{c}" = Callaway table)
CASES = {
    "material_m8": ["material", "{m}", "0"],
    "material_m8_stationary": ["material", "{m}", "1"],
    "box_trace": ["box"],
    "rta_fixed": ["rta", "{m}", "0"],
    "rta_local": ["rta", "{m}", "1"],
    "linearized_rta": ["lincoll", "{m}"],
    "callaway_evolve": ["callaway"],
    "rough_nonconservative": ["rough", "{m}", "0"],
    "rough_conservative": ["rough", "{m}", "1"],
    "gradient_drive": ["gradient", "{m}"],
    "reservoir": ["reservoir", "{m}"],
}


def build(ref: str) -> None:
    subprocess.run(["make", "-s", "-j8", f"REF={ref}"], cwd=os.path.join(ROOT, "oracle", "ref"),
                   check=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    build(args.ref)
    tmp = os.path.join(ROOT, "oracle", "_ref")
    mpath = os.path.join(tmp, "m8.pmat")
    cpath = os.path.join(tmp, "m8c.pmat")
    synthetic.write_pmat(mpath, synthetic.make_material(mesh=8))
    synthetic.write_pmat(cpath, synthetic.make_material(mesh=8, callaway=True))
    for name, argv in CASES.items():
        if args.only and name not in args.only:
            continue
        cmd = [HARNESS] + [a.format(m=mpath, c=cpath) for a in argv]
        out = subprocess.run(cmd, check=True, capture_output=True, text=True).stdout
        data = json.loads(out)
        data["_harness_args"] = argv
        with gzip.open(os.path.join(HERE, name + ".json.gz"), "wt") as f:
            json.dump(data, f)
        print(name, "ok")


if __name__ == "__main__":
    main()
