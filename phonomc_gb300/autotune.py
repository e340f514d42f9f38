"""Autotuner of the device carrier loop's launch and scheduling defaults.

Sweeps, on one GPU and one carrier population per workload, the knobs that
change no physics:

  transport_block          threads per CTA of the carrier pass (128, 256, 512)
  transport_blocks_per_sm  resident CTAs per SM of the carrier pass, which sets
                           how many carriers each thread walks
  carrier_sort_interval    steps between stable (mode, cell) carrier sorts
  tally_aggregation        warp-summed bin tallies (1) or one atomic per carrier (-1)
  transport_pipeline       mixed state: carrier tiles staged in shared memory by
                           bulk asynchronous copies (1, 256 threads) or loaded
                           directly (-1)

for the plain FP64 and the mixed-precision carrier state, then the smallest
population at which sorting pays. Each point is timed over whole timesteps
(graph replays, host clock around a synchronised run) starting on a sort step
and covering whole sort intervals, so a sort's cost is counted at its share.
Unsorted points are timed first, on the fresh population, before any sort has
ordered it.

  python -m phonomc_gb300.autotune --out DIR [--particles 5e7] [--quick]

writes DIR/tuning_record.json (every point) and DIR/phmc_tuning.h (the chosen
defaults, the header the library compiles with, csrc/phmc_tuning.h).
"""

from __future__ import annotations

import argparse
import ctypes as C
import itertools
import json
import os
import time

import numpy as np

BLOCKS = (128, 256, 512)
PER_SM = (2, 4, 8, 16)
SORTS = (10, 25, 50, 100, 200)
AGG = (-1, 1)


def _solver(lib, abi, precision, particles, seed=777):
    from . import synthetic, workloads
    m = abi.Material(lib, "phmc_", synthetic.make_material(mesh=16), 0.1, True, False)
    cfg = workloads.scaled(workloads.inplane_gradient(precision=precision), particles, random_seed=seed,
                           carrier_sort_interval=-1)
    return abi.Solver(lib, "phmc_", cfg, [m]), m


def _time_point(lib, s, sort, block, per_sm, agg, min_steps, pipe=-1):
    """Seconds per step of one schedule: two settling steps after the change
    (graph capture), then whole sort intervals from a sort step."""
    s.check(lib.phmc_solver_set_schedule(s.h, sort, block, per_sm, agg, pipe))
    s.run(2)
    if sort > 0:
        cur = s.stats()["current_timestep"]
        s.run((-cur) % sort)
        steps = sort * max(1, -(-min_steps // sort))
    else:
        steps = min_steps
    s.check(lib.phmc_solver_synchronize(s.h))
    t0 = time.perf_counter()
    s.run(steps)
    s.check(lib.phmc_solver_synchronize(s.h))
    return (time.perf_counter() - t0) / steps, steps


def sweep(lib, abi, precision, particles, quick=False, log=print):
    s, _m = _solver(lib, abi, precision, particles)
    n = s.stats()["particle_count"]
    blocks = (256,) if quick else BLOCKS
    per_sm = (4, 8) if quick else PER_SM
    sorts = (25, 100) if quick else SORTS
    points = []

    def rec(sort, b, p, a, min_steps, pipe=-1):
        sec, steps = _time_point(lib, s, sort, b, p, a, min_steps, pipe)
        pt = {"carrier_sort_interval": sort, "transport_block": b, "transport_blocks_per_sm": p,
              "tally_aggregation": a, "transport_pipeline": pipe, "ms_per_step": 1e3 * sec,
              "carrier_steps_per_s": n / sec, "steps": steps}
        points.append(pt)
        log(json.dumps({"precision": precision, **pt}))
    pipes = (-1, 1) if precision == "mixed" else (-1,)
    # unsorted population first: every schedule without sorts
    for pipe in pipes:
        for b, p, a in itertools.product((256,) if pipe > 0 else blocks, per_sm, AGG):
            rec(-1, b, p, a, 30, pipe)
    for pipe in pipes:
        for k, b, p, a in itertools.product(sorts, (256,) if pipe > 0 else blocks, per_sm, AGG):
            rec(k, b, p, a, 60, pipe)
    s.close()
    best = min(points, key=lambda q: q["ms_per_step"])
    return {"precision": precision, "particles": n, "workload": "inplane_gradient", "points": points, "best": best}


def population_threshold(lib, abi, best, precision="mixed", sizes=(2e5, 1e6, 4e6), log=print):
    """Sorted (best schedule) against never sorted at smaller populations."""
    rows = []
    for n in sizes:
        s, _m = _solver(lib, abi, precision, n)
        never, _ = _time_point(lib, s, -1, best["transport_block"], best["transport_blocks_per_sm"],
                               best["tally_aggregation"], 60, best.get("transport_pipeline", -1))
        k = best["carrier_sort_interval"]
        if k <= 0:
            k = 50
        sorted_, _ = _time_point(lib, s, k, best["transport_block"], best["transport_blocks_per_sm"],
                                 best["tally_aggregation"], 100, best.get("transport_pipeline", -1))
        rows.append({"particles": n, "ms_never": 1e3 * never, "ms_sorted": 1e3 * sorted_, "interval": k})
        log(json.dumps(rows[-1]))
        s.close()
    return rows


def mesh_sort_sweep(lib, abi, particles=2e7, sorts=(25, 50, 100, 200), steps=100, log=print):
    """Sort interval of surface-mesh domains: the FinFET with its heat source,
    a fresh population per point (a long FinFET run can lose a carrier through
    its top surface, which ends the run), timed over `steps` steps from a sort step."""
    import tempfile
    from . import synthetic, workloads
    stl = workloads.finfet_stl(os.path.join(tempfile.mkdtemp(prefix="phmc_tune_"), "finfet.stl"))
    rows = []
    for prec in ("mixed", "fp64"):
        for k in sorts:
            m = abi.Material(lib, "phmc_", synthetic.make_material(mesh=16), 0.1, False, False)
            cfg = workloads.finfet_mesh(stl, particles=particles, precision=prec)
            cfg["carrier_sort_interval"] = k
            s = abi.Solver(lib, "phmc_", cfg, [m])
            s.run(3)
            s.run((-s.stats()["current_timestep"]) % k + 1)
            s.check(lib.phmc_solver_synchronize(s.h))
            t0 = time.perf_counter()
            s.run(steps)
            s.check(lib.phmc_solver_synchronize(s.h))
            rows.append({"precision": prec, "carrier_sort_interval": k,
                         "ms_per_step": 1e3 * (time.perf_counter() - t0) / steps})
            log(json.dumps(rows[-1]))
            s.close()
            m.close()
    return rows


HEADER = """// Launch and scheduling defaults of the device carrier loop, chosen by
// phonomc_gb300/autotune.py from timed sweeps on a GB300 (the sweep record it
// writes sits beside it, phonomc_gb300/tuning_record.json). A configuration
// field of 0 selects these values; none of them changes the physics.
// Index [0] is the plain FP64 carrier state, [1] the mixed-precision one.
#pragma once

namespace phmc {{
namespace tuning {{
// Threads per CTA of the carrier pass (128, 256 or 512).
constexpr int kTransportBlock[2] = {{{b0}, {b1}}};
// Resident CTAs per SM of the carrier pass (grid = SMs x this, fewer for
// small populations): sets the carriers each thread walks.
constexpr int kTransportBlocksPerSm[2] = {{{p0}, {p1}}};
// Steps between carrier sorts by (mode, cell), or by (cell, mode) in mesh
// domains (0: never), and the smallest population that is sorted at all.
constexpr int kSortInterval[2] = {{{k0}, {k1}}};
constexpr double kSortMinCarriers = {nmin:.6g};
// The same for surface-mesh domains (FinFET sweep of the record's "mesh_sorts").
constexpr int kSortIntervalMesh[2] = {{{m0}, {m1}}};
// Bin tallies of the carrier pass: 1 sums runs of equal (cell, bin) across
// the lanes of a warp before one FP64 atomic per run, 0 one atomic per carrier.
constexpr int kTallyAggregation[2] = {{{a0}, {a1}}};
// Mixed carrier pass: carrier tiles staged in shared memory by bulk
// asynchronous copies one tile ahead (1), or loaded directly (0).
constexpr int kTransportPipeline = {pipe};
}} // namespace tuning
}} // namespace phmc
"""


def write_outputs(out, record):
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(out, "tuning_record.json"), "w") as f:
        json.dump(record, f, indent=1)
    b = {r["precision"]: r["best"] for r in record["sweeps"]}
    thr = record.get("threshold", [])
    # sorting counts as a win only when it is at least 1% faster (timing noise)
    wins = [r["particles"] for r in thr if r["ms_sorted"] < 0.99 * r["ms_never"]]
    nmin = min(wins) if wins else 2e6

    def val(prec, key, default):
        v = b.get(prec, {}).get(key, default)
        return default if v is None else v

    def sort_of(prec):
        k = val(prec, "carrier_sort_interval", 50)
        return max(0, k)

    def mesh_sort_of(prec):
        rows = [r for r in record.get("mesh_sorts", []) if r["precision"] == prec]
        return min(rows, key=lambda r: r["ms_per_step"])["carrier_sort_interval"] if rows else 25

    text = HEADER.format(b0=val("fp64", "transport_block", 256), b1=val("mixed", "transport_block", 256),
                         p0=val("fp64", "transport_blocks_per_sm", 8), p1=val("mixed", "transport_blocks_per_sm", 8),
                         k0=sort_of("fp64"), k1=sort_of("mixed"), nmin=float(nmin),
                         m0=mesh_sort_of("fp64"), m1=mesh_sort_of("mixed"),
                         a0=max(0, val("fp64", "tally_aggregation", 1)), a1=max(0, val("mixed", "tally_aggregation", 1)),
                         pipe=max(0, val("mixed", "transport_pipeline", 1)))
    with open(os.path.join(out, "phmc_tuning.h"), "w") as f:
        f.write(text)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--particles", type=float, default=5e7)
    ap.add_argument("--precisions", nargs="*", default=["mixed", "fp64"])
    ap.add_argument("--quick", action="store_true", help="a reduced grid (smoke of the tuner itself)")
    ap.add_argument("--mesh", action="store_true", help="also sweep the sort interval of mesh domains (FinFET)")
    args = ap.parse_args()
    from . import abi
    from . import lib as load
    lib = load()
    record = {"workload": "inplane_gradient film (rough walls, G = 1e7 K/m, 100 z-cells, linearized RTA)",
              "timing": "host clock around synchronised graph-replayed steps, whole sort intervals from a sort step",
              "sweeps": []}
    log_path = os.path.join(args.out, "tuning_log.jsonl")
    os.makedirs(args.out, exist_ok=True)
    with open(log_path, "w") as logf:
        def log(line):
            print(line, flush=True)
            logf.write(line + "\n")
            logf.flush()
        for prec in args.precisions:
            record["sweeps"].append(sweep(lib, abi, prec, args.particles, args.quick, log))
        mixed = [r for r in record["sweeps"] if r["precision"] == "mixed"]
        if mixed:
            record["threshold"] = population_threshold(lib, abi, mixed[0]["best"], log=log)
        if args.mesh:
            record["mesh_sorts"] = mesh_sort_sweep(lib, abi, log=log)
    try:
        import subprocess
        record["gpu"] = subprocess.run(["nvidia-smi", "--query-gpu=name,clocks.max.sm", "--format=csv,noheader"],
                                       capture_output=True, text=True).stdout.strip()
    except Exception:
        pass
    write_outputs(args.out, record)
    print(json.dumps({r["precision"]: r["best"] for r in record["sweeps"]}))


if __name__ == "__main__":
    main()
