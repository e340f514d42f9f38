"""Throughput of the PhonoMC carrier loop on one GB300: carrier-steps/s.

Default workload: in-plane periodic-gradient film (100 nm thick, rough 1 nm
walls, G = 1e7 K/m, 100 z-cells, linearized RTA at 300 K, dt = 0.5 ps) with
5e7 carriers on the seeded synthetic 16^3 x 6 phonon table. A step is one
MonteCarloSolver timestep over every carrier. Carrier state (>= 2 GB) is far
larger than the 129 MB L2, so timed steps do not run from cache.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload inplane_gradient|cross_plane_film|bilayer_callaway] [--particles P]
                  [--precision fp64|mixed]

Prints one JSON line. `--impl reference` times the CPU restatement of the
reference algorithm (oracle/, the reference's own C++ cannot be built on the
GPU host) on the host cores: independent replicas, one per core.
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "carrier-steps/s on 1 GB300: batched mixed-prec vs plain FP64 at equal kappa error"
UNIT = "carrier-steps/s"
# Algorithmic bytes per carrier-step of the transport pass: read position,
# occupation, mode and cell; write position, occupation and cell.
BYTES_PER_CARRIER = {"fp64": 76, "mixed": 52}  # FP64 state / FP32 cell-local offsets
# mesh domains: the wall-cache time of each carrier (FP64, read and written)
# and its mirror facet (read)
MESH_EXTRA_BYTES = 20


_STL = {}


def finfet_stl_path():
    """The procedural FinFET surface, written once per process to a temporary file."""
    if "path" not in _STL:
        import tempfile
        from phonomc_gb300 import workloads
        d = tempfile.mkdtemp(prefix="phmc_finfet_")
        _STL["path"] = workloads.finfet_stl(os.path.join(d, "finfet.stl"))
    return _STL["path"]


def workload_config(name, particles, precision, seed=12345):
    from phonomc_gb300 import workloads
    if name == "finfet_mesh":
        return workloads.finfet_mesh(finfet_stl_path(), particles=particles, seed=seed, precision=precision)
    base = getattr(workloads, name)()
    return workloads.scaled(base, particles, random_seed=seed, precision=precision)


def workload_materials(name):
    """(material tables, include stationary modes, complete the Callaway BZ) per material."""
    from phonomc_gb300 import synthetic, workloads
    if name == "bilayer_callaway":
        return [(d, True, True) for d in workloads.bilayer_materials(8)]
    if name == "nonlinear_callaway_film":
        return [(synthetic.make_material(mesh=8, callaway=True), True, True)]
    return [(synthetic.make_material(mesh=16), name == "inplane_gradient", False)]


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(workload, precision, particles):
    """DRAM bytes (read + write) of one carrier pass from the committed ncu
    summary of that workload, or None when no capture matches its size."""
    path = os.path.join(ROOT, "profiles", f"k_transport_{workload}_{precision}.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    vals = {}
    for line in text.splitlines():
        if "=" in line and line.split("=")[0].strip() in ("pass_traffic_bytes", "carriers"):
            k, v = line.split("=", 1)
            vals[k.strip()] = float(v)
    if "pass_traffic_bytes" not in vals or int(vals.get("carriers", -1)) != int(particles):
        return None
    return vals["pass_traffic_bytes"]


class ClockSampler:
    """SM clock and clock-event reasons sampled DURING the timed region.

    A thread polls NVML (libnvidia-ml through ctypes) every 10 ms, so even a
    timed region of a few milliseconds gets samples; where NVML cannot be
    loaded it falls back to `nvidia-smi -lms 200`."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReasons bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
            "hw_power_brake_slowdown": 0x80}

    def __init__(self, index=0):
        self.index = index
        self.rows = []          # (sm_mhz, max_mhz, reasons bitmask)
        self.proc = None
        self.nvml = None
        self.stop = threading.Event()

    def _nvml_open(self):
        try:
            nv = C.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return False
            h = C.c_void_p()
            if nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
                return False
            self.nvml, self.handle = nv, h
            self.reason_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
            return True
        except (OSError, AttributeError):
            return False

    def _nvml_sample(self):
        cur, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        if self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, C.byref(cur)) != 0:
            return
        self.nvml.nvmlDeviceGetMaxClockInfo(self.handle, 1, C.byref(mx))
        self.reason_fn(self.handle, C.byref(rs))
        self.rows.append((float(cur.value), float(mx.value), int(rs.value)))

    def _nvml_loop(self):
        while not self.stop.is_set():
            self._nvml_sample()
            self.stop.wait(0.01)

    def __enter__(self):
        if self._nvml_open():
            self._nvml_sample()
            self.t = threading.Thread(target=self._nvml_loop, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._smi_read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _smi_read(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.proc.stdout:
            r = [x.strip() for x in line.split(",")]
            if len(r) < 9 or not r[1].replace(".", "").isdigit():
                continue
            bits = 0
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    bits |= self.BITS[name]
            self.rows.append((float(r[1]), float(r[2]) if r[2].replace(".", "").isdigit() else 0.0, bits))

    def __exit__(self, *a):
        if self.nvml is not None:
            self._nvml_sample()
            self.stop.set()
            self.t.join(timeout=5)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        reasons = sorted({name for _, _, bits in self.rows for name, b in self.BITS.items() if bits & b})
        return {"sm_mhz": float(np.median([r[0] for r in self.rows])), "sm_max_mhz": max(r[1] for r in self.rows),
                "reasons": reasons, "samples": len(self.rows), "source": "nvml" if self.nvml else "nvidia-smi"}


def _oracle_replica(args):
    """One CPU replica of the workload sample (separate process): init, warm-up
    steps, then `samples` timed windows of `steps` timesteps each."""
    name, particles, steps, samples, warmup, seed = args
    import oracle
    from phonomc_gb300 import abi
    lib = oracle.load()
    cfg = workload_config(name, particles, "fp64", seed)
    m = [abi.Material(lib, "orc_", d, 0.1, st, bz) for d, st, bz in workload_materials(name)]
    s = abi.Solver(lib, "orc_", cfg, m)
    s.run(max(1, warmup))
    cs, dt = 0, 0.0
    for _ in range(samples):
        n0 = s.stats()["particle_count"]
        t0 = time.perf_counter()
        s.run(steps)
        dt += time.perf_counter() - t0
        cs += 0.5 * (n0 + s.stats()["particle_count"]) * steps
    return cs, dt


def cpu_baseline(name, particles, steps, samples, warmup, procs):
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_replica, [(name, particles, steps, samples, warmup, 1000 + k) for k in range(procs)])
    cs = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    return cs / busy, {"carrier_steps": cs, "busy_s": busy}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = max(1, os.cpu_count() or 1)
    particles, steps = 20000, 4
    # the batched sweep's films are cross-plane films: their CPU path is the film's
    name = "cross_plane_film" if args.workload == "batched_films" else args.workload
    value, info = cpu_baseline(name, particles, steps, args.steps, args.warmup, procs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * info["busy_s"] / (args.steps * steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "particles_per_replica": particles, "replicas": procs,
                   "timesteps_per_step": steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": f"{procs} independent replicas x {particles} carriers, {steps} timesteps per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _time_arm(lib, abi, cfg, materials, steps, warmup):
    """Warm-up, then `steps` timed steps. When the solver sorts its carriers
    every K steps, the warm-up is extended so that the timed window starts on
    a sort step: the window holds ceil(steps / K) sorts, at least the share
    of a long run."""
    m = [abi.Material(lib, "phmc_", d, 0.1, st, bz) for d, st, bz in materials]
    s = abi.Solver(lib, "phmc_", cfg, m)
    k = C.c_int32()
    s.check(lib.phmc_solver_sort_interval(s.h, C.byref(k)))
    K = int(k.value)
    profiled = max(1, min(steps, 3))  # eager steps timed_run spends on the carrier-pass events
    extra = (K - (warmup + profiled) % K) % K if K > 0 else 0
    s.run(warmup + extra)
    first = warmup + extra + profiled
    sorts = sum(1 for t in range(first, first + steps) if K > 0 and t % K == 0)
    tot, kern, launches, n0, n1 = C.c_double(), C.c_double(), C.c_int64(), C.c_int64(), C.c_int64()
    with ClockSampler() as clk:
        s.check(lib.phmc_solver_timed_run(s.h, steps, C.byref(tot), C.byref(kern), C.byref(launches), C.byref(n0),
                                          C.byref(n1)))
    n0, n1 = n0.value, n1.value
    return {"solver": s, "material": m, "ms": tot.value, "kernel_ms_per_launch": kern.value,
            "launches": int(launches.value), "carrier_steps": 0.5 * (n0 + n1) * steps, "carriers": n0,
            "clocks": clk.summary(), "sort_interval": K, "sorts_timed": sorts}


def kappa_window(s, first, last, every=10):
    """Mean of kappa = -q/G over the flux passes of steps first..last (every
    `every` steps; the solver's convergence interval), continuing the run."""
    cur = s.stats()["current_timestep"]
    start = max(cur, first - 1)
    start += (-start) % every
    if start > cur:
        s.run(start - cur)
    vals = []
    step = start
    while step + every <= last:
        s.run(every)
        step += every
        if step >= first:
            vals.append(s.stats()["kappa_endpoints"])
    return float(np.mean(vals)), len(vals)


def measure_batch(lib, precision, steps, warmup, plain=True):
    """512 independent cross-plane films of log-uniform thickness advancing
    together (phmc_batch_*): whole-batch carrier-steps/s, `precision` and,
    unless plain is False, the plain FP64 arm."""
    from phonomc_gb300 import abi, synthetic, workloads
    m = abi.Material(lib, "phmc_", synthetic.make_material(mesh=16), 0.1, False, False)
    out = {}
    for prec in ([precision, "fp64"] if plain and precision != "fp64" else [precision]):
        films = workloads.batched_films(precision=prec)
        b = abi.Batch(lib, films, [m])
        b.run(warmup)
        n = steps if prec == precision else max(3, steps // 2)
        with ClockSampler() as clk:
            ms, cs, launches = b.timed_run(n)
        out[prec] = {"value": cs / (ms * 1e-3), "ms_per_step": ms / n, "launches": launches,
                     "clocks": clk.summary(), "carriers": sum(c["particle_count"] for c in films), "steps": n}
        b.close()
    return out


def run_batch(args):
    """512 independent cross-plane films of log-uniform thickness advancing
    together (phmc_batch_*): whole-batch carrier-steps/s, mixed and plain."""
    import phonomc_gb300
    lib = phonomc_gb300.lib()
    out = measure_batch(lib, args.precision, args.steps, args.warmup, plain=not args.no_plain)
    main = out[args.precision]
    line = {
        "metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": {"workload": "batched_films", "instances": 512, "carriers": int(main["carriers"]),
                   "thickness_nm": "log-uniform 10-2000 (seed 0)", "cells": "10-200 per film",
                   "precision": args.precision, "material": "synthetic 16^3 x 6 modes (seed 0)",
                   "l2": "carrier state larger than L2 (no flush needed)"},
        "gpu_launches": main["launches"],
        "e2e": {"value": None, "unit": UNIT,
                "note": "batched sweep: the default workload measures the host-buffer end-to-end path"},
        "clocks": main["clocks"],
    }
    if "fp64" in out and args.precision != "fp64":
        line["plain_fp64"] = {"value": out["fp64"]["value"], "unit": UNIT, "ms_per_step": out["fp64"]["ms_per_step"],
                              "mixed_over_plain": main["value"] / out["fp64"]["value"],
                              "clocks": out["fp64"]["clocks"]}
    print(json.dumps(line))


def run_ours(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    import phonomc_gb300
    from phonomc_gb300 import abi
    lib = phonomc_gb300.lib()
    materials = workload_materials(args.workload)
    seed = 12345 + rank
    # headline: the requested precision (mixed by default); comparison arm: plain FP64
    main_arm = _time_arm(lib, abi, workload_config(args.workload, args.particles, args.precision, seed), materials,
                         args.steps, args.warmup)
    plain = None
    kappa = None
    if args.precision == "mixed" and not args.no_plain:
        plain = _time_arm(lib, abi, workload_config(args.workload, args.particles, "fp64", seed), materials,
                          max(3, args.steps // 4), args.warmup)
        if args.kappa_steps > 0 and args.workload == "inplane_gradient":
            # kappa = -q/G of both arms (same seed, same draws) over the late half
            # of a kappa_steps run, outside the timed regions
            first = args.kappa_steps // 2 + 1
            km, nm = kappa_window(main_arm["solver"], first, args.kappa_steps)
            kp, npl = kappa_window(plain["solver"], first, args.kappa_steps)
            kappa = {"window_steps": [first, args.kappa_steps], "samples": min(nm, npl), "mixed": km, "fp64": kp,
                     "rel_err": abs(km - kp) / abs(kp), "bar": 0.005,
                     "unit": "W/(m K)", "note": "kappa = -q/G (src/solver/Observables.cpp:75-80), mean over flux "
                                                 "passes every 10 steps; both arms from the same seed"}
        plain["solver"].close()
    ms, carrier_steps = main_arm["ms"], main_arm["carrier_steps"]
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("gloo")
        t = torch.tensor([ms, carrier_steps], dtype=torch.float64)
        mx, sm = t.clone(), t.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        ms, carrier_steps = float(mx[0]), float(sm[1])
    value = carrier_steps / (ms * 1e-3)
    bpc = BYTES_PER_CARRIER[args.precision] + (MESH_EXTRA_BYTES if args.workload == "finfet_mesh" else 0)
    kavg = main_arm["kernel_ms_per_launch"]
    achieved = bpc * main_arm["carriers"] / (kavg * 1e-3) / 1e9
    peak, peak_kind = measured_peak()

    # end to end through the C ABI from pinned host buffers: every step uploads
    # the carriers (positions, occupation, mode), runs one timestep and reads
    # the cell temperatures back
    s = main_arm["solver"]
    Tout = np.zeros(s.cells()[0].size)
    n, e2e_value = 0, None
    if not args.no_e2e:
        c = s.carriers()
        live = c["alive"] == 1
        host = {k: np.ascontiguousarray(c[k][live]) for k in ("x", "y", "z", "occ")}
        host["mode"] = np.ascontiguousarray(c["mode"][live])
        n = host["x"].size
        for a in host.values():
            lib.phmc_host_register(a.ctypes.data, a.nbytes)
        e2e_steps = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            s.check(lib.phmc_solver_run_from_host(s.h, n, abi.dptr(host["x"]), abi.dptr(host["y"]),
                                                  abi.dptr(host["z"]), abi.dptr(host["occ"]),
                                                  host["mode"].ctypes.data_as(abi.c_uint32_p), 1, abi.dptr(Tout)))
        e2e_s = time.perf_counter() - t0
        for a in host.values():
            lib.phmc_host_unregister(a.ctypes.data)
        e2e_value = n * e2e_steps / e2e_s * (world if world > 1 else 1)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64", "data": "synthetic",
        "config": {"workload": args.workload, "particles": int(args.particles), "precision": args.precision,
                   "material": ("two synthetic 8^3 x 6 tables, second 0.7x frequency 0.75x velocity, Callaway BZ "
                                "completed (24552 modes)" if args.workload == "bilayer_callaway"
                                else "synthetic 8^3 x 6 Callaway table, BZ completed (24552 modes)"
                                if args.workload == "nonlinear_callaway_film"
                                else "synthetic 16^3 x 6 modes (seed 0)"), "cells": int(Tout.size),
                   **({"mesh": "procedural FinFET, 6304 triangles, 2245 facets (seed 0)", "voxels": "64x32x32",
                       "heat_source": "gaussian 1e20 W/m^3, sigma 5 nm, fin top, thermal spectrum"}
                      if args.workload == "finfet_mesh" else {}),
                   "l2": "carrier state larger than L2 (no flush needed)", "replicas": world},
        "gpu_launches": main_arm["launches"],
        "roofline": {"bound": "hbm", "kernel": ("k_transport_mesh + k_mesh_events (the carrier pass of a step; the wall "
                                                "events are FP64-pipe bound)" if args.workload == "finfet_mesh" else
                                                "k_transport + k_deferred (the one carrier pass of a step)"),
                     "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_carrier": bpc, "kernel_ms_per_launch": kavg,
                     "traffic": profiled_traffic(args.workload, args.precision, args.particles),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one carrier pass "
                                       "(profiles/k_transport_<workload>_<precision>.md)"},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(n * (4 * 8 + 4)), "d2h_bytes_per_step": int(Tout.size * 8)},
        "clocks": main_arm["clocks"],
    }
    line["config"]["carrier_sort"] = {"interval_steps": main_arm["sort_interval"],
                                      "sorts_in_timed_steps": main_arm["sorts_timed"]}
    if plain is not None:
        pv = plain["carrier_steps"] / (plain["ms"] * 1e-3)
        pk = plain["kernel_ms_per_launch"]
        line["plain_fp64"] = {"value": pv, "unit": UNIT, "ms_per_step": plain["ms"] / max(3, args.steps // 4),
                              "mixed_over_plain": value / pv,
                              "roofline_frac": 76 * plain["carriers"] / (pk * 1e-3) / 1e9 / peak,
                              "kernel_ms_per_launch": pk, "sorts_in_timed_steps": plain["sorts_timed"],
                              "clocks": plain["clocks"]}
    if kappa is not None:
        line["kappa"] = kappa
    if not args.no_batch and world == 1:
        b = measure_batch(lib, args.precision, args.steps, args.warmup, plain=not args.no_plain)
        bm = b[args.precision]
        line["batched"] = {"workload": "batched_films", "instances": 512, "carriers": int(bm["carriers"]),
                           "value": bm["value"], "unit": UNIT, "ms_per_step": bm["ms_per_step"],
                           "steps": bm["steps"], "gpu_launches": bm["launches"], "clocks": bm["clocks"],
                           "thickness_nm": "log-uniform 10-2000 (seed 0)", "cells": "10-200 per film"}
        if "fp64" in b and args.precision != "fp64":
            line["batched"]["plain_fp64"] = {"value": b["fp64"]["value"], "ms_per_step": b["fp64"]["ms_per_step"],
                                             "steps": b["fp64"]["steps"], "clocks": b["fp64"]["clocks"]}
            line["batched"]["mixed_over_plain"] = bm["value"] / b["fp64"]["value"]
    if rank == 0 and not args.no_cpu_baseline:
        cp, cstep = (50000, 4) if args.workload == "finfet_mesh" else (200000, 10)
        cb, info = cpu_baseline(args.workload, cp, cstep, 3, 1, 1)
        line["cpu_baseline"] = {"value": cb, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"{args.workload}, {cp} carriers x {3 * cstep} timed steps, serial CPU oracle"}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: one whole carrier-sort interval of the mixed state on boxes (200
    # steps), so a sort weighs in the timed window at its share of a long run;
    # the FinFET mesh 100 (four of its 25-step sort intervals: the synthetic
    # FinFET loses a carrier through its jittered top surface every few hundred
    # steps at 2e7 carriers, which ends a run, as in the reference)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="inplane_gradient",
                    choices=["inplane_gradient", "cross_plane_film", "bilayer_callaway", "heated_film",
                             "batched_films", "finfet_mesh", "nonlinear_callaway_film"])
    ap.add_argument("--particles", type=float, default=None)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison arm")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-films sub-measurement")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--kappa-steps", type=int, default=2000,
                    help="in-plane gradient: steps of the mixed-vs-FP64 kappa comparison (0: skip)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 100 if args.workload == "finfet_mesh" else 200
    if args.particles is None:
        args.particles = {"inplane_gradient": 5e7, "finfet_mesh": 2e7, "nonlinear_callaway_film": 1e7,
                          "bilayer_callaway": 1e8}.get(args.workload, 1e6)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched_films":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
