"""CPU calibration: the reference's own step loop against the oracle port.

The timed CPU arm of bench.py is the oracle port (oracle/phmc_oracle.cpp),
because the reference's sources do not exist on the machine that runs the
GPU. This script relates the two on one machine that has both: it times
MonteCarloSolver::run_timestep of the reference build in oracle/_ref
(`ref_harness time`, OpenMP with 1 thread and with every core) and the serial
oracle on the same scaled workloads and synthetic 16^3 x 6 table:

  cross_plane_film   the 1e6-carrier cross-plane film (reservoirs 301/299 K,
                     50 cells, dt 1 ps), scaled to --particles carriers
  inplane_gradient   the 5e7-carrier in-plane gradient film (rough walls,
                     G = 1e7 K/m, 100 cells, dt 0.5 ps), scaled the same way

Each run does --warm steps, then times --steps steps; carrier-steps count the
carriers present at the start of each timed step. One JSON line per
(workload, implementation, threads).

    python oracle/ref/calibrate_cpu.py [--particles 200000] [--warm 2] [--steps 6]
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def _toml(workload, particles, steps, out):
    import make_golden
    if workload == "cross_plane_film":
        return make_golden.CROSS_PLANE_TOML.format(particles=int(particles), steps=steps, seed=5, out=out)
    return make_golden.INPLANE_TOML.format(particles=int(particles), steps=steps, seed=5, cells=100, out=out)


def time_reference(workload, pmat, particles, warm, steps, threads, tmp):
    folder = os.path.join(tmp, f"{workload}_{threads}")
    os.makedirs(folder, exist_ok=True)
    toml = os.path.join(folder, "input.toml")
    with open(toml, "w") as f:
        f.write(_toml(workload, particles, warm + steps, folder))
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([HARNESS, "time", pmat, toml, str(warm), str(steps)], check=True, capture_output=True,
                       text=True, env=env)
    return json.loads(r.stdout)


def time_port(workload, particles, warm, steps):
    import oracle
    from phonomc_gb300 import abi, synthetic, workloads
    lib = oracle.load()
    stationary = workload == "inplane_gradient"
    m = abi.Material(lib, "orc_", synthetic.make_material(mesh=16), 0.1, stationary, False)
    cfg = workloads.scaled(getattr(workloads, workload)(), particles, random_seed=5)
    s = abi.Solver(lib, "orc_", cfg, [m])
    s.run(warm)
    carrier_steps = 0.0
    busy = 0.0
    for _ in range(steps):
        carrier_steps += s.stats()["particle_count"]
        t0 = time.perf_counter()
        s.run(1)
        busy += time.perf_counter() - t0
    s.close()
    return {"carrier_steps": carrier_steps, "seconds": busy, "carrier_steps_per_s": carrier_steps / busy,
            "threads": 1}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--particles", type=float, default=2e5)
    ap.add_argument("--warm", type=int, default=2)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--workloads", nargs="*", default=["cross_plane_film", "inplane_gradient"])
    args = ap.parse_args()
    if not os.path.exists(HARNESS):
        sys.exit("oracle/_ref/ref_harness is not built (needs the reference sources)")
    from phonomc_gb300 import synthetic
    cores = os.cpu_count() or 1
    with tempfile.TemporaryDirectory() as tmp:
        pmat = os.path.join(tmp, "m16.pmat")
        synthetic.write_pmat(pmat, synthetic.make_material(mesh=16))
        for w in args.workloads:
            for threads in sorted({1, cores}):
                r = time_reference(w, pmat, args.particles, args.warm, args.steps, threads, tmp)
                print(json.dumps({"workload": w, "impl": "reference (oracle/_ref, OpenMP)", "particles": args.particles,
                                  **r}), flush=True)
            r = time_port(w, args.particles, args.warm, args.steps)
            print(json.dumps({"workload": w, "impl": "port (oracle, serial)", "particles": args.particles, **r}),
                  flush=True)


if __name__ == "__main__":
    main()
