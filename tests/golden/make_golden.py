"""Regenerate the golden fixtures in this folder from the reference solver.

Run in a container that has the reference sources (it builds them first):

    python tests/golden/make_golden.py --ref <reference checkout>   (or PHONOMC_REFERENCE=<checkout>)

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
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from phonomc_gb300 import synthetic, workloads  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# name -> harness arguments ("{m}" = plain 8^3 table, "{c}" = Callaway table)
CASES = {
    "ncallaway_unique": ["ncallaway", "11", "48", "48", "1"],
    "ncallaway_shared": ["ncallaway", "12", "40", "200", "0"],
    "ncallaway_large": ["ncallaway", "13", "600", "900", "0"],
    "material_m8": ["material", "{m}", "0"],
    "material_m8_stationary": ["material", "{m}", "1"],
    "material_m8c_stationary": ["material", "{c}", "1", "1"],
    "box_trace": ["box"],
    "rta_fixed": ["rta", "{m}", "0"],
    "rta_local": ["rta", "{m}", "1"],
    "linearized_rta": ["lincoll", "{m}"],
    "callaway_evolve": ["callaway"],
    "rough_nonconservative": ["rough", "{m}", "0"],
    "rough_conservative": ["rough", "{m}", "1"],
    "gradient_drive": ["gradient", "{m}"],
    "reservoir": ["reservoir", "{m}"],
    "source_thermal": ["source", "{m}", "0", "0"],
    "source_thermal_linearized": ["source", "{m}", "0", "1"],
    "source_weighted": ["source", "{m}", "1", "0"],
    "source_gaussian": ["source", "{m}", "2", "0"],
    "mesh_finfet": ["mesh", "{f}"],
    "domain_finfet": ["domain", "{t}"],
    "domain_prism": ["domain", "{p}", "600"],
    "interface_dmm": ["interface", "{m}", "{s}", "0"],
    "interface_dmm_linearized": ["interface", "{m}", "{s}", "1"],
    "interface_amm": ["amm", "{m}", "{s}", "1", "1.0", "0"],
    "interface_amm_linearized": ["amm", "{m}", "{s}", "1", "1.0", "1"],
    "interface_mmm": ["amm", "{m}", "{s}", "2", "0.4", "0"],
}


CROSS_PLANE_TOML = """[geometry]
model = "box"
sizes = [100, 100, 100]

[simulation]
particle_count = {particles}
time_step = 1.0
iterations = {steps}
random_seed = {seed}
compute_kappa = true
transport_axis = "z"
initial_temperature = "linear"
background_temperature = 300
lifetime_temperature = 300
grid_xyz = [1, 1, 50]
convergence_write_interval = 1

[boundary]
boundary_position = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1],
  [0,0,-0.01,1,1,0.01], [0,0,0.99,1,1,1.01]
]
boundary_conditions = ["P","P","P","P","T","T"]
boundary_values = [0,0,0,0,301,299]
periodic_pair = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1]
]

[io]
material_folder = "unused"
output_folder = "{out}"
"""

# Extruded L-shaped prism (phonomc_gb300.synthetic.prism_mesh, lengths in nm):
# constant-height prism with exact cut-cell volumes, heat flowing from the
# 310 K top to the 300 K bottom, rough side walls.
PRISM_TOML = """[geometry]
model = "{stl}"
extruded_z = true

[simulation]
particle_count = {particles}
time_step = 0.5
iterations = {steps}
random_seed = {seed}
compute_kappa = false
initial_temperature = 305
background_temperature = 305
lifetime_temperature = 305
grid_xyz = [8, 6, 5]
convergence_write_interval = 1

[boundary]
boundary_position = [
  [-0.01, -0.01, -0.01, 1.01, 1.01, 1.01],
  [-0.01, -0.01, -0.001, 1.01, 1.01, 0.001],
  [-0.01, -0.01, 0.999, 1.01, 1.01, 1.001]
]
boundary_conditions = ["R", "T", "T"]
boundary_values = [1.0, 300.0, 310.0]

[io]
material_folder = "unused"
output_folder = "{out}"
"""

# FinFET mesh domain in the reference's TOML form (lengths in nm), the same
# geometry and regions as phonomc_gb300.workloads.finfet_mesh.
FINFET_TOML = """[geometry]
model = "{stl}"

[simulation]
particle_count = {particles}
time_step = 0.1
iterations = {steps}
random_seed = {seed}
compute_kappa = false
initial_temperature = 300
background_temperature = 300
lifetime_temperature = "local"
grid_xyz = [{nx}, {ny}, {nz}]
convergence_write_interval = 1

[boundary]
boundary_position = [
  [0.0, 0.0, 0.001, 1.0, 1.0, 1.01],
  [-0.001, 0.0, 0.0, 0.001, 1.0, 1.0], [0.999, 0.0, 0.0, 1.001, 1.0, 1.0],
  [0.0, -0.001, 0.0, 1.0, 0.001, 1.0], [0.0, 0.999, 0.0, 1.0, 1.001, 1.0],
  [0.0, 0.0, -0.001, 1.0, 1.0, 0.001]
]
boundary_conditions = ["R", "P", "P", "P", "P", "T"]
boundary_values = [1.0, 0.0, 0.0, 0.0, 0.0, 300.0]
periodic_pair = [
  [-0.001, 0.0, 0.0, 0.001, 1.0, 1.0], [0.999, 0.0, 0.0, 1.001, 1.0, 1.0],
  [0.0, -0.001, 0.0, 1.0, 0.001, 1.0], [0.0, 0.999, 0.0, 1.0, 1.001, 1.0]
]
{source}
[io]
material_folder = "unused"
output_folder = "{out}"
"""

FINFET_SOURCE_TOML = """
[heat_source]
enabled = true
profile = "gaussian"
min = [90.0, 0.0, 70.0]
max = [110.0, 100.0, 91.0]
center = [100.0, 50.0, 90.0]
sigma = [5.0, 5.0, 5.0]
power_density = 1.0e20
spectrum = "thermal"
"""


# Full reference runs of the scaled cross-plane film (same geometry and physics
# as phonomc_gb300.workloads.cross_plane_film, 2e4 carriers): per seed, the
# cell temperatures and heat flux averaged over the second half of the run.
STAT_SEEDS = 16
STAT_PARTICLES = 20000
STAT_STEPS = 200


def full_runs(mpath: str, tmp: str) -> dict:
    import numpy as np
    out = {"seeds": [], "T_mean": [], "flux_mean": [], "kappa_eff_mean": [], "particles_mean": [],
           "particles": STAT_PARTICLES, "steps": STAT_STEPS, "average_from_step": STAT_STEPS // 2 + 1}
    for k in range(STAT_SEEDS):
        seed = 101 + k
        folder = os.path.join(tmp, f"run{seed}")
        os.makedirs(folder, exist_ok=True)
        toml = os.path.join(folder, "c1.toml")
        with open(toml, "w") as f:
            f.write(CROSS_PLANE_TOML.format(particles=STAT_PARTICLES, steps=STAT_STEPS, seed=seed, out=folder))
        res = json.loads(subprocess.run([HARNESS, "run", mpath, toml, str(STAT_STEPS)], check=True,
                                        capture_output=True, text=True).stdout)
        rows = np.asarray(res["convergence"])
        late = rows[rows[:, 0] >= STAT_STEPS // 2 + 1]
        out["seeds"].append(seed)
        out["T_mean"].append(late[:, 2:52].mean(axis=0).tolist())
        out["flux_mean"].append(float(late[:, 52].mean()))
        out["kappa_eff_mean"].append(float(late[:, 54].mean()))
        out.setdefault("kappa_fit_mean", []).append(float(late[:, 53].mean()))
        out["particles_mean"].append(float(late[:, 55].mean()))
        out.setdefault("balance_residual_total", []).append(res["balance_residual_total"][-1])
    return out


# Full reference runs of the FinFET mesh domain with its heat source (8^3
# table, 2e4 carriers, 32 x 8 x 16 voxels, 200 steps of 0.1 ps): per seed, the
# late-time means (steps 101-200) of the region temperatures (fin above the
# 50 nm slab, upper and lower slab halves), the thermal energy and the
# absorbed carriers per step, and the heat-source energy at the end.
FINFET_SEEDS = 16
FINFET_PARTICLES = 20000
FINFET_STEPS = 200
FINFET_GRID = (32, 8, 16)


def full_runs_finfet(mpath: str, fpath: str, tmp: str) -> dict:
    import numpy as np
    out = {"seeds": [], "particles": FINFET_PARTICLES, "steps": FINFET_STEPS, "grid": list(FINFET_GRID),
           "average_from_step": FINFET_STEPS // 2 + 1}
    for k in range(FINFET_SEEDS):
        seed = 101 + k
        folder = os.path.join(tmp, f"ff{seed}")
        os.makedirs(folder, exist_ok=True)
        toml = os.path.join(folder, "c3.toml")
        with open(toml, "w") as f:
            f.write(FINFET_TOML.format(stl=fpath, particles=FINFET_PARTICLES, steps=FINFET_STEPS, seed=seed,
                                       nx=FINFET_GRID[0], ny=FINFET_GRID[1], nz=FINFET_GRID[2],
                                       source=FINFET_SOURCE_TOML, out=folder))
        res = json.loads(subprocess.run([HARNESS, "run", mpath, toml, str(FINFET_STEPS)], check=True,
                                        capture_output=True, text=True).stdout)
        rows = np.asarray(res["convergence"])
        nc = len(res["grid_centers"])
        agg = workloads.finfet_aggregates(rows[:, 2:2 + nc], res["thermal_energy"], res["absorbed_total"],
                                res["grid_centers"], out["average_from_step"])
        out["seeds"].append(seed)
        for key, v in agg.items():
            out.setdefault(key, []).append(v)
        out.setdefault("source_total_end", []).append(res["heat_source_total"][-1])
        out.setdefault("balance_residual_total", []).append(res["balance_residual_total"][-1])
    return out


# Full reference runs of a scaled bilayer (phonomc_gb300.workloads.bilayer_callaway
# at 2e4 carriers, 20 cells; 8^3 Callaway tables, the second material softened):
# per seed, late-time means (steps 101-200) of the cell temperatures, heat flux,
# kappa_eff and carrier count, and the interface counts over the run.
BILAYER_SEEDS = 16
BILAYER_PARTICLES = 20000
BILAYER_STEPS = 200
BILAYER_CELLS = 20
BILAYER_TOML = """[geometry]
model = "box"
sizes = [100, 100, 200]

[simulation]
particle_count = {particles}
time_step = 0.5
iterations = {steps}
random_seed = {seed}
compute_kappa = true
transport_axis = "z"
initial_temperature = "linear"
background_temperature = 300
lifetime_temperature = 300
grid_xyz = [1, 1, {cells}]
convergence_write_interval = 1

[scattering]
model = "callaway"

[boundary]
boundary_position = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1],
  [0,0,-0.01,1,1,0.01], [0,0,0.99,1,1,1.01]
]
boundary_conditions = ["P","P","P","P","T","T"]
boundary_values = [0,0,0,0,310,290]
periodic_pair = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1]
]

[materials]
folders = ["a", "b"]
interface_axis = "z"
interface_positions = [100]
interface_model = "dmm"

[io]
material_folder = "unused"
output_folder = "{out}"
"""


def full_runs_bilayer(pmats: str, tmp: str) -> dict:
    import numpy as np
    out = {"seeds": [], "particles": BILAYER_PARTICLES, "steps": BILAYER_STEPS, "cells": BILAYER_CELLS,
           "average_from_step": BILAYER_STEPS // 2 + 1}
    nc = BILAYER_CELLS
    for k in range(BILAYER_SEEDS):
        seed = 101 + k
        folder = os.path.join(tmp, f"bl{seed}")
        os.makedirs(folder, exist_ok=True)
        toml = os.path.join(folder, "c5.toml")
        with open(toml, "w") as f:
            f.write(BILAYER_TOML.format(particles=BILAYER_PARTICLES, steps=BILAYER_STEPS, seed=seed, cells=nc,
                                        out=folder))
        res = json.loads(subprocess.run([HARNESS, "run", pmats, toml, str(BILAYER_STEPS)], check=True,
                                        capture_output=True, text=True).stdout)
        rows = np.asarray(res["convergence"])
        late = rows[rows[:, 0] >= out["average_from_step"]]
        out["seeds"].append(seed)
        out.setdefault("T_mean", []).append(late[:, 2:2 + nc].mean(axis=0).tolist())
        out.setdefault("flux_mean", []).append(float(late[:, 2 + nc].mean()))
        out.setdefault("kappa_eff_mean", []).append(float(late[:, 4 + nc].mean()))
        out.setdefault("kappa_fit_mean", []).append(float(late[:, 3 + nc].mean()))
        out.setdefault("particles_mean", []).append(float(late[:, 5 + nc].mean()))
        out.setdefault("interface_events", []).append(res["interface_events"])
        out.setdefault("interface_transmitted", []).append(res["interface_transmitted"])
        out.setdefault("balance_residual_total", []).append(res["balance_residual_total"][-1])
    return out


# Full reference runs of the bilayer with the acoustic-mismatch interface
# (phonomc_gb300.workloads.bilayer_amm at 2e4 carriers, 20 cells, nonlinear RTA,
# plain 8^3 tables): the late-time fields of full_runs_bilayer.
def full_runs_bilayer_amm(pmats: str, tmp: str) -> dict:
    global BILAYER_TOML
    saved = BILAYER_TOML
    BILAYER_TOML = saved.replace('[scattering]\nmodel = "callaway"\n', '[scattering]\nmodel = "rta"\n').replace(
        'interface_model = "dmm"', 'interface_model = "amm"\nmass_densities_kg_m3 = [2329.0, 5323.0]')
    try:
        return full_runs_bilayer(pmats, tmp)
    finally:
        BILAYER_TOML = saved


# Full reference runs of the cross-plane film with nonlinear Callaway
# collisions (8^3 Callaway table, 8000 carriers, 120 steps of 1 ps): per seed
# the late-time (steps 61-120) cell temperatures, heat flux and kappa_eff.
NCL_SEEDS = 16
NCL_PARTICLES = 8000
NCL_STEPS = 120


def full_runs_ncallaway(mpath: str, tmp: str) -> dict:
    import numpy as np
    out = {"seeds": [], "particles": NCL_PARTICLES, "steps": NCL_STEPS, "average_from_step": NCL_STEPS // 2 + 1}
    for k in range(NCL_SEEDS):
        seed = 101 + k
        folder = os.path.join(tmp, f"ncl{seed}")
        os.makedirs(folder, exist_ok=True)
        toml = os.path.join(folder, "ncl.toml")
        text = CROSS_PLANE_TOML.format(particles=NCL_PARTICLES, steps=NCL_STEPS, seed=seed, out=folder)
        text = text.replace("[boundary]", '[scattering]\nmodel = "callaway"\ncallaway_formulation = "nonlinear"\n\n'
                            "[boundary]", 1)
        with open(toml, "w") as f:
            f.write(text)
        res = json.loads(subprocess.run([HARNESS, "run", mpath, toml, str(NCL_STEPS)], check=True,
                                        capture_output=True, text=True).stdout)
        rows = np.asarray(res["convergence"])
        late = rows[rows[:, 0] >= out["average_from_step"]]
        out["seeds"].append(seed)
        out.setdefault("T_mean", []).append(late[:, 2:52].mean(axis=0).tolist())
        out.setdefault("flux_mean", []).append(float(late[:, 52].mean()))
        out.setdefault("kappa_eff_mean", []).append(float(late[:, 54].mean()))
        out.setdefault("kappa_fit_mean", []).append(float(late[:, 53].mean()))
        out.setdefault("lifetime_residual_total", []).append(res["lifetime_residual_total"])
        out.setdefault("balance_residual_total", []).append(res["balance_residual_total"][-1])
    return out


# Full reference runs of the in-plane periodic-gradient film
# (phonomc_gb300.workloads.inplane_gradient at 2e4 carriers: 100 nm film,
# rough 1 nm z walls, G = 1e7 K/m along x, 100 z-cells, linearized RTA at
# 300 K, dt = 0.5 ps, 2000 steps): per seed the late-time (steps 1001-2000)
# cell temperatures, heat flux and kappa = -q/G, kappa over every window of
# 100 steps (the approach to steady state), and the energy closure.
GRAD_SEEDS = 16
GRAD_PARTICLES = 20000
GRAD_STEPS = 2000
GRAD_CELLS = 100
GRAD_WINDOW = 100
INPLANE_TOML = """[geometry]
model = "box"
sizes = [100, 100, 100]

[simulation]
particle_count = {particles}
time_step = 0.5
iterations = {steps}
random_seed = {seed}
compute_kappa = true
transport_axis = "x"
initial_temperature = 300
background_temperature = 300
lifetime_temperature = 300
grid_xyz = [1, 1, {cells}]
convergence_write_interval = 1

[driving]
temperature_gradient = 1.0e7

[boundary]
boundary_position = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1],
  [0,0,-0.01,1,1,0.01], [0,0,0.99,1,1,1.01]
]
boundary_conditions = ["P","P","P","P","R","R"]
boundary_values = [0,0,0,0,1,1]
periodic_pair = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1]
]

[io]
material_folder = "unused"
output_folder = "{out}"
"""


def full_runs_inplane(mpath: str, tmp: str) -> dict:
    import numpy as np
    nc = GRAD_CELLS
    out = {"seeds": [], "particles": GRAD_PARTICLES, "steps": GRAD_STEPS, "cells": nc, "gradient": 1.0e7,
           "average_from_step": GRAD_STEPS // 2 + 1, "window": GRAD_WINDOW}
    for k in range(GRAD_SEEDS):
        seed = 101 + k
        folder = os.path.join(tmp, f"grad{seed}")
        os.makedirs(folder, exist_ok=True)
        toml = os.path.join(folder, "c2.toml")
        with open(toml, "w") as f:
            f.write(INPLANE_TOML.format(particles=GRAD_PARTICLES, steps=GRAD_STEPS, seed=seed, cells=nc, out=folder))
        res = json.loads(subprocess.run([HARNESS, "run", mpath, toml, str(GRAD_STEPS)], check=True,
                                        capture_output=True, text=True).stdout)
        rows = np.asarray(res["convergence"])
        rows = rows[rows[:, 0] >= 1]
        assert rows.shape[0] == GRAD_STEPS, rows.shape
        late = rows[rows[:, 0] >= out["average_from_step"]]
        kappa = rows[:, 4 + nc]
        out["seeds"].append(seed)
        out.setdefault("T_mean", []).append(late[:, 2:2 + nc].mean(axis=0).tolist())
        out.setdefault("flux_mean", []).append(float(late[:, 2 + nc].mean()))
        out.setdefault("kappa_eff_mean", []).append(float(late[:, 4 + nc].mean()))
        out.setdefault("kappa_fit_mean", []).append(float(late[:, 3 + nc].mean()))
        out.setdefault("kappa_windows", []).append(kappa.reshape(-1, GRAD_WINDOW).mean(axis=1).tolist())
        out.setdefault("gradient_energy_total", []).append(res["gradient_energy_total"])
        out.setdefault("balance_residual_total", []).append(res["balance_residual_total"][-1])
        shutil.rmtree(folder, ignore_errors=True)  # 2,000 rows of 100 cells per seed
    return out


# Output files of a short FinFET run with its heat source and per-cell heat
# flux rows (simulation.write_cell_heat_flux): convergence.txt,
# grid_heat_flux.csv and heat_source_ledger.txt as the reference writes them.
FILES_STEPS = 2


def output_files_finfet(mpath: str, fpath: str, tmp: str) -> dict:
    folder = os.path.join(tmp, "files_finfet")
    os.makedirs(folder, exist_ok=True)
    toml = os.path.join(folder, "c3.toml")
    text = FINFET_TOML.format(stl=fpath, particles=2000, steps=FILES_STEPS, seed=5, nx=FINFET_GRID[0],
                              ny=FINFET_GRID[1], nz=FINFET_GRID[2], source=FINFET_SOURCE_TOML, out=folder)
    text = text.replace("convergence_write_interval = 1\n", "convergence_write_interval = 1\nwrite_cell_heat_flux = true\n", 1)
    assert "write_cell_heat_flux" in text
    with open(toml, "w") as f:
        f.write(text)
    res = json.loads(subprocess.run([HARNESS, "run", mpath, toml, str(FILES_STEPS)], check=True,
                                    capture_output=True, text=True).stdout)
    return {"particles": 2000, "seed": 5, "steps": FILES_STEPS, "grid": list(FINFET_GRID),
            "files": {k[5:]: v for k, v in res.items() if k.startswith("file:")}}


def build(ref: str) -> None:
    subprocess.run(["make", "-s", "-j8", f"REF={ref}"], cwd=os.path.join(ROOT, "oracle", "ref"),
                   check=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PHONOMC_REFERENCE"),
                    help="the reference checkout (default: $PHONOMC_REFERENCE)")
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set PHONOMC_REFERENCE to the reference checkout")
    build(args.ref)
    tmp = os.path.join(ROOT, "oracle", "_ref")
    mpath = os.path.join(tmp, "m8.pmat")
    cpath = os.path.join(tmp, "m8c.pmat")
    synthetic.write_pmat(mpath, synthetic.make_material(mesh=8))
    synthetic.write_pmat(cpath, synthetic.make_material(mesh=8, callaway=True))
    fpath = os.path.join(tmp, "finfet.stl")
    synthetic.write_stl(fpath, *synthetic.finfet_mesh())
    spath = os.path.join(tmp, "m8s.pmat")
    synthetic.write_pmat(spath, synthetic.make_material(mesh=8, freq_scale=0.7, vel_scale=0.75))
    ppath = os.path.join(tmp, "prism.stl")
    synthetic.write_stl(ppath, *synthetic.prism_mesh())
    prism_toml = os.path.join(tmp, "prism_domain.toml")
    with open(prism_toml, "w") as f:
        f.write(PRISM_TOML.format(stl=ppath, particles=2000, steps=1, seed=5, out=os.path.join(tmp, "prism_out")))
    tpath = os.path.join(tmp, "finfet_domain.toml")
    with open(tpath, "w") as f:
        f.write(FINFET_TOML.format(stl=fpath, particles=2000, steps=1, seed=5, nx=64, ny=32, nz=32,
                                   source=FINFET_SOURCE_TOML, out=os.path.join(tmp, "finfet_domain_out")))
    if not args.only or "fullrun_cross_plane" in args.only:
        m16 = os.path.join(tmp, "m16.pmat")
        synthetic.write_pmat(m16, synthetic.make_material(mesh=16))
        data = full_runs(m16, os.path.join(tmp, "fullrun"))
        data["_harness_args"] = ["run", "{m16}", "<cross-plane toml>", str(STAT_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_cross_plane.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_cross_plane ok")
    if not args.only or "fullrun_inplane_gradient" in args.only:
        m16s = os.path.join(tmp, "m16.pmat")
        synthetic.write_pmat(m16s, synthetic.make_material(mesh=16))
        data = full_runs_inplane(m16s, os.path.join(tmp, "fullrun_inplane"))
        data["_harness_args"] = ["run", "{m16}", "<in-plane gradient toml>", str(GRAD_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_inplane_gradient.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_inplane_gradient ok")
    if not args.only or "fullrun_bilayer" in args.only:
        cs = os.path.join(tmp, "m8cs.pmat")
        synthetic.write_pmat(cs, synthetic.make_material(mesh=8, freq_scale=0.7, vel_scale=0.75, callaway=True))
        data = full_runs_bilayer(cpath + "," + cs, os.path.join(tmp, "fullrun_bilayer"))
        data["_harness_args"] = ["run", "{c},{cs}", "<bilayer toml>", str(BILAYER_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_bilayer.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_bilayer ok")
    if not args.only or "fullrun_bilayer_amm" in args.only:
        data = full_runs_bilayer_amm(mpath + "," + spath, os.path.join(tmp, "fullrun_bilayer_amm"))
        data["_harness_args"] = ["run", "{m},{s}", "<bilayer toml, rta, amm>", str(BILAYER_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_bilayer_amm.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_bilayer_amm ok")
    if not args.only or "fullrun_finfet" in args.only:
        data = full_runs_finfet(mpath, fpath, os.path.join(tmp, "fullrun_finfet"))
        data["_harness_args"] = ["run", "{m}", "<FinFET toml>", str(FINFET_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_finfet.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_finfet ok")
    if not args.only or "fullrun_ncallaway" in args.only:
        data = full_runs_ncallaway(cpath, os.path.join(tmp, "fullrun_ncallaway"))
        data["_harness_args"] = ["run", "{c}", "<cross-plane toml, nonlinear Callaway>", str(NCL_STEPS)]
        with gzip.open(os.path.join(HERE, "fullrun_ncallaway.json.gz"), "wt") as f:
            json.dump(data, f)
        print("fullrun_ncallaway ok")
    if not args.only or "files_finfet" in args.only:
        data = output_files_finfet(mpath, fpath, tmp)
        data["_harness_args"] = ["run", "{m}", "<FinFET toml, write_cell_heat_flux>", str(FILES_STEPS)]
        with gzip.open(os.path.join(HERE, "files_finfet.json.gz"), "wt") as f:
            json.dump(data, f)
        print("files_finfet ok")
    for name, argv in CASES.items():
        if args.only and name not in args.only:
            continue
        cmd = [HARNESS] + [a.format(m=mpath, c=cpath, s=spath, f=fpath, t=tpath, p=prism_toml) for a in argv]
        out = subprocess.run(cmd, check=True, capture_output=True, text=True).stdout
        data = json.loads(out)
        data["_harness_args"] = argv
        with gzip.open(os.path.join(HERE, name + ".json.gz"), "wt") as f:
            json.dump(data, f)
        print(name, "ok")


if __name__ == "__main__":
    main()
