"""Named workloads (SimulationConfig dicts in internal units: Angstrom, ps, K).

cross_plane_film   100 nm box, periodic in x/y, reservoirs 301/299 K on the z
                   faces, 50 z-cells, nonlinear RTA with lifetimes fixed at
                   300 K, 1e6 carriers, dt = 1 ps (2000 steps in the full run).
inplane_gradient   100 nm film, periodic in x/y, rough z walls (1 nm RMS),
                   periodic-gradient drive G = 1e7 K/m along x, 100 z-cells,
                   linearized RTA at 300 K, 5e7 carriers, dt = 0.5 ps.

bilayer_callaway  200 nm stack of two materials (the second with 0.7x
                   frequencies and 0.75x velocities), interface at 100 nm,
                   diffuse-mismatch interface, linearized Callaway collisions,
                   reservoirs 310/290 K on the z faces, 100 z-cells, 1e8
                   carriers, dt = 0.5 ps.

bilayer_amm       the bilayer stack with the acoustic-mismatch interface and
                   nonlinear RTA (plain 8^3 tables).

heated_film       the cross-plane film with both reservoirs at 300 K and a
                   prescribed lattice heat source: Gaussian along z (sigma
                   10 nm, centred at 50 nm, uniform in x and y), 1e18 W/m^3
                   peak, thermal spectrum; nonlinear RTA with local
                   lifetimes, 1e6 carriers, dt = 1 ps.

batched_films     512 independent cross-plane films (see batched_films()).

The lateral repeat cell is 100 nm x 100 nm in all of them. `scaled()` keeps the
geometry and physics and shrinks the carrier count for tests.
"""

from __future__ import annotations

import copy

LATERAL_A = 1000.0
THICKNESS_A = 1000.0


def cross_plane_film(particles: float = 1e6, seed: int = 12345, precision: str = "fp64") -> dict:
    return {
        "name": "cross_plane_film",
        "sizes": (LATERAL_A, LATERAL_A, THICKNESS_A),
        "particle_count": particles,
        "time_step": 1.0,
        "iterations": 2000,
        "random_seed": seed,
        "compute_kappa": True,
        "transport_axis": 2,
        "background_temperature": 300.0,
        "lifetime_temperature": 300.0,
        "initial_temperature": "linear",
        "grid": (1, 1, 50),
        "faces": ("P", "P", "P", "P", "T", "T"),
        "face_values": (0, 0, 0, 0, 301.0, 299.0),
        "precision": precision,
    }


def nonlinear_callaway_film(particles: float = 1e7, seed: int = 12345, precision: str = "fp64") -> dict:
    """The cross-plane film with nonlinear Callaway collisions
    (scattering.callaway_formulation = "nonlinear"; absolute occupations,
    conservative boundaries, fixed 300 K rates); 8^3 Callaway table."""
    c = cross_plane_film(particles, seed, precision)
    c.update(name="nonlinear_callaway_film", collision_model="callaway", callaway_formulation="nonlinear")
    return c


def inplane_gradient(particles: float = 5e7, seed: int = 12345, precision: str = "fp64") -> dict:
    return {
        "name": "inplane_gradient",
        "sizes": (LATERAL_A, LATERAL_A, THICKNESS_A),
        "particle_count": particles,
        "time_step": 0.5,
        "iterations": 4000,
        "random_seed": seed,
        "compute_kappa": True,
        "transport_axis": 0,
        "temperature_gradient": 1e7,
        "background_temperature": 300.0,
        "lifetime_temperature": 300.0,
        "initial_temperature": 300.0,
        "grid": (1, 1, 100),
        "faces": ("P", "P", "P", "P", "R", "R"),
        "face_values": (0, 0, 0, 0, 1.0, 1.0),
        "precision": precision,
    }


def bilayer_callaway(particles: float = 1e8, seed: int = 12345, precision: str = "fp64") -> dict:
    return {
        "name": "bilayer_callaway",
        "sizes": (LATERAL_A, LATERAL_A, 2.0 * THICKNESS_A),
        "particle_count": particles,
        "time_step": 0.5,
        "iterations": 3000,
        "random_seed": seed,
        "compute_kappa": True,
        "transport_axis": 2,
        "background_temperature": 300.0,
        "lifetime_temperature": 300.0,
        "initial_temperature": "linear",
        "grid": (1, 1, 100),
        "faces": ("P", "P", "P", "P", "T", "T"),
        "face_values": (0, 0, 0, 0, 310.0, 290.0),
        "collision_model": "callaway",
        "material_interface_axis": 2,
        "material_interface_positions": [THICKNESS_A],
        "interface_frequency_bin_thz": 0.1,
        "precision": precision,
    }


def bilayer_amm(particles: float = 1e7, seed: int = 12345, precision: str = "fp64", model: str = "amm",
                amm_fraction: float = 1.0) -> dict:
    """The bilayer stack with the acoustic-mismatch interface model (or the
    mixed model with `amm_fraction`): nonlinear RTA with lifetimes fixed at
    300 K, mass densities 2329 / 5323 kg/m^3, the plain 8^3 synthetic table and
    its softened copy (bilayer_materials(8, callaway=False))."""
    c = bilayer_callaway(particles, seed, precision)
    c.update(name="bilayer_amm", collision_model="rta", interface_model=model, mass_densities_kg_m3=[2329.0, 5323.0])
    if model == "mmm":
        c["interface_amm_fraction"] = amm_fraction
    return c


def heated_film(particles: float = 1e6, seed: int = 12345, precision: str = "fp64", spectrum: str = "thermal") -> dict:
    c = cross_plane_film(particles, seed, precision)
    c.update(name="heated_film", face_values=(0, 0, 0, 0, 300.0, 300.0), initial_temperature=300.0,
             lifetime_temperature="local")
    hs = {"profile": "gaussian", "center": (0.5 * LATERAL_A, 0.5 * LATERAL_A, 0.5 * THICKNESS_A),
          "sigma": (0.0, 0.0, 100.0), "power_density": 1e18, "spectrum": spectrum}
    if spectrum == "weighted":
        hs.update(branch_weights=[1.0, 1.0, 2.0, 0.5, 0.5, 0.5])
    if spectrum == "gaussian":
        hs.update(frequency_center=6.0, frequency_sigma=2.0)
    c["heat_source"] = hs
    return c


def batched_films(n: int = 512, seed: int = 0, precision: str = "mixed", particles_per_10nm: float = 5e3) -> list:
    """Thickness sweep of independent cross-plane films: thickness log-uniform
    in 10-2000 nm from `seed`, one cell per 10 nm clamped to 10-200 cells,
    carriers proportional to thickness clamped to 1e4-1e6 (about 1e8 in all
    for 512 films), reservoirs 301/299 K, fixed 300 K lifetimes, dt = 1 ps,
    a distinct random seed per film."""
    import numpy as np
    rng = np.random.default_rng(seed)
    t_nm = np.exp(rng.uniform(np.log(10.0), np.log(2000.0), size=n))
    films = []
    for k, t in enumerate(t_nm):
        c = cross_plane_film(precision=precision)
        c["name"] = "batched_films"
        c["sizes"] = (LATERAL_A, LATERAL_A, float(t) * 10.0)
        c["grid"] = (1, 1, int(min(200, max(10, round(t / 10.0)))))
        c["particle_count"] = float(min(1e6, max(1e4, round(particles_per_10nm * t / 10.0))))
        c["random_seed"] = 1000 + k
        films.append(c)
    return films


def bilayer_materials(mesh: int = 8, callaway: bool = True):
    """The two synthetic materials of the bilayer (Callaway linewidth split
    unless callaway is False). Callaway tables are completed over the first
    Brillouin zone as the reference does: 8^3 q-points x 6 branches become
    24,552 modes."""
    from . import synthetic
    return [synthetic.make_material(mesh=mesh, callaway=callaway),
            synthetic.make_material(mesh=mesh, freq_scale=0.7, vel_scale=0.75, callaway=callaway)]


def scaled(cfg: dict, particles: float, **over) -> dict:
    c = copy.deepcopy(cfg)
    c["particle_count"] = particles
    c.update(over)
    return c


# FinFET mesh domain (10 nm fin, 40 nm tall, on a 200 x 100 x 50 nm slab):
# x and y sides periodic, the slab bottom a 300 K heat sink, every other wall
# rough (1 nm). Regions are relative boxes over the bounding box, in order.
FINFET_REGIONS = [
    ((0.0, 0.0, 0.001, 1.0, 1.0, 1.01), "R", 1.0),
    ((-0.001, 0.0, 0.0, 0.001, 1.0, 1.0), "P", 0.0), ((0.999, 0.0, 0.0, 1.001, 1.0, 1.0), "P", 0.0),
    ((0.0, -0.001, 0.0, 1.0, 0.001, 1.0), "P", 0.0), ((0.0, 0.999, 0.0, 1.0, 1.001, 1.0), "P", 0.0),
    ((0.0, 0.0, -0.001, 1.0, 1.0, 0.001), "T", 300.0),
]
FINFET_PAIRS = [r[0] for r in FINFET_REGIONS[1:5]]
# Gaussian heat source at the fin top (lengths in Angstrom)
FINFET_SOURCE = {"profile": "gaussian", "center": (1000.0, 500.0, 900.0), "sigma": (50.0, 50.0, 50.0),
                 "min": (900.0, 0.0, 700.0), "max": (1100.0, 1000.0, 910.0), "power_density": 1e20,
                 "spectrum": "thermal"}


def finfet_stl(path: str, seed: int = 0) -> str:
    """Writes the procedural FinFET surface (about 6,300 triangles) as binary STL."""
    from . import synthetic
    synthetic.write_stl(path, *synthetic.finfet_mesh(seed=seed))
    return path


def finfet_mesh(stl_path: str, particles: float = 2e7, seed: int = 12345, precision: str = "fp64",
                grid=(64, 32, 32), heat_source: bool = True, time_step: float = 0.1) -> dict:
    """FinFET with localized heating: the mesh domain read from `stl_path`,
    local RTA lifetimes, 300 K background and start, Gaussian 1e20 W/m^3 source
    of sigma 5 nm at the fin top with thermal spectrum."""
    c = {"name": "finfet_mesh", "particle_count": float(particles), "time_step": time_step, "iterations": 3000,
         "random_seed": seed, "compute_kappa": False, "background_temperature": 300.0,
         "lifetime_temperature": "local", "initial_temperature": 300.0, "grid": tuple(grid), "precision": precision,
         "mesh": {"model": stl_path, "regions": FINFET_REGIONS, "periodic_pair": FINFET_PAIRS}}
    if heat_source:
        c["heat_source"] = dict(FINFET_SOURCE)
    return c


# Extruded L-shaped prism (synthetic.prism_mesh): 310 K top, 300 K bottom,
# rough (1 nm) side walls; a constant-height prism gridded by exact cut cells.
PRISM_REGIONS = [
    ((-0.01, -0.01, -0.01, 1.01, 1.01, 1.01), "R", 1.0),
    ((-0.01, -0.01, -0.001, 1.01, 1.01, 0.001), "T", 300.0),
    ((-0.01, -0.01, 0.999, 1.01, 1.01, 1.001), "T", 310.0),
]


def prism_stl(path: str) -> str:
    """Writes the L-shaped prism (14 vertices, 24 triangles) as binary STL."""
    from . import synthetic
    synthetic.write_stl(path, *synthetic.prism_mesh())
    return path


def prism_film(stl_path: str, particles: float = 2e4, seed: int = 5, precision: str = "fp64",
               grid=(8, 6, 5)) -> dict:
    """Cross-plane heat flow through the extruded L prism (geometry.extruded_z)."""
    return {"name": "prism_film", "particle_count": float(particles), "time_step": 0.5, "iterations": 2000,
            "random_seed": seed, "compute_kappa": False, "background_temperature": 305.0,
            "lifetime_temperature": 305.0, "initial_temperature": 305.0, "grid": tuple(grid),
            "precision": precision,
            "mesh": {"model": stl_path, "regions": PRISM_REGIONS, "extruded_z": True}}


def finfet_regions(centers):
    """Cell masks of the FinFET: the fin above the 50 nm slab, the upper and the
    lower half of the slab (cell centres in Angstrom)."""
    import numpy as np
    z = np.asarray(centers)[:, 2]
    return {"fin": z > 500.0, "top": (z > 250.0) & (z <= 500.0), "bottom": z <= 250.0}


def finfet_aggregates(T_steps, energy, absorbed_total, centers, first_step):
    """Late-time means from step `first_step` on: region temperatures, thermal
    energy, and absorbed carriers per step (inputs indexed by step - 1)."""
    import numpy as np
    T = np.asarray(T_steps)[first_step - 1:]
    out = {k: float(T[:, m].mean()) for k, m in finfet_regions(centers).items()}
    out["energy"] = float(np.mean(np.asarray(energy)[first_step - 1:]))
    a = np.asarray(absorbed_total, dtype=float)
    out["absorbed_per_step"] = float((a[-1] - a[first_step - 2]) / (len(a) - first_step + 1))
    return out
