"""Named workloads (SimulationConfig dicts in internal units: Angstrom, ps, K).

cross_plane_film   100 nm box, periodic in x/y, reservoirs 301/299 K on the z
                   faces, 50 z-cells, nonlinear RTA with lifetimes fixed at
                   300 K, 1e6 carriers, dt = 1 ps (2000 steps in the full run).
inplane_gradient   100 nm film, periodic in x/y, rough z walls (1 nm RMS),
                   periodic-gradient drive G = 1e7 K/m along x, 100 z-cells,
                   linearized RTA at 300 K, 5e7 carriers, dt = 0.5 ps.

The lateral repeat cell is 100 nm x 100 nm in both. `scaled()` keeps the
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


def scaled(cfg: dict, particles: float, **over) -> dict:
    c = copy.deepcopy(cfg)
    c["particle_count"] = particles
    c.update(over)
    return c
