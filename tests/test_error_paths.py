"""Failure detection without a GPU fault: invalid states made on the host.

Every failure the reference raises from inside the carrier loop has a device
counterpart that records an error word and returns (no trap, no hang); the
host raises the reference's exception text at its next synchronisation and the
solver stays latched, as MonteCarloSolver::run_timestep does after a throw
(src/MonteCarloSolver.cpp:349-354). Each case runs on the CPU oracle here and
on the device under -m gpu:

* more than 64 wall events in one step: a 1 nm periodic cube crossed many
  times per 10 ps step (src/solver/TransportOperator.cpp:252-284);
* a non-finite occupation in the population (GridStatistics.cpp:140-161);
* a carrier outside the domain: a moving one fails its wall trace
  (TransportOperator.cpp:252-284), a stationary one is found by the
  containment check of step 0 (TransportOperator.cpp:364-402);
* a surface mesh with a collapsed triangle, rejected on the host when the
  domain is built (src/SurfaceMesh.cpp:305-313).
"""

import numpy as np
import pytest

from phonomc_gb300 import abi, synthetic, workloads

LATCHED = "Cannot resume a failed timestep"


def _libs(which):
    if which == "oracle":
        import oracle
        return oracle.load(), "orc_"
    import phonomc_gb300
    return phonomc_gb300.lib(), "phmc_"


def _tiny_periodic_cube(seed=3):
    c = workloads.scaled(workloads.cross_plane_film(), 2000, random_seed=seed)
    c.update(sizes=(10.0, 10.0, 10.0), grid=(1, 1, 1), time_step=10.0, faces=("P",) * 6, face_values=(0.0,) * 6,
             initial_temperature=300.0, compute_kappa=False, transport_axis=-1)
    return c


def _run_expect(s, steps, text):
    with pytest.raises(abi.LibError) as e:
        s.run(steps)
        s.stats()  # device errors surface at the next synchronisation
    assert text in str(e.value), str(e.value)
    with pytest.raises(abi.LibError) as e2:
        s.run(1)
    assert LATCHED in str(e2.value), str(e2.value)


def _too_many_events(which):
    lib, pre = _libs(which)
    m = abi.Material(lib, pre, synthetic.make_material(mesh=8), 0.1, False, False)
    s = abi.Solver(lib, pre, _tiny_periodic_cube(), [m])
    _run_expect(s, 1, "exceeded 64 transport events in one timestep")


def _non_finite_occupation(which):
    lib, pre = _libs(which)
    m = abi.Material(lib, pre, synthetic.make_material(mesh=8), 0.1, False, False)
    s = abi.Solver(lib, pre, workloads.scaled(workloads.cross_plane_film(), 3000, random_seed=4), [m])
    c = s.carriers()
    live = np.flatnonzero(c["alive"] == 1)
    c = {k: v[live].copy() for k, v in c.items()}
    c["occ"][17] = np.nan
    # the population's statistics are refreshed when it is replaced: the
    # error comes from set_carriers or, at the latest, from the first step
    with pytest.raises(abi.LibError) as e:
        s.set_carriers(c)
        s.run(1)
        s.stats()
    assert "Invalid particle in grid energy statistics." in str(e.value), str(e.value)
    with pytest.raises(abi.LibError) as e2:
        s.run(1)
        s.stats()


def _outside_carrier(which, stationary):
    """One carrier moved 49 repeat cells beyond the film in x. A moving carrier
    finds no wall ahead that it could reach inside the box: the wall trace
    fails. A carrier of a zero-velocity mode (the in-plane gradient film keeps
    them) drifts without events, and the containment check of step 0 reports it."""
    lib, pre = _libs(which)
    mat = synthetic.make_material(mesh=8)
    m = abi.Material(lib, pre, mat, 0.1, True, False)
    cfg = workloads.scaled(workloads.inplane_gradient(), 3000, random_seed=6)
    s = abi.Solver(lib, pre, cfg, [m])
    c = s.carriers()
    live = np.flatnonzero(c["alive"] == 1)
    c = {k: v[live].copy() for k, v in c.items()}
    if stationary:
        flats = np.flatnonzero(np.asarray(mat.frequency_thz).ravel() > 0.0)  # active modes, in order
        v = np.asarray(mat.group_velocity).reshape(-1, 3)[flats]
        c["mode"][5] = np.uint32(np.flatnonzero(np.all(v == 0.0, axis=1))[0])
    else:
        v = np.asarray(mat.group_velocity).reshape(-1, 3)[np.flatnonzero(np.asarray(mat.frequency_thz).ravel() > 0.0)]
        assert np.any(v[c["mode"][5] & 0xFFFFFF] != 0.0)
    c["x"][5] = 5.0e4
    s.set_carriers(c)
    _run_expect(s, 1, "escaped the domain" if stationary else "Boundary intersection failed")


def _open_mesh(which, tmp_path):
    lib, pre = _libs(which)
    m = abi.Material(lib, pre, synthetic.make_material(mesh=8), 0.1, False, False)
    v, f = synthetic.finfet_mesh()
    f = np.array(f)
    f[-1, 2] = f[-1, 0]  # one triangle collapsed onto an edge: zero area, open edges
    path = str(tmp_path / "open.stl")
    synthetic.write_stl(path, v, f)
    cfg = workloads.finfet_mesh(path, particles=2000, seed=1, grid=(8, 4, 4), heat_source=False)
    with pytest.raises(abi.LibError) as e:
        abi.Solver(lib, pre, cfg, [m])
    assert "Degenerate triangle" in str(e.value) or "Surface mesh" in str(e.value), str(e.value)


CASES = {"too_many_events": _too_many_events, "non_finite_occupation": _non_finite_occupation,
         "escaped_carrier": lambda w: _outside_carrier(w, True), "lost_carrier": lambda w: _outside_carrier(w, False)}


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_error_paths(case):
    CASES[case]("oracle")


def test_oracle_rejects_open_mesh(tmp_path):
    _open_mesh("oracle", tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_device_error_paths(case):
    CASES[case]("gpu")


@pytest.mark.gpu
def test_device_rejects_open_mesh(tmp_path):
    _open_mesh("gpu", tmp_path)


@pytest.mark.gpu
def test_device_error_paths_mixed():
    """The FP32 flight raises the same errors: too many events, escaped carrier."""
    lib, pre = _libs("gpu")
    m = abi.Material(lib, pre, synthetic.make_material(mesh=8), 0.1, False, False)
    s = abi.Solver(lib, pre, dict(_tiny_periodic_cube(), precision="mixed"), [m])
    _run_expect(s, 1, "exceeded 64 transport events in one timestep")
