"""Extruded-prism domains (geometry.extruded_z) against the reference's
SimulationDomain (golden domain_prism: tests/golden/make_golden.py, the L
prism of phonomc_gb300.synthetic.prism_mesh).

The host domain reads the STL, validates the prism (vertical sides, flat top
and bottom), grids it by exact cut cells (the top triangles clipped to each
voxel column, long-double areas and centroids) and traces it by its facets
(src/SimulationDomain.cpp:206-260, 344-396, 650-740). Facets, conditions,
cells, volumes, the voxel map, membership (the ray cast alone) and 600 traces
from inside points are compared with the reference's; the device trace (FP64
edge functions where the reference takes long double) and whole timesteps of
a prism film are compared with the host and the oracle under -m gpu.
"""
import numpy as np
import pytest

from conftest import golden


@pytest.fixture(scope="module")
def prism(tmp_path_factory):
    from phonomc_gb300 import abi, native, workloads
    stl = workloads.prism_stl(str(tmp_path_factory.mktemp("prism") / "prism.stl"))
    d = abi.Domain(native.lib(), workloads.prism_film(stl))
    yield d
    d.close()


def test_prism_surface_facets_and_conditions(prism):
    g = golden("domain_prism")
    assert prism.volume == g["volume"]
    assert prism.bounds.ravel().tolist() == g["bounds"]
    V = np.asarray(g["vertices"])
    assert np.array_equal(V[np.asarray(g["faces"]).reshape(-1, 3)], prism.faces()["triangles"])
    F = prism.facets()
    assert np.array_equal(np.asarray(g["facet_normals"]), F["normal"])
    assert np.array_equal(np.asarray(g["facet_centroids"]), F["centroid"])
    assert F["condition"] == g["conditions"]
    assert np.array_equal(np.asarray(g["values"]), F["value"])


def test_prism_cut_cells(prism):
    """Cut-cell centres and volumes exact; they close to the prism volume."""
    g = golden("domain_prism")
    C = prism.cells()
    assert prism.n_cells == len(g["grid_volumes"])
    assert np.array_equal(np.asarray(g["grid_centers"]), C["centers"])
    assert np.array_equal(np.asarray(g["grid_volumes"]), C["volumes"])
    assert np.array_equal(np.asarray(g["voxel_cell"]), C["voxel_cell"])
    assert abs(C["volumes"].sum() - g["volume"]) < 1e-8 * g["volume"]
    # partial columns at the inner corner: not every cell holds a full voxel
    assert len(np.unique(np.round(C["volumes"], 6))) > 2


def test_prism_membership_and_cells_of_points(prism):
    g = golden("domain_prism")
    P = np.asarray(g["points"])
    assert np.array_equal(np.asarray(g["inside"]), prism.contains(P))
    assert np.array_equal(np.asarray(g["cell"]), prism.grid_index(P))


def test_prism_traces(prism):
    """The facet-scan trace: facets exact, hit points and times to 1e-12."""
    g = golden("domain_prism")
    hit, t, f = prism.trace(np.asarray(g["trace_p"]), np.asarray(g["trace_v"]))
    assert np.array_equal(np.asarray(g["trace_facet"]), f)
    assert np.max(np.abs(hit - np.asarray(g["trace_hit"]))) <= 1e-12 * 1000.0
    assert np.allclose(t, np.asarray(g["trace_t"]), rtol=1e-12, atol=0)


def test_prism_rejects_a_non_prism(tmp_path):
    from phonomc_gb300 import abi, native, workloads
    stl = workloads.finfet_stl(str(tmp_path / "f.stl"))
    cfg = workloads.finfet_mesh(stl)
    cfg["mesh"] = dict(cfg["mesh"], extruded_z=True)
    with pytest.raises(abi.LibError, match="extruded_z requires vertical sides and planar top/bottom"):
        abi.Domain(native.lib(), cfg)


def test_oracle_prism_film_closes_energy(tmp_path):
    """The oracle steps a prism film: injection from both reservoirs, rough
    side walls, energy closing to round-off."""
    import oracle
    from phonomc_gb300 import abi, synthetic, workloads
    lib = oracle.load()
    stl = workloads.prism_stl(str(tmp_path / "p.stl"))
    m = abi.Material(lib, "orc_", synthetic.make_material(mesh=8), 0.1, False, False)
    s = abi.Solver(lib, "orc_", workloads.prism_film(stl, particles=5000), [m])
    s.run(20)
    st = s.stats()
    assert st["absorbed_total"] > 0 and st["injected_total"] > 0
    assert abs(st["total_energy_balance_residual_ev"]) < 1e-9 * abs(st["total_thermal_energy_ev"])
    T, _, _ = s.cells()
    assert np.all((T > 295) & (T < 315))


@pytest.mark.gpu
def test_device_prism_traces_match_host(prism):
    from phonomc_gb300 import abi
    g = golden("domain_prism")
    P, V = np.asarray(g["trace_p"]), np.asarray(g["trace_v"])
    hit, t, f = prism.device_trace(P, V)
    assert np.array_equal(np.asarray(g["trace_facet"]), f)
    assert np.max(np.abs(hit - np.asarray(g["trace_hit"]))) <= 1e-12 * 1000.0
    assert np.allclose(t, np.asarray(g["trace_t"]), rtol=1e-12, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_prism_film_steps(tmp_path, precision):
    """Whole timesteps of the prism film: the plain state matches the oracle
    (alive, modes, cells exact; positions and temperatures to 1e-11); the
    mixed state closes energy and tracks the plain cells."""
    import oracle
    import phonomc_gb300
    from phonomc_gb300 import abi, synthetic, workloads
    gpu, orc = phonomc_gb300.lib(), oracle.load()
    stl = workloads.prism_stl(str(tmp_path / "p.stl"))
    mat = synthetic.make_material(mesh=8)
    cfg = workloads.prism_film(stl, particles=20000, precision=precision)
    sg = abi.Solver(gpu, "phmc_", cfg, [abi.Material(gpu, "phmc_", mat, 0.1, False, False)])
    so = abi.Solver(orc, "orc_", dict(cfg, precision="fp64"), [abi.Material(orc, "orc_", mat, 0.1, False, False)])
    sg.run(6)
    so.run(6)
    cg, co = sg.carriers(), so.carriers()
    Tg, _, _ = sg.cells()
    To, _, _ = so.cells()
    st = sg.stats()
    assert abs(st["total_energy_balance_residual_ev"]) < 1e-9 * abs(st["total_thermal_energy_ev"])
    if precision == "fp64":
        assert np.array_equal(cg["alive"], co["alive"])
        a = cg["alive"] == 1
        assert np.array_equal(cg["mode"][a], co["mode"][a])
        assert np.array_equal(cg["cell"][a], co["cell"][a])
        for k in ("x", "y", "z"):
            assert np.max(np.abs(cg[k][a] - co[k][a])) <= 1e-11 * 1000.0
        assert np.allclose(Tg, To, rtol=1e-11, atol=0)
    else:
        assert np.mean(np.abs(Tg - To) < 1e-3) > 0.95
