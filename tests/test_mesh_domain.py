"""Mesh-domain host geometry against the reference's SimulationDomain
(golden domain_finfet: tests/golden/make_golden.py, the FinFET TOML).

The STL is regenerated from its seed; the library reads it, merges vertices,
orients and groups the faces, assigns the boundary regions and periodic pairs
and builds the cells and voxel map. Everything is compared bit for bit: the
oriented triangles, face -> facet map, facet normals / centroids / areas,
conditions and values, periodic partners and shifts, cell centres, volumes,
the voxel -> cell map, and membership, nearest facet and cell of random
points."""
import numpy as np
import pytest

from conftest import golden


@pytest.fixture(scope="module")
def finfet(tmp_path_factory):
    from phonomc_gb300 import abi, native, workloads
    stl = workloads.finfet_stl(str(tmp_path_factory.mktemp("mesh") / "finfet.stl"))
    d = abi.Domain(native.lib(), workloads.finfet_mesh(stl))
    yield d
    d.close()


def test_surface_and_facets(finfet):
    g = golden("domain_finfet")
    assert finfet.volume == g["volume"]
    assert finfet.bounds.ravel().tolist() == g["bounds"]
    V = np.asarray(g["vertices"])
    tri = V[np.asarray(g["faces"]).reshape(-1, 3)]
    fa = finfet.faces()
    assert np.array_equal(tri, fa["triangles"])  # same merge, shift and winding
    assert np.array_equal(np.asarray(g["face_to_facet"]), fa["face_to_facet"])
    F = finfet.facets()
    assert np.array_equal(np.asarray(g["facet_normals"]), F["normal"])
    assert np.array_equal(np.asarray(g["facet_centroids"]), F["centroid"])
    assert np.array_equal(np.asarray(g["facet_areas"]), F["area"])


def test_boundary_assignment(finfet):
    g = golden("domain_finfet")
    F = finfet.facets()
    assert F["condition"] == g["conditions"]
    assert np.array_equal(np.asarray(g["values"]), F["value"])
    assert np.array_equal(np.asarray(g["pair"]), F["pair"])
    assert np.array_equal(np.asarray(g["shift"]), F["shift"])
    assert F["condition"].count("P") == 4 and F["condition"].count("T") == 1


def test_cells_and_queries(finfet):
    g = golden("domain_finfet")
    C = finfet.cells()
    assert finfet.n_cells == len(g["grid_volumes"])
    assert np.array_equal(np.asarray(g["grid_centers"]), C["centers"])
    assert np.array_equal(np.asarray(g["grid_volumes"]), C["volumes"])
    assert np.array_equal(np.asarray(g["voxel_cell"]), C["voxel_cell"])
    P = np.asarray(g["points"])
    assert np.array_equal(np.asarray(g["inside"]), finfet.contains(P))
    assert np.array_equal(np.asarray(g["nearest_facet"]), finfet.nearest_facet(P))
    assert np.array_equal(np.asarray(g["cell"]), finfet.grid_index(P))


def test_interior_voxels_lie_inside(finfet):
    """Voxels flagged interior (no face's bounding box reaches them, centre
    inside) hold only inside points -- the containment check of the carrier
    loop skips the ray cast there. Random points of every interior voxel,
    including its corners, are inside by the reference's membership test, and
    the flags cover most of the inside voxels."""
    I = finfet.voxel_interior()
    C = finfet.cells()
    assert I.shape == finfet.shape
    inside_voxels = C["voxel_cell"].reshape(finfet.shape) >= 0
    flagged = np.argwhere(I == 1)
    assert len(flagged) > 0.5 * finfet.n_cells
    lo, hi = finfet.bounds
    size = (hi - lo) / np.asarray(finfet.shape)
    rng = np.random.default_rng(3)
    pick = flagged[rng.choice(len(flagged), size=min(len(flagged), 4000), replace=False)]
    u = rng.random((len(pick), 3))
    u[:200] = np.round(u[:200])  # box corners
    P = lo + (pick + u) * size
    assert finfet.contains(P).all()
    # an interior voxel's centre makes a cell (membership of its centre)
    assert inside_voxels[I == 1].all()


def test_region_errors(tmp_path):
    """Configuration errors surface with the reference's messages."""
    from phonomc_gb300 import abi, native, workloads
    stl = workloads.finfet_stl(str(tmp_path / "f.stl"))
    cfg = workloads.finfet_mesh(stl)
    cfg["mesh"] = dict(cfg["mesh"], periodic_pair=cfg["mesh"]["periodic_pair"][:2])
    with pytest.raises(abi.LibError, match="is not assigned to a periodic pair"):
        abi.Domain(native.lib(), cfg)
    cfg = workloads.finfet_mesh(stl)
    cfg["mesh"] = dict(cfg["mesh"], regions=cfg["mesh"]["regions"] + [((0.5, 0.5, -1.0, 0.5, 0.5, -0.9), "T", 300.0)])
    with pytest.raises(abi.LibError, match="did not match any mesh facet"):
        abi.Domain(native.lib(), cfg)


def test_domain_summary_and_grid_centers(tmp_path):
    """summary.txt (domain part) and grid_centers.csv as the reference's
    SimulationDomain writes them for the FinFET TOML; only the paths differ."""
    from phonomc_gb300 import abi, native, workloads
    g = golden("domain_finfet")
    stl = workloads.finfet_stl(str(tmp_path / "finfet.stl"))
    out = tmp_path / "out"
    cfg = workloads.finfet_mesh(stl, particles=2000, seed=5)
    cfg.update(iterations=1, convergence_write_interval=1, output_folder=str(out), material_folder="unused")
    d = abi.Domain(native.lib(), cfg)
    mine = (out / "summary.txt").read_text().splitlines()
    ref = g["domain_summary"].splitlines()
    path_keys = ("model = ", "output_folder = ", "grid_centers_csv = ")
    assert len(mine) == len(ref)
    for a, b in zip(mine, ref):
        if a.startswith(path_keys):
            assert a.split(" = ")[0] == b.split(" = ")[0]
        else:
            assert a == b
    rows = (out / "grid_centers.csv").read_text().splitlines()
    assert rows[0] == "index,x_nm,y_nm,z_nm,volume_nm3"
    C, V = g["grid_centers"], g["grid_volumes"]
    assert len(rows) == len(C) + 1
    for i in (0, 1, len(C) // 2, len(C) - 1):
        c = C[i]
        assert rows[i + 1] == "%d,%g,%g,%g,%g" % (i, c[0] / 10.0, c[1] / 10.0, c[2] / 10.0, V[i] / 1000.0)
    d.close()
