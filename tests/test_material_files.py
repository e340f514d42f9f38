"""Material tables in the reference's on-disk layout (POSCAR + HDF5), read and
written without libhdf5 (phonomc_gb300/csrc/phmc_hdf5.cpp).

* Round trip: a synthetic Callaway table (gamma_N, gamma_U, gamma_isotope)
  written by phmc_material_save is read back dataset by dataset bit for bit,
  and a material loaded from the folder (phmc_material_load, the reference's
  read_material_data + PhononMaterial path) has the same modes and lattice as
  the in-memory one.
* The reference's bundled Si tables (chunked, deflate-compressed phono3py
  files; read only where the reference checkout is present): the full-zone
  file and the irreducible file agree bit for bit through the full-zone file's
  own source-index map; the stored per-mode conductivity equals
  C v(x)v / gamma times half the stored unit conversion, which ties four
  datasets of the file together; the reference's shape checks and file choice
  accept the folder and its messages reject a broken one.
"""

import os

import numpy as np
import pytest

import oracle

from phonomc_gb300 import abi, synthetic

REF = oracle.reference_root() or ""
SI = os.path.join(REF, "material", "Si")


@pytest.fixture(scope="module")
def lib():
    from phonomc_gb300 import native
    return native.lib()


def test_material_folder_round_trip(lib, tmp_path):
    d = synthetic.make_material(mesh=8, callaway=True)
    folder = str(tmp_path / "m8c")
    abi.save_material(lib, d, folder)
    h5 = os.path.join(folder, "kappa-fbz.hdf5")
    nq, nb = d.qpoints, d.branches
    assert np.array_equal(abi.h5_read(lib, h5, "frequency"), np.asarray(d.frequency_thz).reshape(nq, nb))
    assert np.array_equal(abi.h5_read(lib, h5, "qpoint"), np.asarray(d.qpoint_fractions).reshape(nq, 3))
    assert np.array_equal(abi.h5_read(lib, h5, "group_velocity"), np.asarray(d.group_velocity).reshape(nq, nb, 3))
    assert np.array_equal(abi.h5_read(lib, h5, "temperature"), np.asarray(d.temperatures))
    nT = len(d.temperatures)
    for name, arr in (("gamma", d.gamma), ("gamma_N", d.gamma_normal), ("gamma_U", d.gamma_umklapp)):
        assert np.array_equal(abi.h5_read(lib, h5, name), np.asarray(arr).reshape(nT, nq, nb)), name
    iso = np.asarray(d.gamma_resistive["gamma_isotope"])
    assert np.array_equal(abi.h5_read(lib, h5, "gamma_isotope").ravel(), iso)
    assert np.array_equal(abi.h5_read(lib, h5, "mesh"), np.asarray(d.mesh, dtype=float))
    assert np.array_equal(abi.h5_read(lib, h5, "weight"), np.ones(nq))
    # the folder as a material: same modes, lattice from the POSCAR
    for stationary, bz in ((False, False), (True, True)):
        mem = abi.Material(lib, "phmc_", d, 0.1, stationary, bz)
        disk = abi.FolderMaterial(lib, folder, 0.1, stationary, bz)
        a, b = abi.C.c_int32(), abi.C.c_int32()
        assert lib.phmc_material_active_count(mem.h, abi.C.byref(a)) == 0
        assert lib.phmc_material_active_count(disk.h, abi.C.byref(b)) == 0
        assert a.value == b.value > 0


def test_material_folder_errors(lib, tmp_path):
    d = synthetic.make_material(mesh=4)
    folder = tmp_path / "m4"
    abi.save_material(lib, d, str(folder))
    os.rename(folder / "kappa-fbz.hdf5", folder / "a.hdf5")
    abi.FolderMaterial(lib, str(folder))  # a single *.hdf5 is accepted
    (folder / "b.hdf5").write_bytes((folder / "a.hdf5").read_bytes())
    with pytest.raises(abi.LibError, match="Ambiguous HDF5 files"):
        abi.FolderMaterial(lib, str(folder))
    os.remove(folder / "POSCAR")
    with pytest.raises(abi.LibError, match="Strict POSCAR loading failed: POSCAR not found"):
        abi.FolderMaterial(lib, str(folder))
    empty = tmp_path / "empty"
    empty.mkdir()
    (empty / "POSCAR").write_text("x\n1.0\n3 0 0\n0 3 0\n0 0 3\nX\n1\nDirect\n0 0 0\n")
    with pytest.raises(abi.LibError, match="No HDF5 file found under material folder"):
        abi.FolderMaterial(lib, str(empty))


@pytest.mark.skipif(not (REF and os.path.isdir(SI)), reason="reference material folders not present")
def test_bundled_si_tables_are_read_consistently(lib):
    full, irr = os.path.join(SI, "kappa-fbz.hdf5"), os.path.join(SI, "kappa.hdf5")
    src = abi.h5_read(lib, full, "_fbz_src_q_index").astype(int)
    for name in ("frequency", "gv_by_gv"):
        a, b = abi.h5_read(lib, full, name), abi.h5_read(lib, irr, name)
        assert np.array_equal(a, b[src]), name
    gf, gi = abi.h5_read(lib, full, "gamma"), abi.h5_read(lib, irr, "gamma")
    assert np.array_equal(gf, gi[:, src])
    w = abi.h5_read(lib, irr, "weight")
    assert w.sum() == src.size and np.all(np.bincount(src, minlength=w.size) == w)
    assert np.array_equal(abi.h5_read(lib, full, "mesh"), [31.0, 31.0, 31.0])
    # mode_kappa = C v(x)v conversion / (2 gamma), mode by mode
    C = abi.h5_read(lib, irr, "heat_capacity")
    gbg = abi.h5_read(lib, irr, "gv_by_gv")
    mk = abi.h5_read(lib, irr, "mode_kappa")
    conv = float(abi.h5_read(lib, irr, "kappa_unit_conversion"))
    for ti in (30, 100):
        m = (gi[ti] > 0) & (C[ti] > 1e-12) & (np.abs(gbg[..., 0]) > 1e-6)
        r = mk[ti][..., 0][m] / (C[ti][m] * gbg[..., 0][m] / gi[ti][m])
        assert abs(np.median(r) / (0.5 * conv) - 1.0) < 1e-6
        assert np.mean(np.abs(r / (0.5 * conv) - 1.0) < 1e-4) > 0.99
    # the folder through the reference's checks: kappa-fbz.hdf5 chosen, a material built
    m = abi.FolderMaterial(lib, SI, 0.1, False, False)
    n = abi.C.c_int32()
    assert lib.phmc_material_active_count(m.h, abi.C.byref(n)) == 0 and n.value > 6 * 29000
