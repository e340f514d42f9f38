"""The drop-in boundary compiled as a maintainer would add it to PhonoMC.

tests/binding/main_gb300.cpp is the reference's main program with the GB300
carrier loop bound through include/phonomc_gb300.h: the reference's own TOML
loader, SimulationDomain and HDF5 material reader (its build in oracle/_ref)
fill phmc_material_data and phmc_config. The program is compiled here against
the reference's headers and linked with libphonomc_gb300.so; its "check" mode
builds the library's host domain and material from those structs and compares
them with the reference's (cells, volumes, centres, box face conditions and
values, active modes). The in-plane gradient film and the cross-plane film
are read from TOML files with their material in the reference's folder layout
(POSCAR + kappa-fbz.hdf5 written by phmc_material_save).

Needs the reference sources (PHONOMC_REFERENCE, or the checkout oracle/_ref
was built from; skipped without them). The
device run of the same program ("run" mode) needs a GPU and the reference
build, which exist together only where the reference is checked out.
"""

import json
import os
import subprocess

import pytest

import oracle

from phonomc_gb300 import abi, synthetic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.reference_root() or ""
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libphonomc_ref.a")

pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "include")) and os.path.exists(REF_LIB)),
                                reason="reference sources or oracle/_ref build not present")

TOML = """[geometry]
model = "box"
sizes = [100, 100, 100]

[simulation]
particle_count = 20000
time_step = {dt}
iterations = 3
random_seed = 5
compute_kappa = true
transport_axis = "{axis}"
initial_temperature = {init}
background_temperature = 300
lifetime_temperature = 300
grid_xyz = [1, 1, {cells}]
convergence_write_interval = 1
{driving}
[boundary]
boundary_position = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1],
  [0,0,-0.01,1,1,0.01], [0,0,0.99,1,1,1.01]
]
boundary_conditions = ["P","P","P","P","{zc}","{zc}"]
boundary_values = [0,0,0,0,{z0},{z1}]
periodic_pair = [
  [-0.01,0,0,0.01,1,1], [0.99,0,0,1.01,1,1],
  [0,-0.01,0,1,0.01,1], [0,0.99,0,1,1.01,1]
]

[io]
material_folder = "{material}"
output_folder = "{out}"
"""

CASES = {
    "inplane_gradient": dict(dt=0.5, axis="x", init=300, cells=100, zc="R", z0=1, z1=1,
                             driving="\n[driving]\ntemperature_gradient = 1.0e7\n"),
    "cross_plane_film": dict(dt=1.0, axis="z", init='"linear"', cells=50, zc="T", z0=301, z1=299, driving=""),
}


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    from phonomc_gb300 import native
    lib_path = native.build()
    out = str(tmp_path_factory.mktemp("binding") / "main_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-w", os.path.join(ROOT, "tests", "binding", "main_gb300.cpp"),
           "-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "include"),
           REF_LIB, "-L", os.path.dirname(lib_path), "-lphonomc_gb300",
           "-Wl,-rpath," + os.path.dirname(lib_path), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_binding_fills_the_library_from_the_reference_config(program, name, tmp_path):
    from phonomc_gb300 import native
    lib = native.lib()
    material = str(tmp_path / "material")
    abi.save_material(lib, synthetic.make_material(mesh=16), material)
    toml = tmp_path / "input.toml"
    toml.write_text(TOML.format(material=material, out=str(tmp_path / "out"), **CASES[name]))
    r = subprocess.run([program, "check", str(toml)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["cells"] == res["ref_cells"] == CASES[name]["cells"]
    assert res["volume_rel_err"] < 1e-12 and res["center_err"] < 1e-9
    assert res["face_mismatch"] == 0, res
    assert res["active"] == res["ref_active"] > 0
    assert res["qpoints"] == 16 ** 3
    zc = CASES[name]["zc"]
    assert res["face_condition"] == "PPPP" + zc + zc
    if zc == "R":  # roughness goes back to nm for phmc_config
        assert res["face_value"][4:] == [1.0, 1.0] and res["gradient"] == 1.0e7
    else:
        assert res["face_value"][4:] == [301.0, 299.0]
