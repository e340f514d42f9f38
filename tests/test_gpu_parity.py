"""CUDA path against the reference's golden vectors (deterministic sub-steps)
and against the CPU oracle (whole timesteps), through the C ABI."""

import ctypes as C

import numpy as np
import pytest

from conftest import golden
from phonomc_gb300 import abi, synthetic, workloads

pytestmark = pytest.mark.gpu

D = abi.dptr
I32 = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731


def _i32(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


@pytest.fixture(scope="module")
def gpu():
    import phonomc_gb300
    lib = phonomc_gb300.lib()
    n = C.c_int32()
    assert lib.phmc_device_count(C.byref(n)) == 0 and n.value > 0, "no CUDA device"
    return lib


@pytest.fixture(scope="module")
def orc():
    import oracle
    return oracle.load()


def test_trace_box_golden(gpu):
    g = golden("box_trace")
    p, v = _f64(g["ray_p"]), _f64(g["ray_v"])
    n = p.shape[0]
    hit, t, f = np.zeros((n, 3)), np.zeros(n), np.zeros(n, dtype=np.int32)
    assert gpu.phmc_dev_trace_box(D(_f64([0, 0, 0])), D(_f64([1000, 800, 600])), n, D(p), D(v), D(hit), D(t),
                                  I32(f)) == 0
    assert np.array_equal(f, np.asarray(g["hit_f"], dtype=np.int32))  # hit facets bit-exact
    ok = f >= 0
    assert np.allclose(t[ok], np.asarray(g["hit_t"])[ok], rtol=1e-12, atol=0)
    assert np.allclose(hit[ok], np.asarray(g["hit_p"])[ok], rtol=1e-12, atol=1e-12)


def test_temperature_from_energy_golden(gpu, m8):
    g = golden("material_m8")
    m = abi.Material(gpu, "phmc_", m8, 0.1, False, False)
    E = _f64(g["inv_E"])
    T = np.zeros(E.size)
    assert gpu.phmc_dev_temperature_from_energy(m.h, E.size, D(E), D(T)) == 0
    assert np.allclose(T, g["inv_T"], rtol=1e-11, atol=1e-9)


@pytest.mark.parametrize("name", ["rta_fixed", "rta_local"])
def test_rta_golden(gpu, m8, name):
    g = golden(name)
    m = abi.Material(gpu, "phmc_", m8, 0.1, False, False)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    cT = _f64(g["cell_T"])
    res = C.c_double()
    rc = gpu.phmc_dev_rta_collide(m.h, flat.size, I32(flat), I32(cell), D(occ), cT.size, D(cT), g["dt"],
                                  g["particle_volume"], int(g["local"]), g["lifetime_T"], C.byref(res))
    assert rc == 0, gpu.phmc_last_error()
    assert np.allclose(occ, g["occ_out"], rtol=1e-12, atol=1e-15)
    assert abs(res.value - g["residual"]) < 1e-11


def test_linearized_rta_golden(gpu, m8):
    g = golden("linearized_rta")
    m = abi.Material(gpu, "phmc_", m8, 0.1, True, False)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    res = C.c_double()
    rc = gpu.phmc_dev_linear_collide(m.h, 0, 300.0, flat.size, I32(flat), I32(cell), D(occ), int(cell.max()) + 1,
                                     g["dt"], g["particle_volume"], C.byref(res))
    assert rc == 0, gpu.phmc_last_error()
    assert np.allclose(occ, g["occ_out"], rtol=1e-12, atol=1e-15)
    assert abs(res.value - g["residual"]) < 1e-13


@pytest.mark.parametrize("name,conservative", [("rough_nonconservative", 0), ("rough_conservative", 1)])
def test_rough_golden(gpu, m8, name, conservative):
    g = golden(name)
    m = abi.Material(gpu, "phmc_", m8, 0.1, bool(conservative), False)
    draws = _f64(g["draws"]).reshape(-1, 3)
    facet = np.asarray(g["facet"])
    for f, (normal, rough) in enumerate([((0, 0, -1), 10.0), ((0, 0, 1), 3.0)]):
        sel = facet == f
        fin = _i32(np.asarray(g["in_flat"])[sel])
        oin = _f64(np.asarray(g["in_occ"])[sel])
        u = _f64(np.clip(draws[sel], 0, None))
        fo, oo = np.zeros(fin.size, dtype=np.int32), np.zeros(fin.size)
        rc = gpu.phmc_dev_rough_reflect(m.h, conservative, 300.0, D(_f64(normal)), rough, fin.size, I32(fin), D(oin),
                                        D(u), I32(fo), D(oo))
        assert rc == 0, gpu.phmc_last_error()
        assert np.array_equal(fo, np.asarray(g["out_flat"])[sel])  # outgoing modes bit-exact
        assert np.allclose(oo, np.asarray(g["out_occ"])[sel], rtol=1e-12, atol=0)


def test_gradient_golden(gpu, m8):
    g = golden("gradient_drive")
    m = abi.Material(gpu, "phmc_", m8, 0.1, True, False)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    e = C.c_double()
    rc = gpu.phmc_dev_gradient_drive(m.h, 0, g["gradient"], 300.0, flat.size, I32(flat), I32(cell), D(occ), 4,
                                     g["dt"], g["particle_volume"], C.byref(e))
    assert rc == 0, gpu.phmc_last_error()
    assert np.allclose(occ, g["occ_out"], rtol=1e-13, atol=1e-16)
    assert abs(e.value - g["energy"]) < 1e-15


# ------------------------------------------------------------ whole steps
def _pair(gpu, orc, cfg, stationary, material):
    mg = abi.Material(gpu, "phmc_", material, 0.1, stationary, False)
    mo = abi.Material(orc, "orc_", material, 0.1, stationary, False)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    return (sg, mg), (so, mo)


def _compare(sg, so, tol=1e-12):
    cg, co = sg.carriers(), so.carriers()
    assert cg["alive"].size == co["alive"].size
    assert np.array_equal(cg["alive"], co["alive"])
    a = cg["alive"] == 1
    assert np.array_equal(cg["mode"][a], co["mode"][a])
    assert np.array_equal(cg["cell"][a], co["cell"][a])
    for k in ("x", "y", "z"):
        assert np.allclose(cg[k][a], co[k][a], rtol=tol, atol=1e-9)
    assert np.allclose(cg["occ"][a], co["occ"][a], rtol=tol, atol=1e-14)
    Tg, Eg, qg = sg.cells()
    To, Eo, qo = so.cells()
    assert np.allclose(Tg, To, rtol=tol, atol=0)
    assert np.allclose(Eg, Eo, rtol=tol, atol=0)
    stg, sto = sg.stats(), so.stats()
    for k in ("particle_count", "absorbed_total", "injected_total", "step_absorbed", "step_injected",
              "collision_cache_corrections", "rough_counts"):
        assert stg[k] == sto[k], k
    for k in ("total_thermal_energy_ev", "step_absorbed_energy_ev", "step_injected_energy_ev"):
        assert abs(stg[k] - sto[k]) <= 1e-10 * max(1.0, abs(sto[k])), k
    return stg, sto


@pytest.mark.parametrize("cell_update", [-1, 1])
def test_cross_plane_steps_match_oracle(gpu, orc, cell_update):
    """RTA film: separate cell kernels (-1) and the fused warp-per-cell update (1)."""
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(workloads.cross_plane_film(), 20000, random_seed=7, rta_cell_update=cell_update)
    (sg, _), (so, _) = _pair(gpu, orc, cfg, False, mat)
    _compare(sg, so)
    for _ in range(3):
        sg.run(2)
        so.run(2)
        _compare(sg, so)


def test_inplane_gradient_steps_match_oracle(gpu, orc):
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(workloads.inplane_gradient(), 20000, random_seed=9)
    (sg, _), (so, _) = _pair(gpu, orc, cfg, True, mat)
    for _ in range(3):
        sg.run(2)
        so.run(2)
        stg, sto = _compare(sg, so)
        # the drive is energy-neutral per cell: both totals are round-off of a zero sum
        scale = abs(sto["total_thermal_energy_ev"])
        assert abs(stg["total_gradient_energy_ev"]) < 1e-17 * scale
        assert abs(sto["total_gradient_energy_ev"]) < 1e-17 * scale
        assert stg["step_gradient_updates"] == sto["step_gradient_updates"]


def test_energy_ledger_closes_on_device(gpu):
    """Energy bookkeeping closes to FP64 round-off at a larger size (property)."""
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(workloads.cross_plane_film(), 400000, random_seed=3)
    m = abi.Material(gpu, "phmc_", mat, 0.1, False, False)
    s = abi.Solver(gpu, "phmc_", cfg, [m])
    s.run(20)
    st = s.stats()
    scale = abs(st["step_absorbed_energy_ev"]) + abs(st["step_injected_energy_ev"]) + 1e-30
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-9 * max(scale, abs(st["total_thermal_energy_ev"]))
    T, _, _ = s.cells()
    assert np.all(T > 298.0) and np.all(T < 302.0)
    assert st["particle_count"] > 0.9 * 400000


# ------------------------------------------------------------ mixed precision
def _mixed_vs_plain(gpu, cfg, stationary, steps):
    mat = synthetic.make_material(mesh=16)
    m = abi.Material(gpu, "phmc_", mat, 0.1, stationary, False)
    sp = abi.Solver(gpu, "phmc_", dict(cfg, precision="fp64"), [m])
    sm = abi.Solver(gpu, "phmc_", dict(cfg, precision="mixed"), [m])
    sp.run(steps)
    sm.run(steps)
    return sp, sm


@pytest.mark.parametrize("name,stationary", [("cross_plane_film", False), ("inplane_gradient", True)])
def test_mixed_tracks_plain_trajectory(gpu, name, stationary):
    """Same seed, same draws: the FP32 flight reproduces the FP64 trajectory up to
    FP32 rounding (positions), and cell temperatures agree to 1e-4 K after 6 steps."""
    cfg = workloads.scaled(getattr(workloads, name)(), 50000, random_seed=21)
    sp, sm = _mixed_vs_plain(gpu, cfg, stationary, 6)
    cp, cm = sp.carriers(), sm.carriers()
    a = (cp["alive"] == 1) & (cm["alive"] == 1)
    assert a.mean() > 0.99
    same_mode = np.mean(cp["mode"][a] == cm["mode"][a])
    assert same_mode > 0.999, same_mode
    assert np.mean(cp["cell"][a] == cm["cell"][a]) > 0.999
    for k in ("x", "y", "z"):
        d = np.abs(cp[k][a] - cm[k][a])
        assert np.median(d) < 1e-3, (k, np.median(d))
    Tp, _, _ = sp.cells()
    Tm, _, _ = sm.cells()
    assert np.max(np.abs(Tp - Tm)) < 1e-3
    st = sm.stats()
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-12 * abs(st["total_thermal_energy_ev"])


@pytest.mark.parametrize("conservative", [0, 1])
def test_rough_table_device_scan_matches_host(gpu, conservative):
    """Rough-table specular matches from the device scan (FP32 screen, FP64
    decision) equal the host loop's for 96 facets of random orientation and
    the synthetic tables: the same outgoing mode for every incoming mode."""
    # conservative walls need the full-zone Callaway bank (8^3 x 6 completed: 24,552 modes)
    mat = synthetic.make_material(mesh=8 if conservative else 16, callaway=bool(conservative))
    m = abi.Material(gpu, "phmc_", mat, 0.1, bool(conservative), bool(conservative))
    na = C.c_int32()
    assert gpu.phmc_material_active_count(m.h, C.byref(na)) == 0
    rng = np.random.default_rng(11)
    nf = 96
    nrm = rng.normal(size=(nf, 3))
    nrm[:6] = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]]  # axis-aligned: many ties
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    nrm = np.ascontiguousarray(nrm)
    rough = np.full(nf, 10.0)
    out = {}
    for dev in (0, 1):
        match = np.zeros(nf * na.value, np.int32)
        rc = gpu.phmc_dev_rough_spec_match(m.h, conservative, 300.0, nf, D(nrm), D(rough), dev, I32(match))
        assert rc == 0, gpu.phmc_last_error()
        out[dev] = match
    assert np.array_equal(out[0], out[1])
    assert (out[1] >= 0).sum() > nf * na.value // 10


def test_mixed_mesh_tracks_plain_trajectory(gpu, tmp_path):
    """FinFET mesh, same seed and draws: the FP32 offsets (from each cell's
    home voxel) follow the FP64 positions up to FP32 rounding, wall events and
    injections pick the same modes, cells agree, and the energy ledger closes."""
    stl = workloads.finfet_stl(str(tmp_path / "finfet.stl"))
    mat = synthetic.make_material(mesh=8)
    m = abi.Material(gpu, "phmc_", mat, 0.1, False, False)
    base = workloads.finfet_mesh(stl, particles=40000, seed=31, grid=(32, 16, 16))
    sp = abi.Solver(gpu, "phmc_", dict(base, precision="fp64"), [m])
    sm = abi.Solver(gpu, "phmc_", dict(base, precision="mixed"), [m])
    c0p, c0m = sp.carriers(), sm.carriers()
    live0 = c0p["alive"] == 1
    for k in ("x", "y", "z"):  # the initial population through the offsets
        assert np.max(np.abs(c0p[k][live0] - c0m[k][live0])) < 1e-3
    assert np.array_equal(c0p["cell"][live0], c0m["cell"][live0])
    sp.run(8)
    sm.run(8)
    cp, cm = sp.carriers(), sm.carriers()
    a = (cp["alive"] == 1) & (cm["alive"] == 1)
    assert a.mean() > 0.99
    assert np.mean(cp["mode"][a] == cm["mode"][a]) > 0.999
    assert np.mean(cp["cell"][a] == cm["cell"][a]) > 0.999
    for k in ("x", "y", "z"):
        d = np.abs(cp[k][a] - cm[k][a])
        assert np.median(d) < 1e-3, (k, np.median(d))
    Tp, _, _ = sp.cells()
    Tm, _, _ = sm.cells()
    # a few carriers per cell: a cell whose one carrier took another event
    # path differs by a carrier's energy; nearly all cells agree to rounding
    assert np.mean(np.abs(Tp - Tm) < 1e-4) > 0.99
    for s in (sp, sm):
        st = s.stats()
        assert abs(st["step_energy_balance_residual_ev"]) < 1e-9 * abs(st["total_thermal_energy_ev"])
    sm.close()
    sp.close()


def test_mixed_energy_conservation_linearized(gpu):
    """The FP32 linear-response exponential is rescaled in FP64: the collision
    changes the carried energy only at round-off (lifetime residual ~ 0)."""
    cfg = workloads.scaled(workloads.inplane_gradient(), 200000, random_seed=4)
    mat = synthetic.make_material(mesh=16)
    m = abi.Material(gpu, "phmc_", mat, 0.1, True, False)
    s = abi.Solver(gpu, "phmc_", dict(cfg, precision="mixed"), [m])
    s.run(5)
    st = s.stats()
    scale = abs(st["total_thermal_energy_ev"])
    assert abs(st["step_lifetime_energy_residual_ev"]) < 1e-13 * scale
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-13 * scale


# ------------------------------------------------------------ Callaway (normal + resistive)
def _callaway_cfg(particles, seed):
    return workloads.scaled(workloads.inplane_gradient(), particles, random_seed=seed, collision_model="callaway")


def test_callaway_steps_match_oracle(gpu, orc):
    """Linear-response collisions with momentum-conserving normal processes
    (four normal gain directions plus the resistive one): whole steps on the
    device against the oracle."""
    mat = synthetic.make_material(mesh=8, callaway=True)
    cfg = _callaway_cfg(20000, 13)
    mg = abi.Material(gpu, "phmc_", mat, 0.1, True, True)
    mo = abi.Material(orc, "orc_", mat, 0.1, True, True)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    for _ in range(2):
        sg.run(2)
        so.run(2)
        _compare(sg, so, tol=1e-11)


def test_mixed_callaway_conserves_energy_and_tracks_plain(gpu):
    """FP32 Callaway exponential (five gain directions) with the FP64 rescale:
    the collision changes the carried energy only at round-off, and cell
    temperatures follow the FP64 path to 1e-3 K."""
    mat = synthetic.make_material(mesh=8, callaway=True)
    cfg = _callaway_cfg(100000, 17)
    m = abi.Material(gpu, "phmc_", mat, 0.1, True, True)
    sp = abi.Solver(gpu, "phmc_", dict(cfg, precision="fp64"), [m])
    sm = abi.Solver(gpu, "phmc_", dict(cfg, precision="mixed"), [m])
    sp.run(5)
    sm.run(5)
    st = sm.stats()
    scale = abs(st["total_thermal_energy_ev"])
    assert abs(st["step_lifetime_energy_residual_ev"]) < 1e-13 * scale
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-13 * scale
    Tp, _, _ = sp.cells()
    Tm, _, _ = sm.cells()
    assert np.max(np.abs(Tp - Tm)) < 1e-3


# ------------------------------------------------------------ host ingest
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_registered_host_ingest_matches_copy_path(gpu, precision):
    """Carriers read by the device straight from registered host arrays give
    the same state and the same steps as the staged copy path."""
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(workloads.inplane_gradient(), 30000, random_seed=5, precision=precision)
    m = abi.Material(gpu, "phmc_", mat, 0.1, True, False)
    src = abi.Solver(gpu, "phmc_", cfg, [m])
    src.run(2)
    c = src.carriers()
    live = c["alive"] == 1
    host = {k: np.ascontiguousarray(c[k][live]) for k in ("x", "y", "z", "occ", "mode")}
    a = abi.Solver(gpu, "phmc_", cfg, [m])
    b = abi.Solver(gpu, "phmc_", cfg, [m])
    a.set_carriers(dict(host, alive=np.ones(host["x"].size, np.uint8)))
    for arr in host.values():
        assert gpu.phmc_host_register(arr.ctypes.data, arr.nbytes) == 0
    try:
        b.set_carriers(dict(host, alive=None))
    finally:
        for arr in host.values():
            gpu.phmc_host_unregister(arr.ctypes.data)
    for s in (a, b):
        s.run(2)
    ca, cb = a.carriers(), b.carriers()
    for k in ("alive", "mode", "cell", "x", "y", "z"):
        assert np.array_equal(ca[k], cb[k]), k
    # bin sums are FP64 atomics in arrival order: collisions agree to round-off
    assert np.allclose(ca["occ"], cb["occ"], rtol=1e-12, atol=1e-15)
    assert np.allclose(a.cells()[0], b.cells()[0], rtol=1e-12, atol=0)


# ------------------------------------------------------------ layered materials
@pytest.mark.parametrize("name,linearized", [("interface_dmm", 0), ("interface_dmm_linearized", 1)])
def test_interface_golden(gpu, name, linearized):
    g = golden(name)
    ma = abi.Material(gpu, "phmc_", synthetic.make_material(mesh=8), 0.1, False, False)
    mb = abi.Material(gpu, "phmc_", synthetic.make_material(mesh=8, freq_scale=0.7, vel_scale=0.75), 0.1, False,
                      False)
    n = len(g["src"])
    src, flat, signs = (_i32(g[k]) for k in ("src", "in_flat", "in_signs"))
    occ, u3 = _f64(g["in_occ"]), _f64(g["draws"])
    act, mat, fo, so = (np.zeros(n, np.int32) for _ in range(4))
    oo = np.zeros(n)
    rc = gpu.phmc_dev_interface(ma.h, mb.h, g["weight_a"], g["weight_b"], g["axis"], g["frequency_bin_thz"],
                                g["reference_temperature"], linearized, n, I32(src), I32(flat), I32(signs), D(occ),
                                D(u3), I32(act), I32(mat), I32(fo), I32(so), D(oo))
    assert rc == 0, gpu.phmc_last_error()
    assert np.array_equal(act, g["action"])
    assert np.array_equal(mat, g["out_material"])
    assert np.array_equal(fo, g["out_flat"])
    assert np.array_equal(oo, np.asarray(g["out_occ"]))


def _bilayer_pair(gpu, orc, particles, seed, precision="fp64"):
    cfg = workloads.scaled(workloads.bilayer_callaway(), particles, random_seed=seed, precision=precision)
    data = workloads.bilayer_materials(8)
    mg = [abi.Material(gpu, "phmc_", d, 0.1, True, True) for d in data]
    mo = [abi.Material(orc, "orc_", d, 0.1, True, True) for d in data]
    return (abi.Solver(gpu, "phmc_", cfg, mg), mg), (abi.Solver(orc, "orc_", cfg, mo), mo)


def test_bilayer_steps_match_oracle(gpu, orc):
    """Two materials, diffuse-mismatch interface, linearized Callaway, reservoirs:
    whole steps on the device against the oracle, interface counters exact."""
    (sg, _), (so, _) = _bilayer_pair(gpu, orc, 20000, 31)
    _compare(sg, so, tol=1e-11)
    for _ in range(3):
        sg.run(2)
        so.run(2)
        stg, sto = _compare(sg, so, tol=1e-11)
        for k in ("interface_events", "interface_transmitted", "interface_reflected"):
            assert stg[k] == sto[k], k
    assert sto["interface_events"] > 0 and sto["interface_transmitted"] > 0


def test_mixed_bilayer_conserves_energy_and_tracks_plain(gpu):
    cfg = workloads.scaled(workloads.bilayer_callaway(), 200000, random_seed=37)
    data = workloads.bilayer_materials(8)
    m = [abi.Material(gpu, "phmc_", d, 0.1, True, True) for d in data]
    sp = abi.Solver(gpu, "phmc_", dict(cfg, precision="fp64"), m)
    sm = abi.Solver(gpu, "phmc_", dict(cfg, precision="mixed"), m)
    sp.run(6)
    sm.run(6)
    st = sm.stats()
    scale = abs(st["total_thermal_energy_ev"])
    assert abs(st["step_lifetime_energy_residual_ev"]) < 1e-13 * scale
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-12 * scale
    assert st["interface_events"] > 0
    Tp, _, _ = sp.cells()
    Tm, _, _ = sm.cells()
    assert np.max(np.abs(Tp - Tm)) < 2e-2
    cp, cm = sp.carriers(), sm.carriers()
    a = (cp["alive"] == 1) & (cm["alive"] == 1)
    assert np.mean(cp["mode"][a] == cm["mode"][a]) > 0.99


# ------------------------------------------------------------ heat source
@pytest.mark.parametrize("spectrum,callaway", [("thermal", False), ("weighted", False), ("gaussian", False),
                                               ("thermal", True)])
def test_heat_source_steps_match_oracle(gpu, orc, spectrum, callaway):
    """Prescribed heat source (both halves per step, budgets kept in cells
    without eligible carriers): device steps against the oracle. The device
    spreads the round-off correction over the correction mode's carriers of the
    cell instead of one carrier, so occupations agree to 1e-11."""
    cfg = workloads.scaled(workloads.heated_film(spectrum=spectrum), 20000, random_seed=43)
    if callaway:
        cfg["collision_model"] = "callaway"
        cfg["lifetime_temperature"] = 300.0
    mat = synthetic.make_material(mesh=8 if callaway else 16, callaway=callaway)
    stationary = spectrum == "gaussian" or callaway
    mg = abi.Material(gpu, "phmc_", mat, 0.1, stationary, callaway)
    mo = abi.Material(orc, "orc_", mat, 0.1, stationary, callaway)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    for _ in range(3):
        sg.run(1)
        so.run(1)
        stg, sto = _compare(sg, so, tol=1e-11)
        for k in ("step_heat_source_energy_ev", "total_heat_source_energy_ev", "prescribed_heat_source_energy_ev",
                  "pending_heat_source_energy_ev"):
            assert abs(stg[k] - sto[k]) <= 1e-12 * max(1.0, abs(sto[k])), k
        assert stg["step_heat_source_updates"] == sto["step_heat_source_updates"]
        scale = abs(sto["total_thermal_energy_ev"])
        assert abs(stg["step_energy_balance_residual_ev"]) < 1e-12 * scale
    assert sto["total_heat_source_energy_ev"] > 0


def test_mixed_heat_source_conserves_energy(gpu):
    cfg = workloads.scaled(workloads.heated_film(), 200000, random_seed=47, precision="mixed")
    m = abi.Material(gpu, "phmc_", synthetic.make_material(mesh=16), 0.1, False, False)
    s = abi.Solver(gpu, "phmc_", cfg, [m])
    s.run(5)
    st = s.stats()
    scale = abs(st["total_thermal_energy_ev"])
    assert st["total_heat_source_energy_ev"] > 0
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-12 * scale


# ------------------------------------------------------------ graphs
@pytest.mark.parametrize("name", ["cross_plane_film", "heated_film", "inplane_gradient"])
def test_graph_replay_matches_eager_steps(gpu, name):
    """Steps replayed from the captured timestep graph equal steps launched
    one kernel at a time (draw counter and source windows live on the device)."""
    cfg = workloads.scaled(getattr(workloads, name)(), 30000, random_seed=53, precision="mixed")
    mat = synthetic.make_material(mesh=16)
    m = abi.Material(gpu, "phmc_", mat, 0.1, name == "inplane_gradient", False)
    a = abi.Solver(gpu, "phmc_", cfg, [m])
    b = abi.Solver(gpu, "phmc_", cfg, [m])
    assert gpu.phmc_solver_set_graphs(b.h, 0) == 0
    for s in (a, b):
        s.run(12)
    ca, cb = a.carriers(), b.carriers()
    for k in ("alive", "mode", "cell"):
        assert np.array_equal(ca[k], cb[k]), k
    live = ca["alive"] == 1
    for k in ("x", "y", "z", "occ"):
        assert np.allclose(ca[k][live], cb[k][live], rtol=1e-12, atol=1e-12), k
    sa, sb = a.stats(), b.stats()
    assert sa["current_timestep"] == sb["current_timestep"] == 12
    assert sa["particle_count"] == sb["particle_count"]
    assert abs(sa["average_heat_flux_along_axis"] - sb["average_heat_flux_along_axis"]) <= 1e-9 * abs(
        sb["average_heat_flux_along_axis"]) + 1e-9
    assert sa["device_launches"] == sb["device_launches"]


# ------------------------------------------------------------ batches
def test_batch_matches_single_instances(gpu):
    """Films advanced together in a batch equal the same films advanced one by one."""
    films = workloads.batched_films(n=4, seed=3, precision="mixed", particles_per_10nm=200)
    m = abi.Material(gpu, "phmc_", synthetic.make_material(mesh=16), 0.1, False, False)
    b = abi.Batch(gpu, films, [m])
    b.run(12)  # past a flux observation (every 10 steps) on the batch's own streams
    for i, cfg in enumerate(films):
        s = abi.Solver(gpu, "phmc_", cfg, [m])
        s.run(12)
        st, sb = s.stats(), b.stats(i)
        for k in ("current_timestep", "particle_count", "absorbed_total", "injected_total"):
            assert st[k] == sb[k], (i, k)
        T, _, _ = s.cells()
        Tb, _, _ = b.cells(i)
        assert np.allclose(T, Tb, rtol=1e-10, atol=0)
    ms, cs, launches = b.timed_run(3)
    assert ms > 0 and cs > 0 and launches > 0


# ------------------------------------------------------------ meshes
def test_mesh_trace_golden(gpu):
    """Device BVH walk through the procedural FinFET surface against the
    reference's SurfaceMesh::trace_boundary_intersection: facet ids, hit times
    and hit points bit-exact."""
    g = golden("mesh_finfet")
    V, F, f2f = _f64(g["vertices"]), _i32(g["faces"]), _i32(g["face_to_facet"])
    P, Vel = _f64(g["origins"]), _f64(g["velocities"])
    n = P.shape[0]
    hit, t, fac = np.zeros((n, 3)), np.zeros(n), np.zeros(n, np.int32)
    rc = gpu.phmc_dev_trace_mesh(V.shape[0], D(V), F.size // 3, I32(F), I32(f2f), n, D(P), D(Vel), D(hit), D(t),
                                 I32(fac))
    assert rc == 0, gpu.phmc_last_error()
    assert np.array_equal(fac, g["facet"])
    assert np.array_equal(t, np.asarray(g["t"]))
    assert np.array_equal(hit, np.asarray(g["hits"]))


@pytest.fixture(scope="module")
def finfet_stl(tmp_path_factory):
    return workloads.finfet_stl(str(tmp_path_factory.mktemp("finfet") / "finfet.stl"))


def test_mesh_domain_device_queries_golden(gpu, finfet_stl):
    """Device membership (BVH ray cast, then star simplices), nearest facet and
    voxel-map cell of the reference's random points, bit-exact."""
    g = golden("domain_finfet")
    dom = abi.Domain(gpu, workloads.finfet_mesh(finfet_stl))
    inside, near, cell = abi.device_domain_query(dom, g["points"])
    assert np.array_equal(inside, np.asarray(g["inside"], dtype=np.uint8))
    assert np.array_equal(near, np.asarray(g["nearest_facet"], dtype=np.int32))
    assert np.array_equal(cell, np.asarray(g["cell"], dtype=np.int32))
    # cell centres: inside, and each maps to its own cell
    C = dom.cells()
    inside, _, cell = abi.device_domain_query(dom, C["centers"])
    assert inside.all()
    assert np.array_equal(cell, np.arange(dom.n_cells, dtype=np.int32))


@pytest.mark.parametrize("cell_update", [-1, 1])
@pytest.mark.parametrize("source", [True, False])
def test_finfet_steps_match_oracle(gpu, orc, finfet_stl, source, cell_update):
    """FinFET mesh domain (BVH walls, rough facets with mirrored outward modes,
    periodic facet pairs, heat sink, Gaussian heat source): device timesteps
    against the oracle on the same initial carriers, with the separate RTA
    cell kernels (-1) and the fused warp-per-cell update (1)."""
    cfg = workloads.finfet_mesh(finfet_stl, particles=20000, seed=11, grid=(32, 8, 16), heat_source=source)
    cfg["rta_cell_update"] = cell_update
    mat = synthetic.make_material(mesh=8)
    (sg, _), (so, _) = _pair(gpu, orc, cfg, False, mat)
    _compare(sg, so, tol=1e-11)
    for _ in range(3):
        sg.run(1)
        so.run(1)
        stg, sto = _compare(sg, so, tol=1e-11)
        if source:
            for k in ("total_heat_source_energy_ev", "prescribed_heat_source_energy_ev"):
                assert abs(stg[k] - sto[k]) <= 1e-12 * max(1.0, abs(sto[k])), k
    assert sto["absorbed_total"] > 0 and sto["injected_total"] > 0


def test_output_files_finfet(gpu, finfet_stl, tmp_path):
    """convergence.txt, grid_heat_flux.csv and heat_source_ledger.txt of a short
    FinFET run with its heat source against the reference's files
    (tests/golden/files_finfet): headers and layouts identical, the
    deterministic columns (steps, times, cell ids and centres, materials, base
    powers, prescribed energies) equal, the stochastic ones closing the ledger
    (prescribed = deposited + pending per cell)."""
    g = golden("files_finfet")
    files = g["files"]
    m = abi.Material(gpu, "phmc_", synthetic.make_material(mesh=8), 0.1, False, False)
    out = tmp_path / "out"
    cfg = workloads.finfet_mesh(finfet_stl, particles=g["particles"], seed=g["seed"], grid=tuple(g["grid"]))
    cfg.update(iterations=g["steps"], convergence_write_interval=1, output_folder=str(out),
               write_cell_heat_flux=True, material_folder="unused")
    s = abi.Solver(gpu, "phmc_", cfg, [m])
    s.run(g["steps"])
    s.close()

    ref = files["convergence.txt"].splitlines()
    mine = (out / "convergence.txt").read_text().splitlines()
    assert mine[0] == ref[0] and len(mine) == len(ref)
    names = ref[0].split()[1:]
    col = {n: i for i, n in enumerate(names)}
    for a, b in zip(mine[1:], ref[1:]):
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb) == len(names)
        assert ta[:2] == tb[:2]
        for key in ("hs_prescribed_total_ev",):
            assert np.isclose(float(ta[col[key]]), float(tb[col[key]]), rtol=1e-12, atol=0)
        assert abs(float(ta[col["hs_ledger_residual_ev"]])) <= 1e-9 * max(1.0, float(tb[col["hs_prescribed_total_ev"]]))

    ref = files["grid_heat_flux.csv"].splitlines()
    mine = (out / "grid_heat_flux.csv").read_text().splitlines()
    assert mine[0] == ref[0] and len(mine) == len(ref)
    for a, b in zip(mine[1:], ref[1:]):
        ta, tb = a.split(","), b.split(",")
        assert len(ta) == 7 and ta[0] == tb[0] and ta[2] == tb[2]
        assert float(ta[1]) == float(tb[1])
        assert all(np.isfinite(float(x)) for x in ta[3:])

    ref = files["heat_source_ledger.txt"].splitlines()
    mine = (out / "heat_source_ledger.txt").read_text().splitlines()
    assert mine[:3] == ref[:3] and len(mine) == len(ref)
    for a, b in zip(mine[3:], ref[3:]):
        ta, tb = a.split(), b.split()
        assert ta[:5] == tb[:5]  # cell, centre (17 digits), material
        pa, pb = [float(x) for x in ta[5:]], [float(x) for x in tb[5:]]
        assert np.isclose(pa[0], pb[0], rtol=1e-12, atol=0)  # base power, W
        assert np.isclose(pa[1], pb[1], rtol=1e-12, atol=0)  # prescribed, eV
        assert np.isclose(pa[2] + pa[3], pa[1], rtol=1e-9, atol=1e-12 * max(1.0, pb[1]))


# ------------------------------------------------------ nonlinear Callaway
@pytest.mark.parametrize("name,rtol", [("ncallaway_unique", 1e-12), ("ncallaway_shared", 1e-10),
                                       ("ncallaway_large", 1e-10)])
def test_nonlinear_callaway_cell_golden(gpu, name, rtol):
    """One cell of nonlinear Callaway on the device (mode bins, moment Newton
    per substep) against the reference's nonlinear_callaway_evolve on the same
    carriers. With one carrier per mode the device arithmetic is the
    reference's in FP64; with shared modes the convergence scale uses the bin
    bound, so agreement is to the Newton tolerance."""
    g = golden(name)
    mode = _i32(g["mode"])
    occ = _f64(g["n"]).copy()
    rc = gpu.phmc_dev_ncallaway_evolve(len(g["omega"]), D(_f64(g["omega"])), D(_f64(g["k"])), D(_f64(g["rn"])),
                                       D(_f64(g["rr"])), mode.size, I32(mode), D(occ), C.c_double(g["T"]),
                                       C.c_double(g["dt"]))
    assert rc == 0, gpu.phmc_last_error()
    assert np.allclose(occ, g["out"], rtol=rtol, atol=0)


@pytest.mark.parametrize("lifetime", [300.0, "local"])
def test_nonlinear_callaway_steps_match_oracle(gpu, orc, lifetime):
    """Whole steps of a cross-plane film with nonlinear Callaway collisions
    (absolute occupations, conservative boundaries) on the device against the
    oracle's per-carrier long-double restatement; N/U rates at the fixed 300 K
    or interpolated at each cell's temperature."""
    mat = synthetic.make_material(mesh=8, callaway=True)
    cfg = workloads.scaled(workloads.cross_plane_film(), 20000, random_seed=17, collision_model="callaway",
                           callaway_formulation="nonlinear", lifetime_temperature=lifetime)
    mg = abi.Material(gpu, "phmc_", mat, 0.1, True, True)
    mo = abi.Material(orc, "orc_", mat, 0.1, True, True)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    for _ in range(3):
        sg.run(2)
        so.run(2)
        stg, sto = _compare(sg, so, tol=1e-9)
        assert abs(stg["total_lifetime_energy_residual_ev"] - sto["total_lifetime_energy_residual_ev"]) < 1e-8
    assert abs(stg["total_energy_balance_residual_ev"]) < 1e-6


def test_nonlinear_callaway_crowded_bins_match_oracle(gpu, orc):
    """Many carriers per (cell, mode) bin: 1e6 carriers in 2 cells of the 8^3
    Callaway table (about 20 per mode and cell). The device's FP64 moment
    Newton over bin sums stops on the reference's 2e-13 relative test, which
    its per-bin scale makes no looser than the reference's per-carrier one;
    the solve must converge (no error) and stay with the oracle's per-carrier
    long-double solve."""
    mat = synthetic.make_material(mesh=8, callaway=True)
    cfg = workloads.scaled(workloads.cross_plane_film(), 1e6, random_seed=23, collision_model="callaway",
                           callaway_formulation="nonlinear", grid=(1, 1, 2))
    mg = abi.Material(gpu, "phmc_", mat, 0.1, True, True)
    mo = abi.Material(orc, "orc_", mat, 0.1, True, True)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    for _ in range(2):
        sg.run(1)
        so.run(1)
        stg, sto = _compare(sg, so, tol=1e-9)
    assert abs(stg["total_energy_balance_residual_ev"]) < 1e-6


def test_callaway_global_mode_slices_match_oracle(gpu, orc):
    """A 16^3 Callaway table completes to 196,584 modes, more than the shared
    memory of a 16-CTA cluster holds per cell: the exponential keeps its
    per-mode vectors in a global work area instead. Whole steps against the
    oracle."""
    mat = synthetic.make_material(mesh=16, callaway=True)
    cfg = workloads.scaled(workloads.inplane_gradient(), 20000, random_seed=19, collision_model="callaway",
                           grid=(1, 1, 10))
    mg = abi.Material(gpu, "phmc_", mat, 0.1, True, True)
    mo = abi.Material(orc, "orc_", mat, 0.1, True, True)
    sg = abi.Solver(gpu, "phmc_", cfg, [mg])
    so = abi.Solver(orc, "orc_", cfg, [mo])
    for _ in range(2):
        sg.run(2)
        so.run(2)
        _compare(sg, so, tol=1e-11)


# ------------------------------------------------------------ carrier sort
@pytest.mark.parametrize("name,stationary,steps", [("cross_plane_film", False, 2), ("inplane_gradient", True, 3)])
def test_sorted_steps_match_oracle(gpu, orc, name, stationary, steps):
    """Carrier slots stably reordered by (mode, cell) at the start of every
    `steps`-th step, on the device (radix sort) and in the oracle
    (std::stable_sort): identical slots, so identical draws, and whole steps
    that still agree carrier by carrier."""
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(getattr(workloads, name)(), 20000, random_seed=31, carrier_sort_interval=steps)
    (sg, _), (so, _) = _pair(gpu, orc, cfg, stationary, mat)
    for _ in range(4):
        sg.run(steps)
        so.run(steps)
        _compare(sg, so)
    # the population is grouped by mode: after a sort, runs of equal active mode
    c = sg.carriers()
    a = c["alive"] == 1
    assert a.sum() == sg.stats()["particle_count"]


def test_sort_orders_slots_by_mode_then_cell(gpu):
    """A fresh solver with sort interval 1 sorts its initial population at the
    start of its first step: after that step the slots hold the initial
    carriers in stable (active mode, cell) order, each still in its mode unless
    a rough wall resampled it."""
    mat = synthetic.make_material(mesh=16)
    cfg = workloads.scaled(workloads.inplane_gradient(), 300000, random_seed=5, carrier_sort_interval=1)
    m = abi.Material(gpu, "phmc_", mat, 0.1, True, False)
    s = abi.Solver(gpu, "phmc_", cfg, [m])
    before = s.carriers()
    s.run(1)
    after = s.carriers()
    # a stable sort of the step-start state by (mode, cell): the modes after the
    # step are those of the sorted start state except where a wall resampled them
    a0 = before["alive"] == 1
    key = (before["mode"][a0].astype(np.int64) & 0xFFFFFF) * 1000 + before["cell"][a0]
    order = np.argsort(key, kind="stable")
    mode_sorted = before["mode"][a0][order] & 0xFFFFFF
    live = after["alive"] == 1
    assert live.sum() == a0.sum()
    same = np.mean((after["mode"][: a0.sum()] & 0xFFFFFF) == mode_sorted)
    assert same > 0.97, same
    assert np.all(np.diff(mode_sorted) >= 0)


@pytest.mark.parametrize("source", [False, True])
def test_sorted_finfet_steps_match_oracle(gpu, orc, finfet_stl, source):
    """Mesh domain with slots sorted by (cell, mode) every step, wall caches and
    mirror facets moving with their carriers."""
    cfg = workloads.finfet_mesh(finfet_stl, particles=20000, seed=13, grid=(32, 8, 16), heat_source=source)
    cfg["carrier_sort_interval"] = 1
    mat = synthetic.make_material(mesh=8)
    (sg, _), (so, _) = _pair(gpu, orc, cfg, False, mat)
    for _ in range(3):
        sg.run(1)
        so.run(1)
        _compare(sg, so, tol=1e-11)


def test_sorted_mixed_path_conserves_energy(gpu):
    """Mixed precision with sorts every 2 steps at 2e6 carriers (several radix
    tiles per digit, three 8-bit passes): the ledger closes to round-off and the
    live count is kept."""
    mat = synthetic.make_material(mesh=16)
    m = abi.Material(gpu, "phmc_", mat, 0.1, True, False)
    cfg = workloads.scaled(workloads.inplane_gradient(precision="mixed"), 2e6, random_seed=17,
                           carrier_sort_interval=2)
    s = abi.Solver(gpu, "phmc_", cfg, [m])
    s.run(7)
    st = s.stats()
    assert st["particle_count"] == 2000000
    scale = abs(st["total_thermal_energy_ev"])
    assert abs(st["step_lifetime_energy_residual_ev"]) < 1e-13 * scale
    assert abs(st["step_energy_balance_residual_ev"]) < 1e-13 * scale


@pytest.mark.parametrize("name,stationary", [("inplane_gradient", True), ("cross_plane_film", False)])
def test_staged_pass_matches_direct_loads(gpu, name, stationary):
    """The mixed carrier pass with carrier tiles staged in shared memory by bulk
    asynchronous copies against the same pass with direct loads, on identical
    draws and 70,001 carriers (a partial last tile): the same carriers, cells
    and modes, occupations and cell temperatures to bin-sum rounding."""
    mat = synthetic.make_material(mesh=16)
    m = abi.Material(gpu, "phmc_", mat, 0.1, stationary, False)
    base = workloads.scaled(getattr(workloads, name)(precision="mixed"), 70001, random_seed=29,
                            carrier_sort_interval=3)
    runs = []
    for pipe in (1, -1):
        s = abi.Solver(gpu, "phmc_", dict(base, transport_pipeline=pipe), [m])
        s.run(7)
        runs.append((s.carriers(), s.cells()[0], s.stats()))
    (ca, Ta, sa), (cb, Tb, sb) = runs
    assert np.array_equal(ca["alive"], cb["alive"])
    a = ca["alive"] == 1
    assert np.array_equal(ca["mode"][a], cb["mode"][a])
    assert np.array_equal(ca["cell"][a], cb["cell"][a])
    for k in ("x", "y", "z"):
        assert np.array_equal(ca[k][a], cb[k][a]), k
    assert np.allclose(ca["occ"][a], cb["occ"][a], rtol=1e-12, atol=1e-14)
    assert np.allclose(Ta, Tb, rtol=1e-12, atol=0)
    for k in ("particle_count", "absorbed_total", "injected_total", "rough_counts"):
        assert sa[k] == sb[k], k


@pytest.mark.parametrize("cell_update", [-1, 1])
@pytest.mark.parametrize("model,fraction", [("amm", 1.0), ("mmm", 0.4)])
def test_bilayer_amm_steps_match_oracle(gpu, orc, model, fraction, cell_update):
    """Acoustic (and mixed) mismatch interface events inside whole device steps
    against the oracle: rows built on the host, sampled on the device with the
    oracle's draws; carriers, cells and interface counters exact. Two RTA
    materials: the separate cell kernels (-1) and the fused warp-per-cell
    update (1), which takes each cell's material and class list."""
    data = workloads.bilayer_materials(8, callaway=False)
    cfg = workloads.scaled(workloads.bilayer_amm(model=model, amm_fraction=fraction), 20000, random_seed=41,
                           grid=(1, 1, 20), rta_cell_update=cell_update)
    mg = [abi.Material(gpu, "phmc_", d, 0.1, False, False) for d in data]
    mo = [abi.Material(orc, "orc_", d, 0.1, False, False) for d in data]
    sg, so = abi.Solver(gpu, "phmc_", cfg, mg), abi.Solver(orc, "orc_", cfg, mo)
    for _ in range(4):
        sg.run(2)
        so.run(2)
        stg, sto = _compare(sg, so)
        for k in ("interface_events", "interface_transmitted", "interface_reflected"):
            assert stg[k] == sto[k], k
    assert sto["interface_transmitted"] > 0
