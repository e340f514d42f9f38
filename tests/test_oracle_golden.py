"""Pin the CPU oracle (and the host tables it shares with the CUDA path) to
golden vectors printed by the reference solver's own code (tests/golden/)."""

import ctypes as C

import numpy as np
import pytest

from conftest import golden
from phonomc_gb300 import abi

D = abi.dptr
I32 = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731


def _mat(lib, data, stationary=False, callaway=False):
    return abi.Material(lib, "orc_", data, 0.1, stationary, callaway)


def _i32(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


@pytest.mark.parametrize("name,stationary,callaway", [("material_m8", False, False),
                                                       ("material_m8_stationary", True, False),
                                                       ("material_m8c_stationary", True, True)])
def test_material_tables(oracle_lib, m8, name, stationary, callaway):
    g = golden(name)
    if callaway:
        from phonomc_gb300 import synthetic
        m = _mat(oracle_lib, synthetic.make_material(mesh=8, callaway=True), stationary, True)
    else:
        m = _mat(oracle_lib, m8, stationary)
    na = int(g["active_mode_count"])
    sc = np.zeros(7)
    act = np.zeros(na, dtype=np.int32)
    oracle_lib.orc_material_scalars(m.h, C.c_double(1234.5), D(sc), I32(act))
    assert int(sc[0]) == na
    assert np.array_equal(act, np.asarray(g["active_flat"], dtype=np.int32))
    assert sc[1] == g["energy_density_normalization"]
    assert abs(sc[2] - g["zero_point_energy_density"]) <= 1e-15 * abs(g["zero_point_energy_density"])
    assert abs(sc[3] - g["bg_energy_weight"]) <= 1e-15 * g["bg_energy_weight"]
    assert abs(sc[4] - g["bg_energy_density"]) <= 1e-14 * g["bg_energy_density"]
    assert abs(sc[5] - g["bg_energy_density_exact"]) <= 1e-13 * g["bg_energy_density_exact"]
    assert abs(sc[6] - g["bg_heat_capacity_density"]) <= 1e-12 * g["bg_heat_capacity_density"]

    def q(what, flat, x, aux=0.0):
        x = _f64(x)
        out = np.zeros(x.size)
        fl = _i32(flat if flat is not None else np.zeros(x.size))
        rc = oracle_lib.orc_material_query(m.h, what, x.size, I32(fl), D(x), C.c_double(aux), D(out))
        assert rc == 0
        return out

    # lookup tables are bit-exact up to the order of the per-mode energy sum
    assert np.allclose(q(4, None, g["table_T"]), g["table_E"], rtol=1e-13, atol=0)
    T = q(5, None, g["inv_E"])
    assert np.allclose(T, g["inv_T"], rtol=1e-11, atol=1e-9)
    assert np.allclose(q(6, None, g["crystal_T"]), g["crystal_E"], rtol=1e-13, atol=0)
    flat, Tq = g["q_mode"], g["q_T"]
    assert np.array_equal(q(0, flat, Tq), np.asarray(g["q_bose"]))
    assert np.array_equal(q(1, flat, Tq), np.asarray(g["q_capacity"]))
    assert np.array_equal(q(2, flat, Tq, 0.5), np.asarray(g["q_relax_dt0p5"]))
    assert np.array_equal(q(3, flat, Tq, 300.0), np.asarray(g["q_linearized_300"]))


def test_box_trace_and_grid(oracle_lib):
    g = golden("box_trace")
    p = _f64(g["ray_p"])
    v = _f64(g["ray_v"])
    n = p.shape[0]
    hit = np.zeros((n, 3))
    t = np.zeros(n)
    f = np.zeros(n, dtype=np.int32)
    lo, hi = _f64([0, 0, 0]), _f64([1000, 800, 600])
    assert oracle_lib.orc_trace_box(D(lo), D(hi), n, D(p), D(v), D(hit), D(t), I32(f)) == 0
    assert np.array_equal(f, np.asarray(g["hit_f"], dtype=np.int32))
    ok = f >= 0
    assert np.array_equal(t[ok], np.asarray(g["hit_t"])[ok])
    assert np.array_equal(hit[ok], np.asarray(g["hit_p"])[ok])
    gi = np.zeros(n, dtype=np.int32)
    sizes = _f64([1000, 800, 600])
    grid = _i32([3, 2, 5])
    assert oracle_lib.orc_grid_index(D(sizes), I32(grid), n, D(p), I32(gi)) == 0
    assert np.array_equal(gi, np.asarray(g["grid_index"], dtype=np.int32))
    # facet order, normals, areas and grid of the reference box
    assert np.array_equal(np.asarray(g["facet_normals"]),
                          np.array([[-1, 0, 0], [1, 0, 0], [0, -1, 0], [0, 1, 0], [0, 0, -1], [0, 0, 1]]))
    assert g["facet_areas"] == [480000, 480000, 600000, 600000, 800000, 800000]
    assert len(g["grid_volumes"]) == 30 and np.allclose(g["grid_volumes"], 480000000 / 30)


@pytest.mark.parametrize("name", ["rta_fixed", "rta_local"])
def test_rta_collision(oracle_lib, m8, name):
    g = golden(name)
    m = _mat(oracle_lib, m8)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    cT = _f64(g["cell_T"])
    res = C.c_double()
    rc = oracle_lib.orc_rta_collide(m.h, flat.size, I32(flat), I32(cell), D(occ), cT.size, D(cT),
                                    C.c_double(g["dt"]), C.c_double(g["particle_volume"]), int(g["local"]),
                                    C.c_double(g["lifetime_T"]), C.byref(res))
    assert rc == 0
    ref = np.asarray(g["occ_out"])
    assert np.allclose(occ, ref, rtol=1e-12, atol=1e-15)
    # the residual is a round-off sized number; compare on the energy scale
    assert abs(res.value - g["residual"]) < 1e-11


def test_linearized_rta(oracle_lib, m8):
    g = golden("linearized_rta")
    m = _mat(oracle_lib, m8, True)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    res = C.c_double()
    rc = oracle_lib.orc_linear_collide(m.h, 0, C.c_double(300.0), flat.size, I32(flat), I32(cell), D(occ),
                                       int(cell.max()) + 1, C.c_double(g["dt"]), C.c_double(g["particle_volume"]),
                                       C.byref(res))
    assert rc == 0, oracle_lib.orc_last_error()
    assert np.allclose(occ, g["occ_out"], rtol=1e-12, atol=1e-15)
    assert abs(res.value - g["residual"]) < 1e-13


def test_callaway_evolve(oracle_lib):
    g = golden("callaway_evolve")
    for case in g["cases"]:
        n = len(case["omega"])
        out = np.zeros(n)
        args = [_f64(case[k]) for k in ("omega", "capacity", "wavevector", "normal_rate", "resistive_rate", "energy")]
        rc = oracle_lib.orc_callaway_evolve(n, *[D(a) for a in args], C.c_double(case["dt"]), D(out))
        assert rc == 0
        ref = np.asarray(case["evolved"])
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name,conservative", [("rough_nonconservative", 0), ("rough_conservative", 1)])
def test_rough_reflection(oracle_lib, m8, name, conservative):
    g = golden(name)
    m = _mat(oracle_lib, m8, bool(conservative))
    draws = _f64(g["draws"]).reshape(-1, 3)
    facet = np.asarray(g["facet"])
    for f, (normal, rough) in enumerate([((0, 0, -1), 10.0), ((0, 0, 1), 3.0)]):
        sel = facet == f
        fin = _i32(np.asarray(g["in_flat"])[sel])
        oin = _f64(np.asarray(g["in_occ"])[sel])
        u = _f64(np.clip(draws[sel], 0, None))
        fo = np.zeros(fin.size, dtype=np.int32)
        oo = np.zeros(fin.size)
        rc = oracle_lib.orc_rough_reflect(m.h, conservative, C.c_double(300.0), D(_f64(normal)), C.c_double(rough),
                                          fin.size, I32(fin), D(oin), D(u), I32(fo), D(oo))
        assert rc == 0
        assert np.array_equal(fo, np.asarray(g["out_flat"])[sel])
        assert np.array_equal(oo, np.asarray(g["out_occ"])[sel])


def test_gradient_drive(oracle_lib, m8):
    g = golden("gradient_drive")
    m = _mat(oracle_lib, m8, True)
    flat, cell = _i32(g["flat"]), _i32(g["cell"])
    occ = _f64(g["occ_in"]).copy()
    e = C.c_double()
    rc = oracle_lib.orc_gradient_drive(m.h, 0, C.c_double(g["gradient"]), C.c_double(300.0), flat.size, I32(flat),
                                       I32(cell), D(occ), 4, C.c_double(g["dt"]), C.c_double(g["particle_volume"]),
                                       C.byref(e))
    assert rc == 0
    assert np.array_equal(occ, np.asarray(g["occ_out"]))
    assert abs(e.value - g["energy"]) < 1e-15


def test_reservoir_cdf(oracle_lib, m8):
    g = golden("reservoir")
    m = _mat(oracle_lib, m8)
    na = m8.qpoints  # upper bound for buffer
    cdf = np.zeros(6 * na)
    exp = C.c_double()
    init = C.c_int32()
    counts = []
    for r, normal in enumerate([(0, 0, -1), (0, 0, 1)]):
        rc = oracle_lib.orc_reservoir_cdf(m.h, D(_f64(normal)), C.c_double(g["area"]), C.c_double(g["density"]),
                                          C.c_double(g["dt"]), D(cdf), C.byref(exp), C.byref(init))
        assert rc == 0
        counts.append(init.value)
        draws = np.asarray(g["draw"])[r * 300:(r + 1) * 300]
        active = 1512
        idx = np.searchsorted(cdf[:active], draws, side="left")
        idx = np.minimum(idx, active - 1)
        assert np.array_equal(idx, np.asarray(g["active_index"])[r * 300:(r + 1) * 300])
    assert counts == g["initial_count"]


def _alias(oracle_lib, w, u):
    w = _f64(w)
    u = _f64(u)
    n = w.size
    prob, alias, out = np.zeros(n), np.zeros(n, np.int32), np.zeros(u.size, np.int32)
    assert oracle_lib.orc_alias_table(D(w), n, D(prob), I32(alias), u.size, D(u), I32(out)) == 0
    return prob, alias, out


def _alias_mass(prob, alias):
    """Probability of each outcome implied by an alias table."""
    n = prob.size
    q = np.clip(prob, 0.0, 1.0).copy()
    np.add.at(q, alias, 1.0 - np.clip(prob, 0.0, 1.0))
    return q / n


def test_reservoir_alias_tables_reproduce_the_emission_cdf(oracle_lib, m8):
    """The emission mode is drawn through an alias table of the reservoir's
    flux weights (one uniform, O(1)) in place of the reference's lower_bound
    over the normalised roulette (ReservoirSampler.cpp:117-146). Same
    distribution: the table's implied probabilities equal the CDF's steps, a
    mode of zero inward flux is never drawn, and 4096 stratified uniforms per
    column reproduce the steps to 1/4096 of a column."""
    g = golden("reservoir")
    m = _mat(oracle_lib, m8)
    cdf = np.zeros(6 * m8.qpoints)
    exp, init = C.c_double(), C.c_int32()
    active = 1512
    for r, normal in enumerate([(0, 0, -1), (0, 0, 1)]):
        assert oracle_lib.orc_reservoir_cdf(m.h, D(_f64(normal)), C.c_double(g["area"]), C.c_double(g["density"]),
                                            C.c_double(g["dt"]), D(cdf), C.byref(exp), C.byref(init)) == 0
        c = cdf[:active]
        step = np.diff(c, prepend=0.0)
        per = 4096
        u = (np.arange(active * per) + 0.5) / (active * per)
        prob, alias, out = _alias(oracle_lib, step, u)
        q = _alias_mass(prob, alias)
        assert np.max(np.abs(q - step / step.sum())) < 1e-15
        zero = step == 0.0
        assert zero.any() and not zero.all()
        assert np.all(prob[zero] == 0.0) and not np.isin(np.flatnonzero(zero), alias[prob < 1.0]).any()
        counts = np.bincount(out, minlength=active)
        assert np.all(counts[zero] == 0)
        targets = np.bincount(alias[prob < 1.0], minlength=active)
        assert np.all(np.abs(counts / u.size - q) <= (1 + targets) / u.size)
        # the reference's own draws all fall on modes the table can draw
        ref_modes = np.asarray(g["active_index"])[r * 300:(r + 1) * 300]
        assert not np.isin(ref_modes, np.flatnonzero(zero)).any()


def test_alias_table_edge_weights(oracle_lib):
    """Zeros, a dominant weight, subnormal-scale weights and a single outcome."""
    rng = np.random.default_rng(5)
    cases = [np.array([0.0, 0.0, 3.0, 0.0]), np.array([1e-300, 1.0, 1e-300, 0.0]), np.array([7.0]),
             np.r_[np.zeros(50), rng.random(2000) ** 8, [1e6], np.zeros(7)], np.ones(1000)]
    for w in cases:
        u = np.r_[rng.random(4096), 0.0, np.nextafter(1.0, 0.0)]
        prob, alias, out = _alias(oracle_lib, w, u)
        q = _alias_mass(prob, alias)
        assert np.max(np.abs(q - w / w.sum())) <= 4e-16 * w.size
        assert np.all(w[out] > 0.0)
    for bad in (np.zeros(3), np.array([1.0, -1.0]), np.array([1.0, np.nan])):
        assert oracle_lib.orc_alias_table(D(_f64(bad)), bad.size, D(np.zeros(bad.size)),
                                          I32(np.zeros(bad.size, np.int32)), 0, D(np.zeros(1)),
                                          I32(np.zeros(1, np.int32))) != 0


@pytest.mark.parametrize("name,linearized", [("interface_dmm", 0), ("interface_dmm_linearized", 1)])
def test_interface_dmm(oracle_lib, name, linearized):
    """Diffuse-mismatch interface events against InterfaceInteraction::interact,
    with the reference engine's draws replayed (bit-exact modes and occupations)."""
    from phonomc_gb300 import synthetic
    g = golden(name)
    ma = abi.Material(oracle_lib, "orc_", synthetic.make_material(mesh=8), 0.1, False, False)
    mb = abi.Material(oracle_lib, "orc_", synthetic.make_material(mesh=8, freq_scale=0.7, vel_scale=0.75), 0.1,
                      False, False)
    n = len(g["src"])
    src, flat, signs = (np.ascontiguousarray(g[k], dtype=np.int32) for k in ("src", "in_flat", "in_signs"))
    occ = np.ascontiguousarray(g["in_occ"], dtype=np.float64)
    u3 = np.ascontiguousarray(g["draws"], dtype=np.float64)
    act, mat, fo, so = (np.zeros(n, np.int32) for _ in range(4))
    oo = np.zeros(n)
    I = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731
    rc = oracle_lib.orc_interface(ma.h, mb.h, g["weight_a"], g["weight_b"], g["axis"], g["frequency_bin_thz"],
                                  g["reference_temperature"], linearized, n, I(src), I(flat), I(signs), D(occ), D(u3),
                                  I(act), I(mat), I(fo), I(so), D(oo))
    assert rc == 0, oracle_lib.orc_last_error()
    assert np.array_equal(act, g["action"])
    assert np.array_equal(mat, g["out_material"])
    assert np.array_equal(fo, g["out_flat"])
    assert np.array_equal(oo, np.asarray(g["out_occ"]))
    # velocity: table velocity of the outgoing mode with the outgoing sign bits
    for k, m in enumerate((ma, mb)):
        sel = mat == k
        if not sel.any():
            continue
        v = np.array(synthetic.make_material(mesh=8, **({} if k == 0 else {"freq_scale": 0.7, "vel_scale": 0.75}))
                     .group_velocity).reshape(-1, 3)[fo[sel]]
        sg = np.stack([1 - 2 * ((so[sel] >> b) & 1) for b in range(3)], axis=1)
        assert np.array_equal(v * sg, np.asarray(g["out_v"]).reshape(-1, 3)[sel])


def _amm_materials(lib):
    from phonomc_gb300 import synthetic
    return (abi.Material(lib, "orc_", synthetic.make_material(mesh=8), 0.1, False, False),
            abi.Material(lib, "orc_", synthetic.make_material(mesh=8, freq_scale=0.7, vel_scale=0.75), 0.1, False,
                         False))


def test_amm_rows_match_reference(oracle_lib):
    """Acoustic-mismatch rows (AcousticInterfaceSampler::configure): mirror
    partners and transmitted destinations exact, probabilities to 1e-12, for
    both sides of the interface between the 8^3 table and its softened copy."""
    g = golden("interface_amm")
    ma, mb = _amm_materials(oracle_lib)
    I = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731
    for side in (0, 1):
        n = len(g[f"reflected_{side}"])
        refl, start = np.zeros(n, np.int32), np.zeros(n + 1, np.int32)
        assert oracle_lib.orc_amm_rows(ma.h, mb.h, g["density_a"], g["density_b"], g["frequency_bin_thz"],
                                       g["parallel_bin_inv_a"], side, I(refl), I(start), None, None) == 0, \
            oracle_lib.orc_last_error()
        dest, prob = np.zeros(start[-1], np.int32), np.zeros(start[-1])
        assert oracle_lib.orc_amm_rows(ma.h, mb.h, g["density_a"], g["density_b"], g["frequency_bin_thz"],
                                       g["parallel_bin_inv_a"], side, I(refl), I(start), I(dest), D(prob)) == 0
        assert np.array_equal(refl, g[f"reflected_{side}"])
        assert np.array_equal(start, g[f"start_{side}"])
        assert np.array_equal(dest, g[f"dest_{side}"])
        assert np.allclose(prob, g[f"prob_{side}"], rtol=1e-12, atol=0)
        assert start[-1] > 0


@pytest.mark.parametrize("name,linearized", [("interface_amm", 0), ("interface_amm_linearized", 1),
                                             ("interface_mmm", 0)])
def test_interface_amm_events(oracle_lib, name, linearized):
    """Acoustic and mixed-mismatch interface events against
    InterfaceInteraction::interact with the reference engine's draws replayed:
    model choice, row sample or diffuse bands, outgoing mode and occupation."""
    g = golden(name)
    ma, mb = _amm_materials(oracle_lib)
    n = len(g["src"])
    src, flat = (np.ascontiguousarray(g[k], dtype=np.int32) for k in ("src", "in_flat"))
    occ = np.ascontiguousarray(g["in_occ"], dtype=np.float64)
    u4 = np.ascontiguousarray(g["draws"], dtype=np.float64)
    act, mat, fo = (np.zeros(n, np.int32) for _ in range(3))
    oo = np.zeros(n)
    I = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731
    rc = oracle_lib.orc_interface_model(ma.h, mb.h, g["weight_a"], g["weight_b"], g["frequency_bin_thz"],
                                        g["reference_temperature"], linearized, g["model"], g["amm_fraction"],
                                        g["density_a"], g["density_b"], g["parallel_bin_inv_a"], n, I(src), I(flat),
                                        D(occ), D(u4), I(act), I(mat), I(fo), D(oo))
    assert rc == 0, oracle_lib.orc_last_error()
    assert np.array_equal(act, g["action"])
    assert np.array_equal(mat, g["out_material"])
    assert np.array_equal(fo, g["out_flat"])
    assert np.array_equal(oo, np.asarray(g["out_occ"]))
    assert (act == 4).sum() == sum(g["transmitted"]) > 0


SOURCE_CASES = {"source_thermal": ("thermal", 0), "source_thermal_linearized": ("thermal", 1),
                "source_weighted": ("weighted", 0), "source_gaussian": ("gaussian", 0)}


def _source_spec(spectrum):
    h = {"profile": "gaussian", "center": (180.0, 130.0, 90.0), "sigma": (160.0, 140.0, 70.0),
         "power_density": 3e19, "spectrum": spectrum, "frequency_max": 14.0}
    if spectrum == "weighted":
        h.update(branch_weights=[1.0, 2.0, 1.5, 0.5, 0.25, 0.0], branches=[0, 1, 2, 3, 4])
    if spectrum == "gaussian":
        h.update(frequency_center=6.0, frequency_sigma=2.5)
    return h


def test_source_cell_rates(oracle_lib):
    """PrescribedHeatSource cell powers of a Gaussian source (bit-exact)."""
    g = golden("source_thermal")
    cfg = {"sizes": (500.0, 400.0, 300.0), "grid": (2, 2, 3), "faces": ("P", "P", "P", "P", "T", "T"),
           "face_values": (0, 0, 0, 0, 301.0, 299.0), "heat_source": _source_spec("thermal")}
    pod, keep = abi.config_pod(cfg)
    rates = np.zeros(64)
    n = C.c_int32()
    assert oracle_lib.orc_source_rates(C.byref(pod), D(rates), C.byref(n)) == 0, oracle_lib.orc_last_error()
    assert np.array_equal(rates[:n.value], np.asarray(g["rates"]))
    assert np.array_equal(rates[:n.value] * g["factor"], np.asarray(g["pending_before"]))


@pytest.mark.parametrize("name", list(SOURCE_CASES))
def test_source_apply(oracle_lib, name):
    """PhononSourceOperator::apply: per-carrier increments in each spectrum, the
    round-off correction carrier, cells without eligible carriers keep their
    budget (occupations within 1e-15 relative: the reference sums capacities and
    Gaussian weights in long double)."""
    from phonomc_gb300 import synthetic
    g = golden(name)
    spectrum, linearized = SOURCE_CASES[name]
    m = abi.Material(oracle_lib, "orc_", synthetic.make_material(mesh=8), 0.1, True, False)
    keep = []
    hs = abi.heat_source_pod(_source_spec(spectrum), keep)
    flat, cell = (np.ascontiguousarray(g[k], dtype=np.int32) for k in ("flat", "cell"))
    occ = np.ascontiguousarray(g["occ_in"], dtype=np.float64).copy()
    pend = np.ascontiguousarray(g["pending_before"], dtype=np.float64).copy()
    cT = np.ascontiguousarray(g["cell_temperature"], dtype=np.float64)
    e, up = C.c_double(), C.c_int64()
    rc = oracle_lib.orc_source_apply(m.h, C.byref(hs), linearized, 300.0, g["particle_volume"], cT.size, D(cT), D(pend),
                                     flat.size, flat.ctypes.data_as(abi.c_int32_p), cell.ctypes.data_as(abi.c_int32_p),
                                     D(occ), C.byref(e), C.byref(up))
    assert rc == 0, oracle_lib.orc_last_error()
    assert up.value == g["updates"]
    assert e.value == g["energy"]
    assert np.array_equal(pend, np.asarray(g["pending_after"]))
    assert np.allclose(occ, g["occ_out"], rtol=1e-15, atol=1e-18)
    assert np.array_equal(occ == np.asarray(g["occ_in"]), np.asarray(g["occ_out"]) == np.asarray(g["occ_in"]))


def test_mesh_trace(oracle_lib):
    """Ray traces through the procedural FinFET surface against the reference's
    SurfaceMesh::trace_boundary_intersection: facet ids and hit times bit-exact."""
    g = golden("mesh_finfet")
    V = np.ascontiguousarray(g["vertices"], dtype=np.float64)
    F = np.ascontiguousarray(g["faces"], dtype=np.int32)
    f2f = np.ascontiguousarray(g["face_to_facet"], dtype=np.int32)
    P = np.ascontiguousarray(g["origins"], dtype=np.float64)
    Vel = np.ascontiguousarray(g["velocities"], dtype=np.float64)
    n = P.shape[0]
    hit, t, fac = np.zeros((n, 3)), np.zeros(n), np.zeros(n, np.int32)
    I = lambda a: a.ctypes.data_as(abi.c_int32_p)  # noqa: E731
    rc = oracle_lib.orc_trace_mesh(V.shape[0], D(V), F.size // 3, I(F), I(f2f), n, D(P), D(Vel), D(hit), D(t), I(fac))
    assert rc == 0, oracle_lib.orc_last_error()
    assert np.array_equal(fac, g["facet"])
    assert np.array_equal(t, np.asarray(g["t"]))
    assert np.array_equal(hit, np.asarray(g["hits"]))


@pytest.mark.parametrize("name", ["ncallaway_unique", "ncallaway_shared", "ncallaway_large"])
def test_nonlinear_callaway_evolve(oracle_lib, name):
    """The oracle's per-carrier nonlinear Callaway (long double, as the
    reference) against src/solver/NonlinearCallawayCollision.cpp's own
    nonlinear_callaway_evolve on seeded single-cell cases."""
    g = golden(name)
    mode = _i32(g["mode"])
    occ = _f64(g["n"]).copy()
    rc = oracle_lib.orc_ncallaway_evolve(len(g["omega"]), D(_f64(g["omega"])), D(_f64(g["k"])), D(_f64(g["rn"])),
                                         D(_f64(g["rr"])), mode.size, I32(mode), D(occ), C.c_double(g["T"]),
                                         C.c_double(g["dt"]))
    assert rc == 0, oracle_lib.orc_last_error()
    assert np.allclose(occ, g["out"], rtol=1e-14, atol=0)


def test_nonlinear_callaway_config(oracle_lib):
    """Nonlinear Callaway needs the Callaway model and no gradient drive
    (src/config/ConfigValidation.cpp:349-354); a film runs with it and its
    energy ledger closes."""
    from phonomc_gb300 import synthetic, workloads
    mat = synthetic.make_material(mesh=8, callaway=True)
    m = abi.Material(oracle_lib, "orc_", mat, 0.1, True, True)
    bad = workloads.scaled(workloads.cross_plane_film(), 2000, callaway_formulation="nonlinear")
    with pytest.raises(abi.LibError, match="Nonlinear Callaway requires model=callaway"):
        abi.Solver(oracle_lib, "orc_", bad, [m])
    cfg = dict(bad, collision_model="callaway")
    s = abi.Solver(oracle_lib, "orc_", cfg, [m])
    s.run(3)
    st = s.stats()
    assert st["current_timestep"] == 3
    assert abs(st["total_energy_balance_residual_ev"]) < 1e-6
    assert st["total_lifetime_energy_residual_ev"] != 0.0
