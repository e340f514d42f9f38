"""ctypes mirror of the C ABI in include/phonomc_gb300.h.

The structs here are byte-for-byte the ones the header declares; `bind()`
attaches argument/return types to every entry point of a loaded library.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import synthetic

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)
c_uint32_p = C.POINTER(C.c_uint32)
c_uint8_p = C.POINTER(C.c_uint8)
c_int64_p = C.POINTER(C.c_int64)


class MaterialDataPOD(C.Structure):
    _fields_ = [
        ("qpoints", C.c_int32), ("branches", C.c_int32), ("mesh", C.c_int32 * 3), ("ntemps", C.c_int32),
        ("volume_a3", C.c_double), ("reciprocal", C.c_double * 9),
        ("frequency_thz", c_double_p), ("qpoint_fractions", c_double_p), ("group_velocity", c_double_p),
        ("temperatures", c_double_p), ("gamma", c_double_p), ("gamma_normal", c_double_p),
        ("gamma_umklapp", c_double_p), ("gamma_isotope", c_double_p), ("gamma_isotope_len", C.c_int64),
    ]


class HeatSourcePOD(C.Structure):
    _fields_ = [
        ("profile", C.c_int32), ("has_box", C.c_int32), ("min", C.c_double * 3), ("max", C.c_double * 3),
        ("n_centers", C.c_int32), ("centers", c_double_p), ("sigma", C.c_double * 3), ("half_width", C.c_double * 3),
        ("power_density", C.c_double), ("has_total_power", C.c_int32), ("total_power", C.c_double),
        ("n_power_densities", C.c_int32), ("power_densities", c_double_p), ("spectrum", C.c_int32),
        ("has_frequency_gaussian", C.c_int32), ("frequency_center", C.c_double), ("frequency_sigma", C.c_double),
        ("frequency_min", C.c_double), ("frequency_max", C.c_double), ("n_branches", C.c_int32),
        ("branches", c_int32_p), ("n_branch_weights", C.c_int32), ("branch_weights", c_double_p),
        ("time_profile", C.c_int32), ("time_start", C.c_double), ("time_end", C.c_double), ("period", C.c_double),
        ("on_duration", C.c_double), ("duty_cycle", C.c_double), ("amplitude", C.c_double),
    ]


def heat_source_pod(h: dict, keep: list) -> HeatSourcePOD:
    """HeatSourcePOD from a dict of [heat_source] fields (lengths in Angstrom, THz, ps)."""
    p = HeatSourcePOD()
    p.profile = 1 if h.get("profile", "uniform") == "gaussian" else 0
    if "min" in h and "max" in h:
        p.has_box = 1
        p.min[:] = list(h["min"])
        p.max[:] = list(h["max"])
    centers = h.get("centers") or ([h["center"]] if "center" in h else [])
    if centers:
        arr = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1))
        keep.append(arr)
        p.n_centers = arr.size // 3
        p.centers = dptr(arr)
    p.sigma[:] = list(h.get("sigma", (0.0, 0.0, 0.0)))
    p.half_width[:] = list(h.get("half_width", (0.0, 0.0, 0.0)))
    p.power_density = float(h.get("power_density", 0.0))
    if "total_power" in h:
        p.has_total_power = 1
        p.total_power = float(h["total_power"])
    if "power_densities" in h:
        arr = np.ascontiguousarray(h["power_densities"], dtype=np.float64)
        keep.append(arr)
        p.n_power_densities = arr.size
        p.power_densities = dptr(arr)
    p.spectrum = {"thermal": 0, "weighted": 1, "gaussian": 2}[h.get("spectrum", "thermal")]
    if "frequency_center" in h or "frequency_sigma" in h:
        p.has_frequency_gaussian = 1
        p.frequency_center = float(h.get("frequency_center", 0.0))
        p.frequency_sigma = float(h.get("frequency_sigma", 0.0))
    p.frequency_min = float(h.get("frequency_min", -1.0))
    p.frequency_max = float(h.get("frequency_max", -1.0))
    if "branches" in h:
        arr = np.ascontiguousarray(h["branches"], dtype=np.int32)
        keep.append(arr)
        p.n_branches = arr.size
        p.branches = arr.ctypes.data_as(c_int32_p)
    if "branch_weights" in h:
        arr = np.ascontiguousarray(h["branch_weights"], dtype=np.float64)
        keep.append(arr)
        p.n_branch_weights = arr.size
        p.branch_weights = dptr(arr)
    p.time_profile = 1 if h.get("time_profile", "constant") == "pulsed" else 0
    p.time_start = float(h.get("time_start", 0.0))
    p.time_end = float(h.get("time_end", -1.0))
    p.period = float(h.get("period", 0.0))
    p.on_duration = float(h.get("on_duration", -1.0))
    p.duty_cycle = float(h.get("duty_cycle", 0.5))
    p.amplitude = float(h.get("amplitude", 1.0))
    return p


class MeshDomainPOD(C.Structure):
    _fields_ = [
        ("model", C.c_char_p), ("n_vertices", C.c_int64), ("vertices", c_double_p), ("n_faces", C.c_int64),
        ("faces", c_int32_p), ("merge_coplanar_facets", C.c_int32), ("n_regions", C.c_int32),
        ("boundary_position", c_double_p), ("boundary_conditions", C.c_char_p), ("boundary_values", c_double_p),
        ("n_periodic_regions", C.c_int32), ("periodic_pair", c_double_p), ("extruded_z", C.c_int32),
    ]


def mesh_domain_pod(m: dict, keep: list) -> MeshDomainPOD:
    """MeshDomainPOD from {"model": path | None, "vertices": [n,3] Angstrom, "faces": [m,3],
    "merge_coplanar_facets": bool, "extruded_z": bool, "regions": [(box6, cond, value)],
    "periodic_pair": [box6, ...]}."""
    p = MeshDomainPOD()
    if m.get("model"):
        b = str(m["model"]).encode()
        keep.append(b)
        p.model = b
    else:
        v = np.ascontiguousarray(m["vertices"], dtype=np.float64).reshape(-1, 3)
        f = np.ascontiguousarray(m["faces"], dtype=np.int32).reshape(-1, 3)
        keep.extend([v, f])
        p.n_vertices, p.vertices = v.shape[0], dptr(v)
        p.n_faces, p.faces = f.shape[0], f.ctypes.data_as(c_int32_p)
    p.merge_coplanar_facets = int(m.get("merge_coplanar_facets", True))
    p.extruded_z = int(m.get("extruded_z", False))
    regions = m.get("regions", [])
    if regions:
        pos = np.ascontiguousarray([r[0] for r in regions], dtype=np.float64).reshape(-1)
        cond = "".join(r[1] for r in regions).encode()
        val = np.ascontiguousarray([r[2] for r in regions], dtype=np.float64)
        keep.extend([pos, cond, val])
        p.n_regions = len(regions)
        p.boundary_position, p.boundary_conditions, p.boundary_values = dptr(pos), cond, dptr(val)
    pairs = m.get("periodic_pair", [])
    if pairs:
        arr = np.ascontiguousarray(pairs, dtype=np.float64).reshape(-1)
        keep.append(arr)
        p.n_periodic_regions = len(pairs)
        p.periodic_pair = dptr(arr)
    return p


class ConfigPOD(C.Structure):
    _fields_ = [
        ("sizes", C.c_double * 3), ("particle_count", C.c_double), ("time_step", C.c_double),
        ("iterations", C.c_int32), ("convergence_write_interval", C.c_int32), ("random_seed", C.c_uint64),
        ("compute_kappa", C.c_int32), ("transport_axis", C.c_int32), ("has_temperature_gradient", C.c_int32),
        ("temperature_gradient", C.c_double), ("temperature_lookup_dt", C.c_double),
        ("background_temperature", C.c_double), ("lifetime_temperature_is_local", C.c_int32),
        ("lifetime_temperature", C.c_double), ("collision_model", C.c_int32),
        ("conservative_boundaries", C.c_int32), ("grid", C.c_int32 * 3),
        ("initial_temperature_linear", C.c_int32), ("initial_temperature", C.c_double),
        ("face_condition", C.c_char * 6), ("face_value", C.c_double * 6), ("output_folder", C.c_char_p),
        ("material_interface_axis", C.c_int32), ("n_interfaces", C.c_int32),
        ("material_interface_positions", c_double_p), ("interface_frequency_bin_thz", C.c_double),
        ("precision", C.c_int32), ("heat_source", C.POINTER(HeatSourcePOD)),
        ("mesh", C.POINTER(MeshDomainPOD)), ("material_folder", C.c_char_p),
        ("write_cell_heat_flux", C.c_int32), ("callaway_nonlinear", C.c_int32),
        ("carrier_sort_interval", C.c_int32), ("transport_block", C.c_int32),
        ("transport_blocks_per_sm", C.c_int32), ("tally_aggregation", C.c_int32),
        ("transport_pipeline", C.c_int32),
        ("interface_model", C.c_int32), ("interface_amm_fraction", C.c_double),
        ("interface_parallel_bin_inv_a", C.c_double), ("n_mass_densities", C.c_int32),
        ("mass_densities_kg_m3", c_double_p), ("rta_cell_update", C.c_int32),
    ]


class StatsPOD(C.Structure):
    _fields_ = [
        ("current_timestep", C.c_int32), ("particle_count", C.c_int64), ("absorbed_total", C.c_int64),
        ("injected_total", C.c_int64), ("step_absorbed", C.c_int64), ("step_injected", C.c_int64),
        ("step_absorbed_energy_ev", C.c_double), ("step_injected_energy_ev", C.c_double),
        ("total_thermal_energy_ev", C.c_double), ("total_lifetime_energy_residual_ev", C.c_double),
        ("step_lifetime_energy_residual_ev", C.c_double), ("total_energy_balance_residual_ev", C.c_double),
        ("step_energy_balance_residual_ev", C.c_double), ("total_gradient_energy_ev", C.c_double),
        ("step_gradient_energy_ev", C.c_double), ("step_gradient_updates", C.c_int64),
        ("average_heat_flux_along_axis", C.c_double), ("kappa_fit", C.c_double),
        ("kappa_endpoints", C.c_double), ("interface_events", C.c_int64),
        ("interface_transmitted", C.c_int64), ("interface_reflected", C.c_int64),
        ("device_launches", C.c_int64), ("total_heat_source_energy_ev", C.c_double),
        ("step_heat_source_energy_ev", C.c_double), ("prescribed_heat_source_energy_ev", C.c_double),
        ("pending_heat_source_energy_ev", C.c_double), ("step_heat_source_updates", C.c_int64),
        ("rough_counts", C.c_int64 * 8), ("collision_cache_corrections", C.c_int64),
    ]

    def as_dict(self) -> dict:
        out = {name: getattr(self, name) for name, _ in self._fields_}
        out["rough_counts"] = list(self.rough_counts)
        return out


def dptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(c_double_p)


def material_pod(d: synthetic.MaterialData):
    """Pack a MaterialData; returns (pod, keepalive) so the arrays outlive the call."""
    keep = []

    def arr(x):
        if x is None:
            return None
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return a

    pod = MaterialDataPOD()
    pod.qpoints = d.qpoints
    pod.branches = d.branches
    for i in range(3):
        pod.mesh[i] = int(d.mesh[i])
    pod.ntemps = int(d.temperatures.size)
    pod.volume_a3 = float(d.volume_a3)
    R = np.asarray(d.reciprocal, dtype=np.float64).reshape(3, 3)
    for i in range(9):
        pod.reciprocal[i] = float(R.reshape(-1)[i])
    pod.frequency_thz = dptr(arr(d.frequency_thz))
    pod.qpoint_fractions = dptr(arr(d.qpoint_fractions))
    pod.group_velocity = dptr(arr(d.group_velocity))
    pod.temperatures = dptr(arr(d.temperatures))
    pod.gamma = dptr(arr(d.gamma))
    pod.gamma_normal = dptr(arr(d.gamma_normal))
    pod.gamma_umklapp = dptr(arr(d.gamma_umklapp))
    iso = d.gamma_resistive.get("gamma_isotope")
    pod.gamma_isotope = dptr(arr(iso))
    pod.gamma_isotope_len = 0 if iso is None else int(np.asarray(iso).size)
    return pod, keep


def config_pod(cfg: dict):
    """Build a ConfigPOD from a dict of SimulationConfig-style fields (internal units)."""
    keep = []
    c = ConfigPOD()
    c.sizes[:] = list(cfg.get("sizes", (200.0, 200.0, 200.0)))
    c.particle_count = float(cfg.get("particle_count", 1e4))
    c.time_step = float(cfg.get("time_step", 1.0))
    c.iterations = int(cfg.get("iterations", 10000))
    c.convergence_write_interval = int(cfg.get("convergence_write_interval", 10))
    c.random_seed = int(cfg.get("random_seed", 12345))
    c.compute_kappa = int(cfg.get("compute_kappa", False))
    c.write_cell_heat_flux = int(cfg.get("write_cell_heat_flux", False))
    c.callaway_nonlinear = int(cfg.get("callaway_formulation", "linearized") == "nonlinear")
    c.carrier_sort_interval = int(cfg.get("carrier_sort_interval", 0))
    c.transport_block = int(cfg.get("transport_block", 0))
    c.transport_blocks_per_sm = int(cfg.get("transport_blocks_per_sm", 0))
    c.tally_aggregation = int(cfg.get("tally_aggregation", 0))
    c.transport_pipeline = int(cfg.get("transport_pipeline", 0))
    c.rta_cell_update = int(cfg.get("rta_cell_update", 0))
    c.interface_model = {"dmm": 0, "amm": 1, "mmm": 2}[cfg.get("interface_model", "dmm")]
    c.interface_amm_fraction = float(cfg.get("interface_amm_fraction", 0.0))
    c.interface_parallel_bin_inv_a = float(cfg.get("interface_parallel_bin_inv_a", 0.0))
    rho = np.ascontiguousarray(cfg.get("mass_densities_kg_m3", []), dtype=np.float64)
    keep.append(rho)
    c.n_mass_densities = int(rho.size)
    c.mass_densities_kg_m3 = dptr(rho) if rho.size else None
    c.transport_axis = int(cfg.get("transport_axis", -1))
    g = cfg.get("temperature_gradient")
    c.has_temperature_gradient = int(g is not None)
    c.temperature_gradient = float(g or 0.0)
    c.temperature_lookup_dt = float(cfg.get("temperature_lookup_dt", 0.1))
    c.background_temperature = float(cfg.get("background_temperature", 300.0))
    lt = cfg.get("lifetime_temperature", "local")
    c.lifetime_temperature_is_local = int(lt == "local")
    c.lifetime_temperature = 300.0 if lt == "local" else float(lt)
    c.collision_model = 1 if cfg.get("collision_model", "rta") == "callaway" else 0
    c.conservative_boundaries = int(cfg.get("conservative_boundaries", False))
    c.grid[:] = list(cfg.get("grid", (1, 1, 1)))
    it = cfg.get("initial_temperature", 300.0)
    c.initial_temperature_linear = int(it == "linear")
    c.initial_temperature = 300.0 if it == "linear" else float(it)
    c.face_condition = "".join(cfg.get("faces", "RRRRRR")).encode()
    c.face_value[:] = [float(v) for v in cfg.get("face_values", (0.0,) * 6)]
    of = cfg.get("output_folder")
    if of:
        b = of.encode()
        keep.append(b)
        c.output_folder = b
    c.material_interface_axis = int(cfg.get("material_interface_axis", 0))
    planes = np.ascontiguousarray(cfg.get("material_interface_positions", []), dtype=np.float64)
    keep.append(planes)
    c.n_interfaces = int(planes.size)
    c.material_interface_positions = dptr(planes) if planes.size else None
    c.interface_frequency_bin_thz = float(cfg.get("interface_frequency_bin_thz", 0.1))
    c.precision = 1 if cfg.get("precision", "fp64") == "mixed" else 0
    if cfg.get("heat_source"):
        hs = heat_source_pod(cfg["heat_source"], keep)
        keep.append(hs)
        c.heat_source = C.pointer(hs)
    if cfg.get("material_folder"):
        b = str(cfg["material_folder"]).encode()
        keep.append(b)
        c.material_folder = b
    if cfg.get("mesh"):
        mp = mesh_domain_pod(cfg["mesh"], keep)
        keep.append(mp)
        c.mesh = C.pointer(mp)
    return c, keep


# Host geometry (phmc_domain_*), product library only.
DOMAIN_PROTOS = {
    "domain_create": (C.c_int, [C.POINTER(ConfigPOD), C.POINTER(C.c_void_p)]),
    "domain_destroy": (None, [C.c_void_p]),
    "domain_info": (C.c_int, [C.c_void_p, c_int32_p, c_int32_p, c_int32_p, c_int32_p, c_double_p, c_double_p]),
    "domain_facets": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p, C.c_char_p, c_double_p, c_int32_p,
                                c_double_p]),
    "domain_cells": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_int32_p]),
    "domain_faces": (C.c_int, [C.c_void_p, c_int32_p, c_double_p]),
    "domain_contains": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_uint8_p]),
    "domain_voxel_interior": (C.c_int, [C.c_void_p, c_uint8_p]),
    "domain_grid_index": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_int32_p]),
    "domain_nearest_facet": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_int32_p]),
    "domain_trace": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p, c_int32_p]),
    "dev_domain_trace": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p, c_int32_p]),
    "dev_domain_query": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_uint8_p, c_int32_p, c_int32_p]),
    # material folders in the reference's layout (POSCAR + HDF5) and HDF5 datasets
    "material_load": (C.c_int, [C.c_char_p, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "material_save": (C.c_int, [C.POINTER(MaterialDataPOD), C.c_char_p]),
    "h5_shape": (C.c_int, [C.c_char_p, C.c_char_p, c_int32_p, c_int64_p]),
    "h5_read": (C.c_int, [C.c_char_p, C.c_char_p, c_double_p]),
}


SOLVER_PROTOS = {
    "last_error": (C.c_char_p, []),
    "material_create": (C.c_int, [C.POINTER(MaterialDataPOD), C.c_double, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "material_destroy": (None, [C.c_void_p]),
    "solver_create": (C.c_int, [C.POINTER(ConfigPOD), C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "solver_destroy": (None, [C.c_void_p]),
    "solver_run": (C.c_int, [C.c_void_p, C.c_int]),
    "solver_stats": (C.c_int, [C.c_void_p, C.POINTER(StatsPOD)]),
    "solver_cell_count": (C.c_int, [C.c_void_p, c_int32_p]),
    "solver_cells": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p]),
    "solver_slot_count": (C.c_int, [C.c_void_p, c_int64_p]),
    "solver_get_carriers": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p, c_uint32_p,
                                      c_int32_p, c_uint8_p]),
    "solver_set_carriers": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p,
                                      c_uint32_p, c_uint8_p]),
}


def bind(lib: C.CDLL, prefix: str, protos: dict) -> None:
    for name, (res, args) in protos.items():
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args


class LibError(RuntimeError):
    pass


class Handle:
    """Thin solver/material wrapper over a library with the solver ABI shape."""

    def __init__(self, lib: C.CDLL, prefix: str):
        self.lib = lib
        self.p = prefix

    def fn(self, name):
        return getattr(self.lib, self.p + name)

    def check(self, rc: int) -> None:
        if rc != 0:
            raise LibError(self.fn("last_error")().decode())


class Material(Handle):
    def __init__(self, lib, prefix, data: synthetic.MaterialData, lookup_dt=0.1, stationary=False,
                 complete_bz=False):
        super().__init__(lib, prefix)
        pod, keep = material_pod(data)
        h = C.c_void_p()
        self.check(self.fn("material_create")(C.byref(pod), lookup_dt, int(stationary), int(complete_bz),
                                              C.byref(h)))
        self.h = h
        self.data = data

    def close(self):
        if getattr(self, "h", None):
            self.fn("material_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FolderMaterial(Material):
    """A material read from a folder in the reference's layout (phmc_material_load)."""

    def __init__(self, lib, folder: str, lookup_dt=0.1, stationary=False, complete_bz=False):
        Handle.__init__(self, lib, "phmc_")
        h = C.c_void_p()
        self.check(lib.phmc_material_load(str(folder).encode(), lookup_dt, int(stationary), int(complete_bz),
                                          C.byref(h)))
        self.h = h
        self.data = None


def save_material(lib, data: synthetic.MaterialData, folder: str) -> None:
    """POSCAR + kappa-fbz.hdf5 of `data` in the reference's layout (phmc_material_save)."""
    pod, keep = material_pod(data)
    if lib.phmc_material_save(C.byref(pod), str(folder).encode()) != 0:
        raise LibError(lib.phmc_last_error().decode())


def h5_read(lib, path: str, name: str) -> np.ndarray:
    """One numeric HDF5 dataset as float64 (phmc_h5_shape / phmc_h5_read)."""
    rank, dims = C.c_int32(), (C.c_int64 * 8)()
    if lib.phmc_h5_shape(str(path).encode(), name.encode(), C.byref(rank), dims) != 0:
        raise LibError(lib.phmc_last_error().decode())
    shape = tuple(dims[k] for k in range(rank.value))
    out = np.zeros(int(np.prod(shape)) if shape else 1)
    if lib.phmc_h5_read(str(path).encode(), name.encode(), dptr(out)) != 0:
        raise LibError(lib.phmc_last_error().decode())
    return out.reshape(shape)


class Solver(Handle):
    def __init__(self, lib, prefix, cfg: dict, materials: Sequence[Material]):
        super().__init__(lib, prefix)
        pod, keep = config_pod(cfg)
        arr = (C.c_void_p * len(materials))(*[m.h for m in materials])
        h = C.c_void_p()
        self.check(self.fn("solver_create")(C.byref(pod), arr, len(materials), C.byref(h)))
        self.h = h
        self.materials = list(materials)
        self.cfg = dict(cfg)

    def run(self, steps: int = 1) -> None:
        self.check(self.fn("solver_run")(self.h, steps))

    def stats(self) -> dict:
        s = StatsPOD()
        self.check(self.fn("solver_stats")(self.h, C.byref(s)))
        return s.as_dict()

    def cells(self):
        n = C.c_int32()
        self.check(self.fn("solver_cell_count")(self.h, C.byref(n)))
        T = np.zeros(n.value)
        E = np.zeros(n.value)
        q = np.zeros((n.value, 3))
        self.check(self.fn("solver_cells")(self.h, dptr(T), dptr(E), dptr(q)))
        return T, E, q

    def carriers(self) -> dict:
        n = C.c_int64()
        self.check(self.fn("solver_slot_count")(self.h, C.byref(n)))
        n = n.value
        out = {k: np.zeros(n) for k in ("x", "y", "z", "occ")}
        out["mode"] = np.zeros(n, dtype=np.uint32)
        out["cell"] = np.zeros(n, dtype=np.int32)
        out["alive"] = np.zeros(n, dtype=np.uint8)
        self.check(self.fn("solver_get_carriers")(
            self.h, dptr(out["x"]), dptr(out["y"]), dptr(out["z"]), dptr(out["occ"]),
            out["mode"].ctypes.data_as(c_uint32_p), out["cell"].ctypes.data_as(c_int32_p),
            out["alive"].ctypes.data_as(c_uint8_p)))
        return out

    def set_carriers(self, c: dict) -> None:
        n = int(c["x"].size)
        arrs = [np.ascontiguousarray(c[k], dtype=np.float64) for k in ("x", "y", "z", "occ")]
        mode = np.ascontiguousarray(c["mode"], dtype=np.uint32)
        alive = c.get("alive", np.ones(n, np.uint8))
        alive = None if alive is None else np.ascontiguousarray(alive, dtype=np.uint8)
        self.check(self.fn("solver_set_carriers")(self.h, n, *[dptr(a) for a in arrs],
                                                  mode.ctypes.data_as(c_uint32_p),
                                                  None if alive is None else alive.ctypes.data_as(c_uint8_p)))

    def close(self):
        if getattr(self, "h", None):
            self.fn("solver_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# Deterministic sub-step entry points; the CUDA library exports them with the
# prefix phmc_dev_ and the oracle with orc_ (same signatures).
SUBSTEP_PROTOS = {
    "ncallaway_evolve": (C.c_int, [C.c_int32, c_double_p, c_double_p, c_double_p, c_double_p, C.c_int64, c_int32_p,
                                   c_double_p, C.c_double, C.c_double]),
    "trace_box": (C.c_int, [c_double_p, c_double_p, C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p,
                            c_int32_p]),
    "temperature_from_energy": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_double_p]),
    "rta_collide": (C.c_int, [C.c_void_p, C.c_int64, c_int32_p, c_int32_p, c_double_p, C.c_int, c_double_p,
                              C.c_double, C.c_double, C.c_int, C.c_double, c_double_p]),
    "linear_collide": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int64, c_int32_p, c_int32_p, c_double_p,
                                 C.c_int, C.c_double, C.c_double, c_double_p]),
    "rough_reflect": (C.c_int, [C.c_void_p, C.c_int, C.c_double, c_double_p, C.c_double, C.c_int64, c_int32_p,
                                c_double_p, c_double_p, c_int32_p, c_double_p]),
    "gradient_drive": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int64, c_int32_p, c_int32_p,
                                 c_double_p, C.c_int, C.c_double, C.c_double, c_double_p]),
    "trace_mesh": (C.c_int, [C.c_int, c_double_p, C.c_int, c_int32_p, c_int32_p, C.c_int64, c_double_p, c_double_p,
                             c_double_p, c_double_p, c_int32_p]),
    "interface": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                            C.c_int64, c_int32_p, c_int32_p, c_int32_p, c_double_p, c_double_p, c_int32_p, c_int32_p,
                            c_int32_p, c_int32_p, c_double_p]),
}

ORACLE_EXTRA_PROTOS = {
    "amm_rows": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                           c_int32_p, c_int32_p, c_int32_p, c_double_p]),
    "interface_model": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                  C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int64, c_int32_p,
                                  c_int32_p, c_double_p, c_double_p, c_int32_p, c_int32_p, c_int32_p, c_double_p]),
    "material_query": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, c_int32_p, c_double_p, C.c_double, c_double_p]),
    "material_scalars": (C.c_int, [C.c_void_p, C.c_double, c_double_p, c_int32_p]),
    "grid_index": (C.c_int, [c_double_p, c_int32_p, C.c_int64, c_double_p, c_int32_p]),
    "callaway_evolve": (C.c_int, [C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p, c_double_p, c_double_p,
                                  C.c_double, c_double_p]),
    "source_rates": (C.c_int, [C.POINTER(ConfigPOD), c_double_p, c_int32_p]),
    "source_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, c_double_p,
                               c_double_p, C.c_int64, c_int32_p, c_int32_p, c_double_p, c_double_p, c_int64_p]),
    "reservoir_cdf": (C.c_int, [C.c_void_p, c_double_p, C.c_double, C.c_double, C.c_double, c_double_p, c_double_p,
                                c_int32_p]),
    "alias_table": (C.c_int, [c_double_p, C.c_int32, c_double_p, c_int32_p, C.c_int32, c_double_p, c_int32_p]),
}

DEVICE_PROTOS = {
    "device_count": (C.c_int, [c_int32_p]),
    "material_active_count": (C.c_int, [C.c_void_p, c_int32_p]),
    "solver_run_timestep": (C.c_int, [C.c_void_p]),
    "solver_synchronize": (C.c_int, [C.c_void_p]),
    "solver_write_outputs": (C.c_int, [C.c_void_p]),
    "solver_append_summary": (C.c_int, [C.c_void_p, C.c_int64]),
    "solver_timed_run": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, c_int64_p, c_int64_p, c_int64_p]),
    "solver_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "solver_sort_interval": (C.c_int, [C.c_void_p, c_int32_p]),
    "solver_carrier_state": (C.c_int, [C.c_void_p, C.c_int64, c_double_p]),
    "solver_set_schedule": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "batch_create": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "batch_size": (C.c_int, [C.c_void_p, c_int32_p]),
    "batch_run": (C.c_int, [C.c_void_p, C.c_int]),
    "batch_timed_run": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, c_int64_p]),
    "batch_stats": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(StatsPOD)]),
    "batch_cells": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p, c_double_p]),
    "batch_cell_count": (C.c_int, [C.c_void_p, C.c_int, c_int32_p]),
    "batch_destroy": (None, [C.c_void_p]),
    "host_register": (C.c_int, [C.c_void_p, C.c_int64]),
    "host_unregister": (C.c_int, [C.c_void_p]),
    "solver_run_from_host": (C.c_int, [C.c_void_p, C.c_int64, c_double_p, c_double_p, c_double_p, c_double_p,
                                       c_uint32_p, C.c_int, c_double_p]),
    **{"dev_" + k: v for k, v in SUBSTEP_PROTOS.items()},
    "dev_trace_box_noalloc": (C.c_int, [c_double_p, c_double_p, C.c_int64, c_double_p, c_double_p, c_double_p,
                                        c_double_p, c_int32_p, c_int64_p]),
    "dev_rough_spec_match": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int32, c_double_p, c_double_p, C.c_int,
                                       c_int32_p]),
}


class Batch:
    """Independent instances advancing together through phmc_batch_* (device only)."""

    def __init__(self, lib, cfgs: list, materials: list):
        self.lib = lib
        pods, self._keep = [], []
        for cfg in cfgs:
            pod, keep = config_pod(cfg)
            pods.append(pod)
            self._keep.append(keep)
        arr = (ConfigPOD * len(pods))(*pods)
        self._keep.append(arr)
        mats = (C.c_void_p * len(materials))(*[m.h for m in materials])
        self._mats = materials
        h = C.c_void_p()
        self.check(lib.phmc_batch_create(C.cast(arr, C.c_void_p), len(pods), mats, len(materials), C.byref(h)))
        self.h = h
        self.n = len(pods)

    def check(self, rc):
        if rc != 0:
            raise LibError(self.lib.phmc_last_error().decode())

    def run(self, steps: int) -> None:
        self.check(self.lib.phmc_batch_run(self.h, steps))

    def timed_run(self, steps: int):
        ms, cs, launches = C.c_double(), C.c_double(), C.c_int64()
        self.check(self.lib.phmc_batch_timed_run(self.h, steps, C.byref(ms), C.byref(cs), C.byref(launches)))
        return ms.value, cs.value, int(launches.value)

    def stats(self, i: int) -> dict:
        st = StatsPOD()
        self.check(self.lib.phmc_batch_stats(self.h, i, C.byref(st)))
        return st.as_dict()

    def cells(self, i: int):
        n = C.c_int32()
        self.check(self.lib.phmc_batch_cell_count(self.h, i, C.byref(n)))
        T, E, q = np.zeros(n.value), np.zeros(n.value), np.zeros(3 * n.value)
        self.check(self.lib.phmc_batch_cells(self.h, i, dptr(T), dptr(E), dptr(q)))
        return T, E, q.reshape(-1, 3)

    def close(self):
        if getattr(self, "h", None):
            self.lib.phmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



class Domain:
    """Host geometry of a configuration through phmc_domain_* (no device work)."""

    def __init__(self, lib, cfg: dict):
        self.lib = lib
        pod, keep = config_pod(cfg)
        h = C.c_void_p()
        if lib.phmc_domain_create(C.byref(pod), C.byref(h)) != 0:
            raise LibError(lib.phmc_last_error().decode())
        self.h = h
        nf, nc, nfa = C.c_int32(), C.c_int32(), C.c_int32()
        shape = (C.c_int32 * 3)()
        vol = C.c_double()
        b = (C.c_double * 6)()
        self._check(lib.phmc_domain_info(h, C.byref(nf), C.byref(nc), C.byref(nfa), shape, C.byref(vol), b))
        self.n_facets, self.n_cells, self.n_faces = nf.value, nc.value, nfa.value
        self.shape = tuple(shape)
        self.volume = vol.value
        self.bounds = np.array(list(b)).reshape(2, 3)

    def _check(self, rc):
        if rc != 0:
            raise LibError(self.lib.phmc_last_error().decode())

    def facets(self) -> dict:
        n = self.n_facets
        normal, centroid, shift = (np.zeros((n, 3)) for _ in range(3))
        area, value = np.zeros(n), np.zeros(n)
        cond = C.create_string_buffer(max(n, 1))
        pair = np.zeros(n, dtype=np.int32)
        self._check(self.lib.phmc_domain_facets(self.h, dptr(normal), dptr(centroid), dptr(area), cond, dptr(value),
                                                pair.ctypes.data_as(c_int32_p), dptr(shift)))
        return {"normal": normal, "centroid": centroid, "area": area, "condition": cond.raw[:n].decode(),
                "value": value, "pair": pair, "shift": shift}

    def cells(self) -> dict:
        centers, vols = np.zeros((self.n_cells, 3)), np.zeros(self.n_cells)
        vc = np.zeros(int(np.prod(self.shape)), dtype=np.int32)
        self._check(self.lib.phmc_domain_cells(self.h, dptr(centers), dptr(vols), vc.ctypes.data_as(c_int32_p)))
        return {"centers": centers, "volumes": vols, "voxel_cell": vc}

    def faces(self) -> dict:
        f2f = np.zeros(self.n_faces, dtype=np.int32)
        tri = np.zeros((self.n_faces, 3, 3))
        self._check(self.lib.phmc_domain_faces(self.h, f2f.ctypes.data_as(c_int32_p), dptr(tri)))
        return {"face_to_facet": f2f, "triangles": tri}

    def trace(self, p, v):
        """(hit points, times, facets) of rays by the host domain."""
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        n = p.shape[0]
        hit, t, f = np.zeros((n, 3)), np.zeros(n), np.zeros(n, dtype=np.int32)
        self._check(self.lib.phmc_domain_trace(self.h, n, dptr(p), dptr(v), dptr(hit), dptr(t),
                                               f.ctypes.data_as(c_int32_p)))
        return hit, t, f

    def device_trace(self, p, v):
        """The same traces by the device code (GPU)."""
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        n = p.shape[0]
        hit, t, f = np.zeros((n, 3)), np.zeros(n), np.zeros(n, dtype=np.int32)
        self._check(self.lib.phmc_dev_domain_trace(self.h, n, dptr(p), dptr(v), dptr(hit), dptr(t),
                                                   f.ctypes.data_as(c_int32_p)))
        return hit, t, f

    def contains(self, p) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(p.shape[0], dtype=np.uint8)
        self._check(self.lib.phmc_domain_contains(self.h, p.shape[0], dptr(p), out.ctypes.data_as(c_uint8_p)))
        return out

    def voxel_interior(self) -> np.ndarray:
        """Voxels whose whole box lies inside the mesh, shape (nx, ny, nz)."""
        out = np.zeros(int(np.prod(self.shape)), dtype=np.uint8)
        self._check(self.lib.phmc_domain_voxel_interior(self.h, out.ctypes.data_as(c_uint8_p)))
        return out.reshape(tuple(self.shape))

    def grid_index(self, p) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(p.shape[0], dtype=np.int32)
        self._check(self.lib.phmc_domain_grid_index(self.h, p.shape[0], dptr(p), out.ctypes.data_as(c_int32_p)))
        return out

    def nearest_facet(self, p) -> np.ndarray:
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(p.shape[0], dtype=np.int32)
        self._check(self.lib.phmc_domain_nearest_facet(self.h, p.shape[0], dptr(p), out.ctypes.data_as(c_int32_p)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.phmc_domain_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def device_domain_query(dom: "Domain", p):
    """(inside, nearest facet, cell) of points by the device code on a mesh domain."""
    p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
    n = p.shape[0]
    inside = np.zeros(n, dtype=np.uint8)
    near = np.zeros(n, dtype=np.int32)
    cell = np.zeros(n, dtype=np.int32)
    dom._check(dom.lib.phmc_dev_domain_query(dom.h, n, dptr(p), inside.ctypes.data_as(c_uint8_p),
                                              near.ctypes.data_as(c_int32_p), cell.ctypes.data_as(c_int32_p)))
    return inside, near, cell
