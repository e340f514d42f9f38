"""Seeded synthetic phonon tables in the reference's MaterialData layout.

The reference reads phono3py-derived full-Brillouin-zone tables
(``src/material/MaterialDataReader.cpp:192-296``) into ``phonomc::MaterialData``
(``include/material/MaterialData.h:17-31``): q-major/branch-minor frequencies
[THz], fractional q points, group velocities [Angstrom/ps], a temperature axis
[K] and linewidths gamma [THz HWHM] laid out (temperature, q, branch).

The workloads here use a synthetic table of that shape, generated from a seed:

* lattice: simple cubic, ``a = 3.4212`` Angstrom (the 40.04 A^3 volume of the
  silicon primitive cell), so the first Brillouin zone is the reduced cube;
* q grid: ``mesh^3`` Gamma-centred points ``q_i = m_i/mesh`` with
  ``m_i`` in ``[-mesh/2, mesh/2)``, equal weight;
* acoustic branches 0-2: ``omega = omega_max * sin(pi*s/2)`` with
  ``omega_max = 8, 8, 12`` THz and the periodic reduced norm
  ``s^2 = (sin^2(pi q1) + sin^2(pi q2) + sin^2(pi q3))/3`` (``s`` in ``[0,1]``);
* optical branches 3-5: flat at 15 THz plus uniform noise in [-0.5, 0.5) THz
  from ``numpy.random.default_rng(seed)``, zero group velocity;
* group velocities are the analytic gradient ``d omega / d k``; the normal
  component vanishes exactly on the zone faces, so ``v(-q) = -v(q)`` and the
  velocity bank is balanced (the gradient drive requires it,
  ``src/solver/TemperatureGradientDrive.cpp:64-67``);
* ``gamma = scale * (A w^2 T + B w^4) / (4 pi) / 1e12`` THz with ``w`` in
  rad/s, ``A = 1e-19`` s/K and ``B = 1e-45`` s^3, on the 0..1000 K axis in
  10 K steps; ``scale`` is fixed so that the kinetic estimate
  ``sum C v_z^2 tau / (N_q V)`` at 300 K is 150 W/(m K) (silicon-like);
* optional Callaway split ``gamma_N = 0.6 gamma``, ``gamma_U = 0.4 gamma`` and
  ``gamma_isotope = scale * C w^4/(4 pi)/1e12`` with ``C = 2e-46`` s^3;
* the second bilayer material scales frequencies by 0.7 and velocities by 0.75.
"""

from __future__ import annotations

import dataclasses
import struct
from typing import Dict, Optional

import numpy as np

HBAR_EV_PS = 6.582119569e-4
KB_EV_K = 8.617333262145e-5
EV_TO_J = 1.602176634e-19

A_COEF = 1e-19  # s / K
B_COEF = 1e-45  # s^3
C_ISOTOPE = 2e-46  # s^3
LATTICE_A = 3.4212  # Angstrom
KAPPA_TARGET = 150.0  # W/(m K)


@dataclasses.dataclass
class MaterialData:
    """In-memory mirror of ``phonomc::MaterialData`` (reference MaterialData.h:17-31)."""

    volume_a3: float
    reciprocal: np.ndarray  # (3,3) columns are b vectors, 1/Angstrom incl. 2*pi
    mesh: tuple
    frequency_thz: np.ndarray  # (nq*nb,)
    qpoint_fractions: np.ndarray  # (nq,3)
    group_velocity: np.ndarray  # (nq*nb,3)
    temperatures: np.ndarray  # (nT,)
    gamma: np.ndarray  # (nT*nq*nb,)
    gamma_normal: Optional[np.ndarray] = None
    gamma_umklapp: Optional[np.ndarray] = None
    gamma_resistive: Dict[str, np.ndarray] = dataclasses.field(default_factory=dict)
    scale: float = 1.0

    @property
    def qpoints(self) -> int:
        return int(self.qpoint_fractions.shape[0])

    @property
    def branches(self) -> int:
        return int(self.frequency_thz.size // self.qpoint_fractions.shape[0])


def _linewidth(omega_rad_s: np.ndarray, temperature: np.ndarray) -> np.ndarray:
    w2 = omega_rad_s * omega_rad_s
    return (A_COEF * w2[None, :] * temperature[:, None] + B_COEF * (w2 * w2)[None, :]) / (
        4.0 * np.pi
    ) / 1e12


def _kinetic_kappa(freq_thz, vel, gamma_300, nq, volume) -> float:
    omega = 2.0 * np.pi * freq_thz  # rad/ps
    hw = HBAR_EV_PS * omega
    x = np.where(hw > 0, hw / (KB_EV_K * 300.0), np.inf)
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        c = np.where(hw > 0, KB_EV_K * x * x * np.exp(-x) / np.expm1(-x) ** 2, 0.0)  # eV/K
        rate = 4.0 * np.pi * gamma_300  # 1/ps
        tau = np.where(rate > 0, 1.0 / rate, 0.0)  # ps
    vz = vel[:, 2]  # Angstrom/ps
    # eV/K * A^2/ps^2 * ps / A^3 = eV/(K ps A) -> W/(m K)
    k = np.sum(c * vz * vz * tau) / (nq * volume)
    return float(k * EV_TO_J / 1e-12 / 1e-10)


def make_material(mesh: int = 16, seed: int = 0, freq_scale: float = 1.0,
                  vel_scale: float = 1.0, callaway: bool = False,
                  temperatures: Optional[np.ndarray] = None) -> MaterialData:
    """Build the seeded synthetic table described in the module docstring."""
    if mesh < 2 or mesh % 2:
        raise ValueError("mesh must be an even integer >= 2")
    rng = np.random.default_rng(seed)
    b = 2.0 * np.pi / LATTICE_A
    reciprocal = np.eye(3) * b
    idx = np.arange(mesh)
    frac1 = ((idx + mesh // 2) % mesh - mesh // 2) / mesh  # 0..mesh/2-1, then -mesh/2..-1
    q = np.stack(np.meshgrid(frac1, frac1, frac1, indexing="ij"), axis=-1).reshape(-1, 3)
    nq = q.shape[0]
    nb = 6
    sin2 = np.sin(np.pi * q) ** 2
    s = np.sqrt(sin2.sum(axis=1) / 3.0)
    s = np.minimum(s, 1.0)
    ds_dq = np.zeros_like(q)
    nz = s > 0
    sin2pq = np.sin(2.0 * np.pi * q)
    sin2pq[np.abs(np.abs(q) - 0.5) < 1e-15] = 0.0  # exact zero normal velocity on zone faces
    ds_dq[nz] = np.pi * sin2pq[nz] / (6.0 * s[nz, None])
    freq = np.zeros((nq, nb))
    vel = np.zeros((nq, nb, 3))
    for br, fmax in enumerate((8.0, 8.0, 12.0)):
        freq[:, br] = fmax * np.sin(0.5 * np.pi * s)
        domega_ds = 2.0 * np.pi * fmax * 0.5 * np.pi * np.cos(0.5 * np.pi * s)  # rad/ps
        vel[:, br, :] = (domega_ds[:, None] * ds_dq) / b
    noise = rng.uniform(-0.5, 0.5, size=(nq, 3))
    freq[:, 3:] = 15.0 + noise
    freq *= freq_scale
    vel *= vel_scale
    freq = freq.reshape(-1)
    vel = vel.reshape(-1, 3)
    if temperatures is None:
        temperatures = np.arange(0.0, 1000.0 + 1e-9, 10.0)
    omega_rad_s = 2.0 * np.pi * freq * 1e12
    base = _linewidth(omega_rad_s, temperatures)  # (nT, nm)
    it300 = int(np.argmin(np.abs(temperatures - 300.0)))
    volume = LATTICE_A ** 3
    kappa1 = _kinetic_kappa(freq, vel, base[it300], nq, volume)
    scale = kappa1 / KAPPA_TARGET if kappa1 > 0 else 1.0
    gamma = (base * scale).reshape(-1)
    data = MaterialData(volume_a3=volume, reciprocal=reciprocal, mesh=(mesh, mesh, mesh),
                        frequency_thz=freq, qpoint_fractions=q, group_velocity=vel,
                        temperatures=np.asarray(temperatures, dtype=np.float64), gamma=gamma,
                        scale=scale)
    if callaway:
        data.gamma_normal = 0.6 * gamma
        data.gamma_umklapp = gamma - data.gamma_normal
        w4 = omega_rad_s ** 4
        data.gamma_resistive["gamma_isotope"] = scale * C_ISOTOPE * w4 / (4.0 * np.pi) / 1e12
    return data


_MAGIC = b"PMAT0001"


def write_pmat(path: str, data: MaterialData) -> None:
    """Write the flat binary table read by the reference harness (oracle/ref).

    Layout: magic, int32 [qpoints, branches, mesh0, mesh1, mesh2, ntemps,
    has_nu, n_resistive], float64 volume, reciprocal (row-major 3x3), then the
    arrays in MaterialData order; each resistive table is a 16-byte name,
    int64 length and values.
    """
    has_nu = data.gamma_normal is not None
    with open(path, "wb") as f:
        f.write(_MAGIC)
        f.write(struct.pack("<8i", data.qpoints, data.branches, *data.mesh,
                            data.temperatures.size, int(has_nu), len(data.gamma_resistive)))
        f.write(struct.pack("<d", data.volume_a3))
        f.write(np.ascontiguousarray(data.reciprocal, dtype="<f8").tobytes())
        for arr in (data.frequency_thz, data.qpoint_fractions, data.group_velocity,
                    data.temperatures, data.gamma):
            f.write(np.ascontiguousarray(arr, dtype="<f8").tobytes())
        if has_nu:
            f.write(np.ascontiguousarray(data.gamma_normal, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(data.gamma_umklapp, dtype="<f8").tobytes())
        for name, values in data.gamma_resistive.items():
            f.write(name.encode().ljust(16, b"\0")[:16])
            f.write(struct.pack("<q", values.size))
            f.write(np.ascontiguousarray(values, dtype="<f8").tobytes())


# ------------------------------------------------------------------ meshes
def finfet_mesh(voxel_nm: float = 5.0, jitter_nm: float = 0.5, seed: int = 0,
                slab_nm=(200.0, 100.0, 50.0), fin_nm=(10.0, 100.0, 40.0)):
    """Procedural FinFET surface: a fin (10 nm wide in x, running the full 100 nm
    along y, 40 nm tall) on a 200 x 100 x 50 nm slab, as the boundary of a voxel
    solid (voxel_nm lattice), two triangles per exposed voxel face, outward
    winding. Vertices off the slab's side and bottom planes (which stay flat so
    periodic pairing and reservoirs keep exact planes) get a uniform jitter of
    +-jitter_nm per component from `seed`. Returns (vertices [nm], faces)."""
    nx, ny, nz = (int(round(s / voxel_nm)) for s in slab_nm)
    fx, fz = int(round(fin_nm[0] / voxel_nm)), int(round(fin_nm[2] / voxel_nm))
    solid = np.zeros((nx, ny, nz + fz), dtype=bool)
    solid[:, :, :nz] = True
    x0 = (nx - fx) // 2
    solid[x0:x0 + fx, :, nz:nz + fz] = True
    index = {}
    verts = []

    def vid(i, j, k):
        key = (i, j, k)
        if key not in index:
            index[key] = len(verts)
            verts.append((i * voxel_nm, j * voxel_nm, k * voxel_nm))
        return index[key]

    faces = []
    shape = solid.shape
    # corner offsets of the quad on each of the six faces, counter-clockwise seen from outside
    quads = {
        (-1, 0, 0): [(0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)],
        (1, 0, 0): [(1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)],
        (0, -1, 0): [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)],
        (0, 1, 0): [(0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)],
        (0, 0, -1): [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)],
        (0, 0, 1): [(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)],
    }
    for i, j, k in zip(*np.nonzero(solid)):
        for d, corners in quads.items():
            a, b, c = i + d[0], j + d[1], k + d[2]
            if 0 <= a < shape[0] and 0 <= b < shape[1] and 0 <= c < shape[2] and solid[a, b, c]:
                continue
            q = [vid(i + o[0], j + o[1], k + o[2]) for o in corners]
            faces.append((q[0], q[1], q[2]))
            faces.append((q[0], q[2], q[3]))
    v = np.array(verts, dtype=np.float64)
    rng = np.random.default_rng(seed)
    keep = ((np.abs(v[:, 0]) < 1e-9) | (np.abs(v[:, 0] - slab_nm[0]) < 1e-9) | (np.abs(v[:, 1]) < 1e-9) |
            (np.abs(v[:, 1] - slab_nm[1]) < 1e-9) | (np.abs(v[:, 2]) < 1e-9))
    jitter = rng.uniform(-jitter_nm, jitter_nm, size=v.shape)
    v[~keep] += jitter[~keep]
    return v, np.array(faces, dtype=np.int64)


def prism_mesh(outline_nm=((0.0, 0.0), (100.0, 0.0), (100.0, 30.0), (37.0, 30.0), (37.0, 80.0), (0.0, 80.0)),
               height_nm: float = 50.0):
    """An L-shaped prism: the counter-clockwise outline (nm) extruded from z = 0
    to `height_nm`, vertical side walls (one quad per outline edge, the x = 0
    edge split at the inner corner's y so every vertex of the top is a vertex
    of the walls) and a flat top and bottom triangulated as the two rectangles
    of the L. Returns (vertices [nm], faces) with outward winding."""
    o = [tuple(map(float, q)) for q in outline_nm]
    (x0, y0), (x1, _), (_, y1), (xn, _), (_, y2), _ = o
    ring = [(x0, y0), (x1, y0), (x1, y1), (xn, y1), (xn, y2), (x0, y2), (x0, y1)]  # counter-clockwise
    n = len(ring)
    verts = [(x, y, 0.0) for x, y in ring] + [(x, y, float(height_nm)) for x, y in ring]
    # top (counter-clockwise seen from +z) as index triangles of the ring
    top = [(0, 1, 2), (0, 2, 3), (0, 3, 6), (6, 3, 4), (6, 4, 5)]
    faces = [(a + n, b + n, c + n) for a, b, c in top] + [(a, c, b) for a, b, c in top]
    for i in range(n):
        j = (i + 1) % n
        faces.append((i, j, j + n))
        faces.append((i, j + n, i + n))
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.int64)


def write_stl(path: str, vertices, faces, name: str = "synthetic") -> None:
    """Binary STL (little-endian: 80-byte header, count, 50-byte records)."""
    import struct
    v = np.asarray(vertices, dtype=np.float64)
    f = np.asarray(faces, dtype=np.int64)
    with open(path, "wb") as out:
        out.write(name.encode()[:80].ljust(80, b" "))
        out.write(struct.pack("<I", len(f)))
        for a, b, c in f:
            n = np.cross(v[b] - v[a], v[c] - v[a])
            ln = np.linalg.norm(n)
            n = n / ln if ln > 0 else n
            out.write(struct.pack("<12fH", *n, *v[a], *v[b], *v[c], 0))
