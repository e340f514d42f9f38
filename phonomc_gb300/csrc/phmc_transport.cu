// Pass A of the timestep: gradient half-step, free flight with wall events,
// cell reassignment and the (cell, mode) histogram; reservoir injection; the
// heat-flux tally. Plain-FP64 carrier state.
//
// Reference: src/solver/TransportOperator.cpp:113-163 (advance loops),
// 287-361 (boundary collision), 405-466 (event loop);
// src/solver/BoundaryInteraction.cpp:53-162; src/solver/ReservoirInjector.cpp:62-132;
// src/solver/TemperatureGradientDrive.cpp:116-171; src/solver/GridStatistics.cpp:269-347.
#include <type_traits>

#include "phmc_kernels.cuh"

namespace phmc {

// Per-block partial ledger sums, flushed once per block.
struct BlockLedger {
    double absorbed_ev;
    double injected_ev;
    double drive_ev;
    unsigned long long drive_updates;
    unsigned int absorbed;
    unsigned int absorbed_res[kMaxReservoirs];
    unsigned int iface_events, iface_transmitted, iface_reflected;
    unsigned int rough[kRoughCounters];
    unsigned int cache_corrections;
};

__device__ __forceinline__ void block_ledger_init(BlockLedger* b) {
    if (threadIdx.x == 0) {
        b->absorbed_ev = 0;
        b->injected_ev = 0;
        b->drive_ev = 0;
        b->drive_updates = 0;
        b->absorbed = 0;
        for (int r = 0; r < kMaxReservoirs; ++r) b->absorbed_res[r] = 0;
        b->iface_events = b->iface_transmitted = b->iface_reflected = 0;
        for (int k = 0; k < kRoughCounters; ++k) b->rough[k] = 0;
        b->cache_corrections = 0;
    }
}

// One rough reflection into the block's diagnostics (flags of rough_sample_dev).
__device__ __forceinline__ void count_rough(BlockLedger* b, unsigned diag) {
    atomicAdd(&b->rough[kRoughCounters - 1], 1u);
    for (int k = 0; k < kRoughCounters - 1; ++k)
        if (diag & (1u << k)) atomicAdd(&b->rough[k], 1u);
}

__device__ __forceinline__ void block_ledger_flush(BlockLedger* b, DevLedger* L) {
    if (threadIdx.x == 0) {
        if (b->absorbed) {
            atomicAdd(&L->step_absorbed, static_cast<unsigned long long>(b->absorbed));
            atomicAdd(&L->step_absorbed_ev, b->absorbed_ev);
            for (int r = 0; r < kMaxReservoirs; ++r)
                if (b->absorbed_res[r]) atomicAdd(&L->absorbed_res[r], b->absorbed_res[r]);
        }
        if (b->drive_updates) {
            atomicAdd(&L->step_drive_ev, b->drive_ev);
            atomicAdd(&L->step_drive_updates, b->drive_updates);
        }
        if (b->injected_ev != 0.0) atomicAdd(&L->step_injected_ev, b->injected_ev);
        for (int k = 0; k < kRoughCounters; ++k)
            if (b->rough[k]) atomicAdd(&L->total_rough[k], static_cast<unsigned long long>(b->rough[k]));
        if (b->cache_corrections)
            atomicAdd(&L->total_cache_corrections, static_cast<unsigned long long>(b->cache_corrections));
        if (b->iface_events) {
            atomicAdd(&L->total_iface_events, static_cast<unsigned long long>(b->iface_events));
            atomicAdd(&L->total_iface_transmitted, static_cast<unsigned long long>(b->iface_transmitted));
            atomicAdd(&L->total_iface_reflected, static_cast<unsigned long long>(b->iface_reflected));
        }
    }
}

__device__ __forceinline__ double axis_of(const double v[3], int axis) {
    return axis == 0 ? v[0] : (axis == 1 ? v[1] : v[2]);
}

// src/solver/LayeredMaterialLayout.cpp:31-60: time to the next material plane
// in the direction of travel (infinite when none or not ahead by > 1e-14 ps).
__device__ __forceinline__ double next_crossing_dev(const DevDomain& D, int n_materials, const double p[3],
                                                    const double v[3], int current, int& destination) {
    destination = -1;
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    if (n_materials <= 1) return inf;
    const double va = axis_of(v, D.layout_axis);
    if (fabs(va) <= 1e-18) return inf;
    double plane;
    int dest;
    if (va > 0.0 && current + 1 < n_materials) {
        plane = D.planes[current];
        dest = current + 1;
    } else if (va < 0.0 && current > 0) {
        plane = D.planes[current - 1];
        dest = current - 1;
    } else {
        return inf;
    }
    const double time = __dadd_rn(plane, -axis_of(p, D.layout_axis)) / va;
    if (!isfinite(time) || time <= 1e-14) return inf;
    destination = dest;
    return time;
}

__device__ __forceinline__ void count_interface(BlockLedger* bl, const IfaceOut& r) {
    atomicAdd(&bl->iface_events, 1u);
    if (r.action == 4) atomicAdd(&bl->iface_transmitted, 1u);
    else if (r.action == 3) atomicAdd(&bl->iface_reflected, 1u);
}

// True when the carrier cannot reach a wall plane within `remaining`: it is
// inside the box and, on every axis it moves along, the distance to the wall
// ahead -- the numerator target - p of the plane time that trace_box divides
// by the velocity -- exceeds its reach |v| remaining by a relative margin of
// 1e-9, far above the rounding of that quotient. The traced flight of such a
// carrier finds its wall beyond `remaining` and drifts; this test gets there
// with multiplications and compares instead of three FP64 divisions.
__device__ __forceinline__ bool clear_of_walls(const DevDomain& D, const double p[3], const double v[3],
                                               double remaining) {
    bool clear = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        clear = clear && p[a] >= D.lo[a] && p[a] <= D.hi[a];
        const double c = v[a];
        if (!(fabs(c) <= 1e-18)) { // an axis the trace considers (a NaN velocity fails the test below)
            const double gap = c > 0.0 ? D.hi[a] - p[a] : D.lo[a] - p[a];
            clear = clear && fabs(gap) > fabs(c) * remaining * (1.0 + 1e-9);
        }
    }
    return clear;
}

// One carrier's flight for `remaining` ps (src/solver/TransportOperator.cpp:405-466).
// Position, mode word and occupation live in registers; returns false when the
// carrier was absorbed.
// A conservative form of clear_of_walls with few FP64 operations (GB300
// retires two FP64 lanes per SM per clock): true only where clear_of_walls is
// true as well. The gaps to the walls are the FP64 differences of the test,
// rounded toward zero to FP32; the reach |v| dt (1 + 2e-6) is rounded up in
// FP32, above the test's |v| dt (1 + 1e-9); signs and the 1e-18 velocity floor
// are read from the bits. `dt_up`: dt rounded up to FP32.
__device__ __forceinline__ bool clear_of_walls32(const DevDomain& D, const double p[3], const double v[3],
                                                 float dt_up) {
    bool clear = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double ghi = dadd(D.hi[a], -p[a]), glo = dadd(p[a], -D.lo[a]);
        const int hh = __double2hiint(ghi), hl = __double2hiint(glo);
        // p in [lo, hi]: both gaps non-negative and finite (a NaN p fails)
        clear = clear && hh >= 0 && hl >= 0 && (hh & 0x7ff00000) != 0x7ff00000 && (hl & 0x7ff00000) != 0x7ff00000;
        const long long cb = __double_as_longlong(v[a]);
        const long long mag = cb & 0x7fffffffffffffffLL;
        if (mag > 0x3C32725DD1D243ACLL) { // |v| > 1e-18, or NaN: an axis the trace considers
            const double g = cb >= 0 ? ghi : glo;
            const float reach = __fmul_ru(__fmul_ru(__double2float_ru(__longlong_as_double(mag)), dt_up), 1.000002f);
            clear = clear && __double2float_rz(g) > reach;
        }
    }
    return clear;
}

// No material-plane crossing within dt (conservative FP32 form of
// next_crossing_dev > dt): true only where the FP64 crossing time is infinite
// or beyond dt. A plane behind the carrier (gap and velocity of opposite
// sign) is never crossed; NaN velocities fail.
__device__ __forceinline__ bool clear_of_planes32(const DevDomain& D, int n_materials, const double p[3],
                                                  const double v[3], int current, float dt_up) {
    const long long cb = __double_as_longlong(axis_of(v, D.layout_axis));
    const long long mag = cb & 0x7fffffffffffffffLL;
    if (mag <= 0x3C32725DD1D243ACLL) return true; // |v| <= 1e-18 along the layout axis
    double plane;
    if (cb >= 0 && current + 1 < n_materials) plane = D.planes[current];
    else if (cb < 0 && current > 0) plane = D.planes[current - 1];
    else return mag <= 0x7ff0000000000000LL; // no plane ahead (a NaN velocity fails)
    const double gap = dadd(plane, -axis_of(p, D.layout_axis));
    if ((__double2hiint(gap) ^ static_cast<int>(cb >> 32)) < 0) return true; // the plane lies behind
    const float reach = __fmul_ru(__fmul_ru(__double2float_ru(__longlong_as_double(mag)), dt_up), 1.000002f);
    return __double2float_rz(fabs(gap)) > reach;
}

__device__ bool advance_carrier(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot, double p[3],
                                uint32_t& w, double& occ, double remaining, uint32_t purpose, uint32_t step) {
    auto counted_cache = [&](int r) {
        if (r == 2) atomicAdd(&bl->cache_corrections, 1u);
        return r != 0;
    };
    const DevDomain& D = T.dom;
    const DevParams& P = T.par;
    int mid = static_cast<int>(w >> 28);
    const DevMaterial* M = &T.mat[mid];
    double v[3];
    mode_velocity(*M, w, v);
    if (P.n_materials <= 1 && clear_of_walls(D, p, v, remaining)) {
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], remaining));
        return true;
    }
    double cp[3], t;
    int f;
    if (!counted_cache(cache_hit(D, P, p, v, M->speed[w & 0x00FFFFFFu], cp, t, f))) {
        raise_error(L, kErrIntersection, slot);
        return true;
    }
    int event = 0;
    for (; remaining > 1e-14 && event < 64; ++event) {
        int destination = -1;
        const double t_cross = next_crossing_dev(D, P.n_materials, p, v, mid, destination);
        const double t_event = t_cross < t ? t_cross : t;
        if (!isfinite(t_event) || t_event > remaining) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], remaining));
            return true;
        }
        // the outer wall wins exact ties
        const bool interface_first = t_cross < t;
        remaining -= fmax(0.0, t_event);
        const int ai = static_cast<int>(w & 0x00FFFFFFu);
        if (interface_first) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], t_cross));
            const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 0);
            const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 1);
            const IfaceOut r = interface_dev(T, mid, ai, (w >> 24) & 7u, occ, destination, d0.a, d0.b, d1.a, d1.b);
            count_interface(bl, r);
            if (r.action >= 5) {
                raise_error(L, r.action == 6 ? kErrAmmRow : kErrModeMapping, slot);
                return true;
            }
            w = static_cast<uint32_t>(r.active) | (r.signs << 24) | (static_cast<uint32_t>(r.material) << 28);
            occ = r.occ;
            mid = r.material;
            M = &T.mat[mid];
            mode_velocity(*M, w, v);
            const double s = M->push[r.active];
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], s));
            if (!counted_cache(cache_hit(D, P, p, v, M->speed[w & 0x00FFFFFFu], cp, t, f))) {
                raise_error(L, kErrIntersection, slot);
                return true;
            }
            continue;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = cp[a];
        const int axis = f >> 1;
        const char cond = D.cond[f];
        if (cond == 'T') {
            const double e = dmul(dmul(M->hw[ai], occ - M->nbg[ai]), M->energy_weight);
            atomicAdd(&bl->absorbed, 1u);
            atomicAdd(&bl->absorbed_ev, e);
            const int r = D.reservoir[f];
            if (r >= 0) atomicAdd(&bl->absorbed_res[r], 1u);
            return false;
        }
        if (cond == 'P' && D.pair[f] >= 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], D.shift[f][a]);
        } else {
            const int table = D.rough_table[mid][f];
            if (P.conservative || (cond == 'R' && table >= 0)) {
                if (table < 0) {
                    raise_error(L, kErrModeMapping, slot);
                    return true;
                }
                const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose,
                                             static_cast<uint32_t>(event), 0);
                const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose,
                                             static_cast<uint32_t>(event), 1);
                double n_out;
                unsigned diag;
                const int out = rough_sample_dev(T.rough[table], *M, ai, occ, P.conservative != 0, d0.a, d0.b, d1.a,
                                                 n_out, diag);
                count_rough(bl, diag);
                const double nsign = (f & 1) ? 1.0 : -1.0;
                const double vn = M->vel[3 * out + axis] * nsign;
                uint32_t signs = 0;
                if (P.conservative) {
                    if (!isfinite(n_out) || !(M->omega[out] > 0.0) || !(vn < 0.0)) {
                        raise_error(L, kErrModeMapping, slot);
                        return true;
                    }
                } else if (vn > 0.0) {
                    signs = 1u << axis;
                }
                w = static_cast<uint32_t>(out) | (signs << 24) | (static_cast<uint32_t>(mid) << 28);
                occ = n_out;
            } else if (cond == 'R') {
                raise_error(L, kErrNoRoughTable, slot);
                return true;
            } else {
                w ^= 1u << (24 + axis);
            }
        }
        mode_velocity(*M, w, v);
        const double s = M->push[w & 0x00FFFFFFu];
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], s));
        if (!counted_cache(cache_hit(D, P, p, v, M->speed[w & 0x00FFFFFFu], cp, t, f))) {
            raise_error(L, kErrIntersection, slot);
            return true;
        }
        if (t < 1e-12) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], 1e-12));
            if (!counted_cache(cache_hit(D, P, p, v, M->speed[w & 0x00FFFFFFu], cp, t, f))) {
                raise_error(L, kErrIntersection, slot);
                return true;
            }
        }
    }
    if (remaining > 1e-14) raise_error(L, kErrTooManyEvents, slot);
    return true;
}

// Persistent wall cache of a mesh carrier (src/solver/TransportOperator.cpp:186-250):
// time to the wall in units of dt, hit point and facet. The point and facet
// are read from HBM only when the carrier reaches its wall.
struct MeshCache {
    double t, x, y, z;
    int f;
    bool loaded, dirty;
};

__device__ __forceinline__ void mesh_cache_load(const DevFacets& F, int slot, MeshCache& c) {
    if (c.loaded) return;
    c.x = F.hit_x[slot];
    c.y = F.hit_y[slot];
    c.z = F.hit_z[slot];
    c.f = F.hit_f[slot];
    c.loaded = true;
}

__device__ __forceinline__ void mesh_cache_store(const DevFacets& F, int slot, const MeshCache& c) {
    F.hit_t[slot] = c.t;
    if (c.dirty) {
        F.hit_x[slot] = c.x;
        F.hit_y[slot] = c.y;
        F.hit_z[slot] = c.z;
        F.hit_f[slot] = c.f;
    }
}

// Trace from p (nudged retries may move it) into the cache; false after raising an error.
__device__ __forceinline__ bool mesh_refresh(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot, double p[3],
                                             const double v[3], MeshCache& c) {
    double cp[3], t;
    int f;
    const int r = mesh_cache_hit(T.fac, T.dom, T.par, p, v, cp, t, f);
    c.loaded = c.dirty = true;
    if (r == 3 && bl) atomicAdd(&bl->cache_corrections, 1u);
    if (r != 0 && r != 3) {
        raise_error(L, r == 2 ? kErrInvalidStatistics : kErrIntersection, slot);
        c.t = __longlong_as_double(0x7ff0000000000000LL);
        c.f = -1;
        return false;
    }
    c.t = t / T.par.dt;
    c.x = cp[0];
    c.y = cp[1];
    c.z = cp[2];
    c.f = f;
    return true;
}

// One carrier's flight in a mesh domain (single material), reference event loop
// on the persistent wall cache: per-facet conditions, rough reflections whose
// outward mode velocity is mirrored in the facet plane (`mir`), the push along
// the velocity actually carried, then a fresh cache
// (src/solver/TransportOperator.cpp:287-361, 405-466).
__device__ bool advance_carrier_mesh(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot, double p[3], uint32_t& w, int& mir, double& occ, MeshCache& c,
                                     double remaining, uint32_t purpose, uint32_t step) {
    const DevFacets& F = T.fac;
    const DevParams& P = T.par;
    const double dt = P.dt;
    const int mid = static_cast<int>(w >> 28);
    const DevMaterial& M = T.mat[mid];
    double v[3];
    mesh_velocity(F, M, w, mir, v);
    int event = 0;
    for (; remaining > 1e-14 && event < 64; ++event) {
        const double t_wall = dmul(c.t, dt);
        if (!isfinite(t_wall) || t_wall > remaining) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], remaining));
            if (isfinite(c.t)) c.t = dadd(c.t, -(remaining / dt));
            return true;
        }
        remaining -= fmax(0.0, t_wall);
        mesh_cache_load(F, slot, c);
        p[0] = c.x;
        p[1] = c.y;
        p[2] = c.z;
        const int f = c.f;
        const int ai = static_cast<int>(w & 0x00FFFFFFu);
        const char cond = F.cond[f];
        if (cond == 'T') {
            const double e = dmul(dmul(M.hw[ai], occ - M.nbg[ai]), M.energy_weight);
            atomicAdd(&bl->absorbed, 1u);
            atomicAdd(&bl->absorbed_ev, e);
            const int r = F.reservoir[f];
            if (r >= 0) atomicAdd(&bl->absorbed_res[r], 1u);
            return false;
        }
        if (cond == 'P' && F.pair[f] >= 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], F.shift[3 * f + a]);
        } else {
            const int table = F.rough_table[mid * F.n + f];
            if (!(P.conservative || (cond == 'R' && table >= 0)) || table < 0) {
                raise_error(L, cond == 'R' && !P.conservative ? kErrNoRoughTable : kErrModeMapping, slot);
                return true;
            }
            const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 0);
            const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 1);
            double n_out;
            unsigned diag;
            const int out = rough_sample_dev(F.rough[table], M, ai, occ, P.conservative != 0, d0.a, d0.b, d1.a, n_out, diag);
            count_rough(bl, diag);
            const double* nf = F.normal + 3 * f;
            const double vo[3] = {M.vel[3 * out], M.vel[3 * out + 1], M.vel[3 * out + 2]};
            const double nn[3] = {nf[0], nf[1], nf[2]};
            const double vn = meshmath::dot(vo, nn);
            mir = -1;
            if (P.conservative) {
                if (!isfinite(n_out) || !(M.omega[out] > 0.0) || !(vn < 0.0)) {
                    raise_error(L, kErrModeMapping, slot);
                    return true;
                }
            } else if (vn > 0.0) {
                mir = f;
            }
            w = static_cast<uint32_t>(out) | (static_cast<uint32_t>(mid) << 28);
            occ = n_out;
        }
        mesh_velocity(F, M, w, mir, v);
        const double s = P.push_eps / fmax(meshmath::norm(v), 1e-12);
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], s));
        if (!mesh_refresh(T, L, bl, slot, p, v, c)) return true;
        if (dmul(c.t, dt) < 1e-12) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], 1e-12));
            if (!mesh_refresh(T, L, bl, slot, p, v, c)) return true;
        }
    }
    if (remaining > 1e-14) raise_error(L, kErrTooManyEvents, slot);
    return true;
}

// ------------------------------------------------------------------ bins
__device__ __forceinline__ int bin_of(const DevMaterial& M, int ai) { return M.bin ? __ldg(M.bin + ai) : ai; }

// Bin record of a carrier after the checks of GridStatistics
// (src/solver/GridStatistics.cpp:95-181): -1, with the error latched, for a cell
// out of range, of another material, or a non-finite occupation.
__device__ __forceinline__ long long bin_slot(const DevTables& T, const CellArrays& C, DevLedger* L, int slot, int cell,
                                              uint32_t w, double occ) {
    const int mid = static_cast<int>(w >> 28);
    const bool finite = (__double2hiint(occ) & 0x7ff00000) != 0x7ff00000;
    if (cell < 0 || cell >= C.ncells || C.cell_material[cell] != mid || !finite) {
        raise_error(L, kErrInvalidStatistics, slot);
        return -1;
    }
    return static_cast<long long>(cell) * C.hist_modes + bin_of(T.mat[mid], static_cast<int>(w & 0x00FFFFFFu));
}

__device__ __forceinline__ void bin_add(const CellArrays& C, long long h, unsigned cnt, double N, double M, bool rta) {
    atomicAdd(&C.bins[h].cnt, cnt);
    atomicAdd(&C.bins[h].N, N);
    if (rta) atomicAdd(C.hM + h, M);
}

__device__ __forceinline__ void bin_carrier(const DevTables& T, const CellArrays& C, DevLedger* L, int slot, int cell,
                                           uint32_t w, double occ, bool rta) {
    const long long h = bin_slot(T, C, L, slot, cell, w, occ);
    if (h >= 0) bin_add(C, h, 1u, occ, fmax(1.0, occ), rta);
}

// Sums of `v` over runs of equal keys in lane order, left at the first lane of
// each run (all 32 lanes call; `heads` marks the first lane of every run). A
// tree over each run: in round o a lane at an even multiple of o within its
// run adds the partial sum of the lane o further on, when that lane is still
// in the run -- every value is added once, so a run of L lanes costs L - 1
// FP64 additions (GB300 retires two FP64 lanes per SM per clock).
// Rounds run while o is below the longest run of the warp (`span`, from
// run_span), so short runs cost one or two rounds instead of five.
template <class T>
__device__ __forceinline__ T run_sum_to_head(T v, unsigned heads, int lane, int span = 32) {
    const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
    const unsigned later = lane == 31 ? 0u : heads & (0xfffffffeu << lane);
    const int end = later ? __ffs(later) - 1 : 32; // first lane past the run
    const int pos = lane - start;
    for (int o = 1; o < span; o <<= 1) { // warp-uniform trip count
        const T w = __shfl_down_sync(0xffffffffu, v, o);
        if ((pos & (2 * o - 1)) == 0 && lane + o < end) v += w;
    }
    return v;
}

// Length of the longest run of the warp (all 32 lanes call).
__device__ __forceinline__ int run_span(unsigned heads, int lane) {
    const unsigned later = lane == 31 ? 0u : heads & (0xfffffffeu << lane);
    const unsigned len = ((heads >> lane) & 1u) ? static_cast<unsigned>((later ? __ffs(later) - 1 : 32) - lane) : 0u;
    return static_cast<int>(__reduce_max_sync(0xffffffffu, len));
}

// Bin tallies of one warp (all 32 lanes call; h < 0: nothing from this lane).
// Runs of equal records in lane order -- the common case once the carriers
// are sorted by (mode, cell) -- are summed (run_sum_to_head) and the first
// lane of each run makes one atomic per field. kAgg false: one atomic per carrier.
template <bool kAgg, bool kRta>
__device__ __forceinline__ void bin_warp(const CellArrays& C, long long h, double occ) {
    if constexpr (!kAgg) {
        if (h >= 0) bin_add(C, h, 1u, occ, fmax(1.0, occ), kRta);
    } else {
        const int lane = threadIdx.x & 31;
        const long long hp = __shfl_up_sync(0xffffffffu, h, 1);
        const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || hp != h);
        unsigned cnt = h >= 0 ? 1u : 0u;
        double N = h >= 0 ? occ : 0.0;
        double M = h >= 0 ? fmax(1.0, occ) : 0.0;
        if (heads != 0xffffffffu) { // warp-uniform: some run is longer than one lane
            const int span = run_span(heads, lane);
            cnt = run_sum_to_head(cnt, heads, lane, span);
            N = run_sum_to_head(N, heads, lane, span);
            if (kRta) M = run_sum_to_head(M, heads, lane, span);
        }
        if (h >= 0 && ((heads >> lane) & 1u)) bin_add(C, h, cnt, N, M, kRta);
    }
}

// Pending (alpha, beta) of the carrier's bin: collision of the previous step
// and the gradient / heat-source halves around this transport.
__device__ __forceinline__ double apply_pending(const DevTables& T, const CellArrays& C, int cell, uint32_t w,
                                                double occ) {
    const int b = bin_of(T.mat[w >> 28], static_cast<int>(w & 0x00FFFFFFu));
    const double2 ab = __ldg(C.ab + static_cast<size_t>(cell) * C.hist_modes + b);
    return fma(ab.x, occ, ab.y);
}

__device__ __forceinline__ double drive_half(const DevTables& T, const CellArrays& C, const DevMaterial& M, int cell,
                                             int ai) {
    if (!M.grad_rate) return 0.0;
    return fma(-M.drive_cap[ai], C.grad_ratio[cell], M.drive_rate[ai]);
}

// ---------------------------------------------------- FP32 flight (mixed)
struct Frame {
    int i[3];       // cell indices per axis
    float cs[3];    // cell size
    float lo[3], hi[3]; // box walls in the frame of the starting cell
};

// Exact quotient of n < 2^31 by d through the host-verified multiplier floor(2^64/d)+1.
__device__ __forceinline__ int magic_div(int n, unsigned long long magic) {
    return magic ? static_cast<int>(__umul64hi(static_cast<unsigned long long>(n), magic)) : n;
}

__device__ __forceinline__ Frame cell_frame(const DevDomain& D, int cell) {
    Frame F;
    F.i[0] = magic_div(cell, D.div_yz);
    const int r = cell - F.i[0] * (D.shape[1] * D.shape[2]);
    F.i[1] = magic_div(r, D.div_z);
    F.i[2] = r - F.i[1] * D.shape[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        F.cs[a] = D.cell_size32[a];
        F.lo[a] = -static_cast<float>(F.i[a]) * F.cs[a];
        F.hi[a] = static_cast<float>(D.shape[a] - F.i[a]) * F.cs[a];
    }
    return F;
}

// FP32 velocity and its reciprocal (0 where a component is 0) from the
// per-mode tables, sign flips on the sign bits.
__device__ __forceinline__ void mode_velocity32(const DevMaterial& M, uint32_t w, float v[3], float iv[3]) {
    const int a = static_cast<int>(w & 0x00FFFFFFu);
    const float4 vv = __ldg(reinterpret_cast<const float4*>(M.vel32) + a);
    const float4 ii = __ldg(reinterpret_cast<const float4*>(M.ivel32) + a);
    const float c[3] = {vv.x, vv.y, vv.z}, r[3] = {ii.x, ii.y, ii.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const unsigned flip = ((w >> (24 + k)) & 1u) << 31;
        v[k] = __uint_as_float(__float_as_uint(c[k]) ^ flip);
        iv[k] = __uint_as_float(__float_as_uint(r[k]) ^ flip);
    }
}

// ------------------------------------- mixed carrier state in mesh domains
// A mesh carrier keeps FP32 offsets from the corner of its cell's home voxel
// (the voxel whose centre made the cell). A carrier may sit in a voxel whose
// centre lies outside the mesh: that voxel belongs to a neighbouring cell
// through the voxel map, and its offsets reach beyond the home voxel by the
// voxels in between.
__device__ __forceinline__ Frame cell_frame_of(const DevTables& T, int cell) {
    return cell_frame(T.dom, T.fac.cell_voxel ? __ldg(T.fac.cell_voxel + cell) : cell);
}

// FP64 position of FP32 offsets in frame F.
__device__ __forceinline__ void frame_point(const DevDomain& D, const Frame& F, const float o[3], double p[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
        p[a] = dadd(dadd(D.lo[a], dmul(static_cast<double>(F.i[a]), D.cell_size[a])), static_cast<double>(o[a]));
}

// FP32 offsets of an FP64 position from the home voxel of its cell; returns the cell.
__device__ __forceinline__ int frame_offsets(const DevTables& T, const double p[3], float o[3]) {
    const int c = cell_at(T, p[0], p[1], p[2]);
    const Frame F = cell_frame_of(T, c);
#pragma unroll
    for (int a = 0; a < 3; ++a)
        o[a] = static_cast<float>(dadd(p[a], -dadd(T.dom.lo[a], dmul(static_cast<double>(F.i[a]), T.dom.cell_size[a]))));
    return c;
}

// FP32 velocity of a mesh carrier: the mode velocity with its sign flips,
// mirrored in the plane of facet `mir` when set.
__device__ __forceinline__ void mesh_velocity32(const DevFacets& Fc, const DevMaterial& M, uint32_t w, int mir,
                                                float v[3]) {
    float iv[3];
    mode_velocity32(M, w, v, iv);
    if (mir >= 0) {
        const double* n = Fc.normal + 3 * mir;
        const float nn[3] = {static_cast<float>(n[0]), static_cast<float>(n[1]), static_cast<float>(n[2])};
        const float s = 2.0f * (v[0] * nn[0] + v[1] * nn[1] + v[2] * nn[2]);
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] -= nn[k] * s;
    }
}

// Cell after an FP32 flight in frame F of a mesh domain: the voxel the point
// ends in (clamped to the grid), its cell through the voxel map, and the
// offsets moved to that cell's home voxel.
__device__ __forceinline__ int settle_mesh(const DevTables& T, const Frame& F, float p[3]) {
    const DevDomain& D = T.dom;
    int j[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int k = F.i[a] + static_cast<int>(floorf(p[a] * D.inv_cell32[a]));
        j[a] = k < 0 ? 0 : (k >= D.shape[a] ? D.shape[a] - 1 : k);
    }
    const int c = __ldg(T.fac.voxel_cell + (j[0] * D.shape[1] + j[1]) * D.shape[2] + j[2]);
    const Frame H = cell_frame_of(T, c);
#pragma unroll
    for (int a = 0; a < 3; ++a) p[a] -= static_cast<float>(H.i[a] - F.i[a]) * F.cs[a];
    return c;
}

// Wall caches of every live carrier after an upload (src/solver/Initialization.cpp:131).
template <bool kMixed>
__global__ void k_mesh_cache_init(const __grid_constant__ DevTables T, CarrierState S, DevLedger* L) {
    const int n = L->n_slots;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!S.alive[i]) continue;
        const uint32_t w = S.mode[i];
        double v[3];
        mesh_velocity(T.fac, T.mat[w >> 28], w, T.fac.mirror[i], v);
        // the uploaded FP64 position, not its FP32 offsets: a carrier within
        // the offsets' rounding of a wall could otherwise trace from outside
        double p[3] = {S.x[i], S.y[i], S.z[i]};
        MeshCache c;
        mesh_refresh(T, L, nullptr, i, p, v, c);
        if (kMixed) {
            float o[3];
            S.cell[i] = frame_offsets(T, p, o);
            S.ox[i] = o[0];
            S.oy[i] = o[1];
            S.oz[i] = o[2];
        } else {
            S.x[i] = p[0];
            S.y[i] = p[1];
            S.z[i] = p[2];
        }
        mesh_cache_store(T.fac, i, c);
    }
}

// Rough (or, with conservative boundaries, any non-periodic) wall hit
// (src/solver/BoundaryInteraction.cpp:53-162): sample the outgoing mode and
// occupation from the wall's table with the draws of (slot, step, purpose,
// event). False when the event raised an error (the carrier then stays where
// it is, as the reference stops its flight with the throw).
__device__ __forceinline__ bool wall_sample_mixed(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot, int plane,
                                                  uint32_t& w, double& occ, int event, uint32_t purpose, uint32_t step) {
    const DevDomain& D = T.dom;
    const DevParams& P = T.par;
    const int mid = static_cast<int>(w >> 28);
    const DevMaterial& M = T.mat[mid];
    const int axis = plane >> 1;
    const int ai = static_cast<int>(w & 0x00FFFFFFu);
    const int table = D.rough_table[mid][plane];
    if (table < 0) {
        raise_error(L, kErrModeMapping, slot);
        return false;
    }
    const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 0);
    const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 1);
    double n_out;
    unsigned diag;
    const int out = rough_sample_dev(T.rough[table], M, ai, occ, P.conservative != 0, d0.a, d0.b, d1.a, n_out, diag);
    count_rough(bl, diag);
    const double vn = M.vel[3 * out + axis] * ((plane & 1) ? 1.0 : -1.0);
    uint32_t signs = 0;
    if (P.conservative) {
        if (!isfinite(n_out) || !(M.omega[out] > 0.0) || !(vn < 0.0)) {
            raise_error(L, kErrModeMapping, slot);
            return false;
        }
    } else if (vn > 0.0) {
        signs = 1u << axis;
    }
    w = static_cast<uint32_t>(out) | (signs << 24) | (static_cast<uint32_t>(mid) << 28);
    occ = n_out;
    return true;
}

enum FlightEnd { kFlightDone = 0, kFlightAbsorbed = 1, kFlightDeferred = 2 };
constexpr int kDeferInterface = 8; // queued plane code 8 + destination material: an interface event

__device__ __forceinline__ float axis_of(const float v[3], int axis) {
    return axis == 0 ? v[0] : (axis == 1 ? v[1] : v[2]);
}

// Diffuse-mismatch interface event of the FP32 flight (same draws as the FP64
// flight: keyed by slot, step, purpose and event). False on an invalid
// outgoing mode (error raised).
__device__ __forceinline__ bool interface_step_mixed(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot,
                                                     int destination, uint32_t& w, double& occ, int event,
                                                     uint32_t purpose, uint32_t step) {
    const DevParams& P = T.par;
    const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 0);
    const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(slot), step, purpose, static_cast<uint32_t>(event), 1);
    const IfaceOut r = interface_dev(T, static_cast<int>(w >> 28), static_cast<int>(w & 0x00FFFFFFu), (w >> 24) & 7u,
                                     occ, destination, d0.a, d0.b, d1.a, d1.b);
    count_interface(bl, r);
    if (r.action >= 5) {
        raise_error(L, r.action == 6 ? kErrAmmRow : kErrModeMapping, slot);
        return false;
    }
    w = static_cast<uint32_t>(r.active) | (r.signs << 24) | (static_cast<uint32_t>(r.material) << 28);
    occ = r.occ;
    return true;
}

// Free flight in FP32 in the frame of the starting cell. Walls are hit
// exactly (the coordinate is set to the wall), so no push-off distance is
// needed; periodic faces map the coordinate to the opposite wall; material
// planes (cell boundaries) are hit exactly the same way, and the plane ahead
// is chosen from the carrier's own layer and direction, so a carrier leaving
// a plane never re-crosses it. With kDefer the flight stops at a wall that
// needs table sampling, or at a material plane, and reports it (plane), the
// time left and the event index, so that the few carriers with such events
// are finished together by k_deferred instead of stalling the whole warp on
// the long FP64 sampling path.
template <bool kDefer>
__device__ __forceinline__ int advance_mixed(const DevTables& T, DevLedger* L, BlockLedger* bl, int slot,
                                             const Frame& F, float p[3], uint32_t& w, double& occ, float& remaining,
                                             int& event, int& plane_out, uint32_t purpose, uint32_t step) {
    const DevDomain& D = T.dom;
    const DevParams& P = T.par;
    int mid = static_cast<int>(w >> 28);
    const DevMaterial* M = &T.mat[mid];
    const int nmat = P.n_materials;
    const int lax = D.layout_axis;
    float v[3], iv[3];
    mode_velocity32(*M, w, v, iv);
    for (; remaining > 0.0f && event < 64; ++event) {
        float t = __int_as_float(0x7f800000);
        int plane = -1;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (v[a] == 0.0f) continue;
            const bool up = v[a] > 0.0f;
            const float h = fmaxf(((up ? F.hi[a] : F.lo[a]) - p[a]) * iv[a], 0.0f);
            if (h < t) {
                t = h;
                plane = 2 * a + (up ? 1 : 0);
            }
        }
        // material plane ahead (src/solver/LayeredMaterialLayout.cpp:31-60); the wall wins ties
        float t_if = __int_as_float(0x7f800000);
        float plane_at = 0.0f;
        int destination = -1;
        if (nmat > 1) {
            const float va = axis_of(v, lax);
            int k = -1;
            if (va > 0.0f && mid + 1 < nmat) k = mid;
            else if (va < 0.0f && mid > 0) k = mid - 1;
            if (k >= 0) {
                const int fi = lax == 0 ? F.i[0] : (lax == 1 ? F.i[1] : F.i[2]);
                const float cs = lax == 0 ? F.cs[0] : (lax == 1 ? F.cs[1] : F.cs[2]);
                plane_at = static_cast<float>(D.plane_cell[k] - fi) * cs;
                const float h = (plane_at - axis_of(p, lax)) * axis_of(iv, lax);
                if (h >= 0.0f) {
                    t_if = h;
                    destination = va > 0.0f ? mid + 1 : mid - 1;
                }
            }
        }
        const bool interface_first = destination >= 0 && t_if < t;
        const float t_event = interface_first ? t_if : t;
        if ((plane < 0 && !interface_first) || t_event > remaining) {
#pragma unroll
            for (int a = 0; a < 3; ++a) p[a] = fmaf(v[a], remaining, p[a]);
            return kFlightDone;
        }
        remaining -= t_event;
        if (interface_first) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                p[a] = fmaf(v[a], t_event, p[a]);
                if (a == lax) p[a] = plane_at;
            }
            if (kDefer) {
                plane_out = kDeferInterface + destination;
                return kFlightDeferred;
            }
            if (!interface_step_mixed(T, L, bl, slot, destination, w, occ, event, purpose, step)) return kFlightDone;
            mid = static_cast<int>(w >> 28);
            M = &T.mat[mid];
            mode_velocity32(*M, w, v, iv);
            continue;
        }
        const int axis = plane >> 1;
        const bool hi_side = (plane & 1) != 0;
        // the hit coordinate lands on the wall (selects keep p and F in registers)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            p[a] = fmaf(v[a], t, p[a]);
            if (a == axis) p[a] = hi_side ? F.hi[a] : F.lo[a];
        }
        const char cond = D.cond[plane];
        if (cond == 'T') {
            const int ai = static_cast<int>(w & 0x00FFFFFFu);
            const double e = M->hw[ai] * (occ - M->nbg[ai]) * M->energy_weight;
            atomicAdd(&bl->absorbed, 1u);
            atomicAdd(&bl->absorbed_ev, e);
            const int r = D.reservoir[plane];
            if (r >= 0) atomicAdd(&bl->absorbed_res[r], 1u);
            return kFlightAbsorbed;
        }
        if (cond == 'P' && D.pair[plane] >= 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (a == axis) p[a] = hi_side ? F.lo[a] : F.hi[a];
            continue;
        }
        if (P.conservative || (cond == 'R' && D.rough_table[mid][plane] >= 0)) {
            if (kDefer) {
                plane_out = plane;
                return kFlightDeferred;
            }
            if (!wall_sample_mixed(T, L, bl, slot, plane, w, occ, event, purpose, step)) return kFlightDone;
        } else if (cond == 'R') {
            raise_error(L, kErrNoRoughTable, slot);
            return kFlightDone;
        } else {
            w ^= 1u << (24 + axis);
        }
        mode_velocity32(*M, w, v, iv);
    }
    if (remaining > 0.0f) raise_error(L, kErrTooManyEvents, slot);
    return kFlightDone;
}

// New cell and offset after an FP32 flight in the frame of cell F.
__device__ __forceinline__ int settle_mixed(const DevDomain& D, const Frame& F, float p[3]) {
    int j[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int k = F.i[a] + static_cast<int>(floorf(p[a] * D.inv_cell32[a]));
        k = k < 0 ? 0 : (k >= D.shape[a] ? D.shape[a] - 1 : k);
        p[a] -= static_cast<float>(k - F.i[a]) * F.cs[a];
        j[a] = k;
    }
    return (j[0] * D.shape[1] + j[1]) * D.shape[2] + j[2];
}

// ------------------------------------------------------ transport pass
// New cell of an FP32 flight; a carrier that ends exactly on a material plane
// (a cell boundary) is given the cell of its own layer.
__device__ __forceinline__ int settle_layer(const DevTables& T, const CellArrays& C, const Frame& F, float p[3],
                                           int mid) {
    int c = settle_mixed(T.dom, F, p);
    if (T.par.n_materials > 1 && C.cell_material[c] != mid) {
        const DevDomain& D = T.dom;
        const int lax = D.layout_axis;
        const int nyz = D.shape[1] * D.shape[2];
        const int stride = lax == 0 ? nyz : (lax == 1 ? D.shape[2] : 1);
        const int idx = lax == 0 ? c / nyz : (lax == 1 ? (c / D.shape[2]) % D.shape[1] : c % D.shape[2]);
        const int n_axis = lax == 0 ? D.shape[0] : (lax == 1 ? D.shape[1] : D.shape[2]);
        const int dir = mid > C.cell_material[c] ? 1 : -1;
        if (idx + dir >= 0 && idx + dir < n_axis && C.cell_material[c + dir * stride] == mid) {
            c += dir * stride;
#pragma unroll
            for (int a = 0; a < 3; ++a)
                if (a == lax) p[a] -= static_cast<float>(dir) * F.cs[a];
        }
    }
    return c;
}

// Common end of a carrier's step: store the state; a live carrier takes its
// new cell and enters the bins.
// Stores the carrier after its flight; returns its bin record (-1: absorbed
// or invalid) for the caller to tally.
// The mode word is stored only when the flight changed it (most carriers keep
// their mode for the step, and unchanged words leave most of its sectors clean).
__device__ __forceinline__ long long finish_mixed(const DevTables& T, const CarrierState& S, const CellArrays& C,
                                                  DevLedger* L, int i, const Frame& F, float p[3], uint32_t w,
                                                  double occ, bool alive, uint32_t w0) {
    const int c = settle_layer(T, C, F, p, static_cast<int>(w >> 28));
    __stcs(S.ox + i, p[0]);
    __stcs(S.oy + i, p[1]);
    __stcs(S.oz + i, p[2]);
    if (w != w0) __stcs(S.mode + i, w);
    __stcs(S.occ + i, occ);
    if (!alive) {
        S.alive[i] = 0;
        return -1;
    }
    __stcs(S.cell + i, c);
    return bin_slot(T, C, L, i, c, w, occ);
}

constexpr int kTransportThreads = 256; // fused batch kernels and the default of the single-instance pass
constexpr int kTransportMaxThreads = 512;
constexpr int kDeferBuffer = 64; // queued wall events per warp before a flush

// The one carrier pass of a timestep: apply the pending update on load, fly,
// bin. Mixed path: carriers that reach a wall needing table sampling are
// queued (per-warp shared buffers, one global atomic per 32 entries) and
// finished by k_deferred.
// One carrier of the mixed pass, called by every thread of the block with its
// fields (in = slot in range): apply the pending update, fly in FP32, store,
// tally its bin over the warp, and queue a wall event that needs table
// sampling (per-warp shared buffer qbuf, one global atomic per 32 entries).
template <bool kRta, bool kAgg>
__device__ __forceinline__ void mixed_carrier(const DevTables& T, const CarrierState& S, const CellArrays& C,
                                              DevLedger* L, BlockLedger& bl, uint32_t step, int i, bool in,
                                              uint8_t alive, uint32_t w, int c0, double occ0, float p[3],
                                              int4 (*qbuf)[kDeferBuffer], int& queued) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool defer = false;
    int4 entry;
    long long h = -1;
    double hocc = 0.0;
    if (in && alive) {
        const uint32_t w0 = w;
        double occ = apply_pending(T, C, c0, w, occ0);
        const Frame F = cell_frame(T.dom, c0);
        float remaining = T.par.dt32;
        int event = 0, plane = -1;
        const int end = advance_mixed<true>(T, L, &bl, i, F, p, w, occ, remaining, event, plane, kDrawTransport, step);
        if (end == kFlightDeferred) {
            // state at the wall, cell unchanged (the frame of the flight)
            __stcs(S.ox + i, p[0]);
            __stcs(S.oy + i, p[1]);
            __stcs(S.oz + i, p[2]);
            __stcs(S.mode + i, w);
            __stcs(S.occ + i, occ);
            defer = true;
            entry = make_int4(i, __float_as_int(remaining), event, plane);
        } else {
            h = finish_mixed(T, S, C, L, i, F, p, w, occ, end != kFlightAbsorbed, w0);
            hocc = occ;
        }
    }
    bin_warp<kAgg, kRta>(C, h, hocc);
    const unsigned mask = __ballot_sync(0xffffffffu, defer);
    if (mask) {
        if (defer) qbuf[warp][queued + __popc(mask & ((1u << lane) - 1u))] = entry;
        queued += __popc(mask);
        __syncwarp();
        if (queued >= 32) {
            int at = 0;
            if (lane == 0) at = atomicAdd(&L->n_deferred, 32);
            at = __shfl_sync(0xffffffffu, at, 0);
            if (at + lane < S.capacity) S.deferred[at + lane] = qbuf[warp][lane];
            else raise_error(L, kErrInvalidStatistics, i);
            __syncwarp();
            const int rest = queued - 32;
            int4 t = make_int4(0, 0, 0, 0);
            if (lane < rest) t = qbuf[warp][32 + lane];
            __syncwarp();
            if (lane < rest) qbuf[warp][lane] = t;
            __syncwarp();
            queued = rest;
        }
    }
}

// The rest of a warp's queued wall events, after its last carrier.
__device__ __forceinline__ void flush_deferred(const CarrierState& S, DevLedger* L, int4 (*qbuf)[kDeferBuffer],
                                               int queued) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (queued > 0) {
        int at = 0;
        if (lane == 0) at = atomicAdd(&L->n_deferred, queued);
        at = __shfl_sync(0xffffffffu, at, 0);
        if (lane < queued) {
            if (at + lane < S.capacity) S.deferred[at + lane] = qbuf[warp][lane];
            else raise_error(L, kErrInvalidStatistics, at + lane);
        }
    }
}

// First queue entry of a thread in an event pass over a queue of length n:
// entry 32 w + lane goes to warp w = (warp in block) x CTAs + CTA, so the
// first entries spread one warp per CTA over every SM instead of filling the
// first CTAs' warps (a short queue would otherwise run on a few SMs). Stride:
// CTAs x block threads.
__device__ __forceinline__ int queue_first(int vbx, int vgx) {
    return ((static_cast<int>(threadIdx.x >> 5) * vgx + vbx) << 5) + static_cast<int>(threadIdx.x & 31);
}

// Queues slot i (lanes with `defer`) for an event pass: one global atomic per
// warp; every lane of the warp calls it.
__device__ __forceinline__ void queue_event(const CarrierState& S, DevLedger* L, bool defer, int i) {
    const unsigned mask = __ballot_sync(0xffffffffu, defer);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    int at = 0;
    if (lane == 0) at = atomicAdd(&L->n_deferred, __popc(mask));
    at = __shfl_sync(0xffffffffu, at, 0);
    if (defer) {
        const int q = at + __popc(mask & ((1u << lane) - 1u));
        if (q < S.capacity) S.deferred[q] = make_int4(i, 0, 0, 0);
        else raise_error(L, kErrInvalidStatistics, i);
    }
}

// Streamed fields of one slot of the mixed state. Every field is loaded before
// alive is looked at, so the loads of a carrier share one memory round trip
// (slots below n_slots are allocated whether alive or not).
struct MixedSlot {
    bool in;
    uint8_t alive;
    uint32_t w;
    int c0;
    double occ0;
    float p[3];
};

__device__ __forceinline__ MixedSlot load_mixed_slot(const CarrierState& S, int i, int n) {
    MixedSlot s;
    s.in = i < n;
    const int ic = s.in ? i : 0;
    s.alive = __ldcs(S.alive + ic);
    s.w = __ldcs(S.mode + ic);
    s.c0 = __ldcs(S.cell + ic);
    s.occ0 = __ldcs(S.occ + ic);
    s.p[0] = __ldcs(S.ox + ic);
    s.p[1] = __ldcs(S.oy + ic);
    s.p[2] = __ldcs(S.oz + ic);
    return s;
}

// qbuf: kDeferBuffer entries per warp of the block (mixed path).
template <bool kMixed, bool kRta, bool kAgg>
__device__ __forceinline__ void k_transport_body(const DevTables& T, CarrierState S, CellArrays C, DevLedger* L, int vbx,
                                                 int vgx, int4 (*qbuf)[kDeferBuffer]) {
    const uint32_t step = L->step_index; // timesteps completed: the draw counter of this step
    __shared__ BlockLedger bl;
    block_ledger_init(&bl);
    __syncthreads();
    const int n = L->n_slots;
    if constexpr (kMixed) {
        int queued = 0; // warp-uniform
        // block-uniform trip count so that every lane reaches the warp-wide
        // ballot; the next slot's streamed fields are in flight while this
        // one flies (each slot belongs to one thread of the pass). With one
        // material the mode word's material bits (always 0 then) are cleared
        // in the copy the carrier works on, so every table index folds to a
        // compile-time 0 and the table fields become constant-bank operands.
        const int stride = vgx * blockDim.x;
        int base = vbx * blockDim.x;
        const bool one_material = T.par.n_materials == 1;
        auto run = [&](MixedSlot& s, int i) {
            if (one_material)
                mixed_carrier<kRta, kAgg>(T, S, C, L, bl, step, i, s.in, s.alive, s.w & 0x0FFFFFFFu, s.c0, s.occ0, s.p,
                                          qbuf, queued);
            else
                mixed_carrier<kRta, kAgg>(T, S, C, L, bl, step, i, s.in, s.alive, s.w, s.c0, s.occ0, s.p, qbuf,
                                          queued);
        };
        MixedSlot cur = load_mixed_slot(S, base + threadIdx.x, n);
        for (; base < n; base += stride) {
            MixedSlot next;
            if (base + stride < n) next = load_mixed_slot(S, base + stride + threadIdx.x, n);
            run(cur, base + threadIdx.x);
            cur = next;
        }
        flush_deferred(S, L, qbuf, queued);
    } else {
        // Carriers that cannot reach a wall (or, layered, the material plane
        // ahead) within the step drift here; the others are queued, with their
        // updated occupation, for k_box_events, so no warp of this pass waits
        // on a few lanes' FP64 wall events.
        // block-uniform trip count so that every lane reaches the warp tally and ballot
        for (int base = vbx * blockDim.x; base < n; base += vgx * blockDim.x) {
            const int i = base + threadIdx.x;
            long long h = -1;
            double occ = 0.0;
            bool defer = false;
            // all streamed fields in one memory round trip, alive included
            const bool in = i < n;
            const int ic = in ? i : 0;
            const uint8_t alive0 = __ldcs(S.alive + ic);
            uint32_t w = __ldcs(S.mode + ic);
            const int c0 = __ldcs(S.cell + ic);
            const double occ0 = __ldcs(S.occ + ic);
            double p[3] = {__ldcs(S.x + ic), __ldcs(S.y + ic), __ldcs(S.z + ic)};
            if (in && alive0) {
                occ = apply_pending(T, C, c0, w, occ0);
                double v[3];
                mode_velocity(T.mat[w >> 28], w, v);
                const double dt = T.par.dt;
                const float dt_up = __double2float_ru(dt);
                // clear of every wall (and, layered, of the material plane ahead)
                // implies advance_carrier's direct flight: the same position bits
                bool clear = clear_of_walls32(T.dom, p, v, dt_up);
                if (T.par.n_materials > 1)
                    clear = clear && clear_of_planes32(T.dom, T.par.n_materials, p, v, static_cast<int>(w >> 28), dt_up);
                if (clear) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], dt));
                    const int c = grid_index(T.dom, p[0], p[1], p[2]);
                    __stcs(S.x + i, p[0]);
                    __stcs(S.y + i, p[1]);
                    __stcs(S.z + i, p[2]);
                    __stcs(S.occ + i, occ);
                    __stcs(S.cell + i, c);
                    h = bin_slot(T, C, L, i, c, w, occ);
                } else {
                    __stcs(S.occ + i, occ);
                    defer = true;
                }
            }
            bin_warp<kAgg, kRta>(C, h, occ);
            queue_event(S, L, defer, i);
        }
    }
    __syncthreads();
    block_ledger_flush(&bl, L);
}

// Plain FP64 wall events queued by the carrier pass: the whole flight of the
// step from its start (occupation already updated) through advance_carrier,
// then the cell and the bin. Every lane of a warp runs an event flight.
template <bool kRta>
__device__ __forceinline__ void k_box_events_body(const DevTables& T, CarrierState S, CellArrays C, DevLedger* L,
                                                  int vbx, int vgx) {
    const uint32_t step = L->step_index;
    __shared__ BlockLedger bl;
    block_ledger_init(&bl);
    __syncthreads();
    const int nq = min(L->n_deferred, S.capacity);
    for (int q = queue_first(vbx, vgx); q < nq; q += vgx * blockDim.x) {
        const int i = S.deferred[q].x;
        if (i < 0 || i >= S.capacity) {
            raise_error(L, kErrInvalidStatistics, i);
            continue;
        }
        uint32_t w = S.mode[i];
        double occ = S.occ[i];
        double p[3] = {S.x[i], S.y[i], S.z[i]};
        const bool alive = advance_carrier(T, L, &bl, i, p, w, occ, T.par.dt, kDrawTransport, step);
        const int c = grid_index(T.dom, p[0], p[1], p[2]);
        S.x[i] = p[0];
        S.y[i] = p[1];
        S.z[i] = p[2];
        S.mode[i] = w;
        S.occ[i] = occ;
        if (!alive) {
            S.alive[i] = 0;
            continue;
        }
        S.cell[i] = c;
        bin_carrier(T, C, L, i, c, w, occ, kRta);
    }
    __syncthreads();
    block_ledger_flush(&bl, L);
}

template <bool kRta>
__global__ void __launch_bounds__(256) k_box_events(const __grid_constant__ DevTables T, CarrierState S, CellArrays C,
                                                    DevLedger* L) {
    k_box_events_body<kRta>(T, S, C, L, blockIdx.x, gridDim.x);
}

// ------------------------------------------- TMA-staged mixed carrier pass
// The carrier fields of a tile of kPipeTile slots arrive in shared memory by
// bulk asynchronous copies (cp.async.bulk, completion counted on an mbarrier)
// one tile ahead: while a CTA flies the carriers of tile k, the copies of
// tile k + grid are in flight into the other of two stages, so the streamed
// loads never sit on the dependent chain of a carrier (load -> pending gather
// -> flight -> store). One elected thread issues the copies; a bounded wait
// on the stage's barrier phase gives every thread the tile.
constexpr int kPipeTile = 256;

struct __align__(16) PipeStage {
    double occ[kPipeTile];
    uint32_t mode[kPipeTile];
    int32_t cell[kPipeTile];
    float ox[kPipeTile], oy[kPipeTile], oz[kPipeTile];
    uint8_t alive[kPipeTile];
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void bulk_to_shared(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// Bytes of a tile's field copy: 16-byte multiples (the arrays are padded by a
// tile past the capacity, so the rounded tail stays inside the allocation).
__device__ __forceinline__ uint32_t tile_bytes(int count, int size) {
    return (static_cast<uint32_t>(count * size) + 15u) & ~15u;
}

__device__ __forceinline__ void issue_tile(const CarrierState& S, int tile, int n, PipeStage* st, uint64_t* bar) {
    const int first = tile * kPipeTile;
    const int count = min(kPipeTile, n - first);
    const uint32_t b8 = tile_bytes(count, 8), b4 = tile_bytes(count, 4), b1 = tile_bytes(count, 1);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_addr(bar)),
                 "r"(b8 + 5 * b4 + b1)
                 : "memory");
    bulk_to_shared(st->occ, S.occ + first, b8, bar);
    bulk_to_shared(st->mode, S.mode + first, b4, bar);
    bulk_to_shared(st->cell, S.cell + first, b4, bar);
    bulk_to_shared(st->ox, S.ox + first, b4, bar);
    bulk_to_shared(st->oy, S.oy + first, b4, bar);
    bulk_to_shared(st->oz, S.oz + first, b4, bar);
    bulk_to_shared(st->alive, S.alive + first, b1, bar);
}

// Waits for a barrier phase for at most about 2^31 SM clocks (~1 s); false on timeout.
__device__ __forceinline__ bool wait_phase(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(smem_addr(bar)), "r"(parity)
                     : "memory");
        if (done) return true;
        if (clock64() - t0 > (1LL << 31)) return false;
    }
}

template <bool kRta, bool kAgg>
__global__ void __launch_bounds__(kPipeTile) k_transport_pipe(const __grid_constant__ DevTables T, CarrierState S,
                                                              CellArrays C, DevLedger* L) {
    __shared__ PipeStage stage[2];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int4 qbuf[kPipeTile / 32][kDeferBuffer];
    __shared__ BlockLedger bl;
    const uint32_t step = L->step_index;
    const int n = L->n_slots;
    const int ntiles = (n + kPipeTile - 1) / kPipeTile;
    block_ledger_init(&bl);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if (static_cast<int>(blockIdx.x) < ntiles) issue_tile(S, blockIdx.x, n, &stage[0], &bar[0]);
    }
    __syncthreads();
    int queued = 0;
    int k = 0;
    uint32_t pending = static_cast<int>(blockIdx.x) < ntiles ? 1u : 0u; // stages with copies in flight (bits)
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k) { // block-uniform
        const int s = k & 1;
        const int next = t + static_cast<int>(gridDim.x);
        if (next < ntiles) {
            if (threadIdx.x == 0) {
                // the other stage was read in the previous iteration (ordered by its closing barrier)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue_tile(S, next, n, &stage[s ^ 1], &bar[s ^ 1]);
            }
            pending |= 1u << (s ^ 1);
        }
        const bool ok = wait_phase(&bar[s], static_cast<uint32_t>((k >> 1) & 1));
        if (!__syncthreads_and(ok)) {
            raise_error(L, kErrPipelineTimeout, t);
            break;
        }
        pending &= ~(1u << s);
        const int i = t * kPipeTile + static_cast<int>(threadIdx.x);
        const PipeStage& st = stage[s];
        float p[3] = {st.ox[threadIdx.x], st.oy[threadIdx.x], st.oz[threadIdx.x]};
        mixed_carrier<kRta, kAgg>(T, S, C, L, bl, step, i, i < n, st.alive[threadIdx.x], st.mode[threadIdx.x],
                                  st.cell[threadIdx.x], st.occ[threadIdx.x], p, qbuf, queued);
        __syncthreads(); // stage s is free for the copies of iteration k + 1
    }
    // after a timeout in iteration k: give copies still in flight a bounded
    // wait before the CTA leaves (stage k & 1 was awaited for iteration k, the
    // other stage was filled for iteration k + 1)
    for (int x = 0; x < 2; ++x) {
        if (!(pending & (1u << x))) continue;
        const int kk = x == (k & 1) ? k : k + 1;
        wait_phase(&bar[x], static_cast<uint32_t>((kk >> 1) & 1));
    }
    flush_deferred(S, L, qbuf, queued);
    __syncthreads();
    block_ledger_flush(&bl, L);
}

// Block size chosen at launch (128, 256 or 512 threads); the wall-event queue
// of the mixed path is dynamic shared memory, kDeferBuffer entries per warp.
template <bool kMixed, bool kRta, bool kAgg>
__global__ void __launch_bounds__(kTransportMaxThreads) k_transport(const __grid_constant__ DevTables T, CarrierState S,
                                                                    CellArrays C, DevLedger* L) {
    extern __shared__ int4 qdyn[];
    k_transport_body<kMixed, kRta, kAgg>(T, S, C, L, blockIdx.x, gridDim.x,
                                         reinterpret_cast<int4 (*)[kDeferBuffer]>(qdyn));
}

// Mesh transport, pass 1 of 2: apply the pending update and drift every
// carrier that does not reach its cached wall within the step (the cache time
// drops by one step); carriers that do are queued, with their updated
// occupation, for k_mesh_events. Warps thus run the FP64 BVH work only on
// compacted event carriers.
template <bool kRta, bool kMixedState>
__global__ void __launch_bounds__(kTransportThreads) k_transport_mesh(const __grid_constant__ DevTables T, CarrierState S,
                                                                      CellArrays C, DevLedger* L) {
    constexpr bool kMixed = kMixedState;
    const int n = L->n_slots;
    const double dt = T.par.dt;
    // every streamed field of a slot in one memory round trip, and the next
    // slot's fields in flight while this one moves (each slot belongs to one
    // thread of the pass)
    struct Slot {
        bool live;
        uint32_t w;
        int c0, mirror;
        double occ0, ht;
        typename std::conditional<kMixed, float, double>::type p[3]; // FP32 offsets (mixed) or positions
    };
    auto load = [&](int i) {
        Slot s;
        const int ic = i < n ? i : 0;
        s.live = i < n && __ldcs(S.alive + ic);
        s.w = __ldcs(S.mode + ic);
        s.c0 = __ldcs(S.cell + ic);
        s.occ0 = __ldcs(S.occ + ic);
        s.ht = __ldcs(T.fac.hit_t + ic);
        s.mirror = __ldcs(T.fac.mirror + ic);
        if (kMixed) {
            s.p[0] = __ldcs(S.ox + ic);
            s.p[1] = __ldcs(S.oy + ic);
            s.p[2] = __ldcs(S.oz + ic);
        } else {
            s.p[0] = __ldcs(S.x + ic);
            s.p[1] = __ldcs(S.y + ic);
            s.p[2] = __ldcs(S.z + ic);
        }
        return s;
    };
    const int stride = gridDim.x * blockDim.x;
    int base = blockIdx.x * blockDim.x;
    Slot cur = load(base + threadIdx.x);
    for (; base < n; base += stride) {
        const int i = base + threadIdx.x;
        Slot next;
        if (base + stride < n) next = load(i + stride);
        bool defer = false;
        long long h = -1;
        double hocc = 0.0;
        if (cur.live) {
            const uint32_t w = cur.w;
            const int c0 = cur.c0;
            const double occ = apply_pending(T, C, c0, w, cur.occ0);
            const double ht = cur.ht;
            const double t_wall = dmul(ht, dt);
            if (!isfinite(t_wall) || t_wall > dt) {
                int c;
                if (kMixed) {
                    // FP32 flight in the frame of the home voxel, then the new cell
                    float v[3];
                    mesh_velocity32(T.fac, T.mat[w >> 28], w, cur.mirror, v);
                    const float dt32 = T.par.dt32;
                    float q[3] = {fmaf(v[0], dt32, cur.p[0]), fmaf(v[1], dt32, cur.p[1]), fmaf(v[2], dt32, cur.p[2])};
                    c = settle_mesh(T, cell_frame_of(T, c0), q);
                    __stcs(S.ox + i, q[0]);
                    __stcs(S.oy + i, q[1]);
                    __stcs(S.oz + i, q[2]);
                } else {
                    double v[3];
                    mesh_velocity(T.fac, T.mat[w >> 28], w, cur.mirror, v);
                    const double p[3] = {dadd(cur.p[0], dmul(v[0], dt)), dadd(cur.p[1], dmul(v[1], dt)),
                                         dadd(cur.p[2], dmul(v[2], dt))};
                    c = cell_at(T, p[0], p[1], p[2]);
                    __stcs(S.x + i, p[0]);
                    __stcs(S.y + i, p[1]);
                    __stcs(S.z + i, p[2]);
                }
                if (isfinite(ht)) __stcs(T.fac.hit_t + i, dadd(ht, -(dt / dt)));
                __stcs(S.occ + i, occ);
                __stcs(S.cell + i, c);
                h = bin_slot(T, C, L, i, c, w, occ);
                hocc = occ;
            } else {
                __stcs(S.occ + i, occ);
                defer = true;
            }
        }
        bin_warp<true, kRta>(C, h, hocc);
        queue_event(S, L, defer, i);
        cur = next;
    }
}

// Mesh transport, pass 2 of 2: the full flight of every queued carrier from
// the start of the step (occupation already updated), then its cell and bin.
template <bool kRta, bool kMixed>
__global__ void __launch_bounds__(kTransportThreads, 2) k_mesh_events(const __grid_constant__ DevTables T, CarrierState S,
                                                                   CellArrays C, DevLedger* L) {
    const uint32_t step = L->step_index;
    __shared__ BlockLedger bl;
    block_ledger_init(&bl);
    __syncthreads();
    const int nq = min(L->n_deferred, S.capacity);
    // each warp takes the next 32 queue entries when it is done with its own,
    // so walks of uneven length do not leave warps idle at the end
    const int lane = threadIdx.x & 31;
    for (;;) {
        int q0 = 0;
        if (lane == 0) q0 = atomicAdd(&L->event_head, 32);
        q0 = __shfl_sync(0xffffffffu, q0, 0);
        if (q0 >= nq) break;
        const int q = q0 + lane;
        if (q >= nq) continue;
        const int i = S.deferred[q].x;
        if (i < 0 || i >= S.capacity) {
            raise_error(L, kErrInvalidStatistics, i);
            continue;
        }
        uint32_t w = S.mode[i];
        double occ = S.occ[i];
        double p[3];
        if (kMixed) {
            // FP64 position of the FP32 offsets; the events run in FP64
            const float o[3] = {S.ox[i], S.oy[i], S.oz[i]};
            frame_point(T.dom, cell_frame_of(T, S.cell[i]), o, p);
        } else {
            p[0] = S.x[i];
            p[1] = S.y[i];
            p[2] = S.z[i];
        }
        const int mir0 = T.fac.mirror[i];
        int mir = mir0;
        MeshCache mc;
        mc.t = T.fac.hit_t[i];
        mc.loaded = mc.dirty = false;
        const bool alive = advance_carrier_mesh(T, L, &bl, i, p, w, mir, occ, mc, T.par.dt, kDrawTransport, step);
        if (mir != mir0) T.fac.mirror[i] = mir;
        mesh_cache_store(T.fac, i, mc);
        int c;
        if (kMixed) {
            float o[3];
            c = frame_offsets(T, p, o);
            S.ox[i] = o[0];
            S.oy[i] = o[1];
            S.oz[i] = o[2];
        } else {
            S.x[i] = p[0];
            S.y[i] = p[1];
            S.z[i] = p[2];
            c = cell_at(T, p[0], p[1], p[2]);
        }
        S.mode[i] = w;
        S.occ[i] = occ;
        if (!alive) {
            S.alive[i] = 0;
            continue;
        }
        S.cell[i] = c;
        bin_carrier(T, C, L, i, c, w, occ, kRta);
    }
    __syncthreads();
    block_ledger_flush(&bl, L);
}

// Wall events queued by the mixed transport pass: sample the wall with the
// draws of the queued event index, finish the flight (further walls inline),
// then settle and bin exactly as the transport pass would have.
template <bool kRta>
__device__ __forceinline__ void k_deferred_body(const DevTables& T, CarrierState S, CellArrays C, DevLedger* L, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const uint32_t step = L->step_index;
    __shared__ BlockLedger bl;
    block_ledger_init(&bl);
    __syncthreads();
    const int nq = min(L->n_deferred, S.capacity);
    for (int q = queue_first(vbx, vgx); q < nq; q += vgx * blockDim.x) {
        const int4 e = S.deferred[q];
        const int i = e.x;
        if (i < 0 || i >= S.capacity) {
            raise_error(L, kErrInvalidStatistics, i);
            continue;
        }
        float remaining = __int_as_float(e.y);
        int event = e.z, plane = e.w;
        uint32_t w = S.mode[i];
        double occ = S.occ[i];
        const Frame F = cell_frame(T.dom, S.cell[i]);
        float p[3] = {S.ox[i], S.oy[i], S.oz[i]};
        int end = kFlightDone;
        bool resumed = false;
        if (plane >= kDeferInterface && plane < kDeferInterface + kMaxMaterials)
            resumed = interface_step_mixed(T, L, &bl, i, plane - kDeferInterface, w, occ, event, kDrawTransport, step);
        else if (plane >= 0 && plane < 6)
            resumed = wall_sample_mixed(T, L, &bl, i, plane, w, occ, event, kDrawTransport, step);
        if (resumed) {
            ++event;
            int unused = -1;
            end = advance_mixed<false>(T, L, &bl, i, F, p, w, occ, remaining, event, unused, kDrawTransport, step);
        }
        const long long h = finish_mixed(T, S, C, L, i, F, p, w, occ, end != kFlightAbsorbed, ~w);
        if (h >= 0) bin_add(C, h, 1u, occ, fmax(1.0, occ), kRta);
    }
    __syncthreads();
    block_ledger_flush(&bl, L);
}

template <bool kRta>
__global__ void __launch_bounds__(kTransportThreads) k_deferred(const __grid_constant__ DevTables T, CarrierState S,
                                                                CellArrays C, DevLedger* L) {
    k_deferred_body<kRta>(T, S, C, L, blockIdx.x, gridDim.x);
}

// Bins of the current population (initial state or after carriers were replaced).
template <bool kRta>
__global__ void k_histogram(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C, DevLedger* L) {
    const int n = L->n_slots;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!S.alive[i]) continue;
        const uint32_t w = S.mode[i];
        bin_carrier(*Tp, C, L, i, S.cell[i], w, S.occ[i], kRta);
    }
}

// Cells (and FP32 offsets) of uploaded carriers, and the live count.
template <bool kMixed>
__global__ void k_init_cells(const DevTables* __restrict__ Tp, CarrierState S, DevLedger* L) {
    const DevDomain& D = Tp->dom;
    const int n = L->n_slots;
    unsigned long long live = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = cell_at(*Tp, S.x[i], S.y[i], S.z[i]);
        S.cell[i] = c;
        if (Tp->fac.mirror) Tp->fac.mirror[i] = -1;
        if (kMixed) {
            const Frame F = cell_frame_of(*Tp, c);
            S.ox[i] = static_cast<float>(S.x[i] - (D.lo[0] + F.i[0] * D.cell_size[0]));
            S.oy[i] = static_cast<float>(S.y[i] - (D.lo[1] + F.i[1] * D.cell_size[1]));
            S.oz[i] = static_cast<float>(S.z[i] - (D.lo[2] + F.i[2] * D.cell_size[2]));
        }
        live += S.alive[i] ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(reinterpret_cast<unsigned long long*>(&L->particle_count), live);
}

// Carriers straight from registered host memory (one pass over the link, no
// device staging): cell, FP32 offsets or FP64 positions, occupation, mode, alive.
template <bool kMixed>
__global__ void k_ingest(const __grid_constant__ DevTables T, CarrierState S, DevLedger* L, HostCarriers H) {
    const DevDomain& D = T.dom;
    const int n = L->n_slots;
    unsigned long long live = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = H.x[i], y = H.y[i], z = H.z[i];
        const int c = cell_at(T, x, y, z);
        S.cell[i] = c;
        if (T.fac.mirror) T.fac.mirror[i] = -1;
        if (kMixed) {
            const Frame F = cell_frame_of(T, c);
            S.ox[i] = static_cast<float>(x - (D.lo[0] + F.i[0] * D.cell_size[0]));
            S.oy[i] = static_cast<float>(y - (D.lo[1] + F.i[1] * D.cell_size[1]));
            S.oz[i] = static_cast<float>(z - (D.lo[2] + F.i[2] * D.cell_size[2]));
        }
        // FP64 positions (the mixed state's staging): mesh wall caches are traced from them
        S.x[i] = x;
        S.y[i] = y;
        S.z[i] = z;
        S.occ[i] = H.occ[i];
        S.mode[i] = H.mode[i];
        const uint8_t a = H.alive ? H.alive[i] : uint8_t(1);
        S.alive[i] = a;
        live += a ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if ((threadIdx.x & 31) == 0 && live) atomicAdd(reinterpret_cast<unsigned long long*>(&L->particle_count), live);
}

// A replaced population continuing the run: new slot range and live count;
// totals, the clock and the previous reservoir counts stay.
__global__ void k_ledger_replace(DevLedger* L, int n) {
    L->n_slots = n;
    L->n_holes = 0;
    L->n_inject = 0;
    L->n_deferred = 0;
    L->particle_count = 0;
    L->error_code = 0;
    L->error_slot = 0;
}

// Absolute FP64 positions of the mixed state into the staging arrays.
__global__ void k_positions_out(const DevTables* __restrict__ Tp, CarrierState S, const DevLedger* L) {
    const DevDomain& D = Tp->dom;
    const int n = L->n_slots;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Frame F = cell_frame_of(*Tp, S.cell[i]);
        S.x[i] = D.lo[0] + F.i[0] * D.cell_size[0] + static_cast<double>(S.ox[i]);
        S.y[i] = D.lo[1] + F.i[1] * D.cell_size[1] + static_cast<double>(S.oy[i]);
        S.z[i] = D.lo[2] + F.i[2] * D.cell_size[2] + static_cast<double>(S.oz[i]);
    }
}

// ------------------------------------------------------------ injection
// Free slots in ascending order: per-block dead counts, one-block scan, write.
constexpr int kHoleBlock = 1024;

__device__ __forceinline__ void k_dead_count_body(CarrierState S, const DevLedger* L, int* block_dead, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const int n = L->n_slots;
    const int i = vbx * kHoleBlock + threadIdx.x;
    const int dead = (i < n && !S.alive[i]) ? 1 : 0;
    const int c = __syncthreads_count(dead);
    if (threadIdx.x == 0) block_dead[vbx] = c;
}

__global__ void __launch_bounds__(kHoleBlock) k_dead_count(CarrierState S, const DevLedger* L, int* block_dead) {
    k_dead_count_body(S, L, block_dead, blockIdx.x, gridDim.x);
}

// Single block: exclusive scan of block counts and emission counts per reservoir
// (src/solver/ReservoirInjector.cpp:281-284, src/solver/ReservoirSampler.cpp:117-124).
__device__ __forceinline__ void k_inject_prepare_body(const DevTables* __restrict__ Tp, DevLedger* L, int* block_dead, int nblocks, int capacity, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const uint32_t step = L->step_index;
    __shared__ int carry;
    __shared__ int warp_sums[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nblocks ? block_dead[i] : 0;
        int x = v;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            int s = warp_sums[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            warp_sums[lane] = s;
        }
        __syncthreads();
        const int excl = carry + (wid ? warp_sums[wid - 1] : 0) + x - v;
        if (i < nblocks) block_dead[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const DevTables& T = *Tp;
        L->n_holes = carry;
        int total = 0;
        for (int r = 0; r < T.par.n_reservoirs; ++r) {
            const DevReservoir& R = T.res[r];
            int count;
            if (T.par.one_to_one) {
                count = static_cast<int>(L->previous_res[r]);
            } else {
                const int base = static_cast<int>(floor(R.expected));
                const double frac = R.expected - base;
                const Uniform2 u = uniform2(T.par.seed, static_cast<uint32_t>(r), step, kDrawInjectCount, 0, 0);
                count = base + ((frac > 0.0 && u.a < frac) ? 1 : 0);
            }
            if (count > 0 && !(R.cdf[R.n_cdf - 1] > 0.0)) {
                raise_error(L, kErrZeroFluxReservoir, r);
                count = 0;
            }
            L->inject_count[r] = count;
            L->inject_offset[r] = total;
            total += count;
        }
        L->inject_offset[T.par.n_reservoirs] = total;
        L->n_inject = total;
        const int extra = total - carry;
        const long long new_slots = static_cast<long long>(L->n_slots) + (extra > 0 ? extra : 0);
        if (new_slots > capacity) {
            raise_error(L, kErrCapacity, static_cast<int>(new_slots > 0x7fffffff ? 0x7fffffff : new_slots));
            L->n_inject = 0;
        }
    }
}

__global__ void __launch_bounds__(1024) k_inject_prepare(const DevTables* __restrict__ Tp, DevLedger* L,
                                                         int* block_dead, int nblocks, int capacity) {
    k_inject_prepare_body(Tp, L, block_dead, nblocks, capacity, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void k_dead_write_body(CarrierState S, const DevLedger* L, const int* block_off, int* holes, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    __shared__ int warp_base[32];
    const int n = L->n_slots;
    const int need = L->n_inject;
    const int i = vbx * kHoleBlock + threadIdx.x;
    const bool dead = i < n && !S.alive[i];
    const unsigned mask = __ballot_sync(0xffffffffu, dead);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_base[wid] = __popc(mask);
    __syncthreads();
    if (threadIdx.x < 32) {
        int x = warp_base[threadIdx.x];
        const int v = x;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (threadIdx.x >= o) x += y;
        }
        warp_base[threadIdx.x] = x - v;
    }
    __syncthreads();
    if (dead) {
        const int rank = block_off[vbx] + warp_base[wid] + __popc(mask & ((1u << lane) - 1u));
        if (rank < need) holes[rank] = i;
    }
}

__global__ void __launch_bounds__(kHoleBlock) k_dead_write(CarrierState S, const DevLedger* L, const int* block_off,
                                                           int* holes) {
    k_dead_write_body(S, L, block_off, holes, blockIdx.x, gridDim.x);
}

template <bool kMixed, bool kRta, bool kMesh = false>
__device__ __forceinline__ void k_inject_body(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C, DevLedger* L, const int* holes, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const uint32_t step = L->step_index;
    __shared__ BlockLedger bl;
    block_ledger_init(&bl);
    __syncthreads();
    const DevTables& T = *Tp;
    const DevParams& P = T.par;
    const int ni = L->n_inject;
    const int nh = L->n_holes;
    const int n_old = L->n_slots;
    for (int j = vbx * blockDim.x + threadIdx.x; j < ni; j += vgx * blockDim.x) {
        int r = 0;
        while (r + 1 < P.n_reservoirs && j >= L->inject_offset[r + 1]) ++r;
        const int e = j - L->inject_offset[r];
        const DevReservoir& R = T.res[r];
        const DevMaterial& M = T.mat[R.material];
        const Uniform2 d0 = uniform2(P.seed, static_cast<uint32_t>(e), step, kDrawInject, static_cast<uint32_t>(r), 0);
        const Uniform2 d1 = uniform2(P.seed, static_cast<uint32_t>(e), step, kDrawInject, static_cast<uint32_t>(r), 1);
        const Uniform2 d2 = uniform2(P.seed, static_cast<uint32_t>(e), step, kDrawInject, static_cast<uint32_t>(r), 2);
        const int m = alias_draw(R.alias, R.n_cdf, d0.a); // emission mode, O(1)
        const double temit = P.dt * d0.b;
        // area-weighted triangle of the facet: first running sum above u * total
        const double target = dmul(d1.a, R.tri_cum[R.n_tri - 1]);
        int lo_t = 0, hi_t = R.n_tri - 1;
        while (lo_t < hi_t) {
            const int mid = (lo_t + hi_t) >> 1;
            if (R.tri_cum[mid] > target) hi_t = mid;
            else lo_t = mid + 1;
        }
        const double* tv = R.tri + 9 * lo_t;
        const double sr1 = sqrt(d1.b);
        const double w0 = 1.0 - sr1, w1 = sr1 * (1.0 - d2.a), w2 = sr1 * d2.a;
        double p[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = dadd(dadd(dmul(w0, tv[a]), dmul(w1, tv[3 + a])), dmul(w2, tv[6 + a]));
        double v[3] = {M.vel[3 * m], M.vel[3 * m + 1], M.vel[3 * m + 2]};
        uint32_t signs = 0;
        if (dadd(dadd(dmul(v[0], R.normal[0]), dmul(v[1], R.normal[1])), dmul(v[2], R.normal[2])) > 0.0) {
            if (P.conservative) raise_error(L, kErrOutwardReservoirMode, j);
            for (int a = 0; a < 3; ++a) v[a] = -v[a];
            signs = 7u;
        }
        const double s = M.push[m];
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = dadd(p[a], dmul(v[a], s));
        double occ = R.occ[m];
        uint32_t w = static_cast<uint32_t>(m) | (signs << 24) | (static_cast<uint32_t>(R.material) << 28);
        const int slot = j < nh ? holes[j] : n_old + (j - nh);
        atomicAdd(&bl.injected_ev, dmul(dmul(M.hw[m], occ - M.nbg[m]), M.energy_weight));
        const double remain = P.dt - temit;
        bool alive = true;
        int c;
        if (kMesh) {
            int mir = -1;
            MeshCache mc;
            mesh_refresh(T, L, &bl, slot, p, v, mc); // src/MonteCarloSolver.cpp:318-327
            if (remain > 1e-14)
                alive = advance_carrier_mesh(T, L, &bl, slot, p, w, mir, occ, mc, remain, kDrawInjected, step);
            T.fac.mirror[slot] = mir;
            mesh_cache_store(T.fac, slot, mc);
            if (kMixed) {
                float o[3];
                c = frame_offsets(T, p, o);
                S.ox[slot] = o[0];
                S.oy[slot] = o[1];
                S.oz[slot] = o[2];
            } else {
                c = cell_at(T, p[0], p[1], p[2]);
                S.x[slot] = p[0];
                S.y[slot] = p[1];
                S.z[slot] = p[2];
            }
        } else if (kMixed) {
            c = grid_index(T.dom, p[0], p[1], p[2]);
            const Frame F = cell_frame(T.dom, c);
            float q[3];
            for (int a = 0; a < 3; ++a) q[a] = static_cast<float>(p[a] - (T.dom.lo[a] + F.i[a] * T.dom.cell_size[a]));
            if (remain > 1e-14) {
                float rem = static_cast<float>(remain);
                int event = 0, plane = -1;
                alive = advance_mixed<false>(T, L, &bl, slot, F, q, w, occ, rem, event, plane, kDrawInjected, step) !=
                        kFlightAbsorbed;
            }
            c = settle_layer(T, C, F, q, static_cast<int>(w >> 28));
            S.ox[slot] = q[0];
            S.oy[slot] = q[1];
            S.oz[slot] = q[2];
        } else {
            if (remain > 1e-14) alive = advance_carrier(T, L, &bl, slot, p, w, occ, remain, kDrawInjected, step);
            c = grid_index(T.dom, p[0], p[1], p[2]);
            S.x[slot] = p[0];
            S.y[slot] = p[1];
            S.z[slot] = p[2];
        }
        S.mode[slot] = w;
        S.occ[slot] = occ;
        S.alive[slot] = alive ? 1 : 0;
        S.cell[slot] = alive ? c : 0;
        if (alive) bin_carrier(T, C, L, slot, c, w, occ, kRta);
    }
    __syncthreads();
    block_ledger_flush(&bl, L);
}

template <bool kMixed, bool kRta, bool kMesh = false>
__global__ void __launch_bounds__(256) k_inject(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C,
                                                DevLedger* L, const int* holes) {
    k_inject_body<kMixed, kRta, kMesh>(Tp, S, C, L, holes, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void k_inject_finish_body(DevLedger* L, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const int extra = L->n_inject - L->n_holes;
    if (extra > 0) L->n_slots += extra;
    L->step_injected += static_cast<unsigned long long>(L->n_inject);
}

__global__ void k_inject_finish(DevLedger* L) {
    k_inject_finish_body(L, blockIdx.x, gridDim.x);
}

// Escaped-carrier check (src/solver/TransportOperator.cpp:364-402).
// Position of carrier i (the mixed state from its cell frame and FP32 offsets).
template <bool kMixed>
__device__ __forceinline__ void contain_position(const DevTables& T, const CarrierState& S, int i, double p[3]) {
    if (kMixed) {
        const DevDomain& D = T.dom;
        const Frame F = cell_frame_of(T, S.cell[i]);
        p[0] = D.lo[0] + F.i[0] * D.cell_size[0] + S.ox[i];
        p[1] = D.lo[1] + F.i[1] * D.cell_size[1] + S.oy[i];
        p[2] = D.lo[2] + F.i[2] * D.cell_size[2] + S.oz[i];
    } else {
        p[0] = S.x[i];
        p[1] = S.y[i];
        p[2] = S.z[i];
    }
}

// Containment check (src/solver/TransportOperator.cpp:364-402), first part:
// the bounds test of every live carrier; mesh carriers outside the interior
// voxels go to `queue` for the membership test (k_contain_cast), so that the
// ray casts run in full warps.
template <bool kMixed>
__global__ void k_contain_screen(const DevTables* __restrict__ Tp, CarrierState S, DevLedger* L, int* queue,
                                 int* count) {
    const DevDomain& D = Tp->dom;
    const int n = L->n_slots;
    const int lane = threadIdx.x & 31;
    // FP32 offsets carry ~1e-7 relative rounding of the cell size
    const double t = kMixed ? 1e-5 * D.scale : 1e-10 * D.scale;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + threadIdx.x;
        bool cast = false;
        if (i < n && S.alive[i]) {
            double p[3];
            contain_position<kMixed>(*Tp, S, i, p);
            bool outside = false;
            for (int a = 0; a < 3; ++a) outside = outside || !isfinite(p[a]) || p[a] < D.lo[a] - t || p[a] > D.hi[a] + t;
            if (outside) raise_error(L, kErrEscaped, i);
            else cast = Tp->fac.n > 0 && !mesh_voxel_interior(Tp->fac, D, p);
        }
        const unsigned want = __ballot_sync(0xffffffffu, cast);
        if (want) {
            int first = 0;
            if (lane == 0) first = atomicAdd(count, __popc(want));
            first = __shfl_sync(0xffffffffu, first, 0);
            if (cast) queue[first + __popc(want & ((1u << lane) - 1u))] = i;
        }
    }
}

// Second part: membership of the queued carriers (SurfaceMesh::contains_point).
template <bool kMixed>
__global__ void k_contain_cast(const DevTables* __restrict__ Tp, CarrierState S, DevLedger* L, const int* queue,
                               const int* count) {
    const DevDomain& D = Tp->dom;
    const int n = *count;
    const double t = kMixed ? 1e-5 * D.scale : 1e-10 * D.scale;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int i = queue[q];
        double p[3];
        contain_position<kMixed>(*Tp, S, i, p);
        const int in = mesh_contains(Tp->fac, p);
        if (in < 0) raise_error(L, kErrInvalidStatistics, i);
        bool outside = in == 0;
        // the mixed state may sit outside a wall by its FP32 rounding:
        // escaped only when farther from the surface than that
        if (kMixed && outside) outside = !mesh_near_surface(Tp->fac, p, t);
        if (outside) raise_error(L, kErrEscaped, i);
    }
}

// Sums of x[0..2] over the lanes of `peers` (the lanes that hold the same
// key), left in the lowest lane of each group: a tree over every group at
// once in at most five rounds (reduce-by-key of warp-aggregated adds).
__device__ __forceinline__ void reduce_peers3(unsigned peers, double x[3]) {
    const int lane = threadIdx.x & 31;
    unsigned rel = __popc(peers & ((1u << lane) - 1u)); // rank in the group
    unsigned above = peers & (0xfffffffeu << lane);      // group lanes above this one
    while (__any_sync(0xffffffffu, above != 0u)) {
        const int next = above ? __ffs(above) - 1 : lane;
        double t[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) t[a] = __shfl_sync(0xffffffffu, x[a], next);
        if (above) {
#pragma unroll
            for (int a = 0; a < 3; ++a) x[a] = dadd(x[a], t[a]);
        }
        // odd ranks have been read by their lower neighbour: out of every group
        above &= ~__ballot_sync(0xffffffffu, rel & 1u);
        rel >>= 1;
    }
}

// Heat-flux tally q_c = sum v e w (src/solver/GridStatistics.cpp:269-347) with the
// end-of-step occupation n = alpha n + beta - (second drive half). Each thread
// walks kFluxRun consecutive slots and keeps one running sum per component
// while the cell stays the same -- sorted carriers come in runs of one cell.
// A run ends when the cell changes or the slots end; on every step in which
// some lane of the warp ends a run, the ending runs are summed by cell across
// the warp (reduce_peers3) and one lane per cell adds the sum to the target:
// `target` 2 one copy of the cell sums per warp in shared memory (plain adds:
// the adding lanes hold distinct cells), 1 one copy per block (shared
// atomics), 0 the global sums. Sorted carriers thus cost the pending update,
// the drive half and three fused multiply-adds per carrier plus a reduction
// every few slots; unsorted ones (one run per carrier) one reduction per slot.
constexpr int kFluxRun = 8;

__global__ void __launch_bounds__(256) k_flux(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C,
                                              const DevLedger* L, int target) {
    extern __shared__ double sq[];
    const DevTables& T = *Tp;
    const int nq = 3 * C.ncells;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (target > 0)
        for (int k = threadIdx.x; k < (target == 2 ? nwarps : 1) * nq; k += blockDim.x) sq[k] = 0.0;
    __syncthreads();
    double* dst = target == 2 ? sq + warp * nq : (target == 1 ? sq : C.flux);
    // every lane calls: lanes with `ending` hand in their run (cell `key`, sums acc)
    auto hand_in = [&](bool ending, int key, double a0, double a1, double a2) {
        if (!__any_sync(0xffffffffu, ending)) return;
        const unsigned peers = __match_any_sync(0xffffffffu, ending ? key : -1);
        double v[3] = {ending ? a0 : 0.0, ending ? a1 : 0.0, ending ? a2 : 0.0};
        reduce_peers3(peers, v);
        if (ending && lane == __ffs(peers) - 1) {
            if (target == 2) {
#pragma unroll
                for (int a = 0; a < 3; ++a) dst[3 * key + a] = dadd(dst[3 * key + a], v[a]);
            } else {
#pragma unroll
                for (int a = 0; a < 3; ++a) atomicAdd(dst + 3 * key + a, v[a]);
            }
        }
        if (target == 2) __syncwarp();
    };
    const int n = L->n_slots;
    const int per_block = blockDim.x * kFluxRun;
    for (int base = blockIdx.x * per_block; base < n; base += gridDim.x * per_block) { // block-uniform
        const int i0 = base + threadIdx.x * kFluxRun;
        int cur = -1;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int k = 0; k < kFluxRun; ++k) { // warp-uniform trip count: every lane reaches hand_in
            const int i = i0 + k;
            const bool live = i < n && S.alive[i];
            const uint32_t w = live ? S.mode[i] : 0u;
            const int c = live ? S.cell[i] : -1;
            const bool change = live && c != cur;
            hand_in(change && cur >= 0, cur, acc[0], acc[1], acc[2]);
            if (change) {
                cur = c;
                acc[0] = acc[1] = acc[2] = 0.0;
            }
            if (!live) continue;
            const DevMaterial& M = T.mat[w >> 28];
            const int ai = static_cast<int>(w & 0x00FFFFFFu);
            double occ = apply_pending(T, C, c, w, S.occ[i]) - drive_half(T, C, M, c, ai);
            if (C.src_next) occ -= C.src_next[static_cast<size_t>(c) * C.hist_modes + bin_of(M, ai)];
            const double x = occ - M.nbg[ai];
            if (T.fac.mirror) {
                double v[3];
                mesh_velocity(T.fac, M, w, T.fac.mirror[i], v);
                const double e = dmul(dmul(M.hw[ai], x), M.energy_weight);
#pragma unroll
                for (int a = 0; a < 3; ++a) acc[a] = fma(v[a], e, acc[a]);
            } else {
                // v hbar omega w per mode: sign flips on the bits
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const double cv = __ldg(M.flux_vel + 3 * ai + a);
                    const double cs = __hiloint2double(__double2hiint(cv) ^ static_cast<int>(((w >> (24 + a)) & 1u) << 31),
                                                       __double2loint(cv));
                    acc[a] = fma(cs, x, acc[a]);
                }
            }
        }
        hand_in(cur >= 0, cur, acc[0], acc[1], acc[2]);
    }
    __syncthreads();
    if (target > 0)
        for (int k = threadIdx.x; k < nq; k += blockDim.x) {
            double sum = 0.0;
            for (int q = 0; q < (target == 2 ? nwarps : 1); ++q) sum = dadd(sum, sq[q * nq + k]);
            if (sum != 0.0) atomicAdd(C.flux + k, sum);
        }
}

// Apply the pending update to the stored occupations, optionally leaving the
// next step's first drive half pending; then reset the table.
__global__ void k_apply_pending(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C, const DevLedger* L,
                                int subtract_drive) {
    const DevTables& T = *Tp;
    const int n = L->n_slots;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!S.alive[i]) continue;
        const uint32_t w = S.mode[i];
        const int ai = static_cast<int>(w & 0x00FFFFFFu);
        const int c = S.cell[i];
        double occ = apply_pending(T, C, c, w, S.occ[i]);
        if (subtract_drive) {
            occ -= drive_half(T, C, T.mat[w >> 28], c, ai);
            if (C.src_next) occ -= C.src_next[static_cast<size_t>(c) * C.hist_modes + bin_of(T.mat[w >> 28], ai)];
        }
        S.occ[i] = occ;
    }
}

__global__ void k_reset_pending(const DevTables* __restrict__ Tp, CellArrays C, int keep_drive) {
    const DevTables& T = *Tp;
    const size_t total = static_cast<size_t>(C.ncells) * C.hist_modes;
    for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < total;
         k += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const int c = static_cast<int>(k / C.hist_modes);
        const int m = static_cast<int>(k % C.hist_modes);
        const DevMaterial& M = T.mat[C.cell_material[c]];
        double D = (keep_drive && m < M.n_active) ? drive_half(T, C, M, c, m) : 0.0;
        if (keep_drive && C.src_next) D += C.src_next[k];
        else if (C.src_next) C.src_next[k] = 0.0;
        C.ab[k] = make_double2(1.0, D);
    }
}

// ----------------------------------------------------------- launchers
template <bool kMixed, bool kRta>
void launch_transport_pass(const LaunchCtx& x, dim3 g) {
    if (kMixed && x.transport_pipe) {
        const dim3 gp(x.pipe_grid);
        if (x.tally_agg) k_transport_pipe<kRta, true><<<gp, kPipeTile, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        else k_transport_pipe<kRta, false><<<gp, kPipeTile, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        return;
    }
    const int threads = x.transport_block;
    const size_t sh = kMixed ? static_cast<size_t>(threads / 32) * kDeferBuffer * sizeof(int4) : 0;
    if (x.tally_agg) k_transport<kMixed, kRta, true><<<g, threads, sh, x.stream>>>(*x.Th, x.S, x.C, x.L);
    else k_transport<kMixed, kRta, false><<<g, threads, sh, x.stream>>>(*x.Th, x.S, x.C, x.L);
}

int launch_transport(const LaunchCtx& x, bool mixed, bool rta) {
    if (x.transport_block != 128 && x.transport_block != 256 && x.transport_block != 512)
        throw std::invalid_argument("transport_block must be 128, 256 or 512 threads");
    const dim3 g(x.grid_blocks), b(kTransportThreads);
    if (mixed && !x.mesh) {
        // the carrier pass at the configured block size; the deferred wall events at 256
        const dim3 gp(x.transport_grid);
        // deferred wall events: two resident CTAs per SM (93 registers), one wave
        const dim3 ge(2 * x.event_grid);
        if (rta) {
            launch_transport_pass<true, true>(x, gp);
            k_deferred<true><<<ge, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        } else {
            launch_transport_pass<true, false>(x, gp);
            k_deferred<false><<<ge, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        }
        return 2;
    }
    if (x.mesh) {
        if (mixed && rta) {
            k_transport_mesh<true, true><<<g, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
            k_mesh_events<true, true><<<dim3(2 * x.event_grid), b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        } else if (mixed) {
            k_transport_mesh<false, true><<<g, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
            k_mesh_events<false, true><<<dim3(2 * x.event_grid), b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        } else if (rta) {
            k_transport_mesh<true, false><<<g, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
            k_mesh_events<true, false><<<dim3(2 * x.event_grid), b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        } else {
            k_transport_mesh<false, false><<<g, b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
            k_mesh_events<false, false><<<dim3(2 * x.event_grid), b, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
        }
        return 2;
    }
    if (rta) launch_transport_pass<false, true>(x, dim3(x.transport_grid));
    else launch_transport_pass<false, false>(x, dim3(x.transport_grid));
    // wall events (and, layered, plane crossings) queued by the pass
    // two resident CTAs per SM (80 registers), one wave
    const dim3 ge(2 * x.event_grid);
    if (rta) k_box_events<true><<<ge, 256, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
    else k_box_events<false><<<ge, 256, 0, x.stream>>>(*x.Th, x.S, x.C, x.L);
    return 2;
}

void launch_histogram(const LaunchCtx& x, bool rta) {
    if (rta) k_histogram<true><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.C, x.L);
    else k_histogram<false><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.C, x.L);
}

void launch_init_cells(const LaunchCtx& x, bool mixed) {
    if (mixed) k_init_cells<true><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.L);
    else k_init_cells<false><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.L);
}

void launch_ingest(const LaunchCtx& x, bool mixed, const HostCarriers& h) {
    if (mixed) k_ingest<true><<<x.grid_blocks, 256, 0, x.stream>>>(*x.Th, x.S, x.L, h);
    else k_ingest<false><<<x.grid_blocks, 256, 0, x.stream>>>(*x.Th, x.S, x.L, h);
}

void launch_ledger_replace(const LaunchCtx& x, int n) { k_ledger_replace<<<1, 1, 0, x.stream>>>(x.L, n); }

// Initial positions in a mesh domain without a volume decomposition, the
// ray-cast branch of initial_carriers (src/geometry/SurfaceSampling.cpp:114-121):
// uniform points of the bounding box kept when the +x ray cast finds them
// inside, at most 200 trials, with the host's counter-based draws and FP64
// operation order. x = NaN: the ray cast overflowed its hit list (the host
// repeats that carrier); x = +inf: no accepted point.
__global__ void k_mesh_initial_positions(const __grid_constant__ DevTables T, int n, uint64_t seed, double3 lo,
                                         double3 hi, double* xyz) {
    const double ex = dadd(hi.x, -lo.x), ey = dadd(hi.y, -lo.y), ez = dadd(hi.z, -lo.z);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int r = 0;
        double p[3] = {0.0, 0.0, 0.0};
        for (uint32_t trial = 0; trial < 200u && r == 0; ++trial) {
            const Uniform2 a = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial, 0);
            const Uniform2 b = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial, 1);
            p[0] = dadd(lo.x, dmul(ex, a.a));
            p[1] = dadd(lo.y, dmul(ey, a.b));
            p[2] = dadd(lo.z, dmul(ez, b.a));
            r = mesh_ray_cast_inside(T.fac, p);
        }
        double* o = xyz + 3 * static_cast<size_t>(i);
        o[0] = r > 0 ? p[0] : (r < 0 ? __longlong_as_double(0x7ff8000000000000LL) : INFINITY);
        o[1] = p[1];
        o[2] = p[2];
    }
}

void launch_mesh_initial_positions(const LaunchCtx& x, int n, uint64_t seed, const double lo[3], const double hi[3],
                                   double* xyz) {
    const int g = std::max(1, std::min(x.grid_blocks, (n + 127) / 128));
    k_mesh_initial_positions<<<g, 128, 0, x.stream>>>(*x.Th, n, seed, make_double3(lo[0], lo[1], lo[2]),
                                                       make_double3(hi[0], hi[1], hi[2]), xyz);
}

int launch_mesh_cache_init(const LaunchCtx& x, bool mixed) {
    if (!x.mesh) return 0;
    if (mixed) k_mesh_cache_init<true><<<x.grid_blocks, 128, 0, x.stream>>>(*x.Th, x.S, x.L);
    else k_mesh_cache_init<false><<<x.grid_blocks, 128, 0, x.stream>>>(*x.Th, x.S, x.L);
    return 1;
}

void launch_positions_out(const LaunchCtx& x) {
    k_positions_out<<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.L);
}

int launch_inject(const LaunchCtx& x, bool mixed, bool rta, int* holes, int* block_dead, int capacity) {
    const int nb = (capacity + kHoleBlock - 1) / kHoleBlock;
    k_dead_count<<<nb, kHoleBlock, 0, x.stream>>>(x.S, x.L, block_dead);
    k_inject_prepare<<<1, 1024, 0, x.stream>>>(x.T, x.L, block_dead, nb, capacity);
    k_dead_write<<<nb, kHoleBlock, 0, x.stream>>>(x.S, x.L, block_dead, holes);
    const dim3 g(x.grid_blocks), b(256);
    if (mixed && x.mesh) {
        if (rta) k_inject<true, true, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
        else k_inject<true, false, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
    } else if (mixed) {
        if (rta) k_inject<true, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
        else k_inject<true, false><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
    } else if (x.mesh) {
        if (rta) k_inject<false, true, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
        else k_inject<false, false, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
    } else {
        if (rta) k_inject<false, true><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
        else k_inject<false, false><<<g, b, 0, x.stream>>>(x.T, x.S, x.C, x.L, holes);
    }
    k_inject_finish<<<1, 1, 0, x.stream>>>(x.L);
    return 5;
}

int launch_containment(const LaunchCtx& x, bool mixed, int* queue, int* count) {
    cudaMemsetAsync(count, 0, sizeof(int), x.stream);
    const dim3 ge(2 * x.event_grid);
    if (mixed) {
        k_contain_screen<true><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.L, queue, count);
        if (x.mesh) k_contain_cast<true><<<ge, kTransportThreads, 0, x.stream>>>(x.T, x.S, x.L, queue, count);
    } else {
        k_contain_screen<false><<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.L, queue, count);
        if (x.mesh) k_contain_cast<false><<<ge, kTransportThreads, 0, x.stream>>>(x.T, x.S, x.L, queue, count);
    }
    return x.mesh ? 2 : 1;
}

void launch_flux(const LaunchCtx& x, bool /*mixed*/) {
    const size_t per_copy = 3 * sizeof(double) * static_cast<size_t>(x.C.ncells);
    // a private copy per warp (8 per CTA) up to 48 KB, else one per CTA up to
    // 32 KB, else the global sums
    const int target = 8 * per_copy <= 49152 ? 2 : (per_copy <= 32768 ? 1 : 0);
    const size_t sh = target == 2 ? 8 * per_copy : (target == 1 ? per_copy : 0);
    k_flux<<<x.grid_blocks, 256, sh, x.stream>>>(x.T, x.S, x.C, x.L, target);
}

void launch_apply_pending(const LaunchCtx& x, bool subtract_drive) {
    k_apply_pending<<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.S, x.C, x.L, subtract_drive ? 1 : 0);
    k_reset_pending<<<x.grid_blocks, 256, 0, x.stream>>>(x.T, x.C, subtract_drive ? 1 : 0);
}

} // namespace phmc

// ------------------------------------------------- fused batch launches
// Persistent CTAs walk the virtual CTAs of all instances; each virtual CTA
// runs the single-instance kernel body for its instance with the instance's
// CTA index and count. The carrier kernels keep the instance's tables in
// shared memory (copied when the instance changes).
namespace phmc {

struct SharedTables {
    __align__(16) unsigned char raw[sizeof(DevTables)];
    int owner;
};

__device__ __forceinline__ const DevTables& stage_tables(SharedTables& st, const BatchDesc& D, int inst) {
    if (st.owner != inst) { // block-uniform
        __syncthreads();
        const unsigned* src = reinterpret_cast<const unsigned*>(D.tables[inst]);
        unsigned* dst = reinterpret_cast<unsigned*>(st.raw);
        for (int k = threadIdx.x; k < static_cast<int>(sizeof(DevTables) / 4); k += blockDim.x) dst[k] = src[k];
        __syncthreads();
        if (threadIdx.x == 0) st.owner = inst;
        __syncthreads();
    }
    return *reinterpret_cast<const DevTables*>(st.raw);
}

template <bool kMixed, bool kRta>
__global__ void __launch_bounds__(kTransportThreads) kf_transport(const BatchDesc D) {
    __shared__ SharedTables st;
    __shared__ int4 qbuf[kMixed ? kTransportThreads / 32 : 1][kDeferBuffer];
    if (threadIdx.x == 0) st.owner = -1;
    __syncthreads();
    for (int vb = blockIdx.x; vb < D.total_carrier_blocks; vb += gridDim.x) {
        const int i = batch_find(D.carrier_block, D.n, vb);
        const int b0 = D.carrier_block[i];
        const DevTables& T = stage_tables(st, D, i);
        k_transport_body<kMixed, kRta, false>(T, D.states[i], D.cells[i], D.ledgers[i], vb - b0,
                                              D.carrier_block[i + 1] - b0, qbuf);
        __syncthreads();
    }
}

template <bool kRta>
__global__ void __launch_bounds__(kTransportThreads) kf_box_events(const BatchDesc D) {
    __shared__ SharedTables st;
    if (threadIdx.x == 0) st.owner = -1;
    __syncthreads();
    for (int vb = blockIdx.x; vb < D.total_carrier_blocks; vb += gridDim.x) {
        const int i = batch_find(D.carrier_block, D.n, vb);
        const int b0 = D.carrier_block[i];
        const DevTables& T = stage_tables(st, D, i);
        k_box_events_body<kRta>(T, D.states[i], D.cells[i], D.ledgers[i], vb - b0, D.carrier_block[i + 1] - b0);
        __syncthreads();
    }
}
template <bool kRta>
__global__ void __launch_bounds__(kTransportThreads) kf_deferred(const BatchDesc D) {
    __shared__ SharedTables st;
    if (threadIdx.x == 0) st.owner = -1;
    __syncthreads();
    for (int vb = blockIdx.x; vb < D.total_carrier_blocks; vb += gridDim.x) {
        const int i = batch_find(D.carrier_block, D.n, vb);
        const int b0 = D.carrier_block[i];
        const DevTables& T = stage_tables(st, D, i);
        k_deferred_body<kRta>(T, D.states[i], D.cells[i], D.ledgers[i], vb - b0, D.carrier_block[i + 1] - b0);
        __syncthreads();
    }
}

// Hole scans of the batch: one warp per 1024-slot hole block, lane l covering
// slots [32 l, 32 l + 32) of it, so ranks still follow the slot order of
// k_dead_count / k_dead_write.
__device__ __forceinline__ unsigned dead_bits(const uint8_t* __restrict__ alive, int k0, int n) {
    unsigned m = 0;
    if (k0 + 32 <= n) { // k0 is a multiple of 32: both 16-byte loads are aligned and in bounds
        const uint4* p = reinterpret_cast<const uint4*>(alive + k0);
        const uint4 a = p[0], b = p[1];
        const unsigned w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (((w[q] >> (8 * t)) & 0xFFu) == 0u) m |= 1u << (4 * q + t);
    } else {
        for (int t = 0; t < 32 && k0 + t < n; ++t)
            if (!alive[k0 + t]) m |= 1u << t;
    }
    return m;
}

__global__ void __launch_bounds__(256) kf_dead_count(const BatchDesc D) {
    const int lane = threadIdx.x & 31;
    const int nw = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int vb = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5); vb < D.total_hole_blocks; vb += nw) {
        const int i = batch_find(D.hole_block, D.n, vb); // warp-uniform
        const int b = vb - D.hole_block[i];
        const int n = D.ledgers[i]->n_slots;
        int c = __popc(dead_bits(D.states[i].alive, b * kHoleBlock + 32 * lane, n));
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) D.hole_counts[i][b] = c;
    }
}

__global__ void __launch_bounds__(1024) kf_inject_prepare(const BatchDesc D) {
    const int i = blockIdx.x;
    k_inject_prepare_body(D.tables[i], D.ledgers[i], D.hole_counts[i], D.hole_block[i + 1] - D.hole_block[i],
                          D.capacity[i], 0, 1);
}

__global__ void __launch_bounds__(256) kf_dead_write(const BatchDesc D) {
    const int lane = threadIdx.x & 31;
    const int nw = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int vb = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5); vb < D.total_hole_blocks; vb += nw) {
        const int i = batch_find(D.hole_block, D.n, vb); // warp-uniform
        const int b = vb - D.hole_block[i];
        const DevLedger* L = D.ledgers[i];
        const int n = L->n_slots, need = L->n_inject;
        if (need == 0 || b * kHoleBlock >= n) continue; // warp-uniform
        const int k0 = b * kHoleBlock + 32 * lane;
        unsigned m = dead_bits(D.states[i].alive, k0, n);
        const int c = __popc(m);
        int x = c;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        int rank = D.hole_counts[i][b] + x - c;
        int* holes = D.holes[i];
        while (m && rank < need) {
            const int t = __ffs(m) - 1;
            m &= m - 1u;
            holes[rank++] = k0 + t;
        }
    }
}

template <bool kMixed, bool kRta>
__global__ void __launch_bounds__(256) kf_inject(const BatchDesc D) {
    for (int vb = blockIdx.x; vb < D.total_inject_blocks; vb += gridDim.x) {
        const int i = batch_find(D.inject_block, D.n, vb);
        const int b0 = D.inject_block[i];
        k_inject_body<kMixed, kRta, false>(D.tables[i], D.states[i], D.cells[i], D.ledgers[i], D.holes[i], vb - b0,
                                           D.inject_block[i + 1] - b0);
        __syncthreads();
    }
}

__global__ void kf_inject_finish(const BatchDesc D) {
    if (threadIdx.x == 0) k_inject_finish_body(D.ledgers[blockIdx.x], 0, 1);
}

int launch_fused_transport(const BatchDesc& D, cudaStream_t s, bool mixed) {
    const int g = std::min(D.total_carrier_blocks, D.persist);
    const int gh = std::min((D.total_hole_blocks + 7) / 8, D.persist);
    const int gi = std::min(D.total_inject_blocks, D.persist);
    if (mixed) {
        kf_transport<true, true><<<g, kTransportThreads, 0, s>>>(D);
        kf_deferred<true><<<g, kTransportThreads, 0, s>>>(D);
    } else {
        kf_transport<false, true><<<g, kTransportThreads, 0, s>>>(D);
        kf_box_events<true><<<g, kTransportThreads, 0, s>>>(D);
    }
    kf_dead_count<<<gh, 256, 0, s>>>(D);
    kf_inject_prepare<<<D.n, 1024, 0, s>>>(D);
    kf_dead_write<<<gh, 256, 0, s>>>(D);
    if (mixed) kf_inject<true, true><<<gi, 256, 0, s>>>(D);
    else kf_inject<false, true><<<gi, 256, 0, s>>>(D);
    kf_inject_finish<<<D.n, 32, 0, s>>>(D);
    return 7;
}

} // namespace phmc
