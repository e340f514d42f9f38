// Device-side data layout and per-carrier functions of the carrier loop.
//
// Carriers are structure-of-arrays in HBM, one slot per carrier:
//   x, y, z  float64 absolute position (plain path) or
//   ox,oy,oz float32 offset from the cell origin (mixed path)
//   occ      float64 occupation
//   mode     uint32  active index | velocity sign bits << 24 | material << 28
//   cell     int32   grid cell
//   alive    uint8   0 for an absorbed (free) slot
// The velocity is never stored: it is the mode's group velocity with the sign
// bits applied, which reproduces the reference's velocity bit-for-bit on an
// axis-aligned box (specular reflection and reservoir inversion only flip
// signs; src/solver/BoundaryInteraction.cpp:146-159,
// src/solver/ReservoirInjector.cpp:97-102).
#pragma once
#include <cstdint>

#include "phmc_rng.h"

namespace phmc {

constexpr int kMaxMaterials = 4;
constexpr int kMaxRoughTables = 24;
constexpr int kMaxReservoirs = 6;

// Outcome flags of one rough reflection, the event classes counted by the
// reference's RoughSampleEvents (src/solver/RoughBoundarySampler.cpp:371-533).
enum : unsigned {
    kRoughSpecular = 1u,        // specular partner taken
    kRoughMissingSpec = 2u,     // specular draw without a partner
    kRoughWindow = 4u,          // residual-flux window of the incoming frequency
    kRoughWindowFallback = 8u,  // window present but without residual flux
    kRoughDiffuse = 16u,        // a diffuse outgoing mode was drawn
    kRoughPool = 32u,           // uniform outgoing-pool fallback
    kRoughRandom = 64u,         // uniform over all modes
};
constexpr int kRoughCounters = 8; // the seven flags above, then the event count
constexpr double kHbar = 6.582119569e-4;
constexpr double kKb = 8.617333262145e-5;

enum ErrorCode : int {
    kErrNone = 0,
    kErrIntersection = 1,
    kErrModeMapping = 2,
    kErrTooManyEvents = 3,
    kErrInvalidStatistics = 4,
    kErrEscaped = 5,
    kErrZeroFluxReservoir = 6,
    kErrCapacity = 7,
    kErrOutwardReservoirMode = 8,
    kErrNonFinite = 9,
    kErrNoRoughTable = 10,
    kErrCollision = 11,
    kErrNclNoConstraint = 12,
    kErrNclSingular = 13,
    kErrNclLineSearch = 14,
    kErrNclNoConverge = 15,
    kErrNclInvalid = 16,
    kErrNclTemperature = 17,
    kErrPipelineTimeout = 18,
    kErrAmmRow = 19,
};

struct DevMaterial {
    int n_active;
    int n_classes;
    int n_lookup;
    int n_temps;
    const double* omega;    // [active]
    const double* hw;       // [active]
    const double* inv_hw;   // [active]
    const double* vel;      // [active*3]
    const double* flux_vel; // [active*3] v * (hbar omega) * energy weight: heat-flux term per unit deviation
    const float* vel32;     // [active*4] (vx, vy, vz, 0) for the mixed path
    const float* ivel32;    // [active*4] (1/vx, 1/vy, 1/vz, 0); 0 where v = 0
    const double* speed;    // [active] |v|
    const double* push;     // [active] push_eps / max(|v|, 1e-12)
    const double* nbg;      // [active]
    const double* cap_bg;   // [active]
    const int* mode_class;  // [active]
    const double* class_omega;
    const double* class_hw;
    const int* class_rep;
    const double* relax_fixed; // [active]
    const double* temps;       // [n_temps]
    const double* gamma;       // [n_temps * active]
    const double* lookup_T;
    const double* lookup_E;
    const double* col_cap;     // [active]
    const double* col_rate;    // total collision rate [active]
    const double* col_rn;      // normal rate [active]
    const double* col_rr;      // resistive rate [active]
    const double* col_k;       // [active*3]
    const double* grad_rate;   // [active]
    const double* drive_rate;  // [active] half dt * rate / hw: drive half-step D = drive_rate - drive_cap * ratio
    const double* drive_cap;   // [active] half dt * capacity / hw
    // heat source: spectral weight (0: not eligible), Gaussian log-weight, and
    // the class of equal frequency among eligible modes for the thermal Newton
    const double* src_weight;  // [active]
    const double* src_logw;    // [active]
    const int* src_class;      // [active], -1 when not eligible
    const double* src_class_omega;
    int n_src_classes;
    // bins per cell: modes sharing every per-cell update share a bin (RTA:
    // equal frequency and linewidths, and source weight); null = one bin per mode
    const int* bin;            // [active] -> bin
    const int* bin_rep;        // [bins] -> representative active mode
    int n_bins;
    double energy_weight;
    double energy_density_bg;
    double heat_capacity_density_bg;
    double zero_point;
};

struct DevRoughTable {
    int strict;
    int n_sorted, n_roulette, n_outgoing;
    const double* specularity;
    const int* spec_match;
    const int* diffuse_begin;
    const int* diffuse_end;
    const int* outgoing_sorted;
    const double* prefix;
    const double* coarse;     // prefix[64 k], k = 0 .. n_sorted / 64 (null: one-level search)
    const int* roulette_active;
    const double* roulette_cdf;
    const int* outgoing_active;
};

struct DevReservoir {
    int facet, material, n_cdf;
    double expected;
    double normal[3];
    int n_tri;             // triangles of the facet
    const double* tri;     // [n_tri][3 vertices][3]
    const double* tri_cum; // running area sum, [n_tri]
    const double* cdf;
    const AliasCell* alias; // the emission distribution as an alias table, [n_cdf]
    const double* occ; // emitted occupation per active mode
};

struct DevDomain {
    double lo[3], hi[3], inv_cell[3], cell_size[3];
    float cell_size32[3];
    float inv_cell32[3];
    // c / (shape[1] shape[2]) and r / shape[2] as __umul64hi(c, magic); 0 means divisor 1
    unsigned long long div_yz, div_z;
    int shape[3];
    int ncells;
    double tol;        // analytic-box position tolerance
    double scale;      // max(1, extents)
    char cond[6];
    double shift[6][3];
    int pair[6];
    int reservoir[6];
    int rough_table[kMaxMaterials][6];
    // layered materials
    int layout_axis;
    int n_planes;
    double planes[kMaxMaterials];
    int plane_cell[kMaxMaterials]; // cell boundary index of each plane along the layout axis
};

struct DevParams {
    double dt;
    float dt32;
    double push_eps;
    uint64_t seed;
    int conservative;
    int linearized;
    int one_to_one;
    int n_materials;
    int n_reservoirs;
    int lifetime_local;
    double lifetime_T;
    double background_T;
    int gradient_axis;
    double gradient_energy_weight;
    int source_enabled;
    int source_spectrum;        // 0 thermal, 1 weighted, 2 gaussian
    int source_linearized;      // thermal spectrum with linearized transport
    int source_pulsed;          // time profile (src/solver/HeatSourceDriving.cpp:12-44)
    double source_time_start, source_time_end, source_period, source_on, source_amplitude;
};

// Per-step accumulators and running totals, all on the device so a step needs
// no host round trip (src/solver/BoundaryLedger.cpp, src/solver/EnergyLedger.cpp).
struct DevLedger {
    int error_code;
    int error_slot;
    int n_slots;            // slots in use [0, n_slots)
    int n_holes;            // free slots below n_slots at injection
    int n_inject;           // carriers injected this step
    int n_deferred;         // wall events queued by the mixed transport pass this step
    int event_head;         // queue entries handed out to the warps of the mesh event pass
    uint32_t step_index;    // timesteps completed (the draw counter of the running step)
    double elapsed;         // ps at the start of the running step
    int inject_count[kMaxReservoirs];
    int inject_offset[kMaxReservoirs + 1];
    unsigned int absorbed_res[kMaxReservoirs];  // this step
    unsigned int previous_res[kMaxReservoirs];  // previous step (one-to-one refill)
    unsigned long long step_absorbed, step_injected;
    double step_absorbed_ev, step_injected_ev;
    double step_lifetime_residual, step_drive_ev;
    unsigned long long step_drive_updates;
    double next_drive_ev;                  // first gradient half-step of the next step
    unsigned long long next_drive_updates;
    double step_source_ev, next_source_ev, total_source_ev;   // heat source deposits
    unsigned long long step_source_updates, next_source_updates, total_source_updates;
    double step_balance_residual;
    double thermal_energy;
    // totals
    unsigned long long total_absorbed, total_injected;
    double total_absorbed_ev, total_injected_ev, total_lifetime_residual, total_balance_residual, total_drive_ev;
    unsigned long long total_drive_updates;
    unsigned long long total_iface_events, total_iface_transmitted, total_iface_reflected;
    unsigned long long total_rough[kRoughCounters]; // rough reflection outcomes, then the event count
    unsigned long long total_cache_corrections;     // wall caches found from a nudged position
    long long particle_count;
};

// Diffuse-mismatch banks (src/solver/InterfaceModeSampler.cpp:11-44).
struct DevInterfaceBank {
    const double* omega;  // sorted
    const int* active;
    const double* prefix; // n + 1
    int n;
};
// Acoustic-mismatch rows of one side of one interface (src/solver/AcousticInterfaceSampler.cpp):
// per incoming active mode its mirror partner (-1: not incoming) and the
// transmitted entries [start[a], start[a+1]) as (destination active, probability).
struct DevAmmRows {
    const int* reflected;
    const int* start;
    const int* dest;
    const double* prob;
};
struct DevInterface {
    int enabled, linearized, axis;
    double band_width;
    DevInterfaceBank bank[kMaxMaterials][2];
    int model;             // 0 dmm, 1 amm, 2 mmm
    double amm_fraction;   // acoustic-model probability per event
    DevAmmRows amm[kMaxMaterials - 1][2];
};

// Face BVH node: bounds, children (-1 for a leaf) and the record range of a leaf.
struct __align__(16) DevBvhNode {
    double bmin[3], bmax[3];
    int left, right, begin, end;
};

// Device layout of the face BVH: nodes in breadth-first order (root at 0),
// and one contiguous record per face in leaf order (the order the traversal
// tests them), so a leaf is a run of records with no index indirection:
// normal xyz, plane offset k, bounds min xyz / max xyz, vertices a, b, c.
constexpr int kFaceRecord = 19;
// FP32 copies for the culling walk: node bounds and face planes / bounds
// rounded outward; `margin` (Angstrom) covers the FP32 rounding of the walk.
struct __align__(8) DevBvhNode32 {
    float bmin[3], bmax[3];
    int left, right, begin, end;
};
// normal xyz, k, bounds min xyz, max xyz, then per edge (AB, BC, CA) its
// in-plane inward unit normal m and offset m.(edge start): a point p is at
// least -(m.p - offset) from the triangle when that is positive
constexpr int kFaceRecord32 = 22;
struct DevMesh {
    const DevBvhNode* nodes;
    const double* face;        // [nfaces][kFaceRecord]
    const int* face_facet;     // facet of each record
    const int* face_id;        // input face index of each record
    const DevBvhNode32* nodes32;
    const float* face32;       // [nfaces][kFaceRecord32]
    float margin;
    int root;                  // -1: no BVH, records in input order and scanned in full
    int nfaces;
    int nnodes;
};
// Boundary data of a mesh domain, per facet (facet count n = 0: analytic box).
struct DevFacets {
    int n;
    const char* cond;              // 'T', 'P', 'R'
    const int* pair;               // periodic partner or -1
    const int* reservoir;          // reservoir index or -1
    const double* shift;           // [n][3] periodic translation
    const double* normal;          // [n][3] outward unit normal
    const int* rough_table;        // [material][n] -> rough table or -1
    const DevRoughTable* rough;    // every rough table of the domain
    const int* voxel_cell;         // voxel -> active cell
    const int* cell_voxel;         // active cell -> home voxel (origin of its FP32 offsets)
    const unsigned char* voxel_interior; // voxel -> 1: every point of its box is inside (null: none)
    DevMesh mesh;                  // oriented faces and their BVH
    int prism;                     // extruded prism: facet-scan trace, ray-cast membership
    const double* facet_centroid;  // [n][3] (prism trace)
    const int* facet_face_begin;   // [n + 1] the facet's triangles in facet_tri (prism trace)
    const double* facet_tri;       // [faces][9] vertices a, b, c of each facet's triangles
    int n_simplex;                 // star decomposition (0: ray cast only)
    const double* simplex;         // [n_simplex][18]: apex xyz, inverse 3x3 row-major, bounds min xyz, max xyz
    double ray_pad;                // padding of the BVH culling in the membership ray cast
    // per-carrier mesh state (kept here so the carrier-state kernel parameter stays small):
    int32_t* mirror;               // facet whose mirror applies to the mode velocity, -1 none
    double* hit_t;                 // wall cache: time to the wall in units of dt
    double* hit_x;                 //   cached hit point
    double* hit_y;
    double* hit_z;
    int32_t* hit_f;                //   cached facet
};

struct DevTables {
    DevMaterial mat[kMaxMaterials];
    DevInterface iface;
    DevRoughTable rough[kMaxRoughTables];
    DevReservoir res[kMaxReservoirs];
    DevDomain dom;
    DevParams par;
    DevFacets fac;
};

struct CarrierState {
    double* x;   // plain path positions; staging for uploads/downloads in the mixed path
    double* y;
    double* z;
    float* ox;   // mixed path: offset from the lower corner of the carrier's cell
    float* oy;
    float* oz;
    double* occ;
    uint32_t* mode;
    int32_t* cell;
    uint8_t* alive;
    int4* deferred; // mixed path: queued wall events (slot, time left, event, wall), capacity entries
    int capacity;
};

// ------------------------------------------------------------ helpers
__device__ __forceinline__ void raise_error(DevLedger* L, int code, int slot) {
    if (atomicCAS(&L->error_code, 0, code) == 0) L->error_slot = slot;
}

__device__ __forceinline__ double bose_dev(double T, double w) {
    if (T <= 0.0 || w <= 0.0) return 0.0;
    const double x = kHbar * w / (kKb * T);
    if (x > 700.0) return 0.0;
    return 1.0 / fmax(exp(x) - 1.0, 1e-12);
}

__device__ __forceinline__ int grid_index(const DevDomain& D, double px, double py, double pz) {
    const double p[3] = {px, py, pz};
    int idx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int n = D.shape[a];
        if (n <= 1) {
            idx[a] = 0;
        } else {
            int i = static_cast<int>(floor((p[a] - D.lo[a]) * D.inv_cell[a]));
            idx[a] = i < 0 ? 0 : (i >= n ? n - 1 : i);
        }
    }
    return (idx[0] * D.shape[1] + idx[1]) * D.shape[2] + idx[2];
}

__device__ __forceinline__ int material_at(const DevDomain& D, const double p[3]) {
    int m = 0;
    while (m < D.n_planes && p[D.layout_axis] >= D.planes[m]) ++m;
    return m;
}

// Analytic box trace (src/SimulationDomain.cpp:399-450); facet -1 on a miss.
__device__ __forceinline__ void trace_box(const DevDomain& D, const double p[3], const double v[3], double cp[3],
                                          double& t, int& facet) {
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    t = inf;
    facet = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        cp[a] = p[a];
        if (!isfinite(p[a]) || p[a] < D.lo[a] - D.tol || p[a] > D.hi[a] + D.tol) return;
    }
    double best = inf;
    int plane = -1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double c = v[a];
        if (!isfinite(c) || fabs(c) <= 1e-18) continue;
        const int side = c > 0.0 ? 1 : 0;
        const double target = side ? D.hi[a] : D.lo[a];
        const double h = (target - p[a]) / c;
        if (isfinite(h) && h > 1e-14 && h < best) {
            best = h;
            plane = 2 * a + side;
        }
    }
    if (plane < 0) return;
    double c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) c[a] = __fma_rn(v[a], best, p[a]);
    const int ha = plane >> 1;
    c[ha] = (plane & 1) ? D.hi[ha] : D.lo[ha];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (!isfinite(c[a]) || c[a] < D.lo[a] - D.tol || c[a] > D.hi[a] + D.tol) return;
        c[a] = fmin(fmax(c[a], D.lo[a]), D.hi[a]);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) cp[a] = c[a];
    t = best;
    facet = plane;
}

__device__ __forceinline__ bool box_contains(const DevDomain& D, const double p[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (!(p[a] >= D.lo[a] && p[a] <= D.hi[a])) return false;
    return true;
}

// Wall-hit cache with the reference's nudged retries (src/solver/TransportOperator.cpp:186-250).
// 0: no wall found; 1: found; 2: found from a nudged position (the carrier moved).
__device__ __forceinline__ int cache_hit(const DevDomain& D, const DevParams& P, double p[3], const double v[3],
                                         double speed, double cp[3], double& t, int& f) {
    if (isfinite(speed) && speed <= 1e-18) {
        t = __longlong_as_double(0x7ff0000000000000LL);
        f = -1;
        return 1;
    }
    trace_box(D, p, v, cp, t, f);
    if (f >= 0 && isfinite(t)) return 1;
    const double eps = fmax(P.push_eps, 1e-10 * D.scale);
    int nearest = 0;
    double bd = 1e300;
    for (int k = 0; k < 6; ++k) {
        const int a = k >> 1;
        const double d = fabs(p[a] - ((k & 1) ? D.hi[a] : D.lo[a]));
        if (d < bd) {
            bd = d;
            nearest = k;
        }
    }
    double cand[4][3];
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) cand[c][a] = p[a];
    const int na = nearest >> 1;
    const double nsign = (nearest & 1) ? 1.0 : -1.0;
    cand[0][na] = p[na] + nsign * eps;
    cand[1][na] = p[na] - nsign * eps;
    if (speed > 0.0 && isfinite(speed)) {
        for (int a = 0; a < 3; ++a) {
            const double d = v[a] * (1.0 / speed);
            cand[2][a] = p[a] + d * eps;
            cand[3][a] = p[a] - d * eps;
        }
    }
    for (int c = 0; c < 4; ++c) {
        if (!box_contains(D, cand[c])) continue;
        trace_box(D, cand[c], v, cp, t, f);
        if (f >= 0 && isfinite(t)) {
            for (int a = 0; a < 3; ++a) p[a] = cand[c][a];
            return 2;
        }
    }
    return 0;
}

__device__ __forceinline__ void mode_velocity(const DevMaterial& M, uint32_t w, double v[3]) {
    const int a = static_cast<int>(w & 0x00FFFFFFu);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double c = __ldg(M.vel + 3 * a + k);
        // sign flip on the sign bit (integer pipe; the same bits as -c)
        v[k] = __hiloint2double(__double2hiint(c) ^ static_cast<int>(((w >> (24 + k)) & 1u) << 31), __double2loint(c));
    }
}

// Rough-wall reflection with supplied uniforms (src/solver/RoughBoundarySampler.cpp:373-533).

__device__ __forceinline__ int rough_sample_dev(const DevRoughTable& R, const DevMaterial& M, int in_ai, double n_in, bool signed_w,
                                double u0, double u1, double u2, double& n_out, unsigned& diag) {
    n_out = n_in;
    diag = 0;
    const int na = M.n_active;
    const double p_spec = fmin(fmax(R.specularity[in_ai], 0.0), 1.0);
    const double nbg_in = M.nbg[in_ai], w_in = M.omega[in_ai];
    if (u0 <= p_spec) {
        const int out = R.spec_match[in_ai];
        diag = (out >= 0 && out < na) ? kRoughSpecular : kRoughMissingSpec;
        if (out >= 0 && out < na) {
            const double mapped = M.nbg[out] + w_in * (n_in - nbg_in) / fmax(1e-30, M.omega[out]);
            if (isfinite(mapped) && (signed_w || mapped >= 0.0)) {
                n_out = mapped;
                return out;
            }
            return in_ai;
        }
    }
    int out = -1;
    const int b = R.diffuse_begin[in_ai], e = R.diffuse_end[in_ai];
    if (b >= 0 && e > b && e <= R.n_sorted) {
        const double fb = R.prefix[b], fe = R.prefix[e];
        const double window = fe - fb;
        if (window > 0.0 && isfinite(window)) {
            const double u = fmin(fmax(u1, 0.0), 0.99999999999999989);
            const double target = fb + u * window;
            // upper_bound over prefix[b+1 .. e]: the block of 64 that holds it
            // from the coarse copy (small enough to stay in L2), then the block;
            // the prefix is non-decreasing, so the bound is the one-level one
            int lo = b + 1, hi = e + 1;
            if (R.coarse) {
                const int klo = (lo + 63) >> 6, khi = (hi - 1) >> 6; // block starts inside [lo, hi)
                int a = klo, z = khi + 1;
                while (a < z) {
                    const int mid = (a + z) >> 1;
                    if (R.coarse[mid] <= target) a = mid + 1;
                    else z = mid;
                }
                if (a > klo) lo = max(lo, ((a - 1) << 6) + 1); // prefix[64 (a - 1)] <= target
                if (a <= khi) hi = min(hi, a << 6);            // prefix[64 a] > target
            }
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (R.prefix[mid] <= target) lo = mid + 1;
                else hi = mid;
            }
            int pos = lo - 1;
            pos = pos < b ? b : (pos > e - 1 ? e - 1 : pos);
            out = R.outgoing_sorted[pos];
            diag |= kRoughWindow;
        } else {
            diag |= kRoughWindowFallback;
        }
    }
    if (out < 0) {
        if (R.strict) return in_ai;
        if (R.n_roulette > 0 && R.roulette_cdf[R.n_roulette - 1] > 0.0) {
            const double r = R.roulette_cdf[R.n_roulette - 1] * u1;
            int lo = 0, hi = R.n_roulette;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (R.roulette_cdf[mid] < r) lo = mid + 1;
                else hi = mid;
            }
            if (lo >= R.n_roulette) lo = R.n_roulette - 1;
            out = R.roulette_active[lo];
        } else if (R.n_outgoing > 0) {
            int k = static_cast<int>(u2 * R.n_outgoing);
            out = R.outgoing_active[k < R.n_outgoing ? k : R.n_outgoing - 1];
            diag |= kRoughPool;
        } else {
            const int k = static_cast<int>(u2 * na);
            out = k < na ? k : na - 1;
            diag |= kRoughRandom;
        }
    }
    diag |= kRoughDiffuse;
    const double mapped = M.nbg[out] + w_in * (n_in - nbg_in) / fmax(1e-30, M.omega[out]);
    if (isfinite(mapped) && (signed_w || mapped >= 0.0)) {
        n_out = mapped;
        return out;
    }
    n_out = n_in;
    return in_ai;
}

__device__ __forceinline__ double table_inverse(const double* E, const double* T, int n, double e) {
    if (n <= 0) return 0.0;
    if (n == 1 || e <= E[0]) return T[0];
    if (e >= E[n - 1]) return T[n - 1];
    int lo = 0, hi = n;
    while (lo < hi) { // upper_bound
        const int mid = (lo + hi) >> 1;
        if (E[mid] <= e) lo = mid + 1;
        else hi = mid;
    }
    const int h = lo, l = h - 1;
    const double x0 = E[l], x1 = E[h];
    if (fabs(x1 - x0) <= 1e-18) return T[l];
    const double t = (e - x0) / (x1 - x0);
    return T[l] * (1.0 - t) + T[h] * t;
}

// Linear interpolation of the linewidth table, clamped (src/material/Thermodynamics.cpp:108-132).
__device__ __forceinline__ double gamma_at(const DevMaterial& M, int a, double T) {
    const int nT = M.n_temps;
    if (T <= M.temps[0]) return M.gamma[a];
    if (T >= M.temps[nT - 1]) return M.gamma[static_cast<size_t>(nT - 1) * M.n_active + a];
    int lo = 0, hi = nT;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (M.temps[mid] <= T) lo = mid + 1;
        else hi = mid;
    }
    const int h = lo, l = h - 1;
    const double x0 = M.temps[l], x1 = M.temps[h];
    const double y0 = M.gamma[static_cast<size_t>(l) * M.n_active + a];
    const double y1 = M.gamma[static_cast<size_t>(h) * M.n_active + a];
    if (fabs(x1 - x0) <= 1e-18) return y0;
    const double t = (T - x0) / (x1 - x0);
    return y0 * (1.0 - t) + y1 * t;
}

// ------------------------------------------------------ interfaces
__device__ __forceinline__ int lower_bound_dev(const double* a, int lo, int hi, double x) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int upper_bound_dev(const double* a, int lo, int hi, double x) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (!(x < a[mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// src/solver/InterfaceModeSampler.cpp:69-108 with the uniform supplied.
__device__ __forceinline__ int interface_band_dev(const DevInterfaceBank& B, double omega, double width, double u,
                                                  bool& drew, double& flux) {
    const double bin = floor(omega / width);
    const double lo = __dmul_rn(bin, width), hi = __dmul_rn(__dadd_rn(bin, 1.0), width);
    const int begin = lower_bound_dev(B.omega, 0, B.n, lo);
    const int end = lower_bound_dev(B.omega, 0, B.n, hi);
    flux = end > begin ? __dadd_rn(B.prefix[end], -B.prefix[begin]) : 0.0;
    drew = false;
    if (!(flux > 0.0)) return -1;
    drew = true;
    const double target = __dadd_rn(B.prefix[begin], __dmul_rn(u, flux));
    int pos = upper_bound_dev(B.prefix, begin + 1, end + 1, target);
    pos = min(max(pos, begin + 1), end) - 1;
    return B.active[pos];
}

struct IfaceOut {
    int action; // 3 reflect, 4 transmit, 5 fail, 6 acoustic row missing (tangent or unsupported state)
    int material, active;
    uint32_t signs;
    double occ;
    int transmitted;
};

// src/solver/InterfaceInteraction.cpp:46-153 with uniforms consumed in the
// reference's order: the model choice (mixed mismatch only), then either the
// acoustic row (AcousticInterfaceSampler::sample) or the diffuse-mismatch
// reflected band, transmitted band and transmission draws.
__device__ __forceinline__ IfaceOut interface_dev(const DevTables& T, int src, int a, uint32_t signs, double occ,
                                                  int next, double u0, double u1, double u2, double u3) {
    const DevInterface& I = T.iface;
    const DevMaterial& S = T.mat[src];
    IfaceOut r;
    r.material = src;
    r.active = a;
    r.signs = signs;
    r.occ = occ;
    r.transmitted = 0;
    const int axis = I.axis;
    const double omega = S.omega[a];
    const double v_axis = ((signs >> axis) & 1u) ? -S.vel[3 * a + axis] : S.vel[3 * a + axis];
    const int incident = v_axis > 0.0 ? 1 : 0;
    const double u[4] = {u0, u1, u2, u3};
    int k = 0;
    const double acoustic_p = I.model == 1 ? 1.0 : (I.model == 2 ? I.amm_fraction : 0.0);
    const bool use_amm = acoustic_p >= 1.0 || (acoustic_p > 0.0 && u[k++] < acoustic_p);
    bool transmit;
    int sel_material, sel;
    if (use_amm) {
        if (fabs(v_axis) < 1e-7) { // tangent: mirrored in the interface plane
            r.signs ^= 1u << axis;
            r.action = 3;
            return r;
        }
        const DevAmmRows& R = I.amm[src < next ? src : next][src < next ? 0 : 1];
        const int refl = R.reflected[a];
        if (refl < 0) {
            r.action = 6;
            return r;
        }
        double x = u[k++];
        int chosen = -1;
        for (int e = R.start[a]; e < R.start[a + 1]; ++e) {
            x = __dadd_rn(x, -R.prob[e]);
            if (x < 0.0) {
                chosen = R.dest[e];
                break;
            }
        }
        transmit = chosen >= 0;
        sel_material = transmit ? next : src;
        sel = transmit ? chosen : refl;
    } else {
        bool drew;
        double source_flux = 0, target_flux = 0;
        const int refl = interface_band_dev(I.bank[src][1 - incident], omega, I.band_width, u[k], drew, source_flux);
        if (drew) ++k;
        const int trans = interface_band_dev(I.bank[next][incident], omega, I.band_width, u[k], drew, target_flux);
        if (drew) ++k;
        const double transmission =
            target_flux > 0 ? target_flux / fmax(1e-300, __dadd_rn(source_flux, target_flux)) : 0.0;
        transmit = trans >= 0 && u[k] < transmission;
        sel_material = transmit ? next : src;
        sel = transmit ? trans : refl;
    }
    if (sel < 0) {
        if (I.linearized) {
            r.action = 5;
            return r;
        }
        r.signs ^= 1u << axis;
        r.action = 3;
        return r;
    }
    const DevMaterial& Dm = T.mat[sel_material];
    const double new_omega = Dm.omega[sel];
    const double old_deviation = __dadd_rn(occ, -S.nbg[a]);
    const double physical = __dmul_rn(__dmul_rn(S.energy_weight, omega), old_deviation);
    const double new_deviation = physical / fmax(1e-300, __dmul_rn(Dm.energy_weight, new_omega));
    const double new_occ = __dadd_rn(Dm.nbg[sel], new_deviation);
    if (I.linearized) {
        const double nv = Dm.vel[3 * sel + axis];
        const int expected = transmit ? incident : 1 - incident;
        if (!isfinite(new_occ) || !isfinite(nv) || (expected ? !(nv > 0.0) : !(nv < 0.0))) {
            r.action = 5;
            return r;
        }
    }
    if (!isfinite(new_occ) || (!I.linearized && new_occ < 0.0)) {
        r.signs ^= 1u << axis;
        r.action = 3;
        return r;
    }
    r.material = sel_material;
    r.active = sel;
    r.signs = 0;
    r.occ = new_occ;
    r.action = transmit ? 4 : 3;
    r.transmitted = transmit ? 1 : 0;
    return r;
}

// ------------------------------------------------------ mesh tracing
// Device copy of a MeshTracer (face planes, bounds, BVH); all arithmetic of
// the trace below is rounded step by step as the host restatement of
// src/SurfaceMesh.cpp:111-223 and :1164-1269 is.

namespace meshmath {
__device__ __forceinline__ double dot(const double a[3], const double b[3]) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ __forceinline__ void sub(const double a[3], const double b[3], double o[3]) {
    for (int i = 0; i < 3; ++i) o[i] = __dadd_rn(a[i], -b[i]);
}
__device__ __forceinline__ void axpy(const double a[3], const double d[3], double s, double o[3]) {
    for (int i = 0; i < 3; ++i) o[i] = __dadd_rn(a[i], __dmul_rn(d[i], s));
}
// src/SurfaceMesh.cpp:111-159
__device__ __forceinline__ void closest(const double p[3], const double a[3], const double b[3], const double c[3],
                                        double o[3]) {
    double ab[3], ac[3], ap[3];
    sub(b, a, ab);
    sub(c, a, ac);
    sub(p, a, ap);
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) {
        for (int i = 0; i < 3; ++i) o[i] = a[i];
        return;
    }
    double bp[3];
    sub(p, b, bp);
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) {
        for (int i = 0; i < 3; ++i) o[i] = b[i];
        return;
    }
    const double vc = __dadd_rn(__dmul_rn(d1, d4), -__dmul_rn(d3, d2));
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
        axpy(a, ab, d1 / __dadd_rn(d1, -d3), o);
        return;
    }
    double cp[3];
    sub(p, c, cp);
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) {
        for (int i = 0; i < 3; ++i) o[i] = c[i];
        return;
    }
    const double vb = __dadd_rn(__dmul_rn(d5, d2), -__dmul_rn(d1, d6));
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
        axpy(a, ac, d2 / __dadd_rn(d2, -d6), o);
        return;
    }
    const double va = __dadd_rn(__dmul_rn(d3, d6), -__dmul_rn(d5, d4));
    const double e43 = __dadd_rn(d4, -d3), e56 = __dadd_rn(d5, -d6);
    if (va <= 0.0 && e43 >= 0.0 && e56 >= 0.0) {
        double bc[3];
        sub(c, b, bc);
        axpy(b, bc, e43 / __dadd_rn(e43, e56), o);
        return;
    }
    const double denom = 1.0 / __dadd_rn(__dadd_rn(va, vb), vc);
    double t[3];
    axpy(a, ab, __dmul_rn(vb, denom), t);
    axpy(t, ac, __dmul_rn(vc, denom), o);
}
// src/SurfaceMesh.cpp:188-223. The per-axis reciprocal 1/d of the reference is
// the same for every box of one ray, so it is computed once (RayInv).
struct RayInv {
    double inv[3];
    bool flat[3]; // |d| <= 1e-14: the slab test on the origin instead
};
__device__ __forceinline__ RayInv ray_inv(const double d[3]) {
    RayInv r;
    for (int a = 0; a < 3; ++a) {
        r.flat[a] = fabs(d[a]) <= 1e-14;
        r.inv[a] = r.flat[a] ? 0.0 : 1.0 / d[a];
    }
    return r;
}
__device__ __forceinline__ bool ray_box(const double o[3], const RayInv& R, const double bmin[3], const double bmax[3],
                                        double t_limit, double& t_near_out) {
    double t_near = 0.0, t_far = t_limit;
    for (int a = 0; a < 3; ++a) {
        if (R.flat[a]) {
            if (o[a] < bmin[a] - 1e-12 || o[a] > bmax[a] + 1e-12) return false;
            continue;
        }
        double t0 = __dmul_rn(__dadd_rn(bmin[a], -o[a]), R.inv[a]), t1 = __dmul_rn(__dadd_rn(bmax[a], -o[a]), R.inv[a]);
        if (t0 > t1) {
            const double s = t0;
            t0 = t1;
            t1 = s;
        }
        t_near = fmax(t_near, t0);
        t_far = fmin(t_far, t1);
        if (t_far < t_near) return false;
    }
    if (t_far <= 1e-10) return false;
    t_near_out = fmax(0.0, t_near);
    return t_near_out <= t_limit;
}
} // namespace meshmath

// Nearest surface hit of the ray x + v t (t > 1e-10) with the near-first BVH
// walk (src/SurfaceMesh.cpp:1164-1269); facet -1 and t = infinity on a miss.
// Exact face test of the reference (src/SurfaceMesh.cpp:1164-1269): plane time
// with eps 1e-10, bounds +-1e-9, closest-point distance <= 1e-7.
struct MeshHit {
    double t;
    int face;
    double p[3];
};
__device__ __forceinline__ void mesh_try_face(const DevMesh& M, int i, const double x[3], const double v[3], MeshHit& h) {
    using namespace meshmath;
    const double* r = M.face + kFaceRecord * i;
    const double nn[3] = {r[0], r[1], r[2]};
    const double denom = dot(v, nn);
    if (fabs(denom) < 1e-10) return;
    const double t = -__dadd_rn(dot(x, nn), r[3]) / denom;
    if (t <= 1e-10 || t >= h.t) return;
    double p[3];
    axpy(x, v, t, p);
    if (p[0] < r[4] - 1e-9 || p[1] < r[5] - 1e-9 || p[2] < r[6] - 1e-9 || p[0] > r[7] + 1e-9 || p[1] > r[8] + 1e-9 ||
        p[2] > r[9] + 1e-9)
        return;
    const double A[3] = {r[10], r[11], r[12]}, B[3] = {r[13], r[14], r[15]}, Cc[3] = {r[16], r[17], r[18]};
    double cp[3], d[3];
    closest(p, A, B, Cc, cp);
    sub(cp, p, d);
    if (sqrt(dot(d, d)) > 1e-7) return;
    h.t = t;
    h.face = i;
    for (int a = 0; a < 3; ++a) h.p[a] = p[a];
}

// Reference BVH walk in FP64: near-first, boxes pruned by the best time so far.
static __device__ __noinline__ void mesh_walk_fp64(const DevMesh& M, const double x[3], const double v[3], MeshHit& h) {
    using namespace meshmath;
    if (M.root < 0) {
        for (int i = 0; i < M.nfaces; ++i) mesh_try_face(M, i, x, v, h);
        return;
    }
    const RayInv R = ray_inv(v);
    int stack[64];
    int top = 0;
    stack[top++] = M.root;
    while (top > 0) {
        const DevBvhNode& nd = M.nodes[stack[--top]];
        double tn = 0.0;
        if (!ray_box(x, R, nd.bmin, nd.bmax, h.t, tn)) continue;
        if (nd.left < 0 && nd.right < 0) {
            for (int pos = nd.begin; pos < nd.end; ++pos) mesh_try_face(M, pos, x, v, h);
            continue;
        }
        int near_child = -1, far_child = -1;
        double near_t = __longlong_as_double(0x7ff0000000000000LL), far_t = near_t;
        const int kids[2] = {nd.left, nd.right};
        for (int s = 0; s < 2; ++s) {
            const int child = kids[s];
            if (child < 0) continue;
            double tc = 0.0;
            if (!ray_box(x, R, M.nodes[child].bmin, M.nodes[child].bmax, h.t, tc)) continue;
            if (tc < near_t) {
                far_child = near_child;
                far_t = near_t;
                near_child = child;
                near_t = tc;
            } else if (tc < far_t) {
                far_child = child;
                far_t = tc;
            }
        }
        if (far_child >= 0 && top < 64) stack[top++] = far_child;
        if (near_child >= 0 && top < 64) stack[top++] = near_child;
    }
}

// The same walk with FP32 culling. Boxes are widened by `margin`, face
// planes are tested in FP32 with an error bound, and only faces FP32 cannot
// rule out go through the exact FP64 test, so FP32 never drops a face the
// FP64 walk would accept. The FP64 walk runs instead for rays with a velocity
// component of magnitude in (0, 1e-10], where FP32 slab times lose meaning.
__device__ inline void mesh_walk_fp32(const DevMesh& M, const double x[3], const double v[3], MeshHit& h) {
    float xf[3], vf[3], invf[3];
    bool flat[3];
    float vmax = 0.0f;
    for (int a = 0; a < 3; ++a) {
        xf[a] = static_cast<float>(x[a]);
        vf[a] = static_cast<float>(v[a]);
        flat[a] = v[a] == 0.0;
        invf[a] = flat[a] ? 0.0f : 1.0f / vf[a];
        vmax = fmaxf(vmax, fabsf(vf[a]));
    }
    const float m = M.margin;
    auto limit = [&]() {
        return isinf(h.t) ? __int_as_float(0x7f800000) : static_cast<float>(h.t) * 1.000001f + 1e-6f;
    };
    auto box = [&](const DevBvhNode32& b, float tlim, float& tnear) {
        float t0 = 0.0f, t1 = tlim;
        for (int a = 0; a < 3; ++a) {
            const float lo = b.bmin[a] - m, hi = b.bmax[a] + m;
            if (flat[a]) {
                if (xf[a] < lo || xf[a] > hi) return false;
                continue;
            }
            float s0 = (lo - xf[a]) * invf[a], s1 = (hi - xf[a]) * invf[a];
            if (s0 > s1) {
                const float s = s0;
                s0 = s1;
                s1 = s;
            }
            t0 = fmaxf(t0, s0);
            t1 = fminf(t1, s1);
            if (t1 < t0) return false;
        }
        if (t1 < 0.0f) return false;
        tnear = t0;
        return true;
    };
    auto face = [&](int pos) {
        const float* r = M.face32 + kFaceRecord32 * pos;
        const float den = vf[0] * r[0] + vf[1] * r[1] + vf[2] * r[2];
        if (fabsf(den) >= 1e-4f * vmax) {
            const float tf = -(xf[0] * r[0] + xf[1] * r[1] + xf[2] * r[2] + r[3]) / den;
            // error of tf: numerator within m, denominator within 4e-7 vmax (relative to |den| >= 1e-4 vmax)
            const float rel = 4e-7f * vmax / fabsf(den) + 1e-6f;
            const float et = m / fabsf(den) + rel * fabsf(tf) + 1e-6f;
            if (tf + et <= 0.0f || tf - et > limit()) return;
            const float ep = vmax * (et + 1e-6f * fabsf(tf)) + m;
            float p[3];
            for (int a = 0; a < 3; ++a) {
                p[a] = xf[a] + vf[a] * tf;
                if (p[a] < r[4 + a] - ep || p[a] > r[7 + a] + ep) return;
            }
            // outside an edge by more than the FP64 test's 1e-7 plus the
            // error of p (ep) and of the FP32 edge functions (4 margins)
            const float tol = ep + 4.0f * m + 1e-7f;
            for (int e = 0; e < 3; ++e) {
                const float* q = r + 10 + 4 * e;
                if (fmaf(q[0], p[0], fmaf(q[1], p[1], q[2] * p[2])) - q[3] < -tol) return;
            }
        }
        mesh_try_face(M, pos, x, v, h);
    };
    int stack[64];
    int top = 0;
    stack[top++] = M.root;
    while (top > 0) {
        const DevBvhNode32 nd = M.nodes32[stack[--top]];
        float tn;
        if (!box(nd, limit(), tn)) continue;
        if (nd.left < 0 && nd.right < 0) {
            for (int pos = nd.begin; pos < nd.end; ++pos) face(pos);
            continue;
        }
        int near_child = -1, far_child = -1;
        float near_t = __int_as_float(0x7f800000), far_t = near_t;
        const int kids[2] = {nd.left, nd.right};
        const float tl = limit();
        for (int s = 0; s < 2; ++s) {
            const int child = kids[s];
            if (child < 0) continue;
            float tc;
            if (!box(M.nodes32[child], tl, tc)) continue;
            if (tc < near_t) {
                far_child = near_child;
                far_t = near_t;
                near_child = child;
                near_t = tc;
            } else if (tc < far_t) {
                far_child = child;
                far_t = tc;
            }
        }
        if (far_child >= 0 && top < 64) stack[top++] = far_child;
        if (near_child >= 0 && top < 64) stack[top++] = near_child;
    }
}

__device__ inline void mesh_trace_dev(const DevMesh& M, const double x[3], const double v[3], double hit[3], double& t_out,
                                      int& facet) {
    MeshHit h;
    h.t = __longlong_as_double(0x7ff0000000000000LL);
    h.face = -1;
    bool tiny = false;
    for (int a = 0; a < 3; ++a) tiny = tiny || (v[a] != 0.0 && fabs(v[a]) <= 1e-10);
    if (M.root >= 0 && M.nodes32 && !tiny) mesh_walk_fp32(M, x, v, h);
    else mesh_walk_fp64(M, x, v, h);
    if (h.face < 0) {
        for (int a = 0; a < 3; ++a) hit[a] = x[a];
        t_out = __longlong_as_double(0x7ff0000000000000LL);
        facet = -1;
        return;
    }
    for (int a = 0; a < 3; ++a) hit[a] = h.p[a];
    t_out = h.t;
    facet = M.face_facet[h.face];
}

// ------------------------------------------------------------ mesh domains
namespace meshmath {
__device__ __forceinline__ void cross(const double a[3], const double b[3], double o[3]) {
    o[0] = __dadd_rn(__dmul_rn(a[1], b[2]), -__dmul_rn(a[2], b[1]));
    o[1] = __dadd_rn(__dmul_rn(a[2], b[0]), -__dmul_rn(a[0], b[2]));
    o[2] = __dadd_rn(__dmul_rn(a[0], b[1]), -__dmul_rn(a[1], b[0]));
}
__device__ __forceinline__ double norm(const double a[3]) { return sqrt(dot(a, a)); }
// src/SurfaceMesh.cpp:162-186: Moller-Trumbore, eps 1e-10, hit when t > eps
__device__ __forceinline__ bool ray_triangle(const double o[3], const double d[3], const double a[3], const double b[3],
                                             const double c[3], double& t) {
    constexpr double eps = 1e-10;
    double e1[3], e2[3], pvec[3], tvec[3], qvec[3];
    sub(b, a, e1);
    sub(c, a, e2);
    cross(d, e2, pvec);
    const double det = dot(e1, pvec);
    if (fabs(det) < eps) return false;
    const double inv_det = 1.0 / det;
    sub(o, a, tvec);
    const double u = __dmul_rn(dot(tvec, pvec), inv_det);
    if (u < -eps || u > 1.0 + eps) return false;
    cross(tvec, e1, qvec);
    const double v = __dmul_rn(dot(d, qvec), inv_det);
    if (v < -eps || __dadd_rn(u, v) > 1.0 + eps) return false;
    t = __dmul_rn(dot(e2, qvec), inv_det);
    return t > eps;
}
} // namespace meshmath

// Vertices of face record i.
__device__ __forceinline__ void mesh_face(const DevMesh& M, int i, double a[3], double b[3], double c[3]) {
    const double* r = M.face + kFaceRecord * i;
    for (int k = 0; k < 3; ++k) {
        a[k] = r[10 + k];
        b[k] = r[13 + k];
        c[k] = r[16 + k];
    }
}

// +x ray-cast membership (src/SurfaceMesh.cpp:1100-1124): the Moller-Trumbore
// hits of every face, sorted, counted as distinct when more than 1e-9 apart;
// odd means inside. The BVH only culls nodes the ray misses by more than
// ray_pad, so the hit set is that of the full face scan. With the FP32 node
// and face records (widened by M.margin, and face planes and edges tested
// with an error bound as in mesh_walk_fp32) only nodes and faces that FP32
// cannot rule out reach the FP64 test, so the hit set is the same. Returns -1
// when more hits than the local list holds (the caller reports an error).
__device__ inline int mesh_ray_cast_inside(const DevFacets& F, const double p[3]) {
    constexpr int kMaxHits = 64;
    const DevMesh& M = F.mesh;
    const double dir[3] = {1.0, 0.0, 0.0};
    double hits[kMaxHits];
    int nh = 0;
    bool overflow = false;
    auto test_face = [&](int i) {
        double a[3], b[3], c[3], t;
        mesh_face(M, i, a, b, c);
        if (!meshmath::ray_triangle(p, dir, a, b, c, t)) return;
        if (nh < kMaxHits) hits[nh++] = t;
        else overflow = true;
    };
    if (M.root >= 0 && M.nodes32) {
        const float m = M.margin;
        const float xf[3] = {static_cast<float>(p[0]), static_cast<float>(p[1]), static_cast<float>(p[2])};
        // a face FP32 cannot rule out for the ray x + (1, 0, 0) t, t > 0
        auto screen = [&](int pos) {
            const float* r = M.face32 + kFaceRecord32 * pos;
            const float den = r[0];
            if (fabsf(den) >= 1e-4f) {
                const float tf = -(xf[0] * r[0] + xf[1] * r[1] + xf[2] * r[2] + r[3]) / den;
                const float et = m / fabsf(den) + (4e-7f / fabsf(den) + 1e-6f) * fabsf(tf) + 1e-6f;
                if (tf + et <= 0.0f) return false;
                const float ep = et + 1e-6f * fabsf(tf) + m;
                const float q[3] = {xf[0] + tf, xf[1], xf[2]};
                for (int a = 0; a < 3; ++a)
                    if (q[a] < r[4 + a] - ep || q[a] > r[7 + a] + ep) return false;
                const float tol = ep + 4.0f * m + 1e-7f;
                for (int e = 0; e < 3; ++e) {
                    const float* g = r + 10 + 4 * e;
                    if (fmaf(g[0], q[0], fmaf(g[1], q[1], g[2] * q[2])) - g[3] < -tol) return false;
                }
            }
            return true;
        };
        int stack[64];
        int top = 0;
        stack[top++] = M.root;
        while (top > 0) {
            const DevBvhNode32 nd = M.nodes32[stack[--top]];
            if (xf[1] < nd.bmin[1] - m || xf[1] > nd.bmax[1] + m || xf[2] < nd.bmin[2] - m ||
                xf[2] > nd.bmax[2] + m || xf[0] > nd.bmax[0] + m)
                continue;
            if (nd.left < 0 && nd.right < 0) {
                for (int pos = nd.begin; pos < nd.end; ++pos)
                    if (screen(pos)) test_face(pos);
                continue;
            }
            if (top + 2 > 64) {
                overflow = true;
                break;
            }
            if (nd.left >= 0) stack[top++] = nd.left;
            if (nd.right >= 0) stack[top++] = nd.right;
        }
    } else if (M.root >= 0) {
        int stack[64];
        int top = 0;
        stack[top++] = M.root;
        const double pad = F.ray_pad;
        while (top > 0) {
            const DevBvhNode& nd = M.nodes[stack[--top]];
            if (p[1] < nd.bmin[1] - pad || p[1] > nd.bmax[1] + pad || p[2] < nd.bmin[2] - pad ||
                p[2] > nd.bmax[2] + pad || p[0] > nd.bmax[0] + pad)
                continue;
            if (nd.left < 0 && nd.right < 0) {
                for (int pos = nd.begin; pos < nd.end; ++pos) test_face(pos);
                continue;
            }
            if (top + 2 > 64) {
                overflow = true;
                break;
            }
            if (nd.left >= 0) stack[top++] = nd.left;
            if (nd.right >= 0) stack[top++] = nd.right;
        }
    } else {
        for (int i = 0; i < M.nfaces; ++i) test_face(i);
    }
    if (overflow) return -1;
    if (nh == 0) return 0;
    for (int i = 1; i < nh; ++i) { // insertion sort, ascending
        const double key = hits[i];
        int j = i - 1;
        while (j >= 0 && hits[j] > key) {
            hits[j + 1] = hits[j];
            --j;
        }
        hits[j + 1] = key;
    }
    int unique = 1;
    for (int i = 1; i < nh; ++i)
        if (fabs(__dadd_rn(hits[i], -hits[i - 1])) > 1e-9) ++unique;
    return unique & 1;
}

// Star-simplex membership with barycentric tolerance 1e-10 (src/SurfaceMesh.cpp:1126-1149).
__device__ inline bool mesh_simplex_inside(const DevFacets& F, const double p[3]) {
    constexpr double tol = 1e-10;
    for (int s = 0; s < F.n_simplex; ++s) {
        const double* S = F.simplex + 18 * s;
        if (p[0] < S[12] - tol || p[1] < S[13] - tol || p[2] < S[14] - tol || p[0] > S[15] + tol ||
            p[1] > S[16] + tol || p[2] > S[17] + tol)
            continue;
        const double d[3] = {__dadd_rn(p[0], -S[0]), __dadd_rn(p[1], -S[1]), __dadd_rn(p[2], -S[2])};
        const double l1 = __dadd_rn(__dadd_rn(__dmul_rn(S[3], d[0]), __dmul_rn(S[4], d[1])), __dmul_rn(S[5], d[2]));
        const double l2 = __dadd_rn(__dadd_rn(__dmul_rn(S[6], d[0]), __dmul_rn(S[7], d[1])), __dmul_rn(S[8], d[2]));
        const double l3 = __dadd_rn(__dadd_rn(__dmul_rn(S[9], d[0]), __dmul_rn(S[10], d[1])), __dmul_rn(S[11], d[2]));
        const double l0 = __dadd_rn(__dadd_rn(__dadd_rn(1.0, -l1), -l2), -l3);
        if (l0 >= -tol && l1 >= -tol && l2 >= -tol && l3 >= -tol && l0 <= 1.0 + tol && l1 <= 1.0 + tol &&
            l2 <= 1.0 + tol && l3 <= 1.0 + tol)
            return true;
    }
    return false;
}

// SurfaceMesh::contains_point: inside a simplex of the decomposition, else the
// ray cast. Evaluated ray cast first (the result is their union). -1 on a
// hit-list overflow.
__device__ inline int mesh_contains(const DevFacets& F, const double p[3]) {
    const int r = mesh_ray_cast_inside(F, p);
    if (r != 0 || F.prism) return r; // a prism answers by the ray cast alone
    return mesh_simplex_inside(F, p) ? 1 : 0;
}

// True when p lies in a voxel whose whole box is inside the mesh (mesh_contains
// answers 1 there; the closed surface does not cross such a box).
__device__ __forceinline__ bool mesh_voxel_interior(const DevFacets& F, const DevDomain& D, const double p[3]) {
    if (!F.voxel_interior) return false;
    int idx[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double u = floor((p[a] - D.lo[a]) * D.inv_cell[a]);
        if (!(u >= 0.0 && u < static_cast<double>(D.shape[a]))) return false;
        idx[a] = static_cast<int>(u);
    }
    return F.voxel_interior[(static_cast<size_t>(idx[0]) * D.shape[1] + idx[1]) * D.shape[2] + idx[2]] != 0;
}

// True when p lies within `tol` of a face: the face BVH culls every node
// whose bounds, widened by tol, miss p, so only the faces near p are tested.
__device__ inline bool mesh_near_surface(const DevFacets& F, const double p[3], double tol) {
    const DevMesh& M = F.mesh;
    auto near_face = [&](int i) {
        const double* r = M.face + kFaceRecord * i;
        for (int a = 0; a < 3; ++a)
            if (p[a] < r[4 + a] - tol || p[a] > r[7 + a] + tol) return false;
        double a[3], b[3], c[3], cp[3], d[3];
        mesh_face(M, i, a, b, c);
        meshmath::closest(p, a, b, c, cp);
        meshmath::sub(p, cp, d);
        return meshmath::norm(d) <= tol;
    };
    if (M.root < 0) {
        for (int i = 0; i < M.nfaces; ++i)
            if (near_face(i)) return true;
        return false;
    }
    int stack[64];
    int top = 0;
    stack[top++] = M.root;
    while (top > 0) {
        const DevBvhNode& nd = M.nodes[stack[--top]];
        bool miss = false;
        for (int a = 0; a < 3; ++a) miss = miss || p[a] < nd.bmin[a] - tol || p[a] > nd.bmax[a] + tol;
        if (miss) continue;
        if (nd.left < 0 && nd.right < 0) {
            for (int pos = nd.begin; pos < nd.end; ++pos)
                if (near_face(pos)) return true;
            continue;
        }
        if (top + 2 > 64) return true; // too deep to decide: treat as near (no false escape)
        if (nd.left >= 0) stack[top++] = nd.left;
        if (nd.right >= 0) stack[top++] = nd.right;
    }
    return false;
}

// Facet of the closest face, first minimum (src/SurfaceMesh.cpp:996-1023).
__device__ inline int mesh_nearest_facet(const DevFacets& F, const double p[3]) {
    const DevMesh& M = F.mesh;
    int best = -1;
    double bd = __longlong_as_double(0x7ff0000000000000LL);
    for (int i = 0; i < M.nfaces; ++i) {
        double a[3], b[3], c[3], cp[3], d[3];
        mesh_face(M, i, a, b, c);
        meshmath::closest(p, a, b, c, cp);
        meshmath::sub(p, cp, d);
        const double dist = meshmath::norm(d);
        // first minimum in input face order (records are in leaf order)
        if (dist < bd || (dist == bd && best >= 0 && M.face_id[i] < M.face_id[best])) {
            bd = dist;
            best = i;
        }
    }
    return best < 0 ? -1 : M.face_facet[best];
}

// Velocity of a carrier in a mesh domain: the mode velocity (with sign flips),
// mirrored in the plane of facet `mir` when set (src/solver/BoundaryInteraction.cpp:121-124).
__device__ __forceinline__ void mesh_velocity(const DevFacets& F, const DevMaterial& M, uint32_t w, int mir,
                                              double v[3]) {
    mode_velocity(M, w, v);
    if (mir >= 0) {
        const double* n = F.normal + 3 * mir;
        const double nn[3] = {n[0], n[1], n[2]};
        const double s = __dmul_rn(2.0, meshmath::dot(v, nn));
        for (int k = 0; k < 3; ++k) v[k] = __dadd_rn(v[k], -__dmul_rn(nn[k], s));
    }
}

// Trace of an extruded prism (src/SimulationDomain.cpp:344-396): every
// facet's plane through its centroid, the nearest positive distance along
// the unit direction, kept when the point lies in one of the facet's
// triangles by edge functions in the projection dropping the normal's
// largest axis, tolerance 1e-12 of the projected area. The reference takes
// the edge functions in long double; here they are FP64, which decides
// differently only for points within about 1e-16 of the domain size of an
// edge.
__device__ inline void prism_trace_dev(const DevFacets& F, const double p[3], const double vel[3], double hit[3],
                                       double& t_out, int& facet) {
    using namespace meshmath;
    const double speed = norm(vel);
    for (int a = 0; a < 3; ++a) hit[a] = p[a];
    t_out = __longlong_as_double(0x7ff0000000000000LL);
    facet = -1;
    if (!(speed > 0)) return;
    const double inv = 1 / speed;
    const double d[3] = {__dmul_rn(vel[0], inv), __dmul_rn(vel[1], inv), __dmul_rn(vel[2], inv)};
    double best = __longlong_as_double(0x7ff0000000000000LL);
    for (int f = 0; f < F.n; ++f) {
        const double n[3] = {F.normal[3 * f], F.normal[3 * f + 1], F.normal[3 * f + 2]};
        const double den = dot(d, n);
        if (den <= 1e-16) continue;
        const double* c = F.facet_centroid + 3 * f;
        const double cs[3] = {__dadd_rn(c[0], -p[0]), __dadd_rn(c[1], -p[1]), __dadd_rn(c[2], -p[2])};
        const double dist = dot(cs, n) / den;
        if (dist <= 1e-12 || dist >= best) continue;
        double q[3];
        axpy(p, d, dist, q);
        int drop = 0;
        for (int j = 1; j < 3; ++j)
            if (fabs(n[j]) > fabs(n[drop])) drop = j;
        const int u = (drop + 1) % 3, v = (drop + 2) % 3;
        auto cross2 = [&](const double* a, const double* b, const double* cc) {
            return __dadd_rn(__dmul_rn(__dadd_rn(b[u], -a[u]), __dadd_rn(cc[v], -a[v])),
                             -__dmul_rn(__dadd_rn(b[v], -a[v]), __dadd_rn(cc[u], -a[u])));
        };
        for (int k = F.facet_face_begin[f]; k < F.facet_face_begin[f + 1]; ++k) {
            const double* T = F.facet_tri + 9 * static_cast<size_t>(k);
            const double area = cross2(T, T + 3, T + 6), tol = 1e-12 * fabs(area);
            const double e0 = cross2(T, T + 3, q), e1 = cross2(T + 3, T + 6, q), e2 = cross2(T + 6, T, q);
            if ((area > 0 && fmin(fmin(e0, e1), e2) >= -tol) || (area < 0 && fmax(fmax(e0, e1), e2) <= tol)) {
                best = dist;
                facet = f;
                for (int a = 0; a < 3; ++a) hit[a] = q[a];
                break;
            }
        }
    }
    t_out = best / speed;
}

// Wall trace of a mesh domain: the face BVH, or the facet scan of a prism.
__device__ inline void domain_trace_dev(const DevFacets& F, const double p[3], const double v[3], double hit[3],
                                        double& t_out, int& facet) {
    if (F.prism) prism_trace_dev(F, p, v, hit, t_out, facet);
    else mesh_trace_dev(F.mesh, p, v, hit, t_out, facet);
}

// Wall-hit cache with nudged retries on the mesh (src/solver/TransportOperator.cpp:186-250).
// Returns 0 on success, 3 on success from a nudged position, 1 when no retry
// found a wall, 2 on a membership overflow.
static __device__ __noinline__ int mesh_cache_hit(const DevFacets& F, const DevDomain& D, const DevParams& P, double p[3],
                                     const double v[3], double cp[3], double& t, int& f) {
    const double speed = meshmath::norm(v);
    if (isfinite(speed) && speed <= 1e-18) {
        for (int a = 0; a < 3; ++a) cp[a] = p[a];
        t = __longlong_as_double(0x7ff0000000000000LL);
        f = -1;
        return 0;
    }
    domain_trace_dev(F, p, v, cp, t, f);
    if (f >= 0 && isfinite(t)) return 0;
    const double eps = fmax(P.push_eps, 1e-10 * D.scale);
    double cand[4][3];
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < 3; ++a) cand[c][a] = p[a];
    const int nearest = mesh_nearest_facet(F, p);
    if (nearest >= 0) {
        const double* n = F.normal + 3 * nearest;
        for (int a = 0; a < 3; ++a) {
            cand[0][a] = __dadd_rn(p[a], __dmul_rn(n[a], eps));
            cand[1][a] = __dadd_rn(p[a], __dmul_rn(n[a], -eps));
        }
    }
    if (speed > 0.0 && isfinite(speed)) {
        const double inv = 1.0 / speed;
        for (int a = 0; a < 3; ++a) {
            const double d = __dmul_rn(v[a], inv);
            cand[2][a] = __dadd_rn(p[a], __dmul_rn(d, eps));
            cand[3][a] = __dadd_rn(p[a], __dmul_rn(d, -eps));
        }
    }
    for (int c = 0; c < 4; ++c) {
        const int in = mesh_contains(F, cand[c]);
        if (in < 0) return 2;
        if (!in) continue;
        domain_trace_dev(F, cand[c], v, cp, t, f);
        if (f >= 0 && isfinite(t)) {
            for (int a = 0; a < 3; ++a) p[a] = cand[c][a];
            return 3;
        }
    }
    return 1;
}

// Active cell of a point: the voxel, through the voxel map on mesh domains
// (src/SimulationDomain.cpp:92-126).
__device__ __forceinline__ int cell_at(const DevTables& T, double x, double y, double z) {
    const int v = grid_index(T.dom, x, y, z);
    return T.fac.voxel_cell ? __ldg(T.fac.voxel_cell + v) : v;
}

// Heat-source energy factor (ps) of [begin, end] under the time profile
// (src/solver/HeatSourceDriving.cpp:12-44), in the same rounding as the host.
__device__ __forceinline__ double source_time_factor(const DevParams& P, double begin_ps, double end_ps) {
    const double begin = fmax(begin_ps, P.source_time_start);
    const double end = P.source_time_end >= 0.0 ? fmin(end_ps, P.source_time_end) : end_ps;
    if (end <= begin) return 0.0;
    if (!P.source_pulsed) return __dmul_rn(P.source_amplitude, __dadd_rn(end, -begin));
    const double period = P.source_period, on = P.source_on;
    if (on <= 0.0) return 0.0;
    auto on_time = [&](double rel) {
        if (!(rel > 0.0)) return 0.0;
        const double cycles = floor(rel / period);
        return __dadd_rn(__dmul_rn(cycles, on), fmin(__dadd_rn(rel, -__dmul_rn(cycles, period)), on));
    };
    const double rb = __dadd_rn(begin, -P.source_time_start), re = __dadd_rn(end, -P.source_time_start);
    return __dmul_rn(P.source_amplitude, fmax(0.0, __dadd_rn(on_time(re), -on_time(rb))));
}

} // namespace phmc
