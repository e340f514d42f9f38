// Shared declarations of the kernel translation units and their launchers.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "phmc_device.cuh"
#include "phmc_solver.h"

namespace phmc {

// Unfused FP64 add/multiply: the plain path keeps the host's rounding order so
// the device trajectory can be compared with the CPU oracle term by term.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

struct LaunchCtx {
    const DevTables* T;  // device copy
    const DevTables* Th; // host copy, passed by value to the carrier kernels
    CarrierState S;
    CellArrays C;
    DevLedger* L;
    cudaStream_t stream;
    int grid_blocks;
    int event_grid = 1; // CTAs per SM x SMs of one resident wave of the event kernels (x1 per SM)
    bool mesh = false;   // surface-mesh domain (plain FP64 carrier state)
    const DevNcl* ncl = nullptr; // host copy, nonlinear Callaway only
    unsigned char* lin_work = nullptr; // linear Callaway: per-CTA mode slices in global memory (null: shared)
    size_t lin_slice = 0;              // bytes per CTA slice of lin_work
    // carrier pass of box domains (k_transport): threads per CTA, CTAs, warp-summed bin tallies
    int transport_block = 256;
    int transport_grid = 1;
    bool tally_agg = true;
    bool transport_pipe = false; // mixed state: TMA-staged carrier tiles (k_transport_pipe)
    int pipe_grid = 1;
};

// Independent box instances advanced by one launch per kernel of the step:
// per-instance device state behind arrays, and prefix sums that assign each
// CTA of a fused launch to an instance (the instance's own grid of CTAs).
// Modes per CTA of the per-(cell, mode) statistics and table kernels.
constexpr int kStatChunk = 4096;

struct BatchDesc {
    int n;                            // instances
    const DevTables* const* tables;   // [n] device copies of each instance's tables
    const CarrierState* states;       // [n]
    const CellArrays* cells;          // [n]
    DevLedger* const* ledgers;        // [n]
    int* const* holes;                // [n] free-slot lists
    int* const* hole_counts;          // [n] per-CTA dead counts of the slot scan
    const int* capacity;              // [n]
    const int* carrier_block;         // [n+1] CTAs of the carrier kernels
    const int* hole_block;            // [n+1] CTAs of the slot scan (1024 threads)
    const int* cell_begin;            // [n+1] cells
    const int* cell_block;            // [n+1] CTAs of the per-cell thread kernels (256 threads)
    const int* inject_block;          // [n+1] CTAs of the injection kernel
    int total_carrier_blocks, total_hole_blocks, total_cells, total_cell_blocks, total_inject_blocks;
    int chunks;                       // mode chunks of the widest instance
    int persist;                      // resident CTAs of the persistent carrier kernels
    int rta_cap;                      // occupied-class list of the fused RTA cell update (0: separate kernels)
};

// Instance owning index x of a prefix-sum array: the last i with prefix[i] <= x.
__device__ __forceinline__ int batch_find(const int* prefix, int n, int x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The launches of one fused timestep of `D` (nonlinear RTA box instances with
// reservoirs): transport, injection, cell solve, ledger. Returns the launch count.
int launch_fused_step(const BatchDesc& D, cudaStream_t stream, bool mixed);
int launch_fused_transport(const BatchDesc& D, cudaStream_t stream, bool mixed);
int launch_fused_cells(const BatchDesc& D, cudaStream_t stream);

int launch_transport(const LaunchCtx& x, bool mixed, bool rta);
int launch_mesh_cache_init(const LaunchCtx& x, bool mixed);
// The specular-match scan of the rough-table build on the device (phmc_rough.cu).
void spec_match_device(const std::vector<Vec3>& velocities, std::vector<SpecMatchJob>& jobs, cudaStream_t stream);
void launch_histogram(const LaunchCtx& x, bool rta);
void launch_init_cells(const LaunchCtx& x, bool mixed);
// Carriers read straight from device-accessible (registered) host arrays.
struct HostCarriers {
    const double *x, *y, *z, *occ;
    const uint32_t* mode;
    const uint8_t* alive; // null: all alive
};
void launch_ingest(const LaunchCtx& x, bool mixed, const HostCarriers& h);
void launch_ledger_replace(const LaunchCtx& x, int n);
void launch_positions_out(const LaunchCtx& x);
int launch_inject(const LaunchCtx& x, bool mixed, bool rta, int* holes, int* block_dead, int capacity);
// Containment check of the live carriers; mesh carriers outside the interior
// voxels are queued in `queue` (capacity: the slots) for the membership test.
int launch_containment(const LaunchCtx& x, bool mixed, int* queue, int* count);
void launch_flux(const LaunchCtx& x, bool mixed);
void launch_apply_pending(const LaunchCtx& x, bool subtract_drive);
void launch_step_begin(const LaunchCtx& x);
// One heat-source half (time window from the device clock): accrue, deposit into the pending updates.
void launch_source(const LaunchCtx& x, bool final_temperature, bool next);
int launch_cell_solve(const LaunchCtx& x, int phase, int collision);
void launch_mesh_initial_positions(const LaunchCtx& x, int n, uint64_t seed, const double lo[3], const double hi[3],
                                   double* xyz);
void launch_ncl_cell(int n_modes, const double* omega, const double* k3, const double* rn, const double* rr,
                     double* cnt, double2* ab, double2* work, int64_t n, const int32_t* mode, double* occ, double T,
                     double dt, int* status, cudaStream_t s);
int linear_cluster_size(const CellArrays& C, bool mixed);
void prepare_linear_solve(const CellArrays& C, bool global);
size_t linear_global_slice(const CellArrays& C, bool mixed);
void launch_cells_final(const LaunchCtx& x, int phase);
// Every 64th entry of a rough table's residual prefix (the first level of the
// device's two-level diffuse search).
inline std::vector<double> coarse_prefix(const std::vector<double>& prefix) {
    std::vector<double> c;
    for (size_t k = 0; k < prefix.size(); k += 64) c.push_back(prefix[k]);
    return c;
}

// Occupied-class list entries per warp of the fused RTA cell kernel for these
// cell arrays (0: separate kernels). mode 1 forces it where the classes fit,
// < 0 turns it off, 0 takes it on grids of 1024 cells or more.
int rta_cell_capacity(const CellArrays& C, int mode);
void prepare_rta_cell(const CellArrays& C);

// collision kinds for launch_cell_solve
enum CollisionKind : int { kCollideNone = 0, kCollideRta = 1, kCollideLinear = 2, kCollideNonlinear = 3 };



// Device layout of a face BVH (DevMesh): nodes renumbered breadth-first, face
// records in the leaf order of the traversal (input order without a BVH).
template <class Upload>
void fill_dev_mesh(const MeshTracer& Tr, DevMesh& D, Upload&& up) {
    const int nf = static_cast<int>(Tr.faces.size());
    std::vector<int> order(nf);
    for (int i = 0; i < nf; ++i) order[i] = Tr.root >= 0 ? Tr.order[i] : i;
    std::vector<double> rec(static_cast<size_t>(nf) * kFaceRecord);
    std::vector<int> facet(nf), id(nf);
    for (int pos = 0; pos < nf; ++pos) {
        const int f = order[pos];
        double* r = rec.data() + static_cast<size_t>(pos) * kFaceRecord;
        for (int a = 0; a < 3; ++a) {
            r[a] = Tr.normals[f][a];
            r[4 + a] = Tr.bounds[f][0][a];
            r[7 + a] = Tr.bounds[f][1][a];
            for (int k = 0; k < 3; ++k) r[10 + 3 * k + a] = Tr.vertices[Tr.faces[f][k]][a];
        }
        r[3] = Tr.k[f];
        facet[pos] = Tr.face_to_facet[f];
        id[pos] = f;
    }
    std::vector<DevBvhNode> nodes;
    if (Tr.root >= 0) {
        std::vector<int> renum(Tr.nodes.size(), -1), bfs;
        bfs.push_back(Tr.root);
        renum[Tr.root] = 0;
        for (size_t k = 0; k < bfs.size(); ++k) {
            const auto& nd = Tr.nodes[bfs[k]];
            for (int child : {nd.left, nd.right})
                if (child >= 0) {
                    renum[child] = static_cast<int>(bfs.size());
                    bfs.push_back(child);
                }
        }
        nodes.resize(bfs.size());
        for (size_t k = 0; k < bfs.size(); ++k) {
            const auto& nd = Tr.nodes[bfs[k]];
            DevBvhNode& o = nodes[k];
            for (int a = 0; a < 3; ++a) {
                o.bmin[a] = nd.bmin[a];
                o.bmax[a] = nd.bmax[a];
            }
            o.left = nd.left >= 0 ? renum[nd.left] : -1;
            o.right = nd.right >= 0 ? renum[nd.right] : -1;
            o.begin = nd.begin;
            o.end = nd.end;
        }
    }
    // FP32 culling copies: bounds rounded outward, margin for the walk's rounding
    auto down = [](double x) {
        float f = static_cast<float>(x);
        return static_cast<double>(f) > x ? std::nextafter(f, -std::numeric_limits<float>::infinity()) : f;
    };
    auto upf = [](double x) {
        float f = static_cast<float>(x);
        return static_cast<double>(f) < x ? std::nextafter(f, std::numeric_limits<float>::infinity()) : f;
    };
    std::vector<DevBvhNode32> nodes32(nodes.size());
    for (size_t k = 0; k < nodes.size(); ++k) {
        for (int a = 0; a < 3; ++a) {
            nodes32[k].bmin[a] = down(nodes[k].bmin[a]);
            nodes32[k].bmax[a] = upf(nodes[k].bmax[a]);
        }
        nodes32[k].left = nodes[k].left;
        nodes32[k].right = nodes[k].right;
        nodes32[k].begin = nodes[k].begin;
        nodes32[k].end = nodes[k].end;
    }
    std::vector<float> rec32(static_cast<size_t>(nf) * kFaceRecord32);
    double scale = 1.0;
    for (int pos = 0; pos < nf; ++pos) {
        const double* r = rec.data() + static_cast<size_t>(pos) * kFaceRecord;
        float* o = rec32.data() + static_cast<size_t>(pos) * kFaceRecord32;
        for (int q = 0; q < 4; ++q) o[q] = static_cast<float>(r[q]);
        for (int a = 0; a < 3; ++a) {
            o[4 + a] = down(r[4 + a]);
            o[7 + a] = upf(r[7 + a]);
            scale = std::max({scale, std::abs(r[4 + a]), std::abs(r[7 + a])});
        }
        // edge functions: inward in-plane unit normals of AB, BC, CA (FP64, then rounded)
        const double* V = r + 10;
        auto sub3 = [](const double* a, const double* b, double* o3) {
            for (int k = 0; k < 3; ++k) o3[k] = a[k] - b[k];
        };
        auto cross3 = [](const double* a, const double* b, double* o3) {
            o3[0] = a[1] * b[2] - a[2] * b[1];
            o3[1] = a[2] * b[0] - a[0] * b[2];
            o3[2] = a[0] * b[1] - a[1] * b[0];
        };
        double ab[3], ac[3], nrm[3];
        sub3(V + 3, V, ab);
        sub3(V + 6, V, ac);
        cross3(ab, ac, nrm);
        for (int e = 0; e < 3; ++e) {
            const double* P0 = V + 3 * e;
            const double* P1 = V + 3 * ((e + 1) % 3);
            double d[3], m[3];
            sub3(P1, P0, d);
            cross3(nrm, d, m);
            const double len = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
            float* q = o + 10 + 4 * e;
            if (!(len > 0.0) || !std::isfinite(len)) { // no edge test: never rejects
                q[0] = q[1] = q[2] = 0.0f;
                q[3] = -1e30f;
                continue;
            }
            for (int k = 0; k < 3; ++k) q[k] = static_cast<float>(m[k] / len);
            q[3] = static_cast<float>((m[0] * P0[0] + m[1] * P0[1] + m[2] * P0[2]) / len);
        }
    }
    D.nodes32 = nodes32.empty() ? nullptr : up(nodes32);
    D.face32 = up(rec32);
    D.margin = static_cast<float>(1e-6 * scale + 1e-4);
    D.nodes = up(nodes);
    D.face = up(rec);
    D.face_facet = up(facet);
    D.face_id = up(id);
    D.root = Tr.root >= 0 ? 0 : -1;
    D.nfaces = nf;
    D.nnodes = static_cast<int>(nodes.size());
}

// Device copy of a mesh domain's geometry: facet conditions, partners, shifts
// and normals, the voxel -> cell map, the faces with their BVH and the star
// simplices. `up(std::vector<T>)` returns a device pointer holding the vector.
template <class Upload>
void fill_dev_facets(const SimulationDomain& dom, double scale, DevFacets& G, Upload&& up) {
    const auto& F = dom.facets();
    const SurfaceMesh& M = *dom.mesh();
    const MeshTracer& Tr = M.tracer();
    const int nf = static_cast<int>(F.size());
    std::vector<char> cond(nf);
    std::vector<int> pair(nf), res(nf);
    std::vector<double> shift(3 * static_cast<size_t>(nf)), normal(3 * static_cast<size_t>(nf));
    for (int f = 0; f < nf; ++f) {
        cond[f] = F[f].condition;
        pair[f] = F[f].pair;
        res[f] = F[f].reservoir;
        for (int a = 0; a < 3; ++a) {
            shift[3 * f + a] = F[f].shift[a];
            normal[3 * f + a] = F[f].normal[a];
        }
    }
    G.n = nf;
    G.cond = up(cond);
    G.pair = up(pair);
    G.reservoir = up(res);
    G.shift = up(shift);
    G.normal = up(normal);
    G.voxel_cell = up(dom.voxel_cells());
    G.cell_voxel = up(dom.cell_voxels());
    if (!dom.voxel_interior().empty()) G.voxel_interior = up(dom.voxel_interior());
    G.prism = dom.is_prism() ? 1 : 0;
    if (dom.is_prism()) {
        std::vector<double> centroid(3 * static_cast<size_t>(nf)), tri;
        std::vector<int> begin(nf + 1, 0);
        for (int f = 0; f < nf; ++f) {
            for (int a = 0; a < 3; ++a) centroid[3 * f + a] = F[f].centroid[a];
            for (const auto& t : F[f].tris)
                for (int k = 0; k < 3; ++k)
                    for (int a = 0; a < 3; ++a) tri.push_back(t[k][a]);
            begin[f + 1] = static_cast<int>(tri.size() / 9);
        }
        G.facet_centroid = up(centroid);
        G.facet_face_begin = up(begin);
        G.facet_tri = up(tri);
    }
    fill_dev_mesh(Tr, G.mesh, up);
    std::vector<double> sx;
    for (const auto& S : M.simplices()) {
        sx.insert(sx.end(), S.v[0].begin(), S.v[0].end());
        for (int r = 0; r < 3; ++r) sx.insert(sx.end(), S.inv[r].begin(), S.inv[r].end());
        sx.insert(sx.end(), S.bounds[0].begin(), S.bounds[0].end());
        sx.insert(sx.end(), S.bounds[1].begin(), S.bounds[1].end());
    }
    G.n_simplex = static_cast<int>(M.simplices().size());
    G.simplex = up(sx);
    G.ray_pad = 1e-9 * scale;
}

} // namespace phmc
