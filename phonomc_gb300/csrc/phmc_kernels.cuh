// Shared declarations of the kernel translation units and their launchers.
#pragma once
#include <cuda_runtime.h>

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
    bool mesh = false;   // surface-mesh domain (plain FP64 carrier state)
};

int launch_transport(const LaunchCtx& x, bool mixed, bool rta);
int launch_mesh_cache_init(const LaunchCtx& x);
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
void launch_containment(const LaunchCtx& x, bool mixed);
void launch_flux(const LaunchCtx& x, bool mixed);
void launch_apply_pending(const LaunchCtx& x, bool subtract_drive);
void launch_step_begin(const LaunchCtx& x);
// One heat-source half (time window from the device clock): accrue, deposit into the pending updates.
void launch_source(const LaunchCtx& x, bool final_temperature, bool next);
int launch_cell_solve(const LaunchCtx& x, int phase, int collision);
int linear_cluster_size(const CellArrays& C, bool mixed);
void prepare_linear_solve(const CellArrays& C);
void launch_cells_final(const LaunchCtx& x, int phase);

// collision kinds for launch_cell_solve
enum CollisionKind : int { kCollideNone = 0, kCollideRta = 1, kCollideLinear = 2 };


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
    std::vector<double> vv, nrm, bnd, nb;
    std::vector<int> ff, links;
    for (const auto& v : Tr.vertices) vv.insert(vv.end(), v.begin(), v.end());
    for (const auto& f : Tr.faces) ff.insert(ff.end(), f.begin(), f.end());
    for (const auto& x : Tr.normals) nrm.insert(nrm.end(), x.begin(), x.end());
    for (const auto& b : Tr.bounds) {
        bnd.insert(bnd.end(), b[0].begin(), b[0].end());
        bnd.insert(bnd.end(), b[1].begin(), b[1].end());
    }
    for (const auto& nd : Tr.nodes) {
        nb.insert(nb.end(), nd.bmin.begin(), nd.bmin.end());
        nb.insert(nb.end(), nd.bmax.begin(), nd.bmax.end());
        links.insert(links.end(), {nd.left, nd.right, nd.begin, nd.end});
    }
    DevMesh& D = G.mesh;
    D.vertices = up(vv);
    D.faces = up(ff);
    D.face_to_facet = up(Tr.face_to_facet);
    D.normals = up(nrm);
    D.k = up(Tr.k);
    D.bounds = up(bnd);
    D.node_bounds = up(nb);
    D.node_links = up(links);
    D.order = up(Tr.order);
    D.root = Tr.root;
    D.nfaces = static_cast<int>(Tr.faces.size());
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
