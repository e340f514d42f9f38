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
};

int launch_transport(const LaunchCtx& x, bool mixed, bool rta);
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

} // namespace phmc
