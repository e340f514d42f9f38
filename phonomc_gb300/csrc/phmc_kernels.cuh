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
    const DevTables* T;
    CarrierState S;
    CellArrays C;
    DevLedger* L;
    cudaStream_t stream;
    int grid_blocks;
};

void launch_transport(const LaunchCtx& x, bool gradient, bool rta, uint32_t step);
void launch_transport_mixed(const LaunchCtx& x, bool gradient, uint32_t step);
void launch_histogram(const LaunchCtx& x, bool rta);
void launch_init_cells(const LaunchCtx& x);
int launch_inject(const LaunchCtx& x, bool rta, int* holes, int* block_dead, int capacity, uint32_t step);
void launch_containment(const LaunchCtx& x);
void launch_flux(const LaunchCtx& x);
void launch_step_begin(const LaunchCtx& x);
void launch_cell_solve(const LaunchCtx& x, int phase, int collision, int n_classes, const int* class_start,
                       const int* class_modes, double* lin_scratch);
void launch_update(const LaunchCtx& x, int collision, bool gradient);
void launch_cells_final(const LaunchCtx& x, int initial);

// collision kinds for launch_cell_solve / launch_update
enum CollisionKind : int { kCollideNone = 0, kCollideRta = 1, kCollideLinear = 2 };

} // namespace phmc
