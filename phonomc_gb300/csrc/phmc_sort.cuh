// Periodic carrier sort (phmc_sort.cu): scratch layout and launcher.
#pragma once
#include <cstddef>
#include <cstdint>

namespace phmc {

struct LaunchCtx;

// Device scratch of one sort, carved from a single allocation: keys and slot
// indices twice (ping-pong passes), the digit-major tile count table, the scan
// partials and an 8-byte-per-slot gather buffer.
struct SortScratch {
    uint32_t *k0 = nullptr, *k1 = nullptr, *v0 = nullptr, *v1 = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* partial = nullptr;
    void* tmp = nullptr;
    int capacity = 0;
    int ntiles = 0;
    static size_t bytes_for(int capacity);
    void carve(void* base, int capacity);
};

// Enqueues the stable sort of the carrier slots of `x` on its stream and the
// gather of every per-slot array (positions or cell offsets, occupation, mode,
// cell, alive, and the mesh wall cache). Keys: active mode * ncells + cell
// (cell * modes + mode when cell_major), dead slots last. Returns the number
// of kernels launched.
int launch_carrier_sort(const LaunchCtx& x, const SortScratch& s, int ncells, int modes, bool cell_major, bool mixed);

} // namespace phmc
