// Periodic carrier sort (phmc_sort.cu): scratch layout and launcher.
#pragma once
#include <cstddef>
#include <cstdint>

namespace phmc {

struct LaunchCtx;

constexpr int kSortMaxFields = 14;

// Device scratch of one sort, carved from a single allocation: keys and slot
// indices twice (ping-pong passes), the digit-major tile count table, the scan
// partials and a sorted copy of every per-slot array (slot_bytes per slot).
struct SortScratch {
    uint32_t *k0 = nullptr, *k1 = nullptr, *v0 = nullptr, *v1 = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* partial = nullptr;
    unsigned char* alt = nullptr;
    int capacity = 0;
    int slot_bytes = 0;
    int ntiles = 0;
    static size_t bytes_for(int capacity, int slot_bytes);
    void carve(void* base, int capacity, int slot_bytes);
};

// Bytes per slot of the arrays a sort moves.
int carrier_slot_bytes(const LaunchCtx& x, bool mixed);

// Enqueues the stable sort of the carrier slots of `x` on its stream and the
// gather of every per-slot array (positions or cell offsets, occupation, mode,
// cell, alive, and the mesh wall cache). Keys: active mode * ncells + cell
// (cell * modes + mode when cell_major), dead slots last. Returns the number
// of kernels launched.
int launch_carrier_sort(const LaunchCtx& x, const SortScratch& s, int ncells, int modes, bool cell_major, bool mixed);

} // namespace phmc
