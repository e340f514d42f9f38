// Periodic carrier sort: a stable LSD radix sort of (key, slot) pairs over the
// carrier slots, then every per-slot array gathered through the permutation.
//
// The reference keeps a per-step counting-sort index of the carriers by cell
// (CellParticleIndex::ensure, src/solver/CellParticleIndex.cpp:14-44) and never
// moves their storage. Here the carrier pass reads the pending (alpha, beta)
// of each carrier's (cell, bin) and adds its occupation to the same record, so
// the storage itself is reordered every few steps: by (active mode, cell) in
// box domains -- carriers of one mode keep their mode until a wall resamples
// it and drift only a few cells per step, so a warp's table accesses stay in a
// few L2 lines for many steps -- and by (cell, mode) in mesh domains, where the
// cell also localises the BVH walk of the wall events. Dead slots sort last.
// The sort is stable, so the permutation is a function of the state alone and
// the CPU oracle reproduces it with std::stable_sort.
//
// Each pass of 8 key bits: per-tile digit histograms (k_radix_hist), one
// exclusive scan over the digit-major count table (k_scan_*), and a stable
// scatter (k_radix_scatter) in which a tile ranks its keys sweep by sweep with
// warp match masks and per-warp digit counts in shared memory.
#include "phmc_kernels.cuh"
#include "phmc_sort.cuh"

#include <type_traits>

namespace phmc {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortRounds = 16;
constexpr int kSortTile = kSortThreads * kSortRounds; // slots per tile
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

__global__ void __launch_bounds__(256) k_sort_keys(CarrierState S, const DevLedger* __restrict__ L,
                                                   uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                   int capacity, uint32_t ncells, uint32_t modes, int cell_major,
                                                   uint32_t dead) {
    const int n = L->n_slots;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < capacity; i += gridDim.x * blockDim.x) {
        uint32_t k = dead;
        if (i < n && S.alive[i]) {
            const uint32_t a = S.mode[i] & 0x00FFFFFFu;
            const uint32_t c = static_cast<uint32_t>(S.cell[i]);
            // a carrier with an out-of-range index has latched an error already;
            // it still gets a key below the dead ones
            if (a < modes && c < ncells) k = cell_major ? c * modes + a : a * ncells + c;
            else k = dead - 1u;
        }
        keys[i] = k;
        vals[i] = static_cast<uint32_t>(i);
    }
}

__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t* __restrict__ keys, int n, int shift,
                                                             uint32_t* __restrict__ counts, int ntiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const int base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortRounds; ++r) {
        const int i = base + r * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[static_cast<size_t>(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Inclusive scan of one value per thread across the block (kScanThreads).
__device__ __forceinline__ uint32_t block_inclusive_scan(uint32_t v, uint32_t* warp_tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = lane < kScanThreads / 32 ? warp_tot[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kScanThreads / 32) warp_tot[lane] = t;
    }
    __syncthreads();
    const uint32_t r = v + (warp > 0 ? warp_tot[warp - 1] : 0u);
    __syncthreads(); // warp_tot is reused by the caller's next scan
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* __restrict__ a, int m,
                                                              uint32_t* __restrict__ partial) {
    __shared__ uint32_t wt[32];
    const int base = blockIdx.x * kScanChunk;
    uint32_t s = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k * kScanThreads + threadIdx.x;
        if (i < m) s += a[i];
    }
    s = block_inclusive_scan(s, wt);
    if (threadIdx.x == kScanThreads - 1) partial[blockIdx.x] = s;
}

// Exclusive scan of the chunk sums in place, one block, groups of kScanThreads.
__global__ void __launch_bounds__(kScanThreads) k_scan_top(uint32_t* __restrict__ partial, int nb) {
    __shared__ uint32_t wt[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (int g = 0; g < nb; g += kScanThreads) {
        const int i = g + threadIdx.x;
        const uint32_t v = i < nb ? partial[i] : 0u;
        const uint32_t inc = block_inclusive_scan(v, wt);
        const uint32_t c = carry;
        if (i < nb) partial[i] = c + inc - v;
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry = c + inc;
        __syncthreads();
    }
}

// Exclusive scan of each chunk (four consecutive values per thread) plus its offset.
__global__ void __launch_bounds__(kScanThreads) k_scan_down(uint32_t* __restrict__ a, int m,
                                                            const uint32_t* __restrict__ partial) {
    __shared__ uint32_t wt[32];
    const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t t = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < m ? a[base + k] : 0u;
        t += v[k];
    }
    uint32_t run = block_inclusive_scan(t, wt) - t + partial[blockIdx.x];
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) a[base + k] = run;
        run += v[k];
    }
}

// Stable scatter of one tile: items in slot order (sweep of the CTA over the
// tile, warp, lane); a key's destination is its digit's offset for this tile,
// plus the digit's items in earlier sweeps, earlier warps of this sweep, and
// earlier lanes of its warp.
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ vin,
                                                                uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                                int n, int shift, const uint32_t* __restrict__ offsets,
                                                                int ntiles) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t whist[kSortWarps][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = offsets[static_cast<size_t>(tid) * ntiles + blockIdx.x];
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kSortRounds; ++r) {
        for (int w = 0; w < kSortWarps; ++w) whist[w][tid] = 0u;
        const int i = blockIdx.x * kSortTile + r * kSortThreads + tid;
        const bool valid = i < n;
        const uint32_t k = valid ? kin[i] : 0u;
        const uint32_t v = valid ? vin[i] : 0u;
        const uint32_t d = (k >> shift) & 255u;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 256u);
        const uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0u) whist[warp][d] = __popc(peers);
        __syncthreads();
        uint32_t s = 0u;
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = whist[w][tid];
            whist[w][tid] = s;
            s += c;
        }
        __syncthreads();
        if (valid) {
            const uint32_t pos = base[d] + whist[warp][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        base[tid] += s;
    }
}

// The per-slot arrays of a carrier population and their sorted copies.
struct SlotFields {
    int count;
    unsigned char* cur[kSortMaxFields];
    unsigned char* alt[kSortMaxFields];
    int size[kSortMaxFields]; // bytes per slot: 1, 4 or 8
};

__device__ __forceinline__ void copy_slot(unsigned char* dst, const unsigned char* src, int size, size_t to,
                                          size_t from) {
    if (size == 8) reinterpret_cast<unsigned long long*>(dst)[to] = reinterpret_cast<const unsigned long long*>(src)[from];
    else if (size == 4) reinterpret_cast<unsigned*>(dst)[to] = reinterpret_cast<const unsigned*>(src)[from];
    else dst[to] = src[from];
}

// Every field of slot perm[i] into slot i of the sorted copies (one read of the permutation).
__global__ void __launch_bounds__(256) k_gather_fields(const uint32_t* __restrict__ perm, const SlotFields F, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t from = perm[i];
        for (int f = 0; f < F.count; ++f) copy_slot(F.alt[f], F.cur[f], F.size[f], static_cast<size_t>(i), from);
    }
}

// The sorted copies back into the carrier arrays (the arrays keep their
// addresses, so captured step graphs stay valid).
__global__ void __launch_bounds__(256) k_copy_fields(const SlotFields F, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int f = 0; f < F.count; ++f) copy_slot(F.cur[f], F.alt[f], F.size[f], static_cast<size_t>(i),
                                                    static_cast<size_t>(i));
}

int bit_length(uint32_t v) {
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

} // namespace

size_t SortScratch::bytes_for(int capacity, int slot_bytes) {
    const size_t ntiles = (static_cast<size_t>(capacity) + kSortTile - 1) / kSortTile;
    const size_t m = 256 * ntiles;
    const size_t nb = (m + kScanChunk - 1) / kScanChunk;
    return 4 * 4 * static_cast<size_t>(capacity) + 4 * (m + nb) +
           static_cast<size_t>(slot_bytes) * static_cast<size_t>(capacity) + (8 + kSortMaxFields) * 256;
}

void SortScratch::carve(void* base, int cap, int slot_bytes_) {
    capacity = cap;
    slot_bytes = slot_bytes_;
    ntiles = (cap + kSortTile - 1) / kSortTile;
    const size_t m = 256 * static_cast<size_t>(ntiles);
    const size_t nb = (m + kScanChunk - 1) / kScanChunk;
    auto* p = static_cast<unsigned char*>(base);
    auto take = [&](size_t bytes) {
        void* q = p;
        p += (bytes + 255) & ~size_t{255};
        return q;
    };
    alt = static_cast<unsigned char*>(take(static_cast<size_t>(slot_bytes) * static_cast<size_t>(cap) +
                                          kSortMaxFields * 256));
    k0 = static_cast<uint32_t*>(take(4 * static_cast<size_t>(cap)));
    k1 = static_cast<uint32_t*>(take(4 * static_cast<size_t>(cap)));
    v0 = static_cast<uint32_t*>(take(4 * static_cast<size_t>(cap)));
    v1 = static_cast<uint32_t*>(take(4 * static_cast<size_t>(cap)));
    counts = static_cast<uint32_t*>(take(4 * m));
    partial = static_cast<uint32_t*>(take(4 * nb));
}

// Visits every per-slot array that a sort moves: positions (FP64) or cell
// offsets (FP32), occupation, mode, cell, alive, and in mesh domains the mirror
// facet and the wall cache.
template <class Visit> void slot_arrays(const LaunchCtx& x, bool mixed, Visit&& visit) {
    if (mixed) {
        visit(x.S.ox);
        visit(x.S.oy);
        visit(x.S.oz);
    } else {
        visit(x.S.x);
        visit(x.S.y);
        visit(x.S.z);
    }
    visit(x.S.occ);
    visit(x.S.mode);
    visit(x.S.cell);
    visit(x.S.alive);
    if (x.mesh) {
        const DevFacets& M = x.Th->fac;
        visit(M.mirror);
        visit(M.hit_t);
        visit(M.hit_x);
        visit(M.hit_y);
        visit(M.hit_z);
        visit(M.hit_f);
    }
}

int launch_carrier_sort(const LaunchCtx& x, const SortScratch& s, int ncells, int modes, bool cell_major, bool mixed) {
    const int cap = x.S.capacity;
    if (cap != s.capacity) throw std::runtime_error("carrier sort scratch does not match the carrier capacity");
    const uint64_t span = static_cast<uint64_t>(ncells) * static_cast<uint64_t>(modes);
    if (span + 1 >= (1ull << 32)) throw std::runtime_error("carrier sort key exceeds 32 bits (cells x modes)");
    // live keys are below span; an out-of-range carrier gets span, dead slots span + 1
    const uint32_t dead = static_cast<uint32_t>(span) + 1u;
    const int bits = bit_length(dead);
    const int passes = (bits + 7) / 8;
    const int g = x.grid_blocks;
    int launches = 0;
    k_sort_keys<<<g, 256, 0, x.stream>>>(x.S, x.L, s.k0, s.v0, cap, static_cast<uint32_t>(ncells),
                                         static_cast<uint32_t>(modes), cell_major ? 1 : 0, dead);
    ++launches;
    const int m = 256 * s.ntiles;
    const int nb = (m + kScanChunk - 1) / kScanChunk;
    uint32_t *kin = s.k0, *vin = s.v0, *kout = s.k1, *vout = s.v1;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<<<s.ntiles, kSortThreads, 0, x.stream>>>(kin, cap, shift, s.counts, s.ntiles);
        k_scan_reduce<<<nb, kScanThreads, 0, x.stream>>>(s.counts, m, s.partial);
        k_scan_top<<<1, kScanThreads, 0, x.stream>>>(s.partial, nb);
        k_scan_down<<<nb, kScanThreads, 0, x.stream>>>(s.counts, m, s.partial);
        k_radix_scatter<<<s.ntiles, kSortThreads, 0, x.stream>>>(kin, vin, kout, vout, cap, shift, s.counts,
                                                                 s.ntiles);
        launches += 5;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    const uint32_t* perm = vin;
    SlotFields F{};
    size_t offset = 0;
    auto field = [&](auto* arr) {
        using T = std::remove_pointer_t<decltype(arr)>;
        if (!arr) return;
        if (F.count >= kSortMaxFields) throw std::runtime_error("too many carrier arrays for the sort");
        F.cur[F.count] = reinterpret_cast<unsigned char*>(arr);
        F.alt[F.count] = s.alt + offset;
        F.size[F.count] = static_cast<int>(sizeof(T));
        offset += (sizeof(T) * static_cast<size_t>(cap) + 255) & ~size_t{255};
        ++F.count;
    };
    slot_arrays(x, mixed, field);
    if (offset > static_cast<size_t>(s.slot_bytes) * static_cast<size_t>(cap) + kSortMaxFields * 256)
        throw std::runtime_error("carrier sort scratch is smaller than the carrier arrays");
    k_gather_fields<<<g, 256, 0, x.stream>>>(perm, F, cap);
    k_copy_fields<<<g, 256, 0, x.stream>>>(F, cap);
    return launches + 2;
}

int carrier_slot_bytes(const LaunchCtx& x, bool mixed) {
    int bytes = 0;
    slot_arrays(x, mixed, [&](auto* arr) {
        if (arr) bytes += static_cast<int>(sizeof(*arr));
    });
    return bytes;
}

} // namespace phmc
