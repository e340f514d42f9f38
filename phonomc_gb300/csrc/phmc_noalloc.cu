// Box ray trace without any device allocation (phmc_dev_trace_box_noalloc).
//
// phmc_dev_trace_box stages its rays in buffers it allocates and frees on
// every call. cudaFree synchronizes the whole device, so a call made while a
// solver is stepping on another stream waits for that stream, and a process
// whose device memory is already held by another allocator (a caching
// allocator, a memory pool sized to the card) may have nothing left for
// cudaMalloc. This variant runs the same trace kernel body on one static
// device scratch block instead: no cudaMalloc, cudaFree or allocating library
// call on any path, and it waits only on its own non-blocking stream.
//
// Limits and sharing:
// * at most kNoAllocMaxRays rays per call; larger n is rejected before any
//   device work;
// * the scratch is one block per device, so calls must not overlap on a
//   device: the entry point holds a process-wide lock for the whole call, and
//   concurrent callers run one after another;
// * the first call on a device resolves the scratch address
//   (cudaGetSymbolAddress) and creates the stream; with lazy module loading
//   that first call is also when the driver places the module's static data,
//   so make it (n = 0 does only this setup) before any phase in which the
//   device must not allocate, e.g. before capturing a stream.
#include "phmc_kernels.cuh"

#include <mutex>
#include <stdexcept>
#include <string>

namespace phmc {

constexpr long long kNoAllocMaxRays = 1 << 16;
constexpr int kNoAllocMaxDevices = 64;

struct __align__(256) TraceScratch {
    double p[3 * kNoAllocMaxRays];
    double v[3 * kNoAllocMaxRays];
    double hit[3 * kNoAllocMaxRays];
    double t[kNoAllocMaxRays];
    int32_t facet[kNoAllocMaxRays];
    unsigned long long misses; // rays without a facet; must start at zero each call
};

// 65536 rays: 5.77 MB of static device memory
static __device__ __align__(256) TraceScratch g_trace_scratch;

__global__ void k_trace_rays_noalloc(DevDomain D, int n, TraceScratch* S) {
    unsigned long long missed = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p[3] = {S->p[3 * i], S->p[3 * i + 1], S->p[3 * i + 2]};
        const double v[3] = {S->v[3 * i], S->v[3 * i + 1], S->v[3 * i + 2]};
        double cp[3], tt;
        int f;
        trace_box(D, p, v, cp, tt, f);
        for (int a = 0; a < 3; ++a) S->hit[3 * i + a] = f >= 0 ? cp[a] : p[a];
        S->t[i] = tt;
        S->facet[i] = f;
        missed += f < 0 ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) missed += __shfl_xor_sync(0xffffffffu, missed, o);
    if ((threadIdx.x & 31) == 0 && missed) atomicAdd(&S->misses, missed);
}

namespace {
std::mutex g_noalloc_lock;
TraceScratch* g_scratch[kNoAllocMaxDevices] = {};
cudaStream_t g_stream[kNoAllocMaxDevices] = {};

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}
} // namespace

void trace_box_noalloc(const double lo[3], const double hi[3], long long n, const double* p3, const double* v3,
                       double* hit3, double* t, int32_t* facet, long long* misses) {
    if (n < 0 || n > kNoAllocMaxRays)
        throw std::invalid_argument("phmc_dev_trace_box_noalloc: n = " + std::to_string(n) + " outside [0, " +
                                    std::to_string(kNoAllocMaxRays) + "]");
    if (n > 0 && (!lo || !hi || !p3 || !v3 || !hit3 || !t || !facet))
        throw std::invalid_argument("phmc_dev_trace_box_noalloc: null array");
    std::lock_guard<std::mutex> hold(g_noalloc_lock);
    int dev = 0;
    check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw std::runtime_error("phmc_dev_trace_box_noalloc: device index out of range");
    if (!g_scratch[dev]) {
        void* addr = nullptr;
        check(cudaGetSymbolAddress(&addr, g_trace_scratch), "cudaGetSymbolAddress");
        if (!addr || (reinterpret_cast<uintptr_t>(addr) & 255u) != 0)
            throw std::runtime_error("phmc_dev_trace_box_noalloc: scratch address missing or misaligned");
        check(cudaStreamCreateWithFlags(&g_stream[dev], cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
        g_scratch[dev] = static_cast<TraceScratch*>(addr);
    }
    TraceScratch* S = g_scratch[dev];
    cudaStream_t st = g_stream[dev];
    if (misses) *misses = 0;
    if (n == 0) return;
    // Once copies are queued, an error must not return while they may still
    // read or write the caller's (possibly pinned) buffers: drain the stream
    // first, whatever its status.
    struct DrainOnThrow {
        cudaStream_t s;
        bool armed = true;
        ~DrainOnThrow() {
            if (armed) cudaStreamSynchronize(s);
        }
    } drain{st};
    DevDomain D{};
    double scale = 1.0;
    for (int a = 0; a < 3; ++a) {
        D.lo[a] = lo[a];
        D.hi[a] = hi[a];
        scale = std::max(scale, std::abs(hi[a] - lo[a]));
    }
    D.scale = scale;
    D.tol = std::max(1e-9, 64.0 * std::numeric_limits<double>::epsilon() * scale);
    const size_t n3 = 3 * static_cast<size_t>(n);
    check(cudaMemsetAsync(&S->misses, 0, sizeof(S->misses), st), "cudaMemsetAsync");
    check(cudaMemcpyAsync(S->p, p3, n3 * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    check(cudaMemcpyAsync(S->v, v3, n3 * sizeof(double), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    k_trace_rays_noalloc<<<256, 256, 0, st>>>(D, static_cast<int>(n), S);
    check(cudaGetLastError(), "k_trace_rays_noalloc");
    unsigned long long missed = 0;
    check(cudaMemcpyAsync(hit3, S->hit, n3 * sizeof(double), cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    check(cudaMemcpyAsync(t, S->t, static_cast<size_t>(n) * sizeof(double), cudaMemcpyDeviceToHost, st),
          "cudaMemcpyAsync");
    check(cudaMemcpyAsync(facet, S->facet, static_cast<size_t>(n) * sizeof(int32_t), cudaMemcpyDeviceToHost, st),
          "cudaMemcpyAsync");
    check(cudaMemcpyAsync(&missed, &S->misses, sizeof missed, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    const cudaError_t done = cudaStreamSynchronize(st);
    drain.armed = false;
    check(done, "cudaStreamSynchronize");
    if (misses) *misses = static_cast<long long>(missed);
}

} // namespace phmc
