// Specular-match scan of the rough-table build on the device
// (src/solver/RoughBoundarySampler.cpp:286-310, the O(modes x window) part of
// RoughBoundarySampler::build). For every incoming mode of every rough facet
// the host hands over its window [begin, end) of the facet's outgoing modes
// in frequency order; the match is the first mode of the window that
// minimises |v_try - v_out| / max(1e-12, |v_try|, |v_out|).
//
// One warp per incoming mode. GB300's FP64 rate is a small fraction of its
// FP32 rate, so the warp first takes the window's smallest metric in FP32
// (m32, within 7.2e-7 + 3e-7 m of the FP64 metric, bound below), then
// evaluates only the modes with m32 <= min + 2.5e-6 + 1e-6 min in FP64, in the
// host's operation order, and keeps the first minimum in window order: the
// same mode the host loop picks.
//
// Bound: with u = 2^-24, rounding v_try and v_out to FP32 moves each component
// of their difference by u(|v_try| + |v_out|) and the FP32 difference, norms,
// maximum and quotient add a few u relative, so |m32 - m| <= 12u + 5u m with
// the denominator >= max(|v_try|, |v_out|). The exact minimiser m* then has
// m32 <= m* + eps(m*) and the FP32 minimum is >= m* - eps(m*), so the
// threshold (3.5 eps) keeps every mode whose FP64 metric equals m*.
#include "phmc_kernels.cuh"

#include <algorithm>
#include <climits>
#include <stdexcept>
#include <string>

namespace phmc {
namespace {

struct SpecTask {
    int list;  // offset of the facet's sorted outgoing list in `lists`
    int begin; // window within that list
    int end;
    int ai;    // incoming active mode
    int job;   // facet (its inward normal in `nin`)
};

__device__ __forceinline__ float metric32(const float vt[3], float nt, float4 v) {
    const float dx = vt[0] - v.x, dy = vt[1] - v.y, dz = vt[2] - v.z;
    const float num = sqrtf(dx * dx + dy * dy + dz * dz);
    const float den = fmaxf(fmaxf(1e-12f, nt), sqrtf(v.x * v.x + v.y * v.y + v.z * v.z));
    return num / den;
}

__device__ __forceinline__ double norm64(const double a[3]) {
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[0], a[0]), __dmul_rn(a[1], a[1])), __dmul_rn(a[2], a[2])));
}

__global__ void __launch_bounds__(256) k_spec_match(const double* __restrict__ v64, const float4* __restrict__ v32,
                                                    const double* __restrict__ nin, const int* __restrict__ lists,
                                                    const SpecTask* __restrict__ tasks, int ntasks,
                                                    int* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int nwarps = static_cast<int>((gridDim.x * blockDim.x) >> 5);
    for (int t = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5); t < ntasks; t += nwarps) {
        const SpecTask T = tasks[t];
        const double* n = nin + 3 * static_cast<size_t>(T.job);
        const double* vi = v64 + 3 * static_cast<size_t>(T.ai);
        // v_try = v - n (2 (v . n)), rounded as the host computes it
        const double vdn = __dadd_rn(__dadd_rn(__dmul_rn(vi[0], n[0]), __dmul_rn(vi[1], n[1])), __dmul_rn(vi[2], n[2]));
        const double s2 = __dmul_rn(2.0, vdn);
        double vt[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) vt[a] = __dadd_rn(vi[a], -__dmul_rn(n[a], s2));
        const double nt = norm64(vt);
        const float vt32[3] = {static_cast<float>(vt[0]), static_cast<float>(vt[1]), static_cast<float>(vt[2])};
        const float nt32 = static_cast<float>(nt);
        const int* L = lists + T.list;
        float mmin = __int_as_float(0x7f800000);
        for (int pos = T.begin + lane; pos < T.end; pos += 32) mmin = fminf(mmin, metric32(vt32, nt32, v32[L[pos]]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mmin = fminf(mmin, __shfl_xor_sync(0xffffffffu, mmin, o));
        const float thr = mmin + 2.5e-6f + 1e-6f * mmin;
        double best = __longlong_as_double(0x7ff0000000000000LL);
        int bpos = INT_MAX;
        for (int pos = T.begin + lane; pos < T.end; pos += 32) {
            const int ao = L[pos];
            if (!(metric32(vt32, nt32, v32[ao]) <= thr)) continue;
            const double* vo = v64 + 3 * static_cast<size_t>(ao);
            const double dv[3] = {__dadd_rn(vt[0], -vo[0]), __dadd_rn(vt[1], -vo[1]), __dadd_rn(vt[2], -vo[2])};
            const double ref = fmax(fmax(1e-12, nt), norm64(vo));
            const double m = __ddiv_rn(norm64(dv), ref);
            if (m < best) { // lanes walk their positions in ascending order
                best = m;
                bpos = pos;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, bpos, o);
            if (ob < best || (ob == best && op < bpos)) {
                best = ob;
                bpos = op;
            }
        }
        if (lane == 0) out[t] = bpos != INT_MAX ? L[bpos] : -1;
    }
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e) + " at " + what);
}

// Device buffer of one chunk, freed on scope exit.
template <class T> struct Buf {
    T* p = nullptr;
    explicit Buf(size_t n) { check(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)), "cudaMalloc"); }
    ~Buf() { cudaFree(p); }
    Buf(const Buf&) = delete;
    Buf& operator=(const Buf&) = delete;
};

} // namespace

void spec_match_device(const std::vector<Vec3>& va, std::vector<SpecMatchJob>& jobs, cudaStream_t stream) {
    const size_t na = va.size();
    if (jobs.empty() || na == 0) return;
    std::vector<double> v64(3 * na);
    std::vector<float4> v32(na);
    for (size_t a = 0; a < na; ++a) {
        for (int k = 0; k < 3; ++k) v64[3 * a + k] = va[a][k];
        v32[a] = make_float4(static_cast<float>(va[a][0]), static_cast<float>(va[a][1]), static_cast<float>(va[a][2]),
                             0.0f);
    }
    Buf<double> d64(v64.size());
    Buf<float4> d32(v32.size());
    check(cudaMemcpyAsync(d64.p, v64.data(), v64.size() * sizeof(double), cudaMemcpyHostToDevice, stream), "copy");
    check(cudaMemcpyAsync(d32.p, v32.data(), v32.size() * sizeof(float4), cudaMemcpyHostToDevice, stream), "copy");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int grid = std::max(1, sms) * 8;
    // facets in chunks of at most ~4M incoming modes
    constexpr size_t kChunkTasks = size_t{1} << 22;
    size_t j0 = 0;
    while (j0 < jobs.size()) {
        std::vector<SpecTask> tasks;
        std::vector<int> lists;
        std::vector<double> nin;
        size_t j1 = j0;
        while (j1 < jobs.size() && (j1 == j0 || tasks.size() + jobs[j1].incoming->size() <= kChunkTasks)) {
            const SpecMatchJob& J = jobs[j1];
            const int list = static_cast<int>(lists.size());
            if (lists.size() + J.sorted->size() > static_cast<size_t>(INT_MAX))
                throw std::runtime_error("specular-match scan: outgoing lists exceed 2^31 entries");
            lists.insert(lists.end(), J.sorted->begin(), J.sorted->end());
            for (int k = 0; k < 3; ++k) nin.push_back(J.n_in[k]);
            for (int ai : *J.incoming) {
                const int ib = (*J.begin)[ai], ie = (*J.end)[ai];
                if (ib < 0 || ie <= ib) continue;
                tasks.push_back(SpecTask{list, ib, ie, ai, static_cast<int>(j1 - j0)});
            }
            ++j1;
        }
        if (!tasks.empty()) {
            Buf<SpecTask> dt(tasks.size());
            Buf<int> dl(lists.size()), dout(tasks.size());
            Buf<double> dn(nin.size());
            check(cudaMemcpyAsync(dt.p, tasks.data(), tasks.size() * sizeof(SpecTask), cudaMemcpyHostToDevice, stream),
                  "copy");
            check(cudaMemcpyAsync(dl.p, lists.data(), lists.size() * sizeof(int), cudaMemcpyHostToDevice, stream),
                  "copy");
            check(cudaMemcpyAsync(dn.p, nin.data(), nin.size() * sizeof(double), cudaMemcpyHostToDevice, stream),
                  "copy");
            const int g = static_cast<int>(std::min<size_t>(grid, (tasks.size() + 7) / 8));
            k_spec_match<<<g, 256, 0, stream>>>(d64.p, d32.p, dn.p, dl.p, dt.p, static_cast<int>(tasks.size()),
                                                dout.p);
            check(cudaGetLastError(), "k_spec_match");
            std::vector<int> best(tasks.size());
            check(cudaMemcpyAsync(best.data(), dout.p, best.size() * sizeof(int), cudaMemcpyDeviceToHost, stream),
                  "copy");
            check(cudaStreamSynchronize(stream), "k_spec_match");
            for (size_t t = 0; t < tasks.size(); ++t)
                if (best[t] >= 0) (*jobs[j0 + tasks[t].job].match)[tasks[t].ai] = best[t];
        }
        j0 = j1;
    }
}

} // namespace phmc
