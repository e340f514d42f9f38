// Counter-based Philox-4x32-10 (Salmon et al., SC'11), host and device.
//
// The reference draws from one std::mt19937_64 per OpenMP worker
// (src/MonteCarloSolver.cpp:153-162), so its stream depends on the thread
// schedule. Here every draw is a pure function of (seed, carrier slot, step,
// purpose, event): the CUDA kernels and the CPU oracle consume identical
// uniforms regardless of launch shape, which is what makes step-level parity
// between them possible.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define PHMC_HD __host__ __device__ __forceinline__
#else
#define PHMC_HD inline
#endif

namespace phmc {

struct U4 {
    uint32_t x, y, z, w;
};

PHMC_HD void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    const uint64_t p = static_cast<uint64_t>(a) * b;
    hi = static_cast<uint32_t>(p >> 32);
    lo = static_cast<uint32_t>(p);
}

PHMC_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c.x, hi0, lo0);
        mulhilo32(M1, c.z, hi1, lo1);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// Draw purposes (third counter word, high byte).
enum : uint32_t {
    kDrawTransport = 1,   // wall events of carriers advanced from the step start
    kDrawInjected = 2,    // wall events of carriers advanced from their emission time
    kDrawInjectCount = 3, // fixed-flux Bernoulli emission count, per reservoir
    kDrawInject = 4,      // mode/time/surface draws of one emission
    kDrawInit = 5,        // initial positions and modes
};

// Two uniforms in [0,1) with 53-bit resolution from one Philox block.
struct Uniform2 {
    double a, b;
};

PHMC_HD Uniform2 uniform2(uint64_t seed, uint32_t slot, uint32_t step, uint32_t purpose,
                          uint32_t event, uint32_t block) {
    const U4 r = philox4x32_10(U4{slot, step, (purpose << 24) | (event & 0xFFFFFFu), block},
                               static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    const uint64_t m0 = ((static_cast<uint64_t>(r.x) << 32) | r.y) >> 11;
    const uint64_t m1 = ((static_cast<uint64_t>(r.z) << 32) | r.w) >> 11;
    constexpr double inv53 = 1.0 / 9007199254740992.0;
    return {static_cast<double>(m0) * inv53, static_cast<double>(m1) * inv53};
}

// One column of a Walker alias table (A. J. Walker, ACM TOMS 3(3):253-256,
// 1977): the column keeps its own outcome with probability `prob` and gives
// `alias` otherwise. 16 bytes, read with one vector load.
struct alignas(16) AliasCell {
    double prob;
    int32_t alias;
    int32_t pad;
};

// A draw from an n-column alias table with one uniform u in [0, 1): column
// i = floor(u n), kept when the fraction u n - i is below its probability.
// The product is rounded once, identically on host and device (no FMA).
PHMC_HD int alias_draw(const AliasCell* t, int n, double u) {
#if defined(__CUDA_ARCH__)
    const double s = __dmul_rn(u, static_cast<double>(n));
#else
    const double s = u * static_cast<double>(n);
#endif
    int i = static_cast<int>(s);
    if (i > n - 1) i = n - 1;
    const AliasCell c = t[i];
#if defined(__CUDA_ARCH__)
    const double f = __dsub_rn(s, static_cast<double>(i));
#else
    const double f = s - static_cast<double>(i);
#endif
    return f < c.prob ? i : c.alias;
}

} // namespace phmc
