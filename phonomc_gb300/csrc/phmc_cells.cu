// Per-cell work of the timestep, from the (cell, mode) bins of the transport pass.
//
//  k_cell_stats    grid over (mode chunk, cell): energy after transport and the
//                  gradient cell sums (src/solver/GridStatistics.cpp:95-181,
//                  src/solver/TemperatureGradientDrive.cpp:131-150); RTA class sums
//  k_cell_state    per cell: energy density -> temperature (src/solver/GridStatistics.cpp:213-226)
//  k_rta_solve     one CTA per cell: pseudo-temperature bracket + Newton over mode
//                  classes (src/solver/RtaCollisionOperator.cpp:79-184)
//  k_linear_solve  one thread-block cluster per cell: exp(dt L) on the cell's
//                  mode-aggregated quadrature (src/material/CallawayOperator.cpp:193-370,
//                  src/solver/CarrierCollisionOperator.cpp:67-126); the cell's vectors
//                  live in the cluster's shared memory, reductions go through DSMEM
//  k_cell_tables   grid over (mode chunk, cell): the pending affine update per
//                  (cell, mode), the step's lifetime residual, drive energy and the
//                  energy at the end of the step; clears the bins
//  k_cells_final   cell temperatures at the end of the step, total thermal energy
//                  and the energy ledger (src/solver/EnergyLedger.cpp:58-90)
//
// Collisions and drive become n' = alpha n + beta per (cell, mode):
//   RTA     alpha = 1 - a,  beta = a n_eq(T*)
//   linear  alpha = e^{-r dt}, beta = (1 - alpha) n_bg + A_m, A_m the common
//           gain of the mode's carriers (exact: within one mode the carriers
//           differ only in x_i, and the rank-G gain term is shared)
#include "phmc_kernels.cuh"

#include <cooperative_groups.h>

#include <stdexcept>
#include <string>

namespace cg = cooperative_groups;

namespace phmc {

constexpr int kStatThreads = 256;
constexpr int kChunk = kStatChunk; // modes per stats/tables block
constexpr int kMaxGains = 5;
constexpr int kLinThreads = 256;

// Sum over the block, result in every thread: shuffles within each warp, then
// warp 0 folds the per-warp sums, so only 2 x 5 shuffle-adds per value reach
// the FP64 pipe in the threads that do them.
template <int N> __device__ __forceinline__ void block_sum(double (&v)[N], double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[k * 32 + wid] = x;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double x = lane < nw ? red[k * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) red[k * 32] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = red[k * 32];
    __syncthreads();
}

__device__ __forceinline__ void k_step_begin_body(DevLedger* L, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    for (int r = 0; r < kMaxReservoirs; ++r) L->absorbed_res[r] = 0;
    L->step_absorbed = L->step_injected = 0;
    L->step_absorbed_ev = L->step_injected_ev = 0;
    L->step_lifetime_residual = 0;
    L->step_drive_ev = L->next_drive_ev;
    L->step_drive_updates = L->next_drive_updates;
    L->next_drive_ev = 0;
    L->next_drive_updates = 0;
    L->step_source_ev = L->next_source_ev;
    L->step_source_updates = L->next_source_updates;
    L->next_source_ev = 0;
    L->next_source_updates = 0;
    L->n_inject = 0;
    L->n_deferred = 0;
    L->event_head = 0;
}

__global__ void k_step_begin(DevLedger* L) {
    k_step_begin_body(L, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ double idx_to_double(int a) { return static_cast<double>(a); }
__device__ __forceinline__ int double_to_idx(double a) { return static_cast<int>(a); }

// ------------------------------------------------------------ statistics
template <bool kRta>
__device__ __forceinline__ void k_cell_stats_body(const DevTables* __restrict__ Tp, CellArrays C, int classes, int vbx, int vgx, int vby) {
    (void)vbx;
    (void)vgx;
    (void)vby;
    __shared__ double red[3 * 32];
    const DevTables& T = *Tp;
    const int c = vby;
    const DevMaterial& M = T.mat[C.cell_material[c]];
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const int m0 = vbx * kChunk, m1 = min(M.n_bins, m0 + kChunk);
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = m0 + threadIdx.x; b < m1; b += blockDim.x) {
        const unsigned k = C.bins[hb + b].cnt;
        if (!k) continue;
        const double N = C.bins[hb + b].N;
        const int m = M.bin_rep ? M.bin_rep[b] : b;
        v[0] += M.hw[m] * (N - k * M.nbg[m]);
        if (M.grad_rate) {
            v[1] += k * M.grad_rate[m];
            v[2] += k * M.cap_bg[m];
        }
    }
    block_sum<3>(v, red);
    if (threadIdx.x == 0 && m0 < M.n_bins) {
        atomicAdd(C.cell_stats + 4 * c, v[0]);
        atomicAdd(C.cell_stats + 4 * c + 1, v[1]);
        atomicAdd(C.cell_stats + 4 * c + 2, v[2]);
    }
}

template <bool kRta>
__global__ void __launch_bounds__(kStatThreads) k_cell_stats(const DevTables* __restrict__ Tp, CellArrays C,
                                                              int classes) {
    k_cell_stats_body<kRta>(Tp, C, classes, blockIdx.x, gridDim.x, blockIdx.y);
}

// phase 2 keeps the supplied temperatures
__device__ __forceinline__ void k_cell_state_body(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L, int phase, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    const DevTables& T = *Tp;
    for (int c = vbx * blockDim.x + threadIdx.x; c < C.ncells; c += vgx * blockDim.x) {
        const DevMaterial& M = T.mat[C.cell_material[c]];
        const double* s = C.cell_stats + 4 * c;
        const double E = s[0] * M.energy_weight / C.volume[c] + M.energy_density_bg;
        if (!isfinite(E)) raise_error(L, kErrNonFinite, c);
        C.energy[c] = E;
        if (phase != 2)
            C.temperature[c] = T.par.linearized
                                   ? T.par.background_T + (E - M.energy_density_bg) / M.heat_capacity_density_bg
                                   : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, E);
        C.grad_ratio[c] = s[2] > 0.0 ? s[1] / s[2] : 0.0;
    }
}

__global__ void k_cell_state(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L, int phase) {
    k_cell_state_body(Tp, C, L, phase, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ RTA
__device__ __forceinline__ void k_rta_solve_body(const DevTables* __restrict__ Tp, CellArrays C, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    __shared__ double red[2 * 32];
    const DevTables& T = *Tp;
    const int c = vbx;
    const DevMaterial& M = T.mat[C.cell_material[c]];
    // the bins of an RTA cell are its mode classes: count, sum of n, sum of max(1, n)
    const int nc = M.n_classes;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const BinSum* bs = C.bins + hb;
    const double* hm = C.hM + hb;
    double2* ab = C.rta_ab + static_cast<size_t>(c) * C.n_classes;
    const double Tc = C.temperature[c];
    const double dt = T.par.dt;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) {
        const int rep = M.class_rep[k];
        double a;
        if (T.par.lifetime_local) {
            const double g = gamma_at(M, rep, Tc);
            a = (g == 0.0 || dt == 0.0) ? 0.0 : -expm1(-(g * dt) * (4.0 * 3.14159265358979323846));
        } else {
            a = M.relax_fixed[rep];
        }
        ab[k].x = a;
    }
    __syncthreads();
    // f(T) = sum_k hw a (N_k - cnt_k n_eq(T)); f' = -sum cnt hw a dn_eq/dT
    auto evaluate = [&](double temperature, bool want_slope, double& slope) {
        const double Tt = fmax(0.0, temperature);
        double v[2] = {0.0, 0.0};
        for (int k = threadIdx.x; k < nc; k += blockDim.x) {
            const double n0 = static_cast<double>(bs[k].cnt);
            if (n0 == 0.0) continue;
            const double w = fmax(0.0, M.class_omega[k]);
            const double hw = kHbar * w;
            const double a = ab[k].x;
            if (!(hw > 0.0) || !(a > 0.0)) continue;
            const double neq = bose_dev(Tt, w);
            v[0] += hw * a * (bs[k].N - n0 * neq);
            if (want_slope && Tt > 0.0) v[1] -= n0 * hw * a * (hw * neq * (neq + 1.0) / (kKb * Tt * Tt));
        }
        block_sum<2>(v, red);
        slope = v[1];
        return v[0];
    };
    double dummy;
    double low = 0.0, high = fmax(1000.0, 2.0 * fmax(1.0, Tc));
    const double f_low = evaluate(low, false, dummy);
    double f_high = evaluate(high, false, dummy);
    for (int k = 0; f_high > 0.0 && k < 20; ++k) {
        high *= 2.0;
        f_high = evaluate(high, false, dummy);
    }
    double Ts = fmin(fmax(Tc, low), high);
    if (f_low <= 0.0) {
        Ts = low;
    } else if (f_high >= 0.0) {
        Ts = high;
    } else {
        double sv[2] = {0.0, 0.0};
        for (int k = threadIdx.x; k < nc; k += blockDim.x) sv[0] += kHbar * fmax(0.0, M.class_omega[k]) * ab[k].x * hm[k];
        block_sum<2>(sv, red);
        const double tol = 1e-13 * fmax(1.0, sv[0]);
        for (int it = 0; it < 40; ++it) {
            double d;
            const double v = evaluate(Ts, true, d);
            if (fabs(v) <= tol) break;
            if (v > 0.0) low = Ts;
            else high = Ts;
            double cand = 0.5 * (low + high);
            if (d < 0.0 && isfinite(d)) {
                const double nt = Ts - v / d;
                if (nt > low && nt < high && isfinite(nt)) cand = nt;
            }
            Ts = cand;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nc; k += blockDim.x) {
        ab[k].y = bose_dev(Ts, fmax(0.0, M.class_omega[k]));
    }
}

__global__ void __launch_bounds__(256) k_rta_solve(const DevTables* __restrict__ Tp, CellArrays C) {
    k_rta_solve_body(Tp, C, blockIdx.x, gridDim.x);
}

// Warp-wide sum with the result of lane 0 broadcast, so every lane continues
// with the same bits (the iteration decisions below stay warp-uniform).
__device__ __forceinline__ double warp_sum_uniform(double x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return __shfl_sync(0xffffffffu, x, 0);
}

// k_rta_solve with one warp per cell: the same bracket and Newton/bisection
// iteration, with warp reductions instead of block barriers. Used when cells
// are many (a mesh grid): a cell's class loop is short and the block-wide
// reductions, not the arithmetic, set the time per iteration.
__device__ __forceinline__ void rta_solve_warp_cell(const DevTables& T, const CellArrays& C, int c, int lane) {
    const DevMaterial& M = T.mat[C.cell_material[c]];
    const int nc = M.n_classes;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const BinSum* bs = C.bins + hb;
    const double* hm = C.hM + hb;
    double2* ab = C.rta_ab + static_cast<size_t>(c) * C.n_classes;
    const double Tc = C.temperature[c];
    const double dt = T.par.dt;
    for (int k = lane; k < nc; k += 32) {
        const int rep = M.class_rep[k];
        double a;
        if (T.par.lifetime_local) {
            const double g = gamma_at(M, rep, Tc);
            a = (g == 0.0 || dt == 0.0) ? 0.0 : -expm1(-(g * dt) * (4.0 * 3.14159265358979323846));
        } else {
            a = M.relax_fixed[rep];
        }
        ab[k].x = a;
    }
    __syncwarp();
    auto evaluate = [&](double temperature, bool want_slope, double& slope) {
        const double Tt = fmax(0.0, temperature);
        double v0 = 0.0, v1 = 0.0;
        for (int k = lane; k < nc; k += 32) {
            const double n0 = static_cast<double>(bs[k].cnt);
            if (n0 == 0.0) continue;
            const double w = fmax(0.0, M.class_omega[k]);
            const double hw = kHbar * w;
            const double a = ab[k].x;
            if (!(hw > 0.0) || !(a > 0.0)) continue;
            const double neq = bose_dev(Tt, w);
            v0 += hw * a * (bs[k].N - n0 * neq);
            if (want_slope && Tt > 0.0) v1 -= n0 * hw * a * (hw * neq * (neq + 1.0) / (kKb * Tt * Tt));
        }
        slope = want_slope ? warp_sum_uniform(v1) : 0.0;
        return warp_sum_uniform(v0);
    };
    double dummy;
    double low = 0.0, high = fmax(1000.0, 2.0 * fmax(1.0, Tc));
    const double f_low = evaluate(low, false, dummy);
    double f_high = evaluate(high, false, dummy);
    for (int k = 0; f_high > 0.0 && k < 20; ++k) {
        high *= 2.0;
        f_high = evaluate(high, false, dummy);
    }
    double Ts = fmin(fmax(Tc, low), high);
    if (f_low <= 0.0) {
        Ts = low;
    } else if (f_high >= 0.0) {
        Ts = high;
    } else {
        double s0 = 0.0;
        for (int k = lane; k < nc; k += 32) s0 += kHbar * fmax(0.0, M.class_omega[k]) * ab[k].x * hm[k];
        const double tol = 1e-13 * fmax(1.0, warp_sum_uniform(s0));
        for (int it = 0; it < 40; ++it) {
            double d;
            const double v = evaluate(Ts, true, d);
            if (fabs(v) <= tol) break;
            if (v > 0.0) low = Ts;
            else high = Ts;
            double cand = 0.5 * (low + high);
            if (d < 0.0 && isfinite(d)) {
                const double nt = Ts - v / d;
                if (nt > low && nt < high && isfinite(nt)) cand = nt;
            }
            Ts = cand;
        }
    }
    for (int k = lane; k < nc; k += 32) ab[k].y = bose_dev(Ts, fmax(0.0, M.class_omega[k]));
}

__global__ void __launch_bounds__(256) k_rta_solve_warp(const DevTables* __restrict__ Tp, CellArrays C) {
    const int c = static_cast<int>((blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5);
    if (c >= C.ncells) return; // warp-uniform
    rta_solve_warp_cell(*Tp, C, c, threadIdx.x & 31);
}

// ----------------------------------------------- RTA cell update (fused)
// One warp per cell for grids of many cells whose class count fits the warp's
// shared-memory list: the bin sums and the cell state (k_cell_stats,
// k_cell_state), the pseudo-temperature (k_rta_solve) and the pending update
// with the step energies (k_cell_tables) in one kernel. After the first scan
// of the bins only the cell's occupied classes are visited: an empty class
// adds nothing to any sum of the solve, and its pending entry is read by no
// carrier (a carrier reads the entry of the bin it was counted in, and every
// reader clears or adds to exactly those entries).
//
// The iteration of src/solver/RtaCollisionOperator.cpp:79-184 is kept: the
// bracket [0, max(1000, 2 max(1, T))] with its doubling, the edge cases, the
// FP64 Newton/bisection steps and the stopping test |f| <= 1e-13 max(1, sum hw
// a max(1, n)). What changes is how f is evaluated and where the iteration
// starts. (1) It starts at an FP32 Newton estimate of the root inside the
// bracket instead of the cell temperature. (2) f and f' at a point T0 come
// from the Bose occupations (one exp per class); at points within 1e-5 T0 of
// T0 they come from the third-order Taylor expansion of each occupation in
// 1/T about T0, which agrees with the direct formula to about 1e-16 relative
// there (the expansion error is (x dT/T)^4 / 24 for x = hw/kT), so the usual
// final Newton step and the test of its result need no further exps.
// (3) f(high) is evaluated in FP64 only when an FP32 bound does not show it
// negative (only its sign enters the iteration). The occupations at the
// accepted T* are the ones the pending update uses.
constexpr int kRtaCellWarps = 4;
constexpr int kRtaCellMaxCap = 512;

struct RtaCellList {
    double* N;   // summed occupation of the class
    double* n0;  // carriers of the class
    double* hw;  // hbar omega of the class
    double* a;   // relaxation probability
    double* p0;  // n_eq at the expansion point
    float4* f32; // (hw, hw a, N, carriers) in FP32; hw a = 0 marks a class without relaxation
    int* cls;    // class (bin) index
};

__device__ __forceinline__ RtaCellList rta_cell_list(int cap) {
    extern __shared__ double rta_smem[];
    const int w = threadIdx.x >> 5;
    const int stride = kRtaCellWarps * cap;
    RtaCellList l;
    l.N = rta_smem + w * cap;
    l.n0 = rta_smem + stride + w * cap;
    l.hw = rta_smem + 2 * stride + w * cap;
    l.a = rta_smem + 3 * stride + w * cap;
    l.p0 = rta_smem + 4 * stride + w * cap;
    l.f32 = reinterpret_cast<float4*>(rta_smem + 5 * stride) + w * cap;
    l.cls = reinterpret_cast<int*>(reinterpret_cast<float4*>(rta_smem + 5 * stride) + stride) + w * cap;
    return l;
}

static size_t rta_cell_smem(int cap) {
    return static_cast<size_t>(kRtaCellWarps) * cap * (5 * sizeof(double) + sizeof(float4) + sizeof(int));
}

// Interval of the linewidth table at temperature T, found once per cell:
// gamma_at(M, a, T) == gamma_in(M, s, a) for every mode a.
struct GammaSpan {
    int l, h;
    double t;
    bool lerp;
};

__device__ __forceinline__ GammaSpan gamma_span(const DevMaterial& M, double T) {
    GammaSpan s{0, 0, 0.0, false};
    const int nT = M.n_temps;
    if (!(T > M.temps[0])) return s; // also a non-finite T: the first row
    if (T >= M.temps[nT - 1]) {
        s.l = nT - 1;
        return s;
    }
    int lo = 0, hi = nT;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (M.temps[mid] <= T) lo = mid + 1;
        else hi = mid;
    }
    const int h = lo, l = h - 1;
    const double x0 = M.temps[l], x1 = M.temps[h];
    s.l = l;
    if (fabs(x1 - x0) <= 1e-18) return s;
    s.h = h;
    s.t = (T - x0) / (x1 - x0);
    s.lerp = true;
    return s;
}

__device__ __forceinline__ double gamma_in(const DevMaterial& M, const GammaSpan& s, int a) {
    const double y0 = M.gamma[static_cast<size_t>(s.l) * M.n_active + a];
    if (!s.lerp) return y0;
    const double y1 = M.gamma[static_cast<size_t>(s.h) * M.n_active + a];
    return y0 * (1.0 - s.t) + y1 * s.t;
}

__device__ __forceinline__ float warp_sum_uniform_f(float x) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return __shfl_sync(0xffffffffu, x, 0);
}

// n_eq(T) of bose_dev from hbar omega (hw = kHbar w, so x is the same product).
__device__ __forceinline__ double bose_hw(double T, double hw) {
    if (T <= 0.0 || hw <= 0.0) return 0.0;
    const double x = hw / (kKb * T);
    if (x > 700.0) return 0.0;
    return 1.0 / fmax(exp(x) - 1.0, 1e-12);
}

// f(T) = sum hw a (N - cnt n_eq(T)) in FP32, its slope and the sum of the
// magnitudes of its terms (all lanes get the warp totals).
__device__ __forceinline__ void rta_eval32(const RtaCellList& Ls, int count, int lane, float t, float& v, float& d,
                                           float& mag) {
    float v0 = 0.f, v1 = 0.f, m0 = 0.f;
    const float ikt = 1.0f / (static_cast<float>(kKb) * t);
    for (int j = lane; j < count; j += 32) {
        const float4 e = Ls.f32[j]; // (hw, hw a, N, cnt)
        if (e.y == 0.f) continue;
        const float x = e.x * ikt;
        const float neq = x > 80.f ? 0.f : 1.0f / expm1f(x);
        v0 += e.y * (e.z - e.w * neq);
        m0 += e.y * (fabsf(e.z) + e.w * neq);
        v1 -= e.w * e.y * (e.x * neq * (neq + 1.0f) * ikt / t);
    }
    v = warp_sum_uniform_f(v0);
    d = warp_sum_uniform_f(v1);
    mag = warp_sum_uniform_f(m0);
}

// f(T) and f'(T) from the Bose occupations; they become the expansion point.
__device__ __forceinline__ double rta_eval_exp(const RtaCellList& Ls, int count, int lane, double T, double& slope) {
    double v0 = 0.0, v1 = 0.0;
    const double ikt2 = T > 0.0 ? 1.0 / (kKb * T * T) : 0.0;
    for (int j = lane; j < count; j += 32) {
        const double hw = Ls.hw[j];
        const double p = bose_hw(T, hw);
        Ls.p0[j] = p;
        const double a = Ls.a[j];
        if (!(hw > 0.0) || !(a > 0.0)) continue;
        const double hwa = hw * a, n0 = Ls.n0[j];
        v0 += hwa * (Ls.N[j] - n0 * p);
        v1 -= n0 * hwa * (hw * p * (p + 1.0) * ikt2);
    }
    slope = warp_sum_uniform(v1);
    return warp_sum_uniform(v0);
}

// n_eq at T from its expansion about T0: y = (hw / k)(1/T - 1/T0),
// n = p0 - q y + r2 y^2 / 2 - r3 y^3 / 6 with q = p0 (p0 + 1),
// r2 = q (2 p0 + 1), r3 = q (6 q + 1) the derivatives of n in x.
struct RtaModel {
    double du; // (1/T - 1/T0) / k
    double ikt2;
};

__device__ __forceinline__ RtaModel rta_model(double T0, double T) {
    RtaModel m;
    m.du = (T0 - T) / (T * T0 * kKb);
    m.ikt2 = 1.0 / (kKb * T * T);
    return m;
}

__device__ __forceinline__ double rta_model_n(const RtaModel& m, double hw, double p0, double& dn) {
    const double q = p0 * (p0 + 1.0);
    const double r2 = q * (2.0 * p0 + 1.0), r3 = q * (6.0 * q + 1.0);
    const double y = hw * m.du;
    dn = -q + y * (r2 - 0.5 * y * r3); // dn/dx
    return p0 + y * (-q + y * (0.5 * r2 - y * (r3 * (1.0 / 6.0))));
}

__device__ __forceinline__ double rta_eval_model(const RtaCellList& Ls, int count, int lane, double T0, double T,
                                                 double& slope) {
    const RtaModel m = rta_model(T0, T);
    double v0 = 0.0, v1 = 0.0;
    for (int j = lane; j < count; j += 32) {
        const double hw = Ls.hw[j];
        const double a = Ls.a[j];
        if (!(hw > 0.0) || !(a > 0.0)) continue;
        double dn;
        const double p = rta_model_n(m, hw, Ls.p0[j], dn);
        const double hwa = hw * a, n0 = Ls.n0[j];
        v0 += hwa * (Ls.N[j] - n0 * p);
        v1 += n0 * hwa * (hw * dn * m.ikt2); // f' = sum hw a cnt (hw / k T^2) dn/dx
    }
    slope = warp_sum_uniform(v1);
    return warp_sum_uniform(v0);
}

// The RTA cell update of cell c by the calling warp (its list is the warp's
// slot of the CTA's dynamic shared memory).
template <bool kCollide>
__device__ __forceinline__ void rta_cell_body(const DevTables& T, const CellArrays& C, DevLedger* L, int phase,
                                              int cap, int c, int lane) {
    const DevMaterial& M = T.mat[C.cell_material[c]];
    const int nb = M.n_bins;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const RtaCellList Ls = rta_cell_list(cap);

    // bin sums of the cell (src/solver/GridStatistics.cpp:95-181) and its occupied classes
    double st[3] = {0.0, 0.0, 0.0};
    int count = 0;
    for (int b0 = 0; b0 < nb; b0 += 32) {
        const int b = b0 + lane;
        unsigned k = 0;
        double N = 0.0;
        if (b < nb) {
            const BinSum bin = C.bins[hb + b];
            k = bin.cnt;
            N = bin.N;
            if (k) {
                const int m = M.bin_rep ? M.bin_rep[b] : b;
                st[0] += M.hw[m] * (N - k * M.nbg[m]);
                if (M.grad_rate) {
                    st[1] += k * M.grad_rate[m];
                    st[2] += k * M.cap_bg[m];
                }
            }
        }
        const unsigned occ = __ballot_sync(0xffffffffu, k != 0);
        if (k) {
            const int j = count + __popc(occ & ((1u << lane) - 1u));
            Ls.cls[j] = b;
            Ls.n0[j] = static_cast<double>(k);
            Ls.N[j] = N;
        }
        count += __popc(occ);
    }
    for (int k = 0; k < 3; ++k) st[k] = warp_sum_uniform(st[k]);
    __syncwarp();

    // cell state (src/solver/GridStatistics.cpp:213-226)
    const double E = st[0] * M.energy_weight / C.volume[c] + M.energy_density_bg;
    double Tc;
    if (phase != 2)
        Tc = T.par.linearized ? T.par.background_T + (E - M.energy_density_bg) / M.heat_capacity_density_bg
                              : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, E);
    else
        Tc = C.temperature[c];
    const double ratio = st[2] > 0.0 ? st[1] / st[2] : 0.0;
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) C.cell_stats[4 * c + k] = st[k];
        if (!isfinite(E)) raise_error(L, kErrNonFinite, c);
        C.energy[c] = E;
        if (phase != 2) C.temperature[c] = Tc;
        C.grad_ratio[c] = ratio;
    }

    // pseudo-temperature over the occupied classes
    double Ts = 0.0;
    int neq_from = 0; // 0 the Bose formula at Ts, 1 the expansion point (T0 == Ts), 2 the expansion about T0
    double T0 = 0.0;
    if (kCollide) {
        const double dt = T.par.dt;
        const GammaSpan span = T.par.lifetime_local ? gamma_span(M, Tc) : GammaSpan{0, 0, 0.0, false};
        double flow = 0.0, scale = 0.0;
        for (int j = lane; j < count; j += 32) {
            const int k = Ls.cls[j];
            const int rep = M.class_rep[k];
            double a;
            if (T.par.lifetime_local) {
                const double g = gamma_in(M, span, rep);
                a = (g == 0.0 || dt == 0.0) ? 0.0 : -expm1(-(g * dt) * (4.0 * 3.14159265358979323846));
            } else {
                a = M.relax_fixed[rep];
            }
            Ls.a[j] = a;
            const double hw = kHbar * fmax(0.0, M.class_omega[k]);
            Ls.hw[j] = hw;
            const bool act = hw > 0.0 && a > 0.0;
            Ls.f32[j] = make_float4(static_cast<float>(hw), act ? static_cast<float>(hw * a) : 0.f,
                                    static_cast<float>(Ls.N[j]), static_cast<float>(Ls.n0[j]));
            scale += hw * a * C.hM[hb + k];
            if (act) flow += hw * a * Ls.N[j]; // f(0): n_eq(0) = 0
        }
        flow = warp_sum_uniform(flow);
        scale = warp_sum_uniform(scale);
        double low = 0.0, high = fmax(1000.0, 2.0 * fmax(1.0, Tc));
        if (!(flow <= 0.0)) {
            // sign of f(high): FP32 value against a bound on its rounding error
            float v32, d32, m32;
            rta_eval32(Ls, count, lane, static_cast<float>(high), v32, d32, m32);
            double f_high = -1.0;
            if (!(v32 < -1e-3f * m32)) {
                double dd;
                f_high = rta_eval_exp(Ls, count, lane, high, dd);
                for (int k = 0; f_high > 0.0 && k < 20; ++k) {
                    high *= 2.0;
                    f_high = rta_eval_exp(Ls, count, lane, high, dd);
                }
            }
            if (f_high >= 0.0) {
                Ts = high;
            } else {
                const double tol = 1e-13 * fmax(1.0, scale);
                Ts = fmin(fmax(Tc, low), high); // the reference's first iterate
                // Where f(Tc) may already pass the test (the FP32 residual at
                // Tc is small against its terms, or the terms themselves are
                // small), the FP64 iteration starts at Tc as the reference's
                // does; elsewhere the reference cannot stop at Tc, and the FP64
                // iteration starts at the FP32 root.
                rta_eval32(Ls, count, lane, static_cast<float>(Ts), v32, d32, m32);
                const bool from_tc = !(fabsf(v32) > 2e-5f * m32 && 1e-5 * static_cast<double>(m32) > tol);
                if (!from_tc) {
                    // FP32 Newton inside [low, high] from Tc
                    float lo = static_cast<float>(low), hi = static_cast<float>(high);
                    float t = static_cast<float>(Ts);
                    for (int it = 0; it < 8 && t > 0.f; ++it) {
                        if (it > 0) rta_eval32(Ls, count, lane, t, v32, d32, m32);
                        if (v32 > 0.f) lo = t;
                        else hi = t;
                        float cand = 0.5f * (lo + hi);
                        const float nt = t - v32 / d32;
                        if (d32 < 0.f && nt > lo && nt < hi && isfinite(nt)) cand = nt;
                        const bool done = fabsf(cand - t) <= 1e-6f * t;
                        t = cand;
                        if (done) break;
                    }
                    Ts = fmin(fmax(static_cast<double>(t), low), high);
                }
                // the FP64 iteration of the reference from there
                bool expanded = false;
                for (int it = 0; it < 40; ++it) {
                    double d, v;
                    const bool near = expanded && Ts > 0.0 && fabs(Ts - T0) <= 1e-5 * T0;
                    if (near) {
                        v = rta_eval_model(Ls, count, lane, T0, Ts, d);
                    } else {
                        v = rta_eval_exp(Ls, count, lane, Ts, d);
                        T0 = Ts;
                        expanded = Ts > 0.0;
                    }
                    if (fabs(v) <= tol) {
                        neq_from = near ? 2 : 1;
                        break;
                    }
                    if (v > 0.0) low = Ts;
                    else high = Ts;
                    double cand = 0.5 * (low + high);
                    if (d < 0.0 && isfinite(d)) {
                        const double nt = Ts - v / d;
                        if (nt > low && nt < high && isfinite(nt)) cand = nt;
                    }
                    Ts = cand;
                }
            }
        }
    }

    // pending update and step energies of the occupied bins (k_cell_tables)
    const RtaModel model = neq_from == 2 ? rta_model(T0, Ts) : RtaModel{0.0, 0.0};
    double s[3] = {0.0, 0.0, 0.0}; // residual, drive, updates
    for (int j = lane; j < count; j += 32) {
        const int b = Ls.cls[j];
        const int m = M.bin_rep ? M.bin_rep[b] : b;
        double a = 1.0, bc = 0.0;
        if (kCollide) {
            const double r = Ls.a[j];
            double n;
            if (neq_from == 1) {
                n = Ls.p0[j];
            } else if (neq_from == 2) {
                double dn;
                n = Ls.hw[j] > 0.0 ? rta_model_n(model, Ls.hw[j], Ls.p0[j], dn) : 0.0;
            } else {
                n = bose_hw(Ts, Ls.hw[j]);
            }
            a = 1.0 - r;
            bc = r * n;
        }
        const double D = M.grad_rate ? fma(-M.drive_cap[m], ratio, M.drive_rate[m]) : 0.0;
        const double k = Ls.n0[j];
        const double hw = M.hw[m];
        s[0] += hw * ((a - 1.0) * Ls.N[j] + k * bc);
        if (D != 0.0) {
            s[1] += k * hw * D;
            s[2] += k;
        }
        C.ab[hb + b] = make_double2(a, kCollide ? bc + 2.0 * D : D);
        if (!T.par.source_enabled) { // with a heat source the bins are cleared after its halves
            BinSum zero;
            zero.N = 0.0;
            zero.cnt = 0;
            zero.pad = 0;
            C.bins[hb + b] = zero;
            C.hM[hb + b] = 0.0;
        }
        if (C.src_next) C.src_next[hb + b] = 0.0;
    }
    for (int k = 0; k < 3; ++k) s[k] = warp_sum_uniform(s[k]);
    if (lane == 0)
        for (int k = 0; k < 3; ++k) C.cell_final[4 * c + k] = s[k];
}

template <bool kCollide>
__global__ void __launch_bounds__(32 * kRtaCellWarps) k_rta_cell(const DevTables* __restrict__ Tp, CellArrays C,
                                                                 DevLedger* L, int phase, int cap) {
    const int c = static_cast<int>((blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5);
    if (c >= C.ncells) return; // warp-uniform
    rta_cell_body<kCollide>(*Tp, C, L, phase, cap, c, threadIdx.x & 31);
}

// The fused update over every cell of a batch (one warp per cell of every
// instance; all instances have `cap` or fewer classes).
__global__ void __launch_bounds__(32 * kRtaCellWarps) kf_rta_cell(const BatchDesc D, int cap) {
    const int g = static_cast<int>((blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5);
    if (g >= D.total_cells) return; // warp-uniform
    const int i = batch_find(D.cell_begin, D.n, g);
    rta_cell_body<true>(*D.tables[i], D.cells[i], D.ledgers[i], 1, cap, g - D.cell_begin[i], threadIdx.x & 31);
}

int rta_cell_capacity(const CellArrays& C, int mode) {
    const int cap = (C.hist_modes + 31) / 32 * 32;
    if (mode < 0 || cap <= 0 || cap > kRtaCellMaxCap) return 0;
    return (mode > 0 || C.ncells >= 1024) ? cap : 0;
}

void prepare_rta_cell(const CellArrays& C) {
    (void)C;
    // the largest list any solver of the process may use, so that solvers of
    // different class counts can coexist
    const int sm = static_cast<int>(rta_cell_smem(kRtaCellMaxCap));
    cudaFuncSetAttribute(reinterpret_cast<const void*>(k_rta_cell<true>), cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(reinterpret_cast<const void*>(k_rta_cell<false>), cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    cudaFuncSetAttribute(reinterpret_cast<const void*>(kf_rta_cell), cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}

// --------------------------------------------------- nonlinear Callaway
// src/solver/NonlinearCallawayCollision.cpp:25-248. Per cell, three BGK
// substeps N(dt/2), R(dt), N(dt/2) move every carrier n <- (1 - a) n + a t,
// a = 1 - exp(-rate dt), t = 1/expm1(phi) a displaced Bose occupation with
// phi = sum_j lambda_j b_j. The basis b_j orthonormalises {hw/kT, k_x, k_y,
// k_z} (energy only for the resistive substep) in the inner product
// sum a n_eq (1 + n_eq) u v; lambda matches the a-weighted moments of n by
// damped Newton on the convex potential sum a (-log(1 - e^-phi) + n phi).
// Carriers of one mode share every factor, so the sums run over the cell's
// mode bins (count c, occupation sum N) and each substep is one affine map
// per mode: the composition (alpha, beta) becomes the cell's pending update.
// The basis is kept as coefficients over the four features, orthonormalised
// through their 4 x 4 Gram matrix. The convergence scale uses
// max(N, c t_eq) per mode for the per-carrier sum of max(n, t_eq) (equal when
// a mode holds one carrier; the scale only normalises the stopping test).
constexpr double kNclHbar = 6.582119569e-4, kNclKb = 8.617333262145e-5;
constexpr int kNclThreads = 256;

__device__ __forceinline__ double ncl_bose(double x) { return x > 700.0 ? 0.0 : 1.0 / expm1(x); }

struct NclBlock {
    double red[16 * 32];
    double part[2][16]; // this CTA's partial sums, read by the cluster (alternating buffers)
    double total[16];
    double B[4][4];   // basis coefficients over (phi0, kx, ky, kz)
    double y[4];      // phi = sum_k y_k f_k for the point being evaluated
    double lambda[4], delta[4], scale[4];
    int dim, status;
};

// Sums over the modes of one cell: one CTA (block_sum), or the CTAs of a
// cluster, each holding the modes m = rank * blockDim + t (mod ranks * blockDim);
// every CTA gets the same totals, so every decision below is cluster-uniform.
struct NclOneBlock {
    __device__ int first() const { return threadIdx.x; }
    __device__ int stride() const { return blockDim.x; }
    template <int N> __device__ void sum(double (&v)[N], NclBlock& sh) { block_sum<N>(v, sh.red); }
};

struct NclCluster {
    int rank, ranks, parity;
    __device__ int first() const { return rank * blockDim.x + threadIdx.x; }
    __device__ int stride() const { return ranks * blockDim.x; }
    template <int N> __device__ void sum(double (&v)[N], NclBlock& sh) {
        static_assert(N <= 16, "cluster sums hold 16 values");
        cg::cluster_group cl = cg::this_cluster();
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int k = 0; k < N; ++k) {
            double x = v[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) sh.red[k * 32 + wid] = x;
        }
        __syncthreads();
        if (wid == 0)
            for (int k = 0; k < N; ++k) {
                double x = lane < nw ? sh.red[k * 32 + lane] : 0.0;
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if (lane == 0) sh.part[parity][k] = x;
            }
        cl.sync();
        if (wid == 0) {
            const double* rp = cl.map_shared_rank(&sh.part[parity][0], lane < ranks ? lane : 0);
            for (int k = 0; k < N; ++k) {
                double x = lane < ranks ? rp[k] : 0.0;
                for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if (lane == 0) sh.total[k] = x;
            }
        }
        __syncthreads();
        for (int k = 0; k < N; ++k) v[k] = sh.total[k];
        __syncthreads();
        parity ^= 1;
    }
};

// Features of mode m in cell temperature T.
template <class Modes>
__device__ __forceinline__ void ncl_features(const Modes& Q, int m, double T, double (&f)[4]) {
    f[0] = kNclHbar * Q.omega(m) / (kNclKb * T);
    f[1] = Q.kx(m, 0);
    f[2] = Q.kx(m, 1);
    f[3] = Q.kx(m, 2);
}

// Potential, gradient and (want_h) Hessian at the point y of sh; returns
// invalid (phi <= 0 or not finite somewhere) as +inf in v[0].
template <class Modes, class Red>
__device__ __forceinline__ void ncl_evaluate(const Modes& Q, NclBlock& sh, Red& rd, double2* work, double T,
                                             bool want_h, double (&v)[16]) {
    for (int k = 0; k < 16; ++k) v[k] = 0.0;
    const int dim = sh.dim;
    for (int m = rd.first(); m < Q.n; m += rd.stride()) {
        const double c = Q.count(m);
        const double a = work[m].y;
        if (c == 0.0 || a == 0.0) continue;
        double f[4];
        ncl_features(Q, m, T, f);
        const double phi = sh.y[0] * f[0] + sh.y[1] * f[1] + sh.y[2] * f[2] + sh.y[3] * f[3];
        if (!(phi > 0.0) || !isfinite(phi)) {
            v[15] = 1.0;
            continue;
        }
        const double e = ncl_bose(phi);
        const double N = work[m].x;
        v[0] += a * (c * -log(-expm1(-phi)) + N * phi);
        double b[4];
        for (int j = 0; j < 4; ++j)
            b[j] = j < dim ? sh.B[j][0] * f[0] + sh.B[j][1] * f[1] + sh.B[j][2] * f[2] + sh.B[j][3] * f[3] : 0.0;
        for (int j = 0; j < 4; ++j) v[1 + j] += a * b[j] * (N - c * e);
        if (want_h) {
            const double h = a * c * e * (1.0 + e);
            int q = 5;
            for (int j = 0; j < 4; ++j)
                for (int l = j; l < 4; ++l) v[q++] += h * b[j] * b[l];
        }
    }
    rd.sum(v, sh);
    if (v[15] != 0.0) v[0] = INFINITY;
}

__device__ __forceinline__ void ncl_set_point(NclBlock& sh, const double* x) {
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) {
            double y = 0.0;
            for (int j = 0; j < sh.dim; ++j) y += x[j] * sh.B[j][k];
            sh.y[k] = y;
        }
    __syncthreads();
}

__device__ __forceinline__ double ncl_error(const NclBlock& sh, const double (&v)[16]) {
    double e = 0.0;
    for (int j = 0; j < sh.dim; ++j) e = fmax(e, fabs(v[1 + j]) / fmax(1e-30, sh.scale[j]));
    return e;
}

// One cell: bins of Q (count, work.x = occupation sum on entry), rates by
// Q.rate(m, normal). Writes (alpha, beta) per mode through Q.out(m, alpha,
// beta); returns 0 or an error code (block-uniform).
template <class Modes, class Red>
__device__ int ncl_solve_cell(const Modes& Q, NclBlock& sh, Red& rd, double2* work, double T, double dt) {
    if (threadIdx.x == 0) sh.status = 0;
    for (int m = rd.first(); m < Q.n; m += rd.stride()) Q.out(m, 1.0, 0.0);
    __syncthreads();
    if (dt == 0.0) return 0;
    for (int sub = 0; sub < 3; ++sub) {
        const bool normal = sub != 1;
        const double h = sub == 1 ? dt : dt * 0.5;
        // relaxation weights, activity and the Gram matrix of the features
        double v[16];
        for (int k = 0; k < 16; ++k) v[k] = 0.0;
        for (int m = rd.first(); m < Q.n; m += rd.stride()) {
            const double a = -expm1(-Q.rate(m, normal) * h);
            work[m].y = a;
            const double c = Q.count(m);
            if (c == 0.0) continue;
            double f[4];
            ncl_features(Q, m, T, f);
            const double e = ncl_bose(f[0]);
            const double w = c * a * e * (1.0 + e);
            v[0] += c * a;
            int q = 1;
            for (int k = 0; k < 4; ++k)
                for (int l = k; l < 4; ++l) v[q++] += w * f[k] * f[l];
        }
        rd.sum(v, sh);
        if (v[0] == 0.0) continue; // no activity
        if (threadIdx.x == 0) {
            double G[4][4];
            int q = 1;
            for (int k = 0; k < 4; ++k)
                for (int l = k; l < 4; ++l) G[k][l] = G[l][k] = v[q++];
            auto gdot = [&](const double* u, const double* w) {
                double s = 0.0;
                for (int k = 0; k < 4; ++k)
                    for (int l = 0; l < 4; ++l) s += u[k] * G[k][l] * w[l];
                return s;
            };
            int dim = 0;
            for (int k = 0; k < 4; ++k) sh.lambda[k] = 0.0;
            for (int j = 0; j < (normal ? 4 : 1); ++j) {
                double u[4] = {0.0, 0.0, 0.0, 0.0};
                if (!(G[j][j] != 0.0)) continue;
                const double norm0 = sqrt(G[j][j]);
                u[j] = 1.0 / norm0;
                for (int pass = 0; pass < 2; ++pass)
                    for (int b = 0; b < dim; ++b) {
                        const double d = gdot(u, sh.B[b]);
                        for (int k = 0; k < 4; ++k) u[k] -= d * sh.B[b][k];
                    }
                const double len = sqrt(gdot(u, u));
                if (len < 1e-12) continue;
                for (int k = 0; k < 4; ++k) sh.B[dim][k] = u[k] / len;
                if (j == 0) sh.lambda[0] = norm0 * len;
                ++dim;
            }
            sh.dim = dim;
            if (dim == 0) sh.status = kErrNclNoConstraint;
        }
        __syncthreads();
        if (sh.status) return sh.status;
        // convergence scales
        for (int k = 0; k < 16; ++k) v[k] = 0.0;
        for (int m = rd.first(); m < Q.n; m += rd.stride()) {
            const double c = Q.count(m);
            if (c == 0.0) continue;
            double f[4];
            ncl_features(Q, m, T, f);
            const double a = work[m].y;
            const double top = fmax(work[m].x, c * ncl_bose(f[0]));
            for (int j = 0; j < sh.dim; ++j) {
                const double b = sh.B[j][0] * f[0] + sh.B[j][1] * f[1] + sh.B[j][2] * f[2] + sh.B[j][3] * f[3];
                v[j] += fabs(a * b) * top;
            }
        }
        rd.sum(v, sh);
        if (threadIdx.x == 0)
            for (int j = 0; j < 4; ++j) sh.scale[j] = v[j];
        __syncthreads();
        // damped Newton
        bool converged = false;
        for (int it = 0; it < 70 && !converged; ++it) {
            ncl_set_point(sh, sh.lambda);
            double g[16];
            ncl_evaluate(Q, sh, rd, work, T, true, g);
            const double F = g[0];
            const double err = ncl_error(sh, g);
            if (err < 2e-13) {
                converged = true;
                break;
            }
            if (threadIdx.x == 0) {
                const int dim = sh.dim;
                double H[4][4], r[4];
                int q = 5;
                for (int j = 0; j < 4; ++j)
                    for (int l = j; l < 4; ++l) H[j][l] = H[l][j] = g[q++];
                for (int j = 0; j < dim; ++j) r[j] = -g[1 + j];
                for (int j = 0; j < dim && !sh.status; ++j) {
                    int p = j;
                    for (int k = j + 1; k < dim; ++k)
                        if (fabs(H[k][j]) > fabs(H[p][j])) p = k;
                    if (!(fabs(H[p][j]) > 1e-30)) {
                        sh.status = kErrNclSingular;
                        break;
                    }
                    for (int l = 0; l < 4; ++l) {
                        const double t = H[j][l];
                        H[j][l] = H[p][l];
                        H[p][l] = t;
                    }
                    const double t = r[j];
                    r[j] = r[p];
                    r[p] = t;
                    for (int k = j + 1; k < dim; ++k) {
                        const double fk = H[k][j] / H[j][j];
                        for (int l = j; l < dim; ++l) H[k][l] -= fk * H[j][l];
                        r[k] -= fk * r[j];
                    }
                }
                if (!sh.status)
                    for (int j = dim - 1; j >= 0; --j) {
                        for (int l = j + 1; l < dim; ++l) r[j] -= H[j][l] * r[l];
                        sh.delta[j] = r[j] / H[j][j];
                    }
            }
            __syncthreads();
            if (sh.status) return sh.status;
            double slope = 0.0;
            for (int j = 0; j < sh.dim; ++j) slope += g[1 + j] * sh.delta[j];
            bool accepted = false;
            for (double t = 1.0; t > 1e-14; t *= 0.5) {
                double trial[4];
                for (int j = 0; j < 4; ++j) trial[j] = sh.lambda[j] + (j < sh.dim ? t * sh.delta[j] : 0.0);
                __syncthreads();
                ncl_set_point(sh, trial);
                double gt[16];
                ncl_evaluate(Q, sh, rd, work, T, false, gt);
                if (isfinite(gt[0]) && (gt[0] <= F + 1e-4 * t * slope || ncl_error(sh, gt) < err * 0.9)) {
                    __syncthreads();
                    if (threadIdx.x == 0)
                        for (int j = 0; j < 4; ++j) sh.lambda[j] = trial[j];
                    __syncthreads();
                    accepted = true;
                    break;
                }
            }
            if (!accepted) return kErrNclLineSearch;
        }
        if (!converged) return kErrNclNoConverge;
        // move the modes: occupation sums and the composed affine map
        ncl_set_point(sh, sh.lambda);
        int bad = 0;
        for (int m = rd.first(); m < Q.n; m += rd.stride()) {
            const double a = work[m].y, c = Q.count(m);
            if (!(a > 0.0) || c == 0.0) continue;
            double f[4];
            ncl_features(Q, m, T, f);
            const double t = ncl_bose(sh.y[0] * f[0] + sh.y[1] * f[1] + sh.y[2] * f[2] + sh.y[3] * f[3]);
            if (!isfinite(t) || t < 0.0) bad = 1;
            work[m].x = (1.0 - a) * work[m].x + a * c * t;
            Q.compose(m, 1.0 - a, a * t);
        }
        double flag[1] = {bad ? 1.0 : 0.0};
        rd.sum(flag, sh);
        if (flag[0] != 0.0) return kErrNclInvalid;
    }
    return 0;
}

// Cell modes of the simulation: bins, material tables, rates at the cell's
// rate temperature (interpolated as src/material/PhononMaterialCollisionData.cpp:168-193).
struct NclSimModes {
    int n;
    const DevMaterial* M;
    const double* kv;
    const double* gn;
    const double* gu;
    const double* gx;
    const BinSum* bins;
    double2* ab;
    int lo, hi;
    double fr;
    __device__ double omega(int m) const { return M->omega[m]; }
    __device__ double kx(int m, int k) const { return kv[3 * m + k]; }
    __device__ double count(int m) const { return static_cast<double>(bins[m].cnt); }
    __device__ double lerp(const double* g, int m) const {
        const size_t na = static_cast<size_t>(M->n_active);
        return 4.0 * 3.14159265358979311600 * ((1.0 - fr) * g[lo * na + m] + fr * g[hi * na + m]);
    }
    __device__ double rate(int m, bool normal) const {
        return normal ? lerp(gn, m) : lerp(gu, m) + (gx ? lerp(gx, m) : 0.0);
    }
    __device__ void out(int m, double alpha, double beta) const { ab[m] = make_double2(alpha, beta); }
    __device__ void compose(int m, double alpha, double beta) const {
        const double2 p = ab[m];
        ab[m] = make_double2(alpha * p.x, alpha * p.y + beta);
    }
};

// One cluster of kNclCluster CTAs per cell: the nonlinear Callaway update of
// the cell's carriers as the pending (alpha, beta) of each mode bin (in
// C.rta_ab, stride hist_modes). The CTAs split the cell's modes; every exit
// passes one cluster barrier so no CTA leaves while another reads its sums.
constexpr int kNclCluster = 8;

__global__ void __launch_bounds__(kNclThreads, 3) k_ncl_solve(const DevTables* __restrict__ Tp, CellArrays C,
                                                            DevLedger* L, const DevNcl X) {
    __shared__ NclBlock sh;
    cg::cluster_group cl = cg::this_cluster();
    NclCluster rd{static_cast<int>(cl.block_rank()), static_cast<int>(cl.num_blocks()), 0};
    const DevTables& T = *Tp;
    const int c = blockIdx.x / rd.ranks;
    const int mid = C.cell_material[c];
    const DevMaterial& M = T.mat[mid];
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    NclSimModes Q;
    Q.n = M.n_bins;
    Q.M = &M;
    Q.kv = X.k[mid];
    Q.gn = X.gamma_n[mid];
    Q.gu = X.gamma_u[mid];
    Q.gx = X.gamma_x[mid];
    Q.bins = C.bins + hb;
    Q.ab = C.rta_ab + hb;
    double2* work = X.work + hb;
    const double Tc = C.temperature[c];
    const double Tr = X.local ? Tc : X.lifetime_T;
    // src/solver/NonlinearCallawayCollision.cpp:309-312 and :218-221
    double carriers[1] = {0.0};
    for (int m = rd.first(); m < Q.n; m += rd.stride()) {
        const BinSum b = Q.bins[m];
        work[m] = make_double2(b.N, 0.0);
        carriers[0] += b.cnt;
    }
    rd.sum(carriers, sh);
    int st = 0;
    bool solved = false;
    if (carriers[0] != 0.0) {
        if (!(Tr > 0.0) || !isfinite(Tr) || Tr < M.temps[0] || Tr > M.temps[M.n_temps - 1] || !(Tc > 0.0) ||
            !isfinite(Tc)) {
            st = kErrNclTemperature;
        } else {
            int hi = 0;
            const int n = M.n_temps;
            while (hi < n && M.temps[hi] < Tr) ++hi; // lower_bound
            Q.hi = hi;
            Q.lo = hi > 0 ? hi - 1 : hi;
            Q.fr = Q.lo == Q.hi ? 0.0 : (Tr - M.temps[Q.lo]) / (M.temps[Q.hi] - M.temps[Q.lo]);
            st = ncl_solve_cell(Q, sh, rd, work, Tc, T.par.dt);
            solved = st == 0;
        }
    }
    if (!solved)
        for (int m = rd.first(); m < Q.n; m += rd.stride()) Q.out(m, 1.0, 0.0);
    if (st != 0 && rd.rank == 0 && threadIdx.x == 0) raise_error(L, st, c);
    cl.sync();
}

// Stand-alone cell for phmc_dev_ncallaway_evolve: per-mode arrays.
struct NclArrayModes {
    int n;
    const double* om;
    const double* kv;
    const double* rn;
    const double* rr;
    const double* cnt;
    double2* ab;
    __device__ double omega(int m) const { return om[m]; }
    __device__ double kx(int m, int k) const { return kv[3 * m + k]; }
    __device__ double count(int m) const { return cnt[m]; }
    __device__ double rate(int m, bool normal) const { return normal ? rn[m] : rr[m]; }
    __device__ void out(int m, double alpha, double beta) const { ab[m] = make_double2(alpha, beta); }
    __device__ void compose(int m, double alpha, double beta) const {
        const double2 p = ab[m];
        ab[m] = make_double2(alpha * p.x, alpha * p.y + beta);
    }
};

// One CTA: bins the carriers by mode (in carrier order), solves, moves them.
__global__ void __launch_bounds__(kNclThreads) k_ncl_cell(NclArrayModes Q, double* cnt, double2* work, int64_t n,
                                                           const int32_t* mode, double* occ, double T, double dt,
                                                           int* status) {
    NclOneBlock rd;
    __shared__ NclBlock sh;
    for (int m = rd.first(); m < Q.n; m += rd.stride()) {
        double c = 0.0, N = 0.0;
        for (int64_t i = 0; i < n; ++i)
            if (mode[i] == m) {
                c += 1.0;
                N += occ[i];
            }
        cnt[m] = c;
        work[m] = make_double2(N, 0.0);
    }
    __syncthreads();
    const int st = ncl_solve_cell(Q, sh, rd, work, T, dt);
    if (threadIdx.x == 0) *status = st;
    if (st != 0) return;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 ab = Q.ab[mode[i]];
        occ[i] = ab.x * occ[i] + ab.y;
    }
}

// ----------------------------------------------------- linear response
// Cluster-wide sum of N doubles: CTA partials in shared memory, read by every
// CTA of the cluster through distributed shared memory.
// Sum over the thread-block cluster, result in every thread. Values are
// summed in V within each warp; warp 0 of each block folds its warps in FP64
// into part[parity][], and after the cluster barrier warp 0 of each block
// folds the blocks' part[parity][] through distributed shared memory into
// total[]. part[] alternates between two buffers, so one cluster barrier per
// sum suffices: a block can only write a buffer again after every block has
// passed the next sum's barrier, i.e. finished reading that buffer.
template <int N, class V>
__device__ __forceinline__ void cluster_sum(V (&v)[N], double* red, double (*part)[kMaxGains], double* total,
                                            int& parity, cg::cluster_group& cl) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        V x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[k * 32 + wid] = static_cast<double>(x);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double x = lane < nw ? red[k * 32 + lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) part[parity][k] = x;
        }
    }
    cl.sync();
    if (wid == 0) {
        const int ranks = static_cast<int>(cl.num_blocks());
        const double* rp = cl.map_shared_rank(part[parity], lane < ranks ? lane : 0);
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double x = lane < ranks ? rp[k] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) total[k] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = static_cast<V>(total[k]);
    parity ^= 1;
}

template <class R, int GMAX>
__global__ void __launch_bounds__(kLinThreads) k_linear_solve(const DevTables* __restrict__ Tp, CellArrays C,
                                                               unsigned char* __restrict__ gslice, size_t slice) {
    // R = float: FP32 exponential from division-free FP32 per-mode tables; FP64
    // only for the bin energies, the conservation sums and the final beta.
    constexpr bool kF32 = sizeof(R) == sizeof(float);
    constexpr int gmax = GMAX;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[kMaxGains * 32];
    __shared__ double part[2][kMaxGains];
    __shared__ double total[kMaxGains];
    int parity = 0;
    cg::cluster_group cl = cg::this_cluster();
    const DevTables& T = *Tp;
    const int CL = static_cast<int>(cl.num_blocks());
    const int rank = static_cast<int>(cl.block_rank());
    const int c = blockIdx.x / CL;
    const int mat = C.cell_material[c];
    const DevMaterial& M = T.mat[mat];
    const int na = M.n_active;
    const size_t mo = static_cast<size_t>(mat) * C.hist_modes; // this material's per-mode constants
    const int per = (C.hist_modes + CL - 1) / CL;
    const int m0 = rank * per, m1 = min(na, m0 + per);
    const int nloc = max(0, m1 - m0);
    // per-mode vectors of this CTA's slice: shared memory, or (tables too
    // large for a 16-CTA cluster) this CTA's slice of a global work area
    unsigned char* base = gslice ? gslice + static_cast<size_t>(blockIdx.x) * slice : smem;
    R* X = reinterpret_cast<R*>(base);
    R* term = X + per;
    R* rate = term + per;
    R* u = rate + per;                                      // gmax vectors
    unsigned* cnt = reinterpret_cast<unsigned*>(u + static_cast<size_t>(gmax) * per);
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const int m = m0 + j;
        const BinSum bin = C.bins[hb + m];
        const unsigned k = bin.cnt;
        cnt[j] = k;
        const double e = k ? M.hw[m] * (bin.N - k * M.nbg[m]) : 0.0;
        if constexpr (kF32) {
            X[j] = static_cast<float>(e) * C.lin32_inv_s[mo + m];
            rate[j] = C.lin32_rate[mo + m];
        } else {
            X[j] = k ? e / C.lin_s[mo + m] : 0.0;
            rate[j] = M.col_rate[m];
        }
    }
    __syncthreads();
    // gain vectors (src/material/CallawayOperator.cpp:193-229), multiplicity-weighted
    int G = 0;
    for (int kind = 0; kind < 2; ++kind) {
        if (kind == 0 && !C.lin_has_normal) continue;
        const double* sq = kind == 0 ? C.lin_sqrt_rn : C.lin_sqrt_rr;
        const float* sq32 = kind == 0 ? C.lin32_sqrt_rn : C.lin32_sqrt_rr;
        const int nbasis = kind == 0 ? 4 : 1;
        const int first = G;
        for (int b = 0; b < nbasis; ++b) {
            R* v = u + static_cast<size_t>(G) * per;
            R nv[1] = {R(0)};
            const float* basis32 = C.lin32_basis + (static_cast<size_t>(mat) * 5 + (kind == 0 ? 1 + b : 0)) * C.hist_modes;
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
                const int m = m0 + j;
                R val = R(0);
                if (cnt[j]) {
                    if constexpr (kF32) {
                        val = basis32[m];
                    } else {
                        const double sv = C.lin_s[mo + m];
                        val = (b == 0 ? sv : sv * M.col_k[3 * m + b - 1] / M.omega[m]) * sq[mo + m];
                    }
                    nv[0] += static_cast<R>(cnt[j]) * val * val;
                }
                v[j] = val;
            }
            cluster_sum<1>(nv, red, part, total, parity, cl);
            const R original = sqrt(nv[0]);
            if (original == R(0)) continue;
            const R inv = R(1) / original;
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) v[j] *= inv;
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                for (int q = first; q < G; ++q) {
                    const R* qv = u + static_cast<size_t>(q) * per;
                    R pr[1] = {R(0)};
                    for (int j = threadIdx.x; j < nloc; j += blockDim.x) pr[0] += static_cast<R>(cnt[j]) * qv[j] * v[j];
                    cluster_sum<1>(pr, red, part, total, parity, cl);
                    const R pq = pr[0];
                    for (int j = threadIdx.x; j < nloc; j += blockDim.x) v[j] -= pq * qv[j];
                    __syncthreads();
                }
            }
            R ln[1] = {R(0)};
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) ln[0] += static_cast<R>(cnt[j]) * v[j] * v[j];
            cluster_sum<1>(ln, red, part, total, parity, cl);
            const R len = sqrt(ln[0]);
            // dependent direction: dropped below 1e-12 (FP64), or below FP32 round-off
            if (len < R(kF32 ? 1e-5 : 1e-12)) continue;
            const R il = R(1) / len;
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) v[j] *= il;
            __syncthreads();
            ++G;
        }
        for (int q = first; q < G; ++q) {
            R* qv = u + static_cast<size_t>(q) * per;
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
                if constexpr (kF32) qv[j] *= sq32[mo + m0 + j];
                else qv[j] *= sq[mo + m0 + j];
            }
        }
        __syncthreads();
    }
    // Taylor series of exp(h L) per substep on (L T)_m = -r_m T_m + cnt_m sum_g u_gm (u_g . T)
    const R h = static_cast<R>(C.lin_h);
    for (int sstep = 0; sstep < C.lin_substeps; ++sstep) {
        for (int j = threadIdx.x; j < nloc; j += blockDim.x) term[j] = X[j];
        __syncthreads();
        for (int k = 1; k <= C.lin_terms; ++k) {
            // per-thread partials and warp sums in R; FP64 only across warps and blocks
            R dl[GMAX];
#pragma unroll
            for (int g = 0; g < GMAX; ++g) dl[g] = R(0);
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
                const R tm = term[j];
#pragma unroll
                for (int g = 0; g < GMAX; ++g)
                    if (g < G) dl[g] += u[static_cast<size_t>(g) * per + j] * tm;
            }
            cluster_sum<GMAX>(dl, red, part, total, parity, cl);
            const R hk = h / static_cast<R>(k);
            for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
                R gain = 0;
#pragma unroll
                for (int g = 0; g < GMAX; ++g)
                    if (g < G) gain += u[static_cast<size_t>(g) * per + j] * dl[g];
                const R t = hk * (-rate[j] * term[j] + static_cast<R>(cnt[j]) * gain);
                term[j] = t;
                X[j] += t;
            }
            __syncthreads();
        }
    }
    // A_m and, for FP32 exponentials, the FP64 rescale that conserves the cell energy
    double cons[2] = {0.0, 0.0};
    double* beta = C.lin_beta + hb;
    for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const int m = m0 + j;
        const unsigned k = cnt[j];
        double A = 0.0;
        if (k) {
            const double e = M.hw[m] * (C.bins[hb + m].N - k * M.nbg[m]);
            if constexpr (kF32) {
                const float x0 = static_cast<float>(e) * C.lin32_inv_s[mo + m];
                A = static_cast<double>(C.lin32_s_over_hw[mo + m] * (X[j] - C.lin32_decay[mo + m] * x0) *
                                        __frcp_rn(static_cast<float>(k)));
                cons[0] += C.lin_omd[mo + m] * e;
            } else {
                const double x0 = e / C.lin_s[mo + m];
                A = C.lin_s[mo + m] * (static_cast<double>(X[j]) - C.lin_decay[mo + m] * x0) / (k * M.hw[m]);
                cons[0] += (1.0 - C.lin_decay[mo + m]) * e;
            }
            cons[1] += k * M.hw[m] * A;
        }
        beta[m] = A;
    }
    double lambda = 1.0;
    if (C.mixed) {
        cluster_sum<2>(cons, red, part, total, parity, cl);
        if (cons[1] != 0.0 && isfinite(cons[0] / cons[1])) lambda = cons[0] / cons[1];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nloc; j += blockDim.x) {
        const int m = m0 + j;
        if constexpr (kF32) beta[m] = fma(lambda, beta[m], C.lin_bg[mo + m]);
        else beta[m] = (1.0 - C.lin_decay[mo + m]) * M.nbg[m] + lambda * beta[m];
    }
    // no block leaves while another block of the cluster may still read its part[]
    cl.sync();
}

// ----------------------------------------------- tables and step energies
template <int kCollision>
__device__ __forceinline__ void k_cell_tables_body(const DevTables* __restrict__ Tp, CellArrays C, int phase, int vbx, int vgx, int vby) {
    (void)vbx;
    (void)vgx;
    (void)vby;
    __shared__ double red[4 * 32];
    const DevTables& T = *Tp;
    const int c = vby;
    const DevMaterial& M = T.mat[C.cell_material[c]];
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const int m0 = vbx * kChunk, m1 = min(M.n_bins, m0 + kChunk);
    const double ratio = C.grad_ratio[c];
    const bool collide = phase >= 1 && kCollision != kCollideNone;
    double s[3] = {0.0, 0.0, 0.0}; // residual, drive, updates
    for (int b = m0 + threadIdx.x; b < m1; b += blockDim.x) {
        const int m = M.bin_rep ? M.bin_rep[b] : b; // representative mode of the bin
        double a = 1.0, bc = 0.0;
        if (collide) {
            if (kCollision == kCollideRta) {
                const double2 r = C.rta_ab[static_cast<size_t>(c) * C.n_classes + b];
                a = 1.0 - r.x;
                bc = r.x * r.y;
            } else if (kCollision == kCollideNonlinear) {
                const double2 r = C.rta_ab[hb + b]; // composed (alpha, beta) of the three substeps
                a = r.x;
                bc = r.y;
            } else {
                a = C.lin_decay[static_cast<size_t>(C.cell_material[c]) * C.hist_modes + b];
                bc = C.lin_beta[hb + b];
            }
        }
        const double D = M.grad_rate ? fma(-M.drive_cap[m], ratio, M.drive_rate[m]) : 0.0;
        const BinSum bin = C.bins[hb + b];
        const unsigned k = bin.cnt;
        if (k) {
            const double hw = M.hw[m];
            s[0] += hw * ((a - 1.0) * bin.N + k * bc);
            if (D != 0.0) {
                s[1] += k * hw * D;
                s[2] += k;
            }
        }
        C.ab[hb + b] = make_double2(a, collide ? bc + 2.0 * D : D);
        if (!T.par.source_enabled) { // with a heat source the bins are cleared after its halves
            BinSum zero;
            zero.N = 0.0;
            zero.cnt = 0;
            zero.pad = 0;
            C.bins[hb + b] = zero;
            if (C.hM) C.hM[hb + b] = 0.0;
        }
        if (C.src_next) C.src_next[hb + b] = 0.0;
    }
    // the step-end energy deviation of the cell is the step-start one (cell
    // statistics) plus the collision change s[0] plus the drive change s[1]
    block_sum<3>(s, red);
    if (threadIdx.x == 0 && m0 < M.n_bins) {
        double* f = C.cell_final + 4 * c;
        atomicAdd(f, s[0]);
        atomicAdd(f + 1, s[1]);
        atomicAdd(f + 2, s[2]);
    }
}

template <int kCollision>
__global__ void __launch_bounds__(kStatThreads) k_cell_tables(const DevTables* __restrict__ Tp, CellArrays C, int phase) {
    k_cell_tables_body<kCollision>(Tp, C, phase, blockIdx.x, gridDim.x, blockIdx.y);
}

// End of step: cell temperatures, total thermal energy and the energy ledger.
// Per cell: the step-end energy and temperature; v gathers the thermal energy,
// lifetime residual, drive energy and drive updates over the cells.
__device__ __forceinline__ void cells_final_cell(const DevTables& T, const CellArrays& C, DevLedger* L, int phase,
                                                 int c, double (&v)[4]) {
    const DevMaterial& M = T.mat[C.cell_material[c]];
    double* f = C.cell_final + 4 * c;
    const double w = M.energy_weight;
    // step-start energy + collision + drive half + heat-source half (f[3])
    const double dev = C.cell_stats[4 * c] + (phase >= 1 ? f[0] + f[1] + f[3] : 0.0);
    const double Ef = dev * w / C.volume[c] + M.energy_density_bg;
    if (!isfinite(Ef)) raise_error(L, kErrNonFinite, c);
    C.energy_final[c] = Ef;
    C.temperature_final[c] =
        phase == 2 ? C.temperature[c]
                   : (T.par.linearized ? T.par.background_T + (Ef - M.energy_density_bg) / M.heat_capacity_density_bg
                                       : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, Ef));
    v[0] += (Ef - M.zero_point) * C.volume[c];
    v[1] += f[0] * w;
    v[2] += f[1] * w;
    v[3] += f[2];
    for (int k = 0; k < 4; ++k) {
        f[k] = 0.0;
        C.cell_stats[4 * c + k] = 0.0;
    }
}

// The ledger update from the grid sums v (one thread).
__device__ __forceinline__ void cells_final_ledger(const DevTables& T, DevLedger* L, int phase, const double (&v)[4]) {
    L->next_drive_ev += v[2];
    L->next_drive_updates += static_cast<unsigned long long>(v[3]);
    if (phase == 0) {
        L->thermal_energy = v[0];
        return;
    }
    L->step_lifetime_residual += v[1];
    L->step_drive_ev += v[2];
    L->step_drive_updates += static_cast<unsigned long long>(v[3]);
    const double residual = v[0] - L->thermal_energy - L->step_source_ev - L->step_drive_ev - L->step_injected_ev +
                            L->step_absorbed_ev - L->step_lifetime_residual;
    L->step_balance_residual = residual;
    L->total_absorbed += L->step_absorbed;
    L->total_injected += L->step_injected;
    L->total_absorbed_ev += L->step_absorbed_ev;
    L->total_injected_ev += L->step_injected_ev;
    L->total_lifetime_residual += L->step_lifetime_residual;
    L->total_balance_residual += residual;
    L->total_drive_ev += L->step_drive_ev;
    L->total_drive_updates += L->step_drive_updates;
    L->total_source_ev += L->step_source_ev;
    L->total_source_updates += L->step_source_updates;
    L->thermal_energy = v[0];
    L->particle_count += static_cast<long long>(L->step_injected) - static_cast<long long>(L->step_absorbed);
    for (int r = 0; r < kMaxReservoirs; ++r) L->previous_res[r] = L->absorbed_res[r];
    L->step_index += 1;
    L->elapsed += T.par.dt;
}

// One CTA over all cells (the batched films: one CTA per film).
__device__ __forceinline__ void k_cells_final_body(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L, int phase, int vbx, int vgx) {
    (void)vbx;
    (void)vgx;
    __shared__ double red[4 * 32];
    const DevTables& T = *Tp;
    double v[4] = {0.0, 0.0, 0.0, 0.0}; // thermal, residual, drive, updates
    for (int c = threadIdx.x; c < C.ncells; c += blockDim.x) cells_final_cell(T, C, L, phase, c, v);
    block_sum<4>(v, red);
    if (threadIdx.x == 0) cells_final_ledger(T, L, phase, v);
}

// The grid over the cells: every CTA leaves its partial sums in C.final_part;
// the CTA that finishes last folds them in CTA order (the same sums for the
// same grid on every run) and updates the ledger.
__global__ void __launch_bounds__(256) k_cells_final(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L,
                                                     int phase) {
    __shared__ double red[4 * 32];
    __shared__ bool last;
    const DevTables& T = *Tp;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C.ncells; c += gridDim.x * blockDim.x)
        cells_final_cell(T, C, L, phase, c, v);
    block_sum<4>(v, red);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 4; ++k) C.final_part[4 * blockIdx.x + k] = v[k];
        __threadfence();
        last = atomicAdd(C.final_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double u[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < static_cast<int>(gridDim.x); b += blockDim.x)
        for (int k = 0; k < 4; ++k) u[k] += __ldcg(C.final_part + 4 * b + k);
    block_sum<4>(u, red);
    if (threadIdx.x == 0) {
        cells_final_ledger(T, L, phase, u);
        *C.final_done = 0u;
    }
}

// ------------------------------------------------------- heat source
// One heat-source half for one cell (src/solver/PrescribedHeatSource.cpp:218-243
// accrual, src/solver/PhononSourceOperator.cpp:119-340 deposit): the cell's
// budget is shared among its eligible carriers by spectrum, the increments
// are added to the pending update of each (cell, mode), and the mode with the
// largest energy increment per carrier takes the round-off correction (spread
// over that mode's carriers in this cell). `next` = the first half of the next
// step (energy booked to that step). Base temperature of the thermal Newton:
// `temperature` (cell temperatures of the current refresh).
__global__ void __launch_bounds__(kStatThreads) k_source(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L,
                                                         const double* temperature, int next) {
    __shared__ double red[4 * 32];
    __shared__ double s_pend;
    __shared__ int s_arg;
    const DevTables& T = *Tp;
    const int c = C.src_cells[blockIdx.x];
    // this half's time window: second half of the running step, or first half of the coming one
    const double t0 = L->elapsed, half = __dmul_rn(0.5, T.par.dt);
    const double factor = next ? source_time_factor(T.par, t0, __dadd_rn(t0, half))
                               : source_time_factor(T.par, __dadd_rn(t0, half), __dadd_rn(t0, T.par.dt));
    if (threadIdx.x == 0) {
        if (next) {
            C.src_step_pending[c] = C.src_pending[c];
            C.src_step_book[c] = C.src_prescribed[c];
            C.src_step_book[C.ncells + c] = C.src_deposited[c];
        }
        if (factor > 0.0) {
            const double e = C.src_rate[c] * factor;
            C.src_prescribed[c] += e;
            C.src_pending[c] += e;
        }
        s_pend = C.src_pending[c];
    }
    __syncthreads();
    const double pend = s_pend;
    if (!(pend > 0.0)) return;
    const int mat = C.cell_material[c];
    const DevMaterial& M = T.mat[mat];
    const int na = M.n_bins; // bins of this cell (modes or classes); rep(b) stands for all its modes
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const double target = pend / M.energy_weight;
    const int spectrum = T.par.source_spectrum;
    // eligible carriers present, and the spectrum's normalization
    double v[4] = {0.0, 0.0, -1.0e300, 0.0}; // count, sum of weights (k w, k C), max log-weight
    auto rep = [&](int b) { return M.bin_rep ? M.bin_rep[b] : b; };
    for (int b = threadIdx.x; b < na; b += blockDim.x) {
        const unsigned k = C.bins[hb + b].cnt;
        const int m = rep(b);
        if (!k || !(M.src_weight[m] > 0.0)) continue;
        v[0] += k;
        if (spectrum == 1) v[1] += k * M.src_weight[m];
        else if (spectrum == 0 && T.par.source_linearized) v[1] += k * M.cap_bg[m];
        if (spectrum == 2) v[2] = fmax(v[2], M.src_logw[m]);
    }
    {
        double sums[2] = {v[0], v[1]};
        block_sum<2>(sums, red);
        v[0] = sums[0];
        v[1] = sums[1];
        // block max of the log-weights
        double x = v[2];
        for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            double y = red[0];
            for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) y = fmax(y, red[w]);
            red[0] = y;
        }
        __syncthreads();
        v[2] = red[0];
        __syncthreads();
    }
    if (!(v[0] > 0.0)) return; // no eligible carrier: the cell keeps its budget
    const double peak = v[2];
    if (spectrum == 2) {
        double g[1] = {0.0};
        for (int b = threadIdx.x; b < na; b += blockDim.x) {
            const unsigned k = C.bins[hb + b].cnt;
            const int m = rep(b);
            if (k && M.src_weight[m] > 0.0) g[0] += k * exp(M.src_logw[m] - peak);
        }
        block_sum<1>(g, red);
        v[1] = g[0];
    }
    // thermal spectrum, nonlinear: pseudo-temperature of the eligible carriers
    double Ts = 0.0, base = 0.0;
    const bool newton = spectrum == 0 && !T.par.source_linearized;
    if (newton) {
        const double Tc = temperature[c];
        base = isfinite(Tc) && Tc >= 0.0 ? Tc : T.par.background_T;
        const int ncls = M.n_src_classes;
        double* cnt = C.src_scratch + static_cast<size_t>(c) * 2 * C.src_classes;
        double* n0 = cnt + C.src_classes;
        for (int k = threadIdx.x; k < ncls; k += blockDim.x) {
            cnt[k] = 0.0;
            n0[k] = bose_dev(base, M.src_class_omega[k]);
        }
        __syncthreads();
        for (int b = threadIdx.x; b < na; b += blockDim.x) {
            const unsigned k = C.bins[hb + b].cnt;
            const int cls = M.src_class[rep(b)];
            if (k && cls >= 0) atomicAdd(cnt + cls, static_cast<double>(k));
        }
        __syncthreads();
        auto energy_at = [&](double temperature_s, bool slope, double& d) {
            double e[2] = {0.0, 0.0};
            for (int k = threadIdx.x; k < ncls; k += blockDim.x) {
                if (cnt[k] == 0.0) continue;
                const double hw = kHbar * fmax(0.0, M.src_class_omega[k]);
                const double nn = bose_dev(temperature_s, M.src_class_omega[k]);
                e[0] += cnt[k] * hw * (nn - n0[k]);
                if (slope && temperature_s > 0.0)
                    e[1] += cnt[k] * hw * (hw * nn * (nn + 1.0) / (kKb * temperature_s * temperature_s));
            }
            block_sum<2>(e, red);
            d = e[1];
            return e[0];
        };
        double d;
        double low = fmax(0.0, base);
        double high = fmax(low + 1.0, 1.05 * low + 1.0);
        double high_e = energy_at(high, false, d);
        for (int k = 0; high_e < target && k < 60; ++k) {
            high = 2.0 * high + 1.0;
            high_e = energy_at(high, false, d);
        }
        if (!(high_e >= target) || !isfinite(high_e)) {
            if (threadIdx.x == 0) raise_error(L, kErrCollision, c);
            return;
        }
        Ts = 0.5 * (low + high);
        const double tol = 1e-12 * fmax(1e-6, target);
        for (int it = 0; it < 60; ++it) {
            const double r = energy_at(Ts, true, d) - target;
            if (fabs(r) <= tol) break;
            if (r > 0.0) high = Ts;
            else low = Ts;
            double cand = 0.5 * (low + high);
            if (d > 0.0 && isfinite(d)) {
                const double nt = Ts - r / d;
                if (nt > low && nt < high && isfinite(nt)) cand = nt;
            }
            Ts = cand;
        }
    }
    auto increment = [&](int m) {
        const double hw = M.hw[m];
        if (spectrum == 2) return target * exp(M.src_logw[m] - peak) / v[1] / hw;
        if (spectrum == 1) return target * (M.src_weight[m] / v[1]) / hw;
        if (!newton) return target * M.cap_bg[m] / v[1] / hw;
        return bose_dev(Ts, M.omega[m]) - bose_dev(base, M.omega[m]);
    };
    // applied energy and the correction mode (largest energy per carrier, lowest index on ties)
    double applied[1] = {0.0};
    double best = -1.0;
    int arg = 0x7fffffff;
    for (int b = threadIdx.x; b < na; b += blockDim.x) {
        const unsigned k = C.bins[hb + b].cnt;
        const int m = rep(b);
        if (!k || !(M.src_weight[m] > 0.0)) continue;
        const double e = M.hw[m] * increment(m);
        applied[0] += k * e;
        if (e > best || (e == best && b < arg)) {
            best = e;
            arg = b;
        }
    }
    block_sum<1>(applied, red);
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, arg, o);
        if (ob > best || (ob == best && oa < arg)) {
            best = ob;
            arg = oa;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = best;
        red[32 + (threadIdx.x >> 5)] = idx_to_double(arg);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = red[0];
        int a = double_to_idx(red[32]);
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) {
            const double ob = red[w];
            const int oa = double_to_idx(red[32 + w]);
            if (ob > b || (ob == b && oa < a)) {
                b = ob;
                a = oa;
            }
        }
        s_arg = a;
    }
    __syncthreads();
    const int corr_bin = s_arg;
    const int corr_mode = rep(corr_bin);
    const double corr = (target - applied[0]) / (M.hw[corr_mode] * C.bins[hb + corr_bin].cnt);
    for (int b = threadIdx.x; b < na; b += blockDim.x) {
        const unsigned k = C.bins[hb + b].cnt;
        const int m = rep(b);
        if (!k || !(M.src_weight[m] > 0.0)) continue;
        double inc = increment(m);
        if (b == corr_bin) inc += corr;
        C.ab[hb + b].y += inc;
        if (next) C.src_next[hb + b] += inc;
    }
    if (threadIdx.x == 0) {
        const double raw = applied[0] + C.bins[hb + corr_bin].cnt * M.hw[corr_mode] * corr;
        C.src_deposited[c] += pend;
        C.src_pending[c] = 0.0;
        if (next) {
            atomicAdd(&L->next_source_ev, pend);
            atomicAdd(&L->next_source_updates, static_cast<unsigned long long>(v[0]));
        } else {
            C.cell_final[4 * c + 3] = raw;
            atomicAdd(&L->step_source_ev, pend);
            atomicAdd(&L->step_source_updates, static_cast<unsigned long long>(v[0]));
        }
    }
}

// ----------------------------------------------------------- launchers
void launch_step_begin(const LaunchCtx& x) { k_step_begin<<<1, 1, 0, x.stream>>>(x.L); }

void launch_source(const LaunchCtx& x, bool final_temperature, bool next) {
    // one CTA per cell of positive power
    if (x.C.n_src_cells > 0)
        k_source<<<x.C.n_src_cells, kStatThreads, 0, x.stream>>>(
            x.T, x.C, x.L, final_temperature ? x.C.temperature_final : x.C.temperature, next ? 1 : 0);
    if (next) {
        // last reader of this step's bins
        const size_t hist = static_cast<size_t>(x.C.ncells) * x.C.hist_modes;
        cudaMemsetAsync(x.C.bins, 0, hist * sizeof(BinSum), x.stream);
        if (x.C.hM) cudaMemsetAsync(x.C.hM, 0, hist * sizeof(double), x.stream);
    }
}

static size_t linear_smem(const CellArrays& C, int cl, int gmax, size_t real) {
    const size_t per = (static_cast<size_t>(C.hist_modes) + cl - 1) / cl;
    return per * ((3 + gmax) * real + sizeof(unsigned));
}

// Cluster size for the linear solve: the smallest of 8, 16 whose per-CTA slice fits.
int linear_cluster_size(const CellArrays& C, bool mixed) {
    const int gmax = C.lin_has_normal ? kMaxGains : 1;
    const size_t real = mixed ? sizeof(float) : sizeof(double);
    for (int cl : {8, 16})
        if (linear_smem(C, cl, gmax, real) <= 200 * 1024) return cl;
    return 0;
}

// Bytes of one CTA's per-mode slice when it lives in global memory (cluster of 16).
size_t linear_global_slice(const CellArrays& C, bool mixed) {
    const int gmax = C.lin_has_normal ? kMaxGains : 1;
    return (linear_smem(C, 16, gmax, mixed ? sizeof(float) : sizeof(double)) + 255) / 256 * 256;
}

void prepare_linear_solve(const CellArrays& C, bool global) {
    const int gmax = C.lin_has_normal ? kMaxGains : 1;
    const size_t sm = global ? 0 : linear_smem(C, C.lin_cluster, gmax, C.mixed ? sizeof(float) : sizeof(double));
    auto set = [&](const void* f) {
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
        if (C.lin_cluster > 8) cudaFuncSetAttribute(f, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    };
    if (C.lin_has_normal) {
        if (C.mixed) set(reinterpret_cast<const void*>(k_linear_solve<float, kMaxGains>));
        else set(reinterpret_cast<const void*>(k_linear_solve<double, kMaxGains>));
    } else {
        if (C.mixed) set(reinterpret_cast<const void*>(k_linear_solve<float, 1>));
        else set(reinterpret_cast<const void*>(k_linear_solve<double, 1>));
    }
}

int launch_cell_solve(const LaunchCtx& x, int phase, int collision) {
    const CellArrays& C = x.C;
    const DevTables* T = x.T;
    const int chunks = (C.hist_modes + kChunk - 1) / kChunk;
    const dim3 grid(chunks, C.ncells);
    const bool rta = collision == kCollideRta;
    if (rta && C.rta_cell_cap) {
        const int cap = C.rta_cell_cap;
        const dim3 g((C.ncells + kRtaCellWarps - 1) / kRtaCellWarps), b(32 * kRtaCellWarps);
        if (phase >= 1) k_rta_cell<true><<<g, b, rta_cell_smem(cap), x.stream>>>(T, C, x.L, phase, cap);
        else k_rta_cell<false><<<g, b, rta_cell_smem(cap), x.stream>>>(T, C, x.L, phase, cap);
        return 1;
    }
    int launches = 3;
    if (rta) k_cell_stats<true><<<grid, kStatThreads, 0, x.stream>>>(T, C, phase >= 1 ? 1 : 0);
    else k_cell_stats<false><<<grid, kStatThreads, 0, x.stream>>>(T, C, 0);
    k_cell_state<<<(C.ncells + 255) / 256, 256, 0, x.stream>>>(T, C, x.L, phase);
    if (phase >= 1 && rta) {
        if (C.ncells >= 1024) // many cells: one warp per cell
            k_rta_solve_warp<<<(C.ncells + 7) / 8, 256, 0, x.stream>>>(T, C);
        else
            k_rta_solve<<<C.ncells, 256, 0, x.stream>>>(T, C);
        ++launches;
    } else if (phase >= 1 && collision == kCollideLinear) {
        const int gmax = C.lin_has_normal ? kMaxGains : 1;
        const int cl = C.lin_cluster;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C.ncells * cl);
        cfg.blockDim = dim3(kLinThreads);
        cfg.dynamicSmemBytes = x.lin_slice ? 0 : linear_smem(C, cl, gmax, C.mixed ? sizeof(float) : sizeof(double));
        cfg.stream = x.stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = cl;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaError_t err;
        unsigned char* gs = x.lin_work;
        const size_t sl = x.lin_slice;
        if (C.lin_has_normal)
            err = C.mixed ? cudaLaunchKernelEx(&cfg, k_linear_solve<float, kMaxGains>, T, C, gs, sl)
                          : cudaLaunchKernelEx(&cfg, k_linear_solve<double, kMaxGains>, T, C, gs, sl);
        else
            err = C.mixed ? cudaLaunchKernelEx(&cfg, k_linear_solve<float, 1>, T, C, gs, sl)
                          : cudaLaunchKernelEx(&cfg, k_linear_solve<double, 1>, T, C, gs, sl);
        if (err != cudaSuccess)
            throw std::runtime_error(std::string("cluster launch of the collision exponential failed: ") +
                                     cudaGetErrorString(err));
        ++launches;
    }
    if (phase >= 1 && collision == kCollideNonlinear) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(C.ncells * kNclCluster);
        cfg.blockDim = dim3(kNclThreads);
        cfg.stream = x.stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kNclCluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const cudaError_t err = cudaLaunchKernelEx(&cfg, k_ncl_solve, T, C, x.L, *x.ncl);
        if (err != cudaSuccess)
            throw std::runtime_error(std::string("cluster launch of the nonlinear Callaway solve failed: ") +
                                     cudaGetErrorString(err));
        ++launches;
    }
    if (phase >= 1 && rta) k_cell_tables<kCollideRta><<<grid, kStatThreads, 0, x.stream>>>(T, C, phase);
    else if (phase >= 1 && collision == kCollideNonlinear)
        k_cell_tables<kCollideNonlinear><<<grid, kStatThreads, 0, x.stream>>>(T, C, phase);
    else if (phase >= 1 && collision == kCollideLinear)
        k_cell_tables<kCollideLinear><<<grid, kStatThreads, 0, x.stream>>>(T, C, phase);
    else k_cell_tables<kCollideNone><<<grid, kStatThreads, 0, x.stream>>>(T, C, phase);
    return launches;
}

void launch_cells_final(const LaunchCtx& x, int phase) {
    k_cells_final<<<x.C.final_blocks, 256, 0, x.stream>>>(x.T, x.C, x.L, phase);
}

} // namespace phmc

// ------------------------------------------------- fused batch launches
namespace phmc {

__global__ void kf_step_begin(const BatchDesc D) {
    if (threadIdx.x == 0) k_step_begin_body(D.ledgers[blockIdx.x], 0, 1);
}

__global__ void __launch_bounds__(kStatThreads) kf_cell_stats(const BatchDesc D) {
    const int i = batch_find(D.cell_begin, D.n, blockIdx.y);
    k_cell_stats_body<true>(D.tables[i], D.cells[i], 1, blockIdx.x, gridDim.x, blockIdx.y - D.cell_begin[i]);
}

__global__ void kf_cell_state(const BatchDesc D, int phase) {
    const int i = batch_find(D.cell_block, D.n, blockIdx.x);
    const int b0 = D.cell_block[i];
    k_cell_state_body(D.tables[i], D.cells[i], D.ledgers[i], phase, blockIdx.x - b0, D.cell_block[i + 1] - b0);
}

// one warp per cell of every instance
__global__ void __launch_bounds__(256) kf_rta_solve(const BatchDesc D) {
    const int g = static_cast<int>((blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x) >> 5);
    if (g >= D.total_cells) return; // warp-uniform
    const int i = batch_find(D.cell_begin, D.n, g);
    rta_solve_warp_cell(*D.tables[i], D.cells[i], g - D.cell_begin[i], threadIdx.x & 31);
}

__global__ void __launch_bounds__(kStatThreads) kf_cell_tables(const BatchDesc D, int phase) {
    const int i = batch_find(D.cell_begin, D.n, blockIdx.y);
    k_cell_tables_body<kCollideRta>(D.tables[i], D.cells[i], phase, blockIdx.x, gridDim.x, blockIdx.y - D.cell_begin[i]);
}

__global__ void __launch_bounds__(1024) kf_cells_final(const BatchDesc D, int phase) {
    const int i = blockIdx.x;
    k_cells_final_body(D.tables[i], D.cells[i], D.ledgers[i], phase, 0, 1);
}

int launch_fused_cells(const BatchDesc& D, cudaStream_t s) {
    if (D.rta_cap > 0) {
        kf_rta_cell<<<(D.total_cells + kRtaCellWarps - 1) / kRtaCellWarps, 32 * kRtaCellWarps,
                      rta_cell_smem(D.rta_cap), s>>>(D, D.rta_cap);
        kf_cells_final<<<D.n, 1024, 0, s>>>(D, 1);
        return 2;
    }
    kf_cell_stats<<<dim3(D.chunks, D.total_cells), kStatThreads, 0, s>>>(D);
    kf_cell_state<<<D.total_cell_blocks, 256, 0, s>>>(D, 1);
    kf_rta_solve<<<(D.total_cells + 7) / 8, 256, 0, s>>>(D);
    kf_cell_tables<<<dim3(D.chunks, D.total_cells), kStatThreads, 0, s>>>(D, 1);
    kf_cells_final<<<D.n, 1024, 0, s>>>(D, 1);
    return 5;
}

int launch_fused_step(const BatchDesc& D, cudaStream_t s, bool mixed) {
    kf_step_begin<<<D.n, 32, 0, s>>>(D);
    return 1 + launch_fused_transport(D, s, mixed) + launch_fused_cells(D, s);
}

// One stand-alone cell of nonlinear Callaway (phmc_dev_ncallaway_evolve).
void launch_ncl_cell(int n_modes, const double* omega, const double* k3, const double* rn, const double* rr,
                     double* cnt, double2* ab, double2* work, int64_t n, const int32_t* mode, double* occ, double T,
                     double dt, int* status, cudaStream_t s) {
    NclArrayModes Q{n_modes, omega, k3, rn, rr, cnt, ab};
    k_ncl_cell<<<1, kNclThreads, 0, s>>>(Q, cnt, work, n, mode, occ, T, dt, status);
}

} // namespace phmc
