// Per-cell work of the timestep, from the (cell, mode) bins of the transport pass.
//
//  k_cell_solve   one CTA per cell:
//    * energy density and temperature after transport
//      (src/solver/GridStatistics.cpp:95-234)
//    * gradient cell sums (src/solver/TemperatureGradientDrive.cpp:131-150)
//    * collision as an affine update per (cell, mode):
//        RTA      pseudo-temperature bracket + Newton over mode classes
//                 (src/solver/RtaCollisionOperator.cpp:79-184): n' = (1-a) n + a n_eq(T*)
//        linear   exp(dt L) on the cell's mode-aggregated quadrature
//                 (src/material/CallawayOperator.cpp:193-370,
//                 src/solver/CarrierCollisionOperator.cpp:67-126):
//                 n' = n_bg + e^{-r dt} (n - n_bg) + A_m
//    * the pending update table, the step's lifetime residual, drive energy
//      and the cell energy/temperature at the end of the step
//  k_cells_final  total thermal energy and the energy ledger (src/solver/EnergyLedger.cpp:58-90)
#include "phmc_kernels.cuh"

namespace phmc {

constexpr int kCellThreads = 512;
constexpr int kMaxGains = 5;

template <int N> __device__ __forceinline__ void block_sum(double (&v)[N], double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[k * 32 + wid] = x;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double x = 0.0;
        for (int w = 0; w < nw; ++w) x += red[k * 32 + w];
        v[k] = x;
    }
    __syncthreads();
}

template <int N> __device__ __forceinline__ void block_sum_f(float (&v)[N], double* red) {
    double d[N];
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = v[k];
    block_sum<N>(d, red);
#pragma unroll
    for (int k = 0; k < N; ++k) v[k] = static_cast<float>(d[k]);
}

__global__ void k_step_begin(DevLedger* L) {
    for (int r = 0; r < kMaxReservoirs; ++r) L->absorbed_res[r] = 0;
    L->step_absorbed = L->step_injected = 0;
    L->step_absorbed_ev = L->step_injected_ev = 0;
    L->step_lifetime_residual = 0;
    L->step_drive_ev = L->next_drive_ev;
    L->step_drive_updates = L->next_drive_updates;
    L->next_drive_ev = 0;
    L->next_drive_updates = 0;
    L->n_inject = 0;
}

// ------------------------------------------------------------------ RTA
__device__ void rta_tables(const DevTables& T, const CellArrays& C, const DevMaterial& M, int c, double Tc,
                           double* red, double* alpha, double* betac) {
    const int nc = C.n_classes;
    double* sc = C.scratch + static_cast<size_t>(c) * nc * 5;
    double* s_cnt = sc;
    double* s_N = sc + nc;
    double* s_M = sc + 2 * nc;
    double* a_tab = sc + 3 * nc;
    double* B_tab = sc + 4 * nc;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const double dt = T.par.dt;
    for (int k = threadIdx.x; k < nc; k += blockDim.x) {
        double n0 = 0, n1 = 0, n2 = 0;
        for (int j = C.class_start[k]; j < C.class_start[k + 1]; ++j) {
            const int m = C.class_modes[j];
            n0 += C.hcnt[hb + m];
            n1 += C.hN[hb + m];
            n2 += C.hM[hb + m];
        }
        s_cnt[k] = n0;
        s_N[k] = n1;
        s_M[k] = n2;
        const int rep = M.class_rep[k];
        double a;
        if (T.par.lifetime_local) {
            const double g = gamma_at(M, rep, Tc);
            a = (g == 0.0 || dt == 0.0) ? 0.0 : -expm1(-(g * dt) * (4.0 * 3.14159265358979323846));
        } else {
            a = M.relax_fixed[rep];
        }
        a_tab[k] = a;
    }
    __syncthreads();
    // f(T) = sum_k hw a (N_k - cnt_k n_eq(T)); f' = -sum cnt hw a dn_eq/dT
    auto evaluate = [&](double temperature, bool want_slope, double& slope) {
        const double Tt = fmax(0.0, temperature);
        double v[2] = {0.0, 0.0};
        for (int k = threadIdx.x; k < nc; k += blockDim.x) {
            const double n0 = s_cnt[k];
            if (n0 == 0.0) continue;
            const double w = fmax(0.0, M.class_omega[k]);
            const double hw = kHbar * w;
            const double a = a_tab[k];
            if (!(hw > 0.0) || !(a > 0.0)) continue;
            const double neq = bose_dev(Tt, w);
            v[0] += hw * a * (s_N[k] - n0 * neq);
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
        double sv[1] = {0.0};
        for (int k = threadIdx.x; k < nc; k += blockDim.x) sv[0] += kHbar * fmax(0.0, M.class_omega[k]) * a_tab[k] * s_M[k];
        block_sum<1>(sv, red);
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
    for (int k = threadIdx.x; k < nc; k += blockDim.x) B_tab[k] = bose_dev(Ts, fmax(0.0, M.class_omega[k]));
    __syncthreads();
    for (int m = threadIdx.x; m < M.n_active; m += blockDim.x) {
        const int k = M.mode_class[m];
        const double a = a_tab[k];
        alpha[m] = 1.0 - a;
        betac[m] = a * B_tab[k];
    }
    __syncthreads();
}

// ----------------------------------------------------- linear response
// exp(dt L) on the aggregated quadrature of cell c. R = double for the plain
// path; R = float for the mixed path, whose result is rescaled in FP64 so the
// collision conserves the cell energy exactly.
template <class R>
__device__ void linear_tables(const DevTables& T, const CellArrays& C, const DevMaterial& M, int c, double* red,
                              double* alpha, double* betac) {
    const int na = M.n_active;
    const size_t H = static_cast<size_t>(C.hist_modes);
    const size_t hb = static_cast<size_t>(c) * H;
    R* base = reinterpret_cast<R*>(C.scratch) + static_cast<size_t>(c) * H * (3 + kMaxGains);
    R* X0 = base;
    R* X = base + H;
    R* term = base + 2 * H;
    R* u = base + 3 * H;
    const unsigned* cnt = C.hcnt + hb;
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        const unsigned k = cnt[m];
        const double e = k ? M.hw[m] * (C.hN[hb + m] - k * M.nbg[m]) : 0.0;
        const R xm = k ? static_cast<R>(e / C.lin_s[m]) : R(0);
        X0[m] = xm;
        X[m] = xm;
    }
    // gain vectors (src/material/CallawayOperator.cpp:193-229), multiplicity-weighted
    int G = 0;
    for (int kind = 0; kind < 2; ++kind) {
        if (kind == 0 && !C.lin_has_normal) continue;
        const double* sq = kind == 0 ? C.lin_sqrt_rn : C.lin_sqrt_rr;
        const int nbasis = kind == 0 ? 4 : 1;
        const int first = G;
        for (int b = 0; b < nbasis; ++b) {
            R* v = u + static_cast<size_t>(G) * H;
            double nv[1] = {0.0};
            for (int m = threadIdx.x; m < na; m += blockDim.x) {
                double val = 0.0;
                if (cnt[m]) {
                    const double s = C.lin_s[m];
                    const double bv = b == 0 ? s : s * M.col_k[3 * m + b - 1] / M.omega[m];
                    val = bv * sq[m];
                    nv[0] += cnt[m] * val * val;
                }
                v[m] = static_cast<R>(val);
            }
            block_sum<1>(nv, red);
            const double original = sqrt(nv[0]);
            if (original == 0.0) continue;
            const R inv = static_cast<R>(1.0 / original);
            for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] *= inv;
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                for (int q = first; q < G; ++q) {
                    const R* qv = u + static_cast<size_t>(q) * H;
                    double pr[1] = {0.0};
                    for (int m = threadIdx.x; m < na; m += blockDim.x) pr[0] += cnt[m] * static_cast<double>(qv[m]) * v[m];
                    block_sum<1>(pr, red);
                    const R p = static_cast<R>(pr[0]);
                    for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] -= p * qv[m];
                    __syncthreads();
                }
            }
            double ln[1] = {0.0};
            for (int m = threadIdx.x; m < na; m += blockDim.x) ln[0] += cnt[m] * static_cast<double>(v[m]) * v[m];
            block_sum<1>(ln, red);
            const double len = sqrt(ln[0]);
            if (len < 1e-12) continue;
            const R il = static_cast<R>(1.0 / len);
            for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] *= il;
            __syncthreads();
            ++G;
        }
        for (int q = first; q < G; ++q) {
            R* qv = u + static_cast<size_t>(q) * H;
            for (int m = threadIdx.x; m < na; m += blockDim.x) qv[m] *= static_cast<R>(sq[m]);
        }
        __syncthreads();
    }
    // Taylor series of exp(h L) per substep on (L T)_m = -r_m T_m + cnt_m sum_g u_gm (u_g . T)
    const R h = static_cast<R>(C.lin_h);
    for (int sstep = 0; sstep < C.lin_substeps; ++sstep) {
        for (int m = threadIdx.x; m < na; m += blockDim.x) term[m] = X[m];
        __syncthreads();
        for (int k = 1; k <= C.lin_terms; ++k) {
            double d[kMaxGains] = {0, 0, 0, 0, 0};
            for (int m = threadIdx.x; m < na; m += blockDim.x) {
                const R tm = term[m];
                for (int g = 0; g < G; ++g) d[g] += static_cast<double>(u[static_cast<size_t>(g) * H + m]) * tm;
            }
            block_sum<kMaxGains>(d, red);
            const R hk = h / static_cast<R>(k);
            R dg[kMaxGains];
            for (int g = 0; g < kMaxGains; ++g) dg[g] = static_cast<R>(d[g]);
            for (int m = threadIdx.x; m < na; m += blockDim.x) {
                R gain = 0;
                for (int g = 0; g < G; ++g) gain += u[static_cast<size_t>(g) * H + m] * dg[g];
                const R t = hk * (-static_cast<R>(M.col_rate[m]) * term[m] + static_cast<R>(cnt[m]) * gain);
                term[m] = t;
                X[m] += t;
            }
            __syncthreads();
        }
    }
    // A_m: the carriers' common additive occupation change beyond the decay
    double cons[2] = {0.0, 0.0};
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        const unsigned k = cnt[m];
        double A = 0.0;
        if (k) {
            A = C.lin_s[m] * (static_cast<double>(X[m]) - C.lin_decay[m] * static_cast<double>(X0[m])) / (k * M.hw[m]);
            cons[0] += (1.0 - C.lin_decay[m]) * M.hw[m] * (C.hN[hb + m] - k * M.nbg[m]);
            cons[1] += k * M.hw[m] * A;
        }
        alpha[m] = C.lin_decay[m];
        betac[m] = A;
    }
    double lambda = 1.0;
    if (C.mixed) {
        // FP64 energy-conservation rescaling of the FP32 gain term
        block_sum<2>(cons, red);
        if (cons[1] != 0.0 && isfinite(cons[0] / cons[1])) lambda = cons[0] / cons[1];
    }
    for (int m = threadIdx.x; m < na; m += blockDim.x) betac[m] = (1.0 - C.lin_decay[m]) * M.nbg[m] + lambda * betac[m];
    __syncthreads();
}

// phase 0: statistics only (initial population; pending table = first drive half);
// 1: full step; 2: as 1 with the cell temperatures supplied in C.temperature.
template <bool kMixed>
__global__ void __launch_bounds__(kCellThreads) k_cell_solve(const DevTables* __restrict__ Tp, CellArrays C,
                                                             DevLedger* L, int phase, int collision) {
    __shared__ double red[kMaxGains * 32];
    const DevTables& T = *Tp;
    const int c = blockIdx.x;
    const int mid = C.cell_material[c];
    const DevMaterial& M = T.mat[mid];
    const int na = M.n_active;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const unsigned* cnt = C.hcnt + hb;
    // ---- energy after transport and gradient sums
    double v[3] = {0.0, 0.0, 0.0};
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        const unsigned k = cnt[m];
        if (!k) continue;
        v[0] += M.hw[m] * (C.hN[hb + m] - k * M.nbg[m]);
        if (M.grad_rate) {
            v[1] += k * M.grad_rate[m];
            v[2] += k * M.cap_bg[m];
        }
    }
    block_sum<3>(v, red);
    const double E = v[0] * M.energy_weight / C.volume[c] + M.energy_density_bg;
    double Tc;
    if (phase == 2) {
        Tc = C.temperature[c];
    } else {
        Tc = T.par.linearized ? T.par.background_T + (E - M.energy_density_bg) / M.heat_capacity_density_bg
                              : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, E);
    }
    const double ratio = v[2] > 0.0 ? v[1] / v[2] : 0.0;
    if (threadIdx.x == 0) {
        if (!isfinite(E)) raise_error(L, kErrNonFinite, c);
        C.energy[c] = E;
        C.temperature[c] = Tc;
        C.grad_ratio[c] = ratio;
    }
    // ---- collision coefficients (alpha, beta) per mode, in a per-cell slice of
    // the scratch placed after the solver's work vectors
    double2* ab = C.ab + hb;
    double* al = nullptr;
    double* be = nullptr;
    const bool collide = phase >= 1 && collision != kCollideNone;
    if (collide) {
        al = C.scratch + static_cast<size_t>(gridDim.x) * (collision == kCollideRta ? 5 * C.n_classes
                                                                                      : C.hist_modes * (3 + kMaxGains)) +
             static_cast<size_t>(c) * 2 * C.hist_modes;
        be = al + C.hist_modes;
        if (collision == kCollideRta) rta_tables(T, C, M, c, Tc, red, al, be);
        else if (kMixed) linear_tables<float>(T, C, M, c, red, al, be);
        else linear_tables<double>(T, C, M, c, red, al, be);
    }
    // ---- pending table, residual, drive energy, end-of-step energy
    const double half = 0.5 * T.par.dt;
    double s[4] = {0.0, 0.0, 0.0, 0.0}; // residual, drive, updates, energy deviation at step end
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        const unsigned k = cnt[m];
        const double a = collide ? al[m] : 1.0;
        const double bc = collide ? be[m] : 0.0;
        const double D = M.grad_rate ? half * (M.grad_rate[m] - M.cap_bg[m] * ratio) * M.inv_hw[m] : 0.0;
        ab[m] = make_double2(a, collide ? bc + 2.0 * D : D);
        if (!k) continue;
        const double N = C.hN[hb + m];
        const double hw = M.hw[m];
        s[0] += hw * ((a - 1.0) * N + k * bc);
        if (D != 0.0) {
            s[1] += k * hw * D;
            s[2] += k;
        }
        const double N1 = a * N + k * (bc + D);
        s[3] += hw * (N1 - k * M.nbg[m]);
    }
    block_sum<4>(s, red);
    if (threadIdx.x == 0) {
        const double w = M.energy_weight;
        if (phase >= 1) {
            atomicAdd(&L->step_lifetime_residual, s[0] * w);
            atomicAdd(&L->step_drive_ev, s[1] * w);
            atomicAdd(&L->step_drive_updates, static_cast<unsigned long long>(s[2]));
        }
        atomicAdd(&L->next_drive_ev, s[1] * w);
        atomicAdd(&L->next_drive_updates, static_cast<unsigned long long>(s[2]));
        const double Ef = (phase >= 1 ? s[3] : v[0]) * w / C.volume[c] + M.energy_density_bg;
        C.energy_final[c] = Ef;
        C.temperature_final[c] =
            phase == 2 ? Tc
                       : (T.par.linearized
                              ? T.par.background_T + (Ef - M.energy_density_bg) / M.heat_capacity_density_bg
                              : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, Ef));
    }
    __syncthreads();
    // ---- clear the bins for the next transport pass
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        C.hcnt[hb + m] = 0;
        C.hN[hb + m] = 0.0;
        if (C.hM) C.hM[hb + m] = 0.0;
    }
}

// End of step: total thermal energy and the energy ledger. One CTA.
__global__ void __launch_bounds__(1024) k_cells_final(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L,
                                                      int initial) {
    __shared__ double red[32];
    const DevTables& T = *Tp;
    double thermal = 0.0;
    for (int c = threadIdx.x; c < C.ncells; c += blockDim.x) {
        const DevMaterial& M = T.mat[C.cell_material[c]];
        thermal += (C.energy_final[c] - M.zero_point) * C.volume[c];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) thermal += __shfl_xor_sync(0xffffffffu, thermal, o);
    if (lane == 0) red[wid] = thermal;
    __syncthreads();
    if (threadIdx.x != 0) return;
    double total = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) total += red[w];
    if (initial) {
        L->thermal_energy = total;
        return;
    }
    const double residual = total - L->thermal_energy - 0.0 - L->step_drive_ev - L->step_injected_ev +
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
    L->thermal_energy = total;
    L->particle_count += static_cast<long long>(L->step_injected) - static_cast<long long>(L->step_absorbed);
    for (int r = 0; r < kMaxReservoirs; ++r) L->previous_res[r] = L->absorbed_res[r];
}

// ----------------------------------------------------------- launchers
void launch_step_begin(const LaunchCtx& x) { k_step_begin<<<1, 1, 0, x.stream>>>(x.L); }

void launch_cell_solve(const LaunchCtx& x, int phase, int collision) {
    if (x.C.mixed) k_cell_solve<true><<<x.C.ncells, kCellThreads, 0, x.stream>>>(x.T, x.C, x.L, phase, collision);
    else k_cell_solve<false><<<x.C.ncells, kCellThreads, 0, x.stream>>>(x.T, x.C, x.L, phase, collision);
}

void launch_cells_final(const LaunchCtx& x, int initial) {
    k_cells_final<<<1, 1024, 0, x.stream>>>(x.T, x.C, x.L, initial);
}

} // namespace phmc
