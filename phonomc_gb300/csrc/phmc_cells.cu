// Per-cell work of the timestep and pass B.
//
//  k_cell_solve  one CTA per cell: energy density and temperature
//                (src/solver/GridStatistics.cpp:95-234), gradient cell sums
//                (src/solver/TemperatureGradientDrive.cpp:131-150), the RTA
//                pseudo-temperature bracket/Newton solve
//                (src/solver/RtaCollisionOperator.cpp:79-165) over mode classes,
//                or the linear-response exponential
//                (src/material/CallawayOperator.cpp:193-370) over the cell's
//                mode-aggregated quadrature.
//  k_update      pass B: collision update, second gradient half-step, tally.
//  k_cells_final temperatures after the step and the energy ledger
//                (src/solver/EnergyLedger.cpp:58-90).
#include "phmc_kernels.cuh"

namespace phmc {

constexpr int kCellThreads = 256;
constexpr int kMaxGains = 5;

template <int N> __device__ __forceinline__ void block_sum(double (&v)[N], double* red) {
    // red: shared scratch of N * 32 doubles
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

__global__ void k_step_begin(DevLedger* L) {
    for (int r = 0; r < kMaxReservoirs; ++r) L->absorbed_res[r] = 0;
    L->step_absorbed = L->step_injected = 0;
    L->step_absorbed_ev = L->step_injected_ev = 0;
    L->step_lifetime_residual = 0;
    L->step_drive_ev = 0;
    L->step_drive_updates = 0;
    L->n_inject = 0;
    L->particle_count = 0;
}

struct ClassCSR {
    const int* start;
    const int* modes;
    int n;
};

// phase 0: refresh only; 1: refresh + collision tables; 2: as 1 with given cell temperatures.
__global__ void __launch_bounds__(kCellThreads) k_cell_solve(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L,
                                                             int phase, int collision, ClassCSR cls, double* lin_scratch,
                                                             double* rta_scratch) {
    __shared__ double red[kMaxGains * 32];
    __shared__ double s_val[4];
    const DevTables& T = *Tp;
    const int c = blockIdx.x;
    const int mid = C.cell_material[c];
    const DevMaterial& M = T.mat[mid];
    const int na = M.n_active;
    const size_t hb = static_cast<size_t>(c) * C.hist_modes;
    const unsigned* cnt = C.hcnt + hb;
    const double* hE = C.hE + hb;
    // ---- tally and gradient sums
    {
        double v[3] = {0.0, 0.0, 0.0};
        for (int m = threadIdx.x; m < na; m += blockDim.x) {
            const unsigned k = cnt[m];
            if (!k) continue;
            v[0] += hE[m];
            if (M.grad_rate) {
                v[1] += k * M.grad_rate[m];
                v[2] += k * M.cap_bg[m];
            }
        }
        block_sum<3>(v, red);
        if (threadIdx.x == 0) {
            double e = dmul(v[0], M.energy_weight) / C.volume[c];
            e += M.energy_density_bg;
            if (!isfinite(e)) raise_error(L, kErrNonFinite, c);
            C.energy[c] = e;
            if (phase != 2)
                C.temperature[c] = T.par.linearized
                                       ? T.par.background_T + (e - M.energy_density_bg) / M.heat_capacity_density_bg
                                       : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, e);
            C.grad_R[c] = v[1];
            C.grad_C[c] = v[2];
        }
        __syncthreads();
    }
    if (phase >= 1 && collision == kCollideRta) {
        // ---- RTA over classes: aggregate counts and occupation sums
        const int nc = cls.n;
        double* s_cnt = rta_scratch + static_cast<size_t>(c) * nc * 3;
        double* s_N = s_cnt + nc;
        double* s_M = s_N + nc;
        const double Tc = C.temperature[c];
        const double dt = T.par.dt;
        double* a_tab = C.rta_a + static_cast<size_t>(c) * nc;
        double* B_tab = C.rta_B + static_cast<size_t>(c) * nc;
        for (int k = threadIdx.x; k < nc; k += blockDim.x) {
            double n0 = 0, n1 = 0, n2 = 0;
            for (int j = cls.start[k]; j < cls.start[k + 1]; ++j) {
                const int m = cls.modes[j];
                n0 += cnt[m];
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
        // f(T) = sum_k hw a (N_k - cnt_k neq_k(T)), slope = -sum cnt hw a dn/dT
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
            for (int k = threadIdx.x; k < nc; k += blockDim.x) {
                const double hw = kHbar * fmax(0.0, M.class_omega[k]);
                sv[0] += hw * a_tab[k] * s_M[k];
            }
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
        if (threadIdx.x == 0) s_val[0] = Ts;
        __syncthreads();
    } else if (phase >= 1 && collision == kCollideLinear) {
        // ---- linear response on the mode-aggregated quadrature
        const size_t stride = static_cast<size_t>(C.hist_modes);
        double* base = lin_scratch + static_cast<size_t>(c) * stride * (3 + kMaxGains);
        double* X0 = base;
        double* X = base + stride;
        double* term = base + 2 * stride;
        double* u = base + 3 * stride;
        int G = 0;
        // X_m = sum over carriers of x_i = e_i / sqrt(C_m)
        for (int m = threadIdx.x; m < na; m += blockDim.x) {
            const double xm = cnt[m] ? hE[m] / sqrt(M.col_cap[m]) : 0.0;
            X0[m] = xm;
            X[m] = xm;
        }
        // gains (src/material/CallawayOperator.cpp:193-229), weighted by multiplicity
        for (int pass_kind = 0; pass_kind < 2; ++pass_kind) {
            const double* rate = pass_kind == 0 ? M.col_rn : M.col_rr;
            const int nbasis = pass_kind == 0 ? 4 : 1;
            const int first = G;
            for (int b = 0; b < nbasis; ++b) {
                double* v = u + static_cast<size_t>(G) * stride;
                double nv[1] = {0.0};
                for (int m = threadIdx.x; m < na; m += blockDim.x) {
                    double val = 0.0;
                    if (cnt[m]) {
                        const double s = sqrt(M.col_cap[m]);
                        const double bv = b == 0 ? s : s * M.col_k[3 * m + b - 1] / M.omega[m];
                        val = bv * sqrt(rate[m]);
                        nv[0] += cnt[m] * val * val;
                    }
                    v[m] = val;
                }
                block_sum<1>(nv, red);
                const double original = sqrt(nv[0]);
                if (original == 0.0) continue;
                for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] /= original;
                __syncthreads();
                for (int pass = 0; pass < 2; ++pass) {
                    for (int q = first; q < G; ++q) {
                        const double* qv = u + static_cast<size_t>(q) * stride;
                        double pr[1] = {0.0};
                        for (int m = threadIdx.x; m < na; m += blockDim.x) pr[0] += cnt[m] * qv[m] * v[m];
                        block_sum<1>(pr, red);
                        for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] -= pr[0] * qv[m];
                        __syncthreads();
                    }
                }
                double ln[1] = {0.0};
                for (int m = threadIdx.x; m < na; m += blockDim.x) ln[0] += cnt[m] * v[m] * v[m];
                block_sum<1>(ln, red);
                const double len = sqrt(ln[0]);
                if (len < 1e-12) continue;
                for (int m = threadIdx.x; m < na; m += blockDim.x) v[m] /= len;
                __syncthreads();
                ++G;
            }
            for (int q = first; q < G; ++q) {
                double* qv = u + static_cast<size_t>(q) * stride;
                for (int m = threadIdx.x; m < na; m += blockDim.x) qv[m] *= sqrt(rate[m]);
            }
            __syncthreads();
        }
        // Taylor series of exp(h L) per substep; L is the aggregated operator
        // (L T)_m = -r_m T_m + cnt_m sum_g u_gm (sum_m' u_gm' T_m').
        const double h = C.lin_h;
        for (int sstep = 0; sstep < C.lin_substeps; ++sstep) {
            for (int m = threadIdx.x; m < na; m += blockDim.x) term[m] = X[m];
            __syncthreads();
            for (int k = 1; k <= C.lin_terms; ++k) {
                double d[kMaxGains] = {0, 0, 0, 0, 0};
                for (int m = threadIdx.x; m < na; m += blockDim.x) {
                    const double tm = term[m];
                    for (int g = 0; g < G; ++g) d[g] += u[static_cast<size_t>(g) * stride + m] * tm;
                }
                block_sum<kMaxGains>(d, red);
                const double hk = h / k;
                for (int m = threadIdx.x; m < na; m += blockDim.x) {
                    double gain = 0.0;
                    for (int g = 0; g < G; ++g) gain += u[static_cast<size_t>(g) * stride + m] * d[g];
                    const double t = hk * (-M.col_rate[m] * term[m] + cnt[m] * gain);
                    term[m] = t;
                    X[m] += t;
                }
                __syncthreads();
            }
        }
        // additive occupation term per (cell, mode)
        double* A = C.lin_A + static_cast<size_t>(c) * stride;
        for (int m = threadIdx.x; m < na; m += blockDim.x) {
            const unsigned k = cnt[m];
            A[m] = k ? sqrt(M.col_cap[m]) * (X[m] - C.lin_decay[m] * X0[m]) / (k * M.hw[m]) : 0.0;
        }
    }
    __syncthreads();
    // ---- clear this cell's histogram for the next pass
    for (int m = threadIdx.x; m < na; m += blockDim.x) {
        C.hcnt[hb + m] = 0;
        C.hE[hb + m] = 0.0;
        if (collision == kCollideRta) {
            C.hN[hb + m] = 0.0;
            C.hM[hb + m] = 0.0;
        }
    }
}

// Pass B: collision update, second gradient half-step, tally for the final refresh.
template <int kCollision, bool kGradient>
__global__ void __launch_bounds__(256) k_update(const DevTables* __restrict__ Tp, CarrierState S, CellArrays C,
                                                DevLedger* L, int use_shared) {
    extern __shared__ double sacc[];
    __shared__ double part[4];
    const DevTables& T = *Tp;
    if (use_shared)
        for (int k = threadIdx.x; k < C.ncells; k += blockDim.x) sacc[k] = 0.0;
    if (threadIdx.x < 4) part[threadIdx.x] = 0.0;
    __syncthreads();
    const int n = L->n_slots;
    const double half = 0.5 * T.par.dt;
    double res = 0.0, drive = 0.0, upd = 0.0, alive_count = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!S.alive[i]) continue;
        alive_count += 1.0;
        const uint32_t w = S.mode[i];
        const DevMaterial& M = T.mat[w >> 28];
        const int ai = static_cast<int>(w & 0x00FFFFFFu);
        const int c = S.cell[i];
        double occ = S.occ[i];
        const double hw = M.hw[ai];
        if (kCollision == kCollideRta) {
            const size_t k = static_cast<size_t>(c) * M.n_classes + M.mode_class[ai];
            const double a = C.rta_a[k];
            const double nn = occ + a * (C.rta_B[k] - occ);
            res += (hw * nn - hw * occ) * M.energy_weight;
            occ = fmax(0.0, nn);
        } else if (kCollision == kCollideLinear) {
            const double nb = M.nbg[ai];
            const double nn = nb + C.lin_decay[ai] * (occ - nb) + C.lin_A[static_cast<size_t>(c) * C.hist_modes + ai];
            res += hw * (nn - occ) * M.energy_weight;
            occ = nn;
        }
        if (kGradient) {
            const double e = half * (M.grad_rate[ai] - C.grad_R[c] * M.cap_bg[ai] / C.grad_C[c]);
            const double next = occ + e / hw;
            drive += hw * (next - occ);
            if (e != 0.0) upd += 1.0;
            occ = next;
        }
        if (!isfinite(occ)) raise_error(L, kErrCollision, i);
        S.occ[i] = occ;
        const double e = dmul(dmul(hw, occ - M.nbg[ai]), M.energy_weight);
        atomicAdd((use_shared ? sacc : C.acc) + c, e);
    }
    double v[4] = {res, drive, upd, alive_count};
    for (int k = 0; k < 4; ++k) {
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&part[k], v[k]);
    }
    __syncthreads();
    if (use_shared)
        for (int k = threadIdx.x; k < C.ncells; k += blockDim.x)
            if (sacc[k] != 0.0) atomicAdd(C.acc + k, sacc[k]);
    if (threadIdx.x == 0) {
        if (part[0] != 0.0) atomicAdd(&L->step_lifetime_residual, part[0]);
        if (part[1] != 0.0) atomicAdd(&L->step_drive_ev, part[1]);
        if (part[2] != 0.0) atomicAdd(&L->step_drive_updates, static_cast<unsigned long long>(part[2]));
        atomicAdd(reinterpret_cast<unsigned long long*>(&L->particle_count),
                  static_cast<unsigned long long>(part[3]));
    }
}

// Final refresh of the step and the energy ledger. One CTA.
__global__ void __launch_bounds__(1024) k_cells_final(const DevTables* __restrict__ Tp, CellArrays C, DevLedger* L,
                                                      int initial) {
    __shared__ double red[32];
    const DevTables& T = *Tp;
    double thermal = 0.0;
    for (int c = threadIdx.x; c < C.ncells; c += blockDim.x) {
        const DevMaterial& M = T.mat[C.cell_material[c]];
        double e = initial ? C.energy[c] : dmul(C.acc[c], 1.0) / C.volume[c] + M.energy_density_bg;
        if (!initial) {
            if (!isfinite(e)) raise_error(L, kErrNonFinite, c);
            C.energy[c] = e;
            C.temperature[c] = T.par.linearized
                                   ? T.par.background_T + (e - M.energy_density_bg) / M.heat_capacity_density_bg
                                   : table_inverse(M.lookup_E, M.lookup_T, M.n_lookup, e);
            C.acc[c] = 0.0;
        }
        thermal += (e - M.zero_point) * C.volume[c];
    }
    double v[1] = {thermal};
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        double x = v[0];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[wid] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w];
            thermal = s;
        }
    }
    if (threadIdx.x == 0) {
        if (initial) {
            L->thermal_energy = thermal;
            return;
        }
        const double residual = thermal - L->thermal_energy - 0.0 - L->step_drive_ev - L->step_injected_ev +
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
        L->thermal_energy = thermal;
        for (int r = 0; r < kMaxReservoirs; ++r) L->previous_res[r] = L->absorbed_res[r];
    }
}

// ----------------------------------------------------------- launchers
void launch_step_begin(const LaunchCtx& x) { k_step_begin<<<1, 1, 0, x.stream>>>(x.L); }

void launch_cell_solve(const LaunchCtx& x, int phase, int collision, int n_classes, const int* class_start,
                       const int* class_modes, double* scratch) {
    ClassCSR cls{class_start, class_modes, n_classes};
    k_cell_solve<<<x.C.ncells, kCellThreads, 0, x.stream>>>(x.T, x.C, x.L, phase, collision, cls,
                                                            collision == kCollideLinear ? scratch : nullptr,
                                                            collision == kCollideRta ? scratch : nullptr);
}

void launch_update(const LaunchCtx& x, int collision, bool gradient) {
    const size_t sh = sizeof(double) * static_cast<size_t>(x.C.ncells);
    const int use_shared = sh <= 32768 ? 1 : 0;
    const size_t shb = use_shared ? sh : 0;
    const dim3 g(x.grid_blocks), b(256);
#define PHMC_UPD(K, G) k_update<K, G><<<g, b, shb, x.stream>>>(x.T, x.S, x.C, x.L, use_shared)
    if (collision == kCollideRta) {
        if (gradient) PHMC_UPD(kCollideRta, true); else PHMC_UPD(kCollideRta, false);
    } else if (collision == kCollideLinear) {
        if (gradient) PHMC_UPD(kCollideLinear, true); else PHMC_UPD(kCollideLinear, false);
    } else {
        if (gradient) PHMC_UPD(kCollideNone, true); else PHMC_UPD(kCollideNone, false);
    }
#undef PHMC_UPD
}

void launch_cells_final(const LaunchCtx& x, int initial) {
    k_cells_final<<<1, 1024, 0, x.stream>>>(x.T, x.C, x.L, initial);
}

} // namespace phmc
