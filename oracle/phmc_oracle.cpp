// CPU oracle for the GB300 carrier loop -- TEST INFRASTRUCTURE ONLY.
//
// A plain, serial FP64 restatement of the reference's per-timestep algorithm
// (PhonoMC src/MonteCarloSolver.cpp:348-398 and the operators it calls). It is
// the checker the CUDA path is compared against and the CPU baseline that
// bench.py times; nothing in the product links or calls it.
//
// Pinning: every deterministic sub-step below is compared in tests/ against
// golden vectors printed by the reference's own code (tests/golden/, made by
// tests/golden/make_golden.py with oracle/ref/ref_harness.cpp).
//
// Restatement choices shared with the CUDA path (they change no physics):
//  * draws come from counter-based Philox (phmc_rng.h), not per-thread
//    mt19937_64, so GPU and oracle consume identical uniforms;
//  * the wall-hit time is recomputed from the current position at the start of
//    each flight instead of being cached across steps (collision_times in the
//    reference); both are the same analytic plane time up to rounding;
//  * dead carrier slots are refilled by injected carriers in ascending slot
//    order instead of a stable compaction; slot order only keys the draws.
#include "../phonomc_gb300/csrc/phmc_host.h"
#include "../phonomc_gb300/csrc/phmc_pod.h"
#include "../phonomc_gb300/csrc/phmc_rng.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <limits>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

using namespace phmc;

namespace {
thread_local std::string g_error;

double dot3(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double norm3(const Vec3& a) { return std::sqrt(dot3(a, a)); }
Vec3 add3(const Vec3& a, const Vec3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
Vec3 mul3(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
Vec3 sub3(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }

double bose(double T, double w) {
    if (T <= 0.0 || w <= 0.0) return 0.0;
    const double x = kHbarEvPs * w / (kBoltzmannEvK * T);
    if (x > 700.0) return 0.0;
    return 1.0 / std::max(std::exp(x) - 1.0, 1e-12);
}

// ---------------------------------------------------------------- rough
struct RoughDraws {
    double u[3];
};
// src/solver/RoughBoundarySampler.cpp:373-533 with the draws supplied.
// Outcome flags as counted by the reference's RoughSampleEvents.
enum : unsigned {
    kRoughSpecular = 1u, kRoughMissingSpec = 2u, kRoughWindow = 4u, kRoughWindowFallback = 8u,
    kRoughDiffuse = 16u, kRoughPool = 32u, kRoughRandom = 64u,
};
int rough_sample(const RoughTable& rd, const MaterialTables& T, int in_ai, double n_in, bool signed_weights,
                 const RoughDraws& d, double& n_out, unsigned* diag_out = nullptr) {
    unsigned diag_local = 0;
    unsigned& diag = diag_out ? *diag_out : diag_local;
    diag = 0;
    n_out = n_in;
    const int na = T.n_active;
    const double p_spec = (in_ai >= 0 && in_ai < na) ? std::clamp(rd.specularity[in_ai], 0.0, 1.0) : 0.0;
    auto remap = [&](int out_ai) {
        const double win = T.omega[in_ai], wout = T.omega[out_ai];
        return T.nbg[out_ai] + win * (n_in - T.nbg[in_ai]) / std::max(1e-30, wout);
    };
    if (in_ai >= 0 && d.u[0] <= p_spec) {
        const int out_ai = rd.spec_match[in_ai];
        diag = (out_ai >= 0 && out_ai < na) ? kRoughSpecular : kRoughMissingSpec;
        if (out_ai >= 0 && out_ai < na) {
            const double mapped = remap(out_ai);
            if (std::isfinite(mapped) && (signed_weights || mapped >= 0.0)) {
                n_out = mapped;
                return out_ai;
            }
            return in_ai;
        }
    }
    int out_ai = -1;
    bool done = false;
    if (in_ai >= 0) {
        const int b = rd.diffuse_begin[in_ai], e = rd.diffuse_end[in_ai];
        if (b >= 0 && e > b && e <= static_cast<int>(rd.outgoing_sorted.size())) {
            const double fb = rd.residual_prefix[b], fe = rd.residual_prefix[e];
            const double window = fe - fb;
            if (window > 0.0 && std::isfinite(window)) {
                const double u = std::clamp(d.u[1], 0.0, std::nextafter(1.0, 0.0));
                const double target = fb + u * window;
                const auto first = rd.residual_prefix.begin() + b + 1, last = rd.residual_prefix.begin() + e + 1;
                const int pos = std::clamp(static_cast<int>(std::upper_bound(first, last, target) -
                                                            rd.residual_prefix.begin()) - 1, b, e - 1);
                out_ai = rd.outgoing_sorted[pos];
                done = true;
                diag |= kRoughWindow;
            } else {
                diag |= kRoughWindowFallback;
            }
        }
    }
    if (!done) {
        if (rd.strict_elastic) return in_ai;
        if (!rd.roulette_active.empty() && rd.roulette_cdf.back() > 0.0) {
            const double r = rd.roulette_cdf.back() * d.u[1];
            size_t pos = static_cast<size_t>(std::lower_bound(rd.roulette_cdf.begin(), rd.roulette_cdf.end(), r) -
                                             rd.roulette_cdf.begin());
            if (pos >= rd.roulette_active.size()) pos = rd.roulette_active.size() - 1;
            out_ai = rd.roulette_active[pos];
        } else if (!rd.outgoing_active.empty()) {
            int k = static_cast<int>(d.u[2] * rd.outgoing_active.size());
            k = std::min(k, static_cast<int>(rd.outgoing_active.size()) - 1);
            out_ai = rd.outgoing_active[k];
            diag |= kRoughPool;
        } else {
            out_ai = std::min(static_cast<int>(d.u[2] * na), na - 1);
            diag |= kRoughRandom;
        }
    }
    diag |= kRoughDiffuse;
    const double mapped = remap(out_ai);
    if (std::isfinite(mapped) && (signed_weights || mapped >= 0.0)) {
        n_out = mapped;
        return out_ai;
    }
    n_out = n_in;
    return in_ai;
}

// --------------------------------------------------- Callaway operator
// src/material/CallawayOperator.cpp (long double throughout, as the reference).
struct Callaway {
    using V = std::vector<long double>;
    V scale, rate;
    std::vector<V> ng, rg;
    long double bound = 0;
    static long double dot(const V& a, const V& b) {
        long double s = 0;
        for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
        return s;
    }
    static std::vector<V> gains(const std::vector<double>& rates, std::vector<V> basis) {
        std::vector<V> orth;
        for (auto v : basis) {
            for (size_t i = 0; i < v.size(); ++i) v[i] *= std::sqrt(static_cast<long double>(rates[i]));
            const auto original = std::sqrt(dot(v, v));
            if (original == 0) continue;
            for (auto& x : v) x /= original;
            for (int pass = 0; pass < 2; ++pass)
                for (const auto& q : orth) {
                    const auto pr = dot(q, v);
                    for (size_t i = 0; i < v.size(); ++i) v[i] -= pr * q[i];
                }
            const auto len = std::sqrt(dot(v, v));
            if (len < 1e-12L) continue;
            for (auto& x : v) x /= len;
            orth.push_back(std::move(v));
        }
        for (auto& q : orth)
            for (size_t i = 0; i < q.size(); ++i) q[i] *= std::sqrt(static_cast<long double>(rates[i]));
        return orth;
    }
    Callaway(const std::vector<double>& omega, const std::vector<double>& cap, const std::vector<Vec3>& k,
             const std::vector<double>& rn, const std::vector<double>& rr) {
        const size_t n = omega.size();
        scale.resize(n);
        rate.resize(n);
        std::vector<V> basis(4, V(n));
        for (size_t i = 0; i < n; ++i) {
            if (!std::isfinite(omega[i]) || omega[i] <= 0 || !std::isfinite(cap[i]) || cap[i] <= 0 || rn[i] < 0 ||
                rr[i] < 0)
                throw std::invalid_argument("Callaway needs positive frequencies/capacities and finite nonnegative rates.");
            scale[i] = std::sqrt(static_cast<long double>(cap[i]));
            basis[0][i] = scale[i];
            for (int a = 0; a < 3; ++a) basis[a + 1][i] = scale[i] * k[i][a] / omega[i];
            rate[i] = static_cast<long double>(rn[i]) + rr[i];
            bound = std::max(bound, rate[i]);
        }
        ng = gains(rn, basis);
        rg = gains(rr, {basis[0]});
    }
    V action(const V& x) const {
        V r(x.size());
        for (size_t i = 0; i < x.size(); ++i) r[i] = -rate[i] * x[i];
        for (const auto* g : {&ng, &rg})
            for (const auto& u : *g) {
                const auto c = dot(u, x);
                for (size_t i = 0; i < x.size(); ++i) r[i] += u[i] * c;
            }
        return r;
    }
    std::vector<double> evolve(const std::vector<double>& e, double dt) const {
        V x(e.size());
        long double mag = 0;
        for (size_t i = 0; i < x.size(); ++i) {
            x[i] = e[i] / scale[i];
            mag = std::max(mag, std::abs(x[i]));
        }
        if (mag == 0 || dt == 0 || bound == 0) return e;
        const long double steps_ld = std::max(1.0L, std::ceil(dt * bound / 4.0L));
        if (!std::isfinite(steps_ld) || steps_ld > 100000 || steps_ld * x.size() > 200000000)
            throw std::runtime_error("Callaway exponential work limit exceeded; reduce time_step.");
        const size_t steps = static_cast<size_t>(steps_ld);
        const long double h = static_cast<long double>(dt) / steps;
        const long double sn = h * bound;
        for (auto& v : x) v /= mag;
        const long double tol = 2e-14L / steps;
        for (size_t s = 0; s < steps; ++s) {
            V sum = x, term = x;
            const long double ref = std::sqrt(dot(x, x));
            bool conv = false;
            for (int k = 1; k <= 40; ++k) {
                term = action(term);
                for (size_t i = 0; i < x.size(); ++i) {
                    term[i] *= h / k;
                    sum[i] += term[i];
                }
                if (sn < k + 2) {
                    const long double tail = std::sqrt(dot(term, term)) * sn / (k + 1) / (1.0L - sn / (k + 2));
                    if (tail <= tol * ref) {
                        conv = true;
                        break;
                    }
                }
            }
            if (!conv) throw std::runtime_error("Callaway exponential did not converge.");
            x = std::move(sum);
        }
        std::vector<double> out(x.size());
        for (size_t i = 0; i < x.size(); ++i) out[i] = static_cast<double>(x[i] * mag * scale[i]);
        return out;
    }
};

// ---------------------------------------------------------- RTA per cell
// src/solver/RtaCollisionOperator.cpp:79-184 for one cell's carriers.
double rta_cell(const std::vector<int>& members, const std::vector<double>& omega_i, const std::vector<double>& a_i,
                std::vector<double>& occ, double cell_T, double cell_weight) {
    if (members.empty()) return 0.0;
    auto evaluate = [&](double temperature, double* deriv) {
        double value = 0.0, slope = 0.0;
        const double T = std::max(0.0, temperature);
        for (int i : members) {
            const double w = std::max(0.0, omega_i[i]);
            const double hw = kHbarEvPs * w;
            const double a = a_i[i];
            if (!(hw > 0.0) || !(a > 0.0)) continue;
            const double neq = bose(T, w);
            value += hw * a * (occ[i] - neq);
            if (T > 0.0) {
                const double dndt = hw * neq * (neq + 1.0) / (kBoltzmannEvK * T * T);
                slope -= hw * a * dndt;
            }
        }
        if (deriv) *deriv = slope;
        return value;
    };
    double low = 0.0, high = std::max(1000.0, 2.0 * std::max(1.0, cell_T));
    const double f_low = evaluate(low, nullptr);
    double f_high = evaluate(high, nullptr);
    for (int k = 0; f_high > 0.0 && k < 20; ++k) {
        high *= 2.0;
        f_high = evaluate(high, nullptr);
    }
    double Ts = std::clamp(cell_T, low, high);
    if (f_low <= 0.0) Ts = low;
    else if (f_high >= 0.0) Ts = high;
    else {
        double scale = 0.0;
        for (int i : members) scale += kHbarEvPs * std::max(0.0, omega_i[i]) * a_i[i] * std::max(1.0, occ[i]);
        for (int it = 0; it < 40; ++it) {
            double d = 0.0;
            const double v = evaluate(Ts, &d);
            if (std::abs(v) <= 1e-13 * std::max(1.0, scale)) break;
            if (v > 0.0) low = Ts;
            else high = Ts;
            double cand = 0.5 * (low + high);
            if (d < 0.0 && std::isfinite(d)) {
                const double nt = Ts - v / d;
                if (nt > low && nt < high && std::isfinite(nt)) cand = nt;
            }
            Ts = cand;
        }
    }
    double eb = 0.0, ea = 0.0;
    for (int i : members) {
        const double w = std::max(0.0, omega_i[i]);
        const double hw = kHbarEvPs * w;
        const double old = occ[i];
        const double nn = old + a_i[i] * (bose(Ts, w) - old);
        eb += hw * old;
        ea += hw * nn;
        occ[i] = std::max(0.0, nn);
    }
    return (ea - eb) * cell_weight;
}

// ------------------------------------------------------ interfaces
// src/solver/InterfaceModeSampler.cpp:69-108: flux-weighted draw inside the
// shared band [floor(w/width) width, +width) of one bank; `drew` tells whether
// the reference consumed a uniform (it does only for a positive band flux).
int interface_sample_band(const InterfaceBank& B, double omega, double width, double u, bool& drew,
                          double& flux_sum) {
    if (!std::isfinite(omega) || omega < 0 || !std::isfinite(width) || width <= 0)
        throw std::invalid_argument("Invalid shared interface frequency band.");
    const double bin = std::floor(omega / width);
    const double lo = bin * width, hi = (bin + 1) * width;
    const size_t begin = static_cast<size_t>(std::lower_bound(B.omega.begin(), B.omega.end(), lo) - B.omega.begin());
    const size_t end = static_cast<size_t>(std::lower_bound(B.omega.begin(), B.omega.end(), hi) - B.omega.begin());
    flux_sum = end > begin ? B.prefix[end] - B.prefix[begin] : 0.0;
    drew = false;
    if (!(flux_sum > 0.0)) return -1;
    drew = true;
    const double target = B.prefix[begin] + (u * (flux_sum - 0.0) + 0.0);
    size_t pos = static_cast<size_t>(std::upper_bound(B.prefix.begin() + static_cast<std::ptrdiff_t>(begin + 1),
                                                      B.prefix.begin() + static_cast<std::ptrdiff_t>(end + 1), target) -
                                     B.prefix.begin());
    pos = std::clamp(pos, begin + 1, end) - 1;
    return B.active[pos];
}

struct InterfaceOutcome {
    int action = 0;          // kInterfaceReflect, kInterfaceTransmit or kInterfaceFail
    int material = 0, active = 0;
    uint32_t signs = 0;
    double occ = 0;
    int events = 0, transmitted = 0, reflected = 0;
};

// src/solver/InterfaceInteraction.cpp:46-153, diffuse mismatch: reflected draw,
// transmitted draw, transmission test, occupation remap conserving w ω Δn.
// Uniforms are consumed in the reference's order from u[0..2].
InterfaceOutcome interface_interact(const InterfaceTables& I, const std::vector<MaterialTables>& mats, int src, int a,
                                    uint32_t signs, double occ, int next, const double u[4]) {
    InterfaceOutcome r;
    r.material = src;
    r.active = a;
    r.signs = signs;
    r.occ = occ;
    const MaterialTables& S = mats[src];
    const int axis = I.axis;
    const double omega = S.omega[a];
    const double v_axis = ((signs >> axis) & 1u) ? -S.vel[3 * a + axis] : S.vel[3 * a + axis];
    const int incident = v_axis > 0.0 ? 1 : 0;
    int k = 0;
    // model choice (mixed mismatch), src/solver/InterfaceInteraction.cpp:60-67
    const double acoustic_p = I.model == 1 ? 1.0 : (I.model == 2 ? I.amm_fraction : 0.0);
    const bool use_amm = acoustic_p >= 1 || (acoustic_p > 0 && u[k++] < acoustic_p);
    bool transmit;
    int sel_material, sel;
    if (use_amm) {
        r.events = 1;
        if (std::abs(v_axis) < 1e-7) { // :68-74
            r.signs ^= 1u << axis;
            r.reflected = 1;
            r.action = kInterfaceReflect;
            return r;
        }
        // AcousticInterfaceSampler::sample, src/solver/AcousticInterfaceSampler.cpp:448-470
        const AmmRow& row = I.amm.faces.at(std::min(src, next)).rows[src < next ? 0 : 1].at(a);
        if (row.reflected < 0) {
            r.action = kInterfaceAmmRow;
            return r;
        }
        double x = u[k++];
        int chosen = -1;
        for (const auto& e : row.transmitted) {
            x -= e.second;
            if (x < 0) {
                chosen = e.first;
                break;
            }
        }
        transmit = chosen >= 0;
        sel_material = transmit ? next : src;
        sel = transmit ? chosen : row.reflected;
    } else {
        bool drew;
        double source_flux = 0, target_flux = 0;
        const int reflected = interface_sample_band(I.banks[src][1 - incident], omega, I.band_width, u[k], drew, source_flux);
        if (drew) ++k;
        const int transmitted = interface_sample_band(I.banks[next][incident], omega, I.band_width, u[k], drew, target_flux);
        if (drew) ++k;
        const double transmission = target_flux > 0 ? target_flux / std::max(1e-300, source_flux + target_flux) : 0;
        transmit = transmitted >= 0 && u[k] < transmission;
        sel_material = transmit ? next : src;
        sel = transmit ? transmitted : reflected;
    }
    r.events = 1;
    if (sel < 0) {
        if (I.linearized) {
            r.action = kInterfaceFail;
            return r;
        }
        r.signs ^= 1u << axis;
        r.reflected = 1;
        r.action = kInterfaceReflect;
        return r;
    }
    const MaterialTables& D = mats[sel_material];
    const double new_omega = D.omega[sel];
    const double old_deviation = occ - S.nbg[a];
    const double physical = S.energy_weight * omega * old_deviation;
    const double new_deviation = physical / std::max(1e-300, D.energy_weight * new_omega);
    const double new_occ = D.nbg[sel] + new_deviation;
    if (I.linearized) {
        const double nv = D.vel[3 * sel + axis];
        const int expected = transmit ? incident : 1 - incident;
        if (!std::isfinite(new_occ) || !std::isfinite(nv) || (expected ? !(nv > 0.0) : !(nv < 0.0))) {
            r.action = kInterfaceFail;
            return r;
        }
    }
    if (!std::isfinite(new_occ) || (!I.linearized && new_occ < 0.0)) {
        r.signs ^= 1u << axis;
        r.reflected = 1;
        r.action = kInterfaceReflect;
        return r;
    }
    r.material = sel_material;
    r.active = sel;
    r.signs = 0;
    r.occ = new_occ;
    if (transmit) {
        r.transmitted = 1;
        r.action = kInterfaceTransmit;
    } else {
        r.reflected = 1;
        r.action = kInterfaceReflect;
    }
    return r;
}

// src/solver/PhononSourceOperator.cpp:119-340 (non-full-matrix branch): the
// pending energy of every cell with eligible carriers is given to them in the
// chosen spectrum, the carrier with the largest energy increment absorbs the
// round-off, and the cell's budget moves to `deposited`.
void source_apply_cells(const HeatSourceTables& S, const std::vector<const PhononMaterial*>& mats,
                    const std::vector<MaterialTables>& tables, const std::vector<int>& cell_material, double Tbg,
                    const std::vector<std::vector<int>>& members, const std::vector<uint32_t>& mode,
                    std::vector<double>& occ, const std::vector<double>& cell_T, std::vector<double>& src_pending,
                    std::vector<double>& src_deposited, long long& updates, double& deposited) {
    double pending_total = 0.0;
    for (double e : src_pending) pending_total += e;
    if (pending_total <= 0.0) return;
    auto fail = [](const std::string& m) { throw std::runtime_error(m); };
    for (size_t c = 0; c < members.size(); ++c) {
        if (src_pending[c] <= 0.0) continue;
        const int mid = cell_material[c];
        const PhononMaterial& M = *mats[mid];
        const MaterialTables& T = tables[mid];
        std::vector<int> idx;
        for (int i : members[c]) {
            if (static_cast<int>(mode[i] >> 28) != mid) fail("Source particle and cell material disagree.");
            const int a = static_cast<int>(mode[i] & kActiveMask);
            const double hw = kHbarEvPs * M.omega(T.active_flat[a]);
            if (std::isfinite(hw) && hw > 1e-14 && S.mode_weight(M, T.active_flat[a]) > 0.0) idx.push_back(i);
        }
        if (idx.empty()) continue;
        const double raw_to_physical = T.energy_weight;
        const double target = src_pending[c] / raw_to_physical;
        if (!std::isfinite(target)) fail("Non-finite heat-source energy per carrier.");
        const size_t n = idx.size();
        std::vector<double> inc(n);
        auto flat_of = [&](int i) { return T.active_flat[mode[i] & kActiveMask]; };
        auto hw_of = [&](int i) { return kHbarEvPs * M.omega(flat_of(i)); };
        if (S.spectrum == HeatSourceSpectrum::Gaussian) {
            std::vector<long double> w(n);
            long double peak = -std::numeric_limits<long double>::infinity();
            for (size_t k = 0; k < n; ++k) {
                const long double f = M.omega(flat_of(idx[k])) / 6.283185307179586476925286766559L;
                const long double z = (f - S.gaussian_center) / S.gaussian_sigma;
                w[k] = -.5L * z * z;
                peak = std::max(peak, w[k]);
            }
            long double sum = 0;
            for (auto& x : w) {
                x = std::exp(x - peak);
                sum += x;
            }
            for (size_t k = 0; k < n; ++k) inc[k] = static_cast<double>(target * w[k] / sum) / hw_of(idx[k]);
        } else if (S.spectrum == HeatSourceSpectrum::Weighted) {
            double sum = 0.0;
            for (int i : idx) sum += S.mode_weight(M, flat_of(i));
            for (size_t k = 0; k < n; ++k)
                inc[k] = target * (S.mode_weight(M, flat_of(idx[k])) / sum) / hw_of(idx[k]);
        } else if (S.linearized_thermal) {
            long double cap = 0;
            for (int i : idx) cap += M.mode_heat_capacity(Tbg, flat_of(i));
            if (!(cap > 0)) fail("Source sample has no thermal capacity.");
            for (size_t k = 0; k < n; ++k)
                inc[k] = static_cast<double>(target * M.mode_heat_capacity(Tbg, flat_of(idx[k])) / cap) /
                         (kHbarEvPs * M.omega(flat_of(idx[k])));
        } else {
            const double base = std::isfinite(cell_T[c]) && cell_T[c] >= 0.0 ? cell_T[c] : Tbg;
            auto energy_at = [&](double temperature, double* slope_out) {
                double e = 0.0, slope = 0.0;
                for (int i : idx) {
                    const int f = flat_of(i);
                    const double hw = kHbarEvPs * std::max(0.0, M.omega(f));
                    const double n0 = M.bose_occupation(base, f);
                    const double nn = M.bose_occupation(temperature, f);
                    e += hw * (nn - n0);
                    if (slope_out && temperature > 0.0) slope += hw * (hw * nn * (nn + 1.0) / (kBoltzmannEvK * temperature * temperature));
                }
                if (slope_out) *slope_out = slope;
                return e;
            };
            double low = std::max(0.0, base);
            double high = std::max(low + 1.0, 1.05 * low + 1.0);
            double high_e = energy_at(high, nullptr);
            for (int k = 0; high_e < target && k < 60; ++k) {
                high = 2.0 * high + 1.0;
                high_e = energy_at(high, nullptr);
            }
            if (!(high_e >= target) || !std::isfinite(high_e))
                fail("Could not bracket the occupation-source pseudo-temperature.");
            double Ts = 0.5 * (low + high);
            const double tol = 1e-12 * std::max(1e-6, target);
            for (int it = 0; it < 60; ++it) {
                double d = 0.0;
                const double r = energy_at(Ts, &d) - target;
                if (std::abs(r) <= tol) break;
                if (r > 0.0) high = Ts;
                else low = Ts;
                double cand = 0.5 * (low + high);
                if (d > 0.0 && std::isfinite(d)) {
                    const double nt = Ts - r / d;
                    if (nt > low && nt < high && std::isfinite(nt)) cand = nt;
                }
                Ts = cand;
            }
            for (size_t k = 0; k < n; ++k)
                inc[k] = M.bose_occupation(Ts, flat_of(idx[k])) - M.bose_occupation(base, flat_of(idx[k]));
        }
        // round-off correction on the carrier with the largest energy increment
        double applied = 0.0, largest = -1.0;
        size_t corr = 0;
        for (size_t k = 0; k < n; ++k) {
            const double e = hw_of(idx[k]) * inc[k];
            applied += e;
            if (e > largest) {
                largest = e;
                corr = k;
            }
        }
        inc[corr] += (target - applied) / hw_of(idx[corr]);
        for (size_t k = 0; k < n; ++k) {
            const double next = occ[idx[k]] + inc[k];
            if (!std::isfinite(inc[k]) || !std::isfinite(next) || next < 0.0)
                fail("Heat source would produce an invalid occupation; cell budget retained.");
        }
        for (size_t k = 0; k < n; ++k) occ[idx[k]] += inc[k];
        const double e = src_pending[c];
        src_deposited[c] += e;
        src_pending[c] = 0.0;
        deposited += e;
        updates += static_cast<long long>(n);
    }
}


// ---------------------------------------------- linearized collision per cell
// src/solver/CarrierCollisionOperator.cpp:67-126 for one cell.
long double linear_cell(const std::vector<int>& members, const MaterialTables& T, const std::vector<int>& active_i,
                        std::vector<double>& occ, double dt, double cell_weight) {
    if (members.empty() || dt == 0) return 0;
    std::vector<double> om, cap, rn, rr, e;
    std::vector<Vec3> k;
    for (int i : members) {
        const int m = active_i[i];
        om.push_back(T.omega[m]);
        cap.push_back(T.col_capacity[m]);
        k.push_back({T.col_k[3 * m], T.col_k[3 * m + 1], T.col_k[3 * m + 2]});
        rn.push_back(T.col_normal[m]);
        rr.push_back(T.col_resistive[m]);
        e.push_back(kHbarEvPs * T.omega[m] * (occ[i] - T.nbg[m]));
    }
    const auto ev = Callaway(om, cap, k, rn, rr).evolve(e, dt);
    long double res = 0;
    std::vector<double> next(members.size());
    for (size_t j = 0; j < members.size(); ++j) {
        const int i = members[j], m = active_i[i];
        const double hw = kHbarEvPs * T.omega[m];
        next[j] = T.nbg[m] + ev[j] / hw;
        if (!std::isfinite(next[j])) throw std::overflow_error("Carrier collision occupation overflow.");
        res += hw * (static_cast<long double>(next[j]) - occ[i]);
    }
    for (size_t j = 0; j < members.size(); ++j) occ[members[j]] = next[j];
    return res * cell_weight;
}

// ------------------------------------------ nonlinear Callaway per cell
// src/solver/NonlinearCallawayCollision.cpp:25-248, per carrier and in long
// double as the reference: three BGK substeps N(dt/2), R(dt), N(dt/2), each
// n <- (1-a) n + a n_target with a = 1 - exp(-rate dt) and n_target a
// displaced Bose distribution 1/expm1(phi), phi = sum_j lambda_j b_j. The
// basis b_j is the a-weighted orthonormalised set {hw/kT, k_x, k_y, k_z}
// (energy only for resistive substeps); lambda solves the moment equations
// sum a b_j (n - n_target) = 0 by damped Newton on the convex potential.
namespace ncl {
using LD = long double;
constexpr double kHbarNcl = 6.582119569e-4, kKbNcl = 8.617333262145e-5;

LD bose(LD x) { return x > 700 ? 0 : 1 / std::expm1(x); }

void substep(const std::vector<double>& omega, const std::vector<std::array<double, 3>>& k,
             const std::vector<double>& rate, double dt, bool normal, double T, std::vector<double>& n) {
    const size_t N = n.size();
    std::vector<LD> a(N), w(N), phi0(N);
    LD activity = 0;
    for (size_t i = 0; i < N; ++i) {
        a[i] = -std::expm1(-rate[i] * dt);
        activity += a[i];
        phi0[i] = kHbarNcl * omega[i] / (kKbNcl * T);
        const LD e = bose(phi0[i]);
        w[i] = a[i] * e * (1 + e);
    }
    if (activity == 0) return;
    auto dot = [&](const std::vector<LD>& u, const std::vector<LD>& v) {
        LD s = 0;
        for (size_t i = 0; i < N; ++i) s += w[i] * u[i] * v[i];
        return s;
    };
    std::vector<std::vector<LD>> basis;
    LD lambda[4] = {0, 0, 0, 0};
    for (int j = 0; j < (normal ? 4 : 1); ++j) {
        std::vector<LD> v(N);
        for (size_t i = 0; i < N; ++i) v[i] = j == 0 ? phi0[i] : static_cast<LD>(k[i][j - 1]);
        const LD norm0 = std::sqrt(dot(v, v));
        if (norm0 == 0) continue;
        for (auto& x : v) x /= norm0;
        for (int pass = 0; pass < 2; ++pass)
            for (const auto& b : basis) {
                const LD d = dot(v, b);
                for (size_t i = 0; i < N; ++i) v[i] -= d * b[i];
            }
        const LD len = std::sqrt(dot(v, v));
        if (len < 1e-12L) continue;
        for (auto& x : v) x /= len;
        if (j == 0) lambda[0] = norm0 * len;
        basis.push_back(std::move(v));
    }
    const int dim = static_cast<int>(basis.size());
    if (dim == 0) throw std::runtime_error("Nonlinear Callaway has no representable energy constraint");
    LD scale[4] = {0, 0, 0, 0};
    for (int j = 0; j < dim; ++j)
        for (size_t i = 0; i < N; ++i)
            scale[j] += std::abs(a[i] * basis[j][i]) * std::max(static_cast<LD>(n[i]), bose(phi0[i]));
    std::vector<LD> target(N);
    // potential F(lambda) = sum a (-log(1 - e^-phi) + n phi), gradient g, Hessian H
    auto potential = [&](const LD* x, LD* g, LD (*H)[4], bool keep) {
        for (int j = 0; j < 4; ++j) {
            g[j] = 0;
            if (H)
                for (int l = 0; l < 4; ++l) H[j][l] = 0;
        }
        LD F = 0;
        for (size_t i = 0; i < N; ++i) {
            if (a[i] == 0) continue;
            LD phi = 0;
            for (int j = 0; j < dim; ++j) phi += x[j] * basis[j][i];
            if (!(phi > 0) || !std::isfinite(phi)) return std::numeric_limits<LD>::infinity();
            const LD e = bose(phi);
            if (keep) target[i] = e;
            F += a[i] * (-std::log(-std::expm1(-phi)) + n[i] * phi);
            for (int j = 0; j < dim; ++j) {
                g[j] += a[i] * basis[j][i] * (n[i] - e);
                if (H)
                    for (int l = 0; l < dim; ++l) H[j][l] += a[i] * basis[j][i] * basis[l][i] * e * (1 + e);
            }
        }
        return F;
    };
    auto residual = [&](const LD* g) {
        LD r = 0;
        for (int j = 0; j < dim; ++j) r = std::max(r, std::abs(g[j]) / std::max(1e-30L, scale[j]));
        return r;
    };
    bool converged = false;
    for (int it = 0; it < 70; ++it) {
        LD g[4], H[4][4];
        const LD F = potential(lambda, g, H, true);
        const LD err = residual(g);
        if (err < 2e-13L) {
            converged = true;
            break;
        }
        LD step_dir[4];
        for (int j = 0; j < dim; ++j) step_dir[j] = -g[j];
        for (int j = 0; j < dim; ++j) { // Gaussian elimination, partial pivoting
            int p = j;
            for (int r = j + 1; r < dim; ++r)
                if (std::abs(H[r][j]) > std::abs(H[p][j])) p = r;
            if (!(std::abs(H[p][j]) > 1e-30L)) throw std::runtime_error("Singular nonlinear Callaway moment Jacobian");
            for (int l = 0; l < 4; ++l) std::swap(H[j][l], H[p][l]);
            std::swap(step_dir[j], step_dir[p]);
            for (int r = j + 1; r < dim; ++r) {
                const LD f = H[r][j] / H[j][j];
                for (int l = j; l < dim; ++l) H[r][l] -= f * H[j][l];
                step_dir[r] -= f * step_dir[j];
            }
        }
        for (int j = dim - 1; j >= 0; --j) {
            for (int l = j + 1; l < dim; ++l) step_dir[j] -= H[j][l] * step_dir[l];
            step_dir[j] /= H[j][j];
        }
        LD slope = 0;
        for (int j = 0; j < dim; ++j) slope += g[j] * step_dir[j];
        bool ok = false;
        for (LD t = 1; t > 1e-14L; t *= .5L) {
            LD trial[4] = {lambda[0], lambda[1], lambda[2], lambda[3]}, gt[4];
            for (int j = 0; j < dim; ++j) trial[j] += t * step_dir[j];
            const LD Ft = potential(trial, gt, nullptr, false);
            if (std::isfinite(Ft) && (Ft <= F + 1e-4L * t * slope || residual(gt) < err * .9L)) {
                for (int j = 0; j < 4; ++j) lambda[j] = trial[j];
                ok = true;
                break;
            }
        }
        if (!ok) throw std::runtime_error("Nonlinear Callaway moment line search failed");
    }
    if (!converged) throw std::runtime_error("Nonlinear Callaway moment solve did not converge");
    for (size_t i = 0; i < N; ++i) {
        if (!(a[i] > 0)) continue;
        n[i] = static_cast<double>((1 - a[i]) * n[i] + a[i] * target[i]);
        if (!std::isfinite(n[i]) || n[i] < 0) throw std::runtime_error("Nonlinear Callaway occupation is invalid");
    }
}

// src/solver/NonlinearCallawayCollision.cpp:216-248
std::vector<double> evolve(const std::vector<double>& omega, const std::vector<std::array<double, 3>>& k,
                           const std::vector<double>& rn, const std::vector<double>& rr, std::vector<double> n, double T,
                           double dt) {
    if (n.empty() || !std::isfinite(T) || T <= 0 || !std::isfinite(dt) || dt < 0)
        throw std::invalid_argument("Invalid nonlinear Callaway state");
    for (size_t i = 0; i < n.size(); ++i)
        if (!std::isfinite(n[i]) || n[i] < 0 || !(omega[i] > 0) || !std::isfinite(omega[i]) || !(rn[i] >= 0) ||
            !(rr[i] >= 0) || !std::isfinite(rn[i]) || !std::isfinite(rr[i]))
            throw std::invalid_argument("Invalid nonlinear Callaway mode");
    if (dt == 0) return n;
    substep(omega, k, rn, 0.5 * dt, true, T, n);
    substep(omega, k, rr, dt, false, T, n);
    substep(omega, k, rn, 0.5 * dt, true, T, n);
    return n;
}
} // namespace ncl

// ---------------------------------------------------------------- solver
struct OracleSolver {
    SimulationConfig cfg;
    std::vector<std::unique_ptr<PhononMaterial>> owned;
    std::vector<const PhononMaterial*> mats;
    std::unique_ptr<SimulationDomain> domain;
    Problem P;
    // carriers (slots)
    std::vector<double> x, y, z, occ;
    std::vector<uint32_t> mode;
    std::vector<int32_t> cell;
    std::vector<uint8_t> alive;
    // mesh domains: facet whose specular mirror applies to the mode velocity (-1: none),
    // and the persistent wall cache of src/solver/TransportOperator.cpp:186-250
    // (time to the wall in units of dt, hit point, facet)
    std::vector<int32_t> mirror;
    std::vector<double> hit_t;
    std::vector<Vec3> hit_p;
    std::vector<int32_t> hit_f;
    // grid
    std::vector<double> cell_T, cell_E;
    std::vector<Vec3> cell_q;
    // ledgers
    std::vector<int> prev_absorbed, cur_absorbed;
    BoundaryBalance step_b, total_b;
    EnergyLedger energy;
    int step = 0;
    double elapsed = 0;
    double avg_flux = 0, kappa_fit = 0, kappa_end = 0;
    long long iface_events = 0, iface_transmitted = 0, iface_reflected = 0;
    long long rough_counts[8] = {0, 0, 0, 0, 0, 0, 0, 0}; // outcome flags, then events
    long long cache_corrections = 0;
    bool failed = false;

    Vec3 velocity(uint32_t w, int32_t mir = -1) const {
        const MaterialTables& T = P.mats[w >> 28];
        const int a = static_cast<int>(w & kActiveMask);
        Vec3 v{T.vel[3 * a], T.vel[3 * a + 1], T.vel[3 * a + 2]};
        for (int k = 0; k < 3; ++k)
            if ((w >> (24 + k)) & 1u) v[k] = -v[k];
        if (mir >= 0) v = reflect(v, domain->facets()[mir].normal);
        return v;
    }
    Vec3 velocity_of(size_t i) const { return velocity(mode[i], mirror.empty() ? -1 : mirror[i]); }

    // src/solver/BoundaryInteraction.cpp:121-124: v - 2 (v.n) n
    static Vec3 reflect(const Vec3& v, const Vec3& n) { return sub3(v, mul3(n, 2.0 * dot3(v, n))); }

    void init(const std::vector<const PhononMaterial*>& m) {
        mats = m;
        domain = std::make_unique<SimulationDomain>(cfg);
        P = build_problem(cfg, *domain, mats);
        const CarrierArrays c = initial_carriers(P, mats);
        x = c.x; y = c.y; z = c.z; occ = c.occ; mode = c.mode; cell = c.cell; alive = c.alive;
        if (domain->is_mesh()) {
            if (mats.size() != 1) throw std::runtime_error("Layered materials are built for box domains only.");
            reset_mesh_state();
        }
        prev_absorbed.resize(P.reservoirs.size());
        for (size_t r = 0; r < P.reservoirs.size(); ++r) prev_absorbed[r] = P.reservoirs[r].initial_count;
        cur_absorbed.assign(P.reservoirs.size(), 0);
        const int nc = domain->grid_count();
        cell_T.assign(nc, 300.0);
        cell_E.assign(nc, 0.0);
        src_pending.assign(nc, 0.0);
        src_prescribed.assign(nc, 0.0);
        src_deposited.assign(nc, 0.0);
        cell_q.assign(nc, {0, 0, 0});
        refresh();
        energy.initialize(total_thermal());
        update_flux();
    }

    // ------------------------------------------------------- transport
    // src/solver/TransportOperator.cpp:186-250
    bool cache(Vec3& p, const Vec3& v, Vec3& cp, double& t, int& f) {
        const double speed = norm3(v);
        if (std::isfinite(speed) && speed <= 1e-18) {
            cp = p; t = std::numeric_limits<double>::infinity(); f = -1;
            return true;
        }
        domain->trace(p, v, cp, t, f);
        if (f < 0 || !std::isfinite(t)) {
            const Vec3 ext{domain->bounds_max()[0] - domain->bounds_min()[0], domain->bounds_max()[1] - domain->bounds_min()[1],
                           domain->bounds_max()[2] - domain->bounds_min()[2]};
            const double scale = std::max({1.0, std::abs(ext[0]), std::abs(ext[1]), std::abs(ext[2])});
            const double eps = std::max(P.push_eps, 1e-10 * scale);
            Vec3 cand[4] = {p, p, p, p};
            const int nf = domain->nearest_facet(p);
            if (nf >= 0) {
                cand[0] = add3(p, mul3(domain->facets()[nf].normal, eps));
                cand[1] = add3(p, mul3(domain->facets()[nf].normal, -eps));
            }
            if (speed > 0.0 && std::isfinite(speed)) {
                const Vec3 d = mul3(v, 1.0 / speed);
                cand[2] = add3(p, mul3(d, eps));
                cand[3] = add3(p, mul3(d, -eps));
            }
            for (const Vec3& c : cand) {
                if (!domain->contains_point(c)) continue;
                domain->trace(c, v, cp, t, f);
                if (f >= 0 && std::isfinite(t)) {
                    p = c;
                    ++cache_corrections;
                    break;
                }
            }
        }
        return f >= 0 && std::isfinite(t);
    }

    void fail(const std::string& msg) {
        failed = true;
        throw std::runtime_error(msg);
    }

    // src/solver/TransportOperator.cpp:287-361 + src/solver/BoundaryInteraction.cpp:53-162.
    // Returns false when the carrier was absorbed.
    bool boundary(int i, int f, Vec3& p, uint32_t purpose, int event) {
        const Facet& F = domain->facets()[f];
        uint32_t w = mode[i];
        const int mid = static_cast<int>(w >> 28);
        const MaterialTables& T = P.mats[mid];
        const int a = static_cast<int>(w & kActiveMask);
        const int axis = f / 2;
        if (F.condition == 'T') {
            const double e = T.hw[a] * (occ[i] - T.nbg[a]) * T.energy_weight;
            step_b.absorbed += 1;
            step_b.absorbed_energy_ev += e;
            if (F.reservoir >= 0) cur_absorbed[F.reservoir] += 1;
            alive[i] = 0;
            return false;
        }
        if (F.condition == 'P' && F.pair >= 0) {
            p = add3(p, F.shift);
        } else {
            const int nfac = static_cast<int>(domain->facets().size());
            const int table = P.rough.facet_table[static_cast<size_t>(mid) * nfac + f];
            if (P.conservative || (F.condition == 'R' && table >= 0)) {
                if (table < 0) fail("Full-matrix boundary mode mapping failed while advancing particles for particle " + std::to_string(i));
                const Uniform2 d0 = uniform2(P.cfg.random_seed, static_cast<uint32_t>(i), static_cast<uint32_t>(step), purpose,
                                             static_cast<uint32_t>(event), 0);
                const Uniform2 d1 = uniform2(P.cfg.random_seed, static_cast<uint32_t>(i), static_cast<uint32_t>(step), purpose,
                                             static_cast<uint32_t>(event), 1);
                RoughDraws dr{{d0.a, d0.b, d1.a}};
                double n_out;
                unsigned diag = 0;
                const int out = rough_sample(P.rough.tables[table], T, a, occ[i], P.conservative, dr, n_out, &diag);
                rough_counts[7] += 1;
                for (int k = 0; k < 7; ++k)
                    if (diag & (1u << k)) rough_counts[k] += 1;
                uint32_t signs = 0;
                const bool mesh = domain->is_mesh();
                const double vn = mesh ? dot3({T.vel[3 * out], T.vel[3 * out + 1], T.vel[3 * out + 2]}, F.normal)
                                       : T.vel[3 * out + axis] * F.normal[axis];
                if (mesh) mirror[i] = -1;
                if (P.conservative) {
                    if (!std::isfinite(n_out) || !(T.omega[out] > 0.0) || !(vn < 0.0))
                        fail("Full-matrix boundary mode mapping failed while advancing particles for particle " + std::to_string(i));
                } else if (vn > 0.0) {
                    if (mesh) mirror[i] = f; // outward mode velocity mirrored in the facet plane
                    else signs = 1u << axis;
                }
                w = mode_word(static_cast<uint32_t>(out), signs, static_cast<uint32_t>(mid));
                occ[i] = n_out;
            } else if (F.condition == 'R') {
                fail("Rough facet without a sampling table is not supported for box geometry.");
            } else if (domain->is_mesh()) {
                fail("Specular reflection without a sampling table is not reachable for mesh facets.");
            } else {
                w ^= 1u << (24 + axis); // specular: exact sign flip of the normal component
            }
            mode[i] = w;
        }
        const Vec3 v = velocity_of(i);
        p = add3(p, mul3(v, P.push_eps / std::max(norm3(v), 1e-12)));
        return true;
    }

    // src/solver/LayeredMaterialLayout.cpp:31-60
    double next_crossing(const Vec3& p, const Vec3& v, int current, int& destination) const {
        destination = -1;
        const int count = static_cast<int>(P.mats.size());
        if (count <= 1) return std::numeric_limits<double>::infinity();
        const int ax = P.layout.axis;
        const double velocity_axis = v[ax];
        if (std::abs(velocity_axis) <= 1e-18) return std::numeric_limits<double>::infinity();
        double plane;
        int dest;
        if (velocity_axis > 0.0 && current + 1 < count) {
            plane = P.layout.planes[current];
            dest = current + 1;
        } else if (velocity_axis < 0.0 && current > 0) {
            plane = P.layout.planes[current - 1];
            dest = current - 1;
        } else {
            return std::numeric_limits<double>::infinity();
        }
        const double time = (plane - p[ax]) / velocity_axis;
        if (!std::isfinite(time) || time <= 1e-14) return std::numeric_limits<double>::infinity();
        destination = dest;
        return time;
    }

    // src/solver/TransportOperator.cpp:468-497
    void material_interface(int i, int destination, uint32_t purpose, int event) {
        const uint32_t w = mode[i];
        const Uniform2 d0 = uniform2(P.cfg.random_seed, static_cast<uint32_t>(i), static_cast<uint32_t>(step), purpose,
                                     static_cast<uint32_t>(event), 0);
        const Uniform2 d1 = uniform2(P.cfg.random_seed, static_cast<uint32_t>(i), static_cast<uint32_t>(step), purpose,
                                     static_cast<uint32_t>(event), 1);
        const double u[4] = {d0.a, d0.b, d1.a, d1.b};
        const InterfaceOutcome r = interface_interact(P.iface, P.mats, static_cast<int>(w >> 28),
                                                      static_cast<int>(w & kActiveMask), (w >> 24) & 7u, occ[i],
                                                      destination, u);
        iface_events += r.events;
        iface_transmitted += r.transmitted;
        iface_reflected += r.reflected;
        if (r.action == kInterfaceAmmRow) fail("AMM incoming state is tangent or unsupported.");
        if (r.action == kInterfaceFail)
            fail("Full-matrix boundary mode mapping failed while advancing particles for particle " + std::to_string(i) +
                 ". An inward discrete material mode and finite signed energy weight are required; no velocity-only "
                 "reflection was applied.");
        mode[i] = mode_word(static_cast<uint32_t>(r.active), r.signs, static_cast<uint32_t>(r.material));
        occ[i] = r.occ;
    }

    // Mesh domains: fresh carriers carry the mode velocity and get their wall cache
    // (src/solver/Initialization.cpp:131).
    void reset_mesh_state() {
        mirror.assign(alive.size(), -1);
        hit_t.assign(alive.size(), std::numeric_limits<double>::infinity());
        hit_p.assign(alive.size(), Vec3{0, 0, 0});
        hit_f.assign(alive.size(), -1);
        for (size_t i = 0; i < alive.size(); ++i)
            if (alive[i]) update_cache(static_cast<int>(i));
    }

    // src/solver/TransportOperator.cpp:186-250: trace from the current position
    // (with nudged retries, which may move the carrier), time stored in units of dt.
    void update_cache(int i) {
        Vec3 p{x[i], y[i], z[i]}, cp;
        double t;
        int f;
        const Vec3 v = velocity_of(i);
        if (!cache(p, v, cp, t, f))
            fail("Boundary intersection failed while updating collision cache for particle " + std::to_string(i) +
                 ". Check that the STL is closed and manifold.");
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        hit_t[i] = t / cfg.time_step;
        hit_p[i] = cp;
        hit_f[i] = f;
    }

    // src/solver/TransportOperator.cpp:405-466 with the persistent wall cache (mesh domains).
    void advance_mesh(int i, double remaining, uint32_t purpose) {
        const double dt = cfg.time_step;
        Vec3 v = velocity_of(i);
        int event = 0;
        for (; remaining > 1e-14 && event < 64; ++event) {
            const double t_wall = hit_t[i] * dt;
            if (!std::isfinite(t_wall) || t_wall > remaining) {
                x[i] += v[0] * remaining; y[i] += v[1] * remaining; z[i] += v[2] * remaining;
                if (std::isfinite(hit_t[i])) hit_t[i] -= remaining / dt;
                return;
            }
            remaining -= std::max(0.0, t_wall);
            Vec3 p = hit_p[i];
            if (!boundary(i, hit_f[i], p, purpose, event)) {
                x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
                return;
            }
            x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
            v = velocity_of(i);
            update_cache(i);
            if (hit_t[i] * dt < 1e-12) {
                x[i] += v[0] * 1e-12; y[i] += v[1] * 1e-12; z[i] += v[2] * 1e-12;
                update_cache(i);
            }
        }
        if (remaining > 1e-14)
            fail("Particle " + std::to_string(i) + " exceeded 64 transport events in one timestep");
    }

    // src/solver/TransportOperator.cpp:405-466
    void advance(int i, double remaining, uint32_t purpose) {
        if (!alive[i]) return;
        if (domain->is_mesh()) {
            advance_mesh(i, remaining, purpose);
            return;
        }
        Vec3 p{x[i], y[i], z[i]};
        Vec3 cp;
        double t;
        int f;
        Vec3 v = velocity_of(i);
        if (!cache(p, v, cp, t, f))
            fail("Boundary intersection failed while advancing particles for particle " + std::to_string(i) +
                 ". Check that the STL is closed and manifold.");
        int event = 0;
        for (; remaining > 1e-14 && event < 64; ++event) {
            int destination = -1;
            const double t_cross = next_crossing(p, v, static_cast<int>(mode[i] >> 28), destination);
            const double t_event = std::min(t, t_cross);
            if (!std::isfinite(t_event) || t_event > remaining) {
                p = add3(p, mul3(v, remaining));
                x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
                return;
            }
            // the outer wall wins exact ties
            const bool interface_first = t_cross < t;
            remaining -= std::max(0.0, t_event);
            if (interface_first) {
                p = add3(p, mul3(v, t_cross));
                material_interface(i, destination, purpose, event);
                v = velocity_of(i);
                const double speed = std::max(norm3(v), 1e-12);
                p = add3(p, mul3(v, P.push_eps / speed));
            } else {
                p = cp;
                if (!boundary(i, f, p, purpose, event)) {
                    x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
                    return;
                }
                v = velocity_of(i);
            }
            if (!cache(p, v, cp, t, f)) fail("Boundary intersection failed while advancing particles for particle " + std::to_string(i));
            if (!interface_first && t < 1e-12) {
                p = add3(p, mul3(v, 1e-12));
                if (!cache(p, v, cp, t, f)) fail("Boundary intersection failed while advancing particles for particle " + std::to_string(i));
            }
        }
        x[i] = p[0]; y[i] = p[1]; z[i] = p[2];
        if (remaining > 1e-14)
            fail("Particle " + std::to_string(i) + " exceeded 64 transport events in one timestep");
    }

    // src/solver/ReservoirInjector.cpp:62-132 with slot refilling.
    void inject(std::vector<std::pair<int, double>>& injected) {
        const double dt = cfg.time_step;
        std::vector<int> holes;
        for (size_t i = 0; i < alive.size(); ++i)
            if (!alive[i]) holes.push_back(static_cast<int>(i));
        size_t next_hole = 0;
        for (size_t r = 0; r < P.reservoirs.size(); ++r) {
            const Reservoir& R = P.reservoirs[r];
            const MaterialTables& T = P.mats[R.material];
            int count;
            if (P.one_to_one) count = prev_absorbed[r];
            else {
                const int base = static_cast<int>(std::floor(R.expected));
                const double frac = R.expected - base;
                const Uniform2 u = uniform2(cfg.random_seed, static_cast<uint32_t>(r), static_cast<uint32_t>(step), kDrawInjectCount, 0, 0);
                count = base + ((frac > 0.0 && u.a < frac) ? 1 : 0);
            }
            if (count > 0 && !(R.cdf.back() > 0.0))
                fail("Cannot sample positive emissions from a zero-flux reservoir.");
            const Facet& F = domain->facets()[R.facet];
            std::vector<double> cum; // running triangle area (src/geometry/SurfaceSampling.cpp:45-58)
            for (double a : F.tri_area) cum.push_back((cum.empty() ? 0.0 : cum.back()) + std::max(a, 0.0));
            for (int e = 0; e < count; ++e) {
                const Uniform2 d0 = uniform2(cfg.random_seed, static_cast<uint32_t>(e), static_cast<uint32_t>(step), kDrawInject, static_cast<uint32_t>(r), 0);
                const Uniform2 d1 = uniform2(cfg.random_seed, static_cast<uint32_t>(e), static_cast<uint32_t>(step), kDrawInject, static_cast<uint32_t>(r), 1);
                const Uniform2 d2 = uniform2(cfg.random_seed, static_cast<uint32_t>(e), static_cast<uint32_t>(step), kDrawInject, static_cast<uint32_t>(r), 2);
                // the emission distribution of ReservoirSampler::sample (its
                // lower_bound over the flux roulette, ReservoirSampler.cpp:117-146)
                // drawn from the same weights' alias table, as the device does
                const size_t m = static_cast<size_t>(alias_draw(R.alias.data(), static_cast<int>(R.alias.size()), d0.a));
                const double temit = dt * d0.b;
                size_t k = static_cast<size_t>(std::upper_bound(cum.begin(), cum.end(), d1.a * cum.back()) - cum.begin());
                if (k >= cum.size()) k = cum.size() - 1;
                const auto& tri = F.tris[k];
                const double sr1 = std::sqrt(d1.b);
                const double w0 = 1.0 - sr1, w1 = sr1 * (1.0 - d2.a), w2 = sr1 * d2.a;
                Vec3 pos{w0 * tri[0][0] + w1 * tri[1][0] + w2 * tri[2][0], w0 * tri[0][1] + w1 * tri[1][1] + w2 * tri[2][1],
                         w0 * tri[0][2] + w1 * tri[1][2] + w2 * tri[2][2]};
                Vec3 v{T.vel[3 * m], T.vel[3 * m + 1], T.vel[3 * m + 2]};
                uint32_t signs = 0;
                if (dot3(v, R.normal) > 0.0) {
                    if (P.conservative) fail("Full-matrix reservoir sampled an outward mode.");
                    v = mul3(v, -1.0);
                    signs = 7u;
                }
                const double speed = std::max(1e-12, norm3(v));
                pos = add3(pos, mul3(v, P.push_eps / speed));
                const double o = P.reservoir_occ[r][m];
                int slot;
                if (next_hole < holes.size()) slot = holes[next_hole++];
                else {
                    slot = static_cast<int>(alive.size());
                    x.push_back(0); y.push_back(0); z.push_back(0); occ.push_back(0); mode.push_back(0);
                    cell.push_back(0); alive.push_back(0);
                    if (domain->is_mesh()) {
                        mirror.push_back(-1);
                        hit_t.push_back(0);
                        hit_p.push_back({0, 0, 0});
                        hit_f.push_back(-1);
                    }
                }
                if (domain->is_mesh()) mirror[slot] = -1;
                x[slot] = pos[0]; y[slot] = pos[1]; z[slot] = pos[2];
                occ[slot] = o;
                mode[slot] = mode_word(static_cast<uint32_t>(m), signs, static_cast<uint32_t>(R.material));
                cell[slot] = domain->fast_grid_index(pos);
                alive[slot] = 1;
                injected.push_back({slot, temit});
                step_b.injected += 1;
                step_b.injected_energy_ev += T.hw[m] * (o - T.nbg[m]) * T.energy_weight;
            }
        }
    }

    void transport() {
        const int n_before = static_cast<int>(alive.size());
        std::fill(cur_absorbed.begin(), cur_absorbed.end(), 0);
        for (int i = 0; i < n_before; ++i) {
            advance(i, cfg.time_step, kDrawTransport);
            if (alive[i]) cell[i] = domain->fast_grid_index({x[i], y[i], z[i]});
        }
        std::vector<std::pair<int, double>> injected;
        inject(injected);
        if (domain->is_mesh())
            for (const auto& inj : injected) update_cache(inj.first); // src/MonteCarloSolver.cpp:318-327
        for (const auto& [slot, temit] : injected) {
            const double remain = cfg.time_step - temit;
            if (remain > 1e-14) advance(slot, remain, kDrawInjected);
            if (alive[slot]) cell[slot] = domain->fast_grid_index({x[slot], y[slot], z[slot]});
        }
        prev_absorbed = cur_absorbed;
        if (step % 100 == 0) containment();
    }

    // src/solver/TransportOperator.cpp:364-402
    void containment() {
        const Vec3& lo = domain->bounds_min();
        const Vec3& hi = domain->bounds_max();
        const double scale = std::max({1.0, hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]});
        const double tol = 1e-10 * scale;
        for (size_t i = 0; i < alive.size(); ++i) {
            if (!alive[i]) continue;
            const double p[3] = {x[i], y[i], z[i]};
            bool outside = false;
            for (int a = 0; a < 3; ++a) outside = outside || !std::isfinite(p[a]) || p[a] < lo[a] - tol || p[a] > hi[a] + tol;
            if (!outside && domain->is_mesh()) outside = !domain->contains_point({p[0], p[1], p[2]});
            if (outside) fail("Particle " + std::to_string(i) + " escaped the domain");
        }
    }

    // ---------------------------------------------------------- grid
    // src/solver/GridStatistics.cpp:95-234
    void refresh() {
        const int nc = domain->grid_count();
        std::vector<double> acc(nc, 0.0);
        for (size_t i = 0; i < alive.size(); ++i) {
            if (!alive[i]) continue;
            const int c = cell[i];
            const int mid = static_cast<int>(mode[i] >> 28);
            if (c < 0 || c >= nc || mid != P.cell_material[c] || !std::isfinite(occ[i]))
                fail("Invalid particle in grid energy statistics.");
            const MaterialTables& T = P.mats[mid];
            const int a = static_cast<int>(mode[i] & kActiveMask);
            acc[c] += T.hw[a] * (occ[i] - T.nbg[a]) * T.energy_weight;
        }
        for (int c = 0; c < nc; ++c) {
            const MaterialTables& T = P.mats[P.cell_material[c]];
            double e = acc[c] / domain->grid_volumes()[c];
            e += T.energy_density_bg;
            if (!std::isfinite(e)) throw std::overflow_error("Non-finite grid energy reduction.");
            cell_E[c] = e;
            cell_T[c] = P.linearized ? cfg.background_temperature + (e - T.energy_density_bg) / T.heat_capacity_density_bg
                                     : PhononMaterial::interp_linear_clamped(T.lookup_E, T.lookup_T, e);
        }
    }

    double total_thermal() const {
        double total = 0.0;
        for (int c = 0; c < domain->grid_count(); ++c)
            total += (cell_E[c] - P.mats[P.cell_material[c]].zero_point) * domain->grid_volumes()[c];
        return total;
    }

    std::vector<std::vector<int>> members_by_cell() const {
        std::vector<std::vector<int>> m(domain->grid_count());
        for (size_t i = 0; i < alive.size(); ++i)
            if (alive[i]) m[cell[i]].push_back(static_cast<int>(i));
        return m;
    }

    // ----------------------------------------------------- collisions
    double collide() {
        const auto members = members_by_cell();
        const double dt = cfg.time_step;
        if (P.linearized) {
            long double sum = 0;
            for (size_t c = 0; c < members.size(); ++c) {
                const MaterialTables& T = P.mats[P.cell_material[c]];
                std::vector<int> act(alive.size());
                for (int i : members[c]) act[i] = static_cast<int>(mode[i] & kActiveMask);
                sum += linear_cell(members[c], T, act, occ, dt, T.energy_weight);
            }
            return static_cast<double>(sum);
        }
        if (cfg.callaway_nonlinear) {
            // src/solver/NonlinearCallawayCollision.cpp:265-343
            long double sum = 0;
            for (size_t c = 0; c < members.size(); ++c) {
                if (members[c].empty()) continue;
                const int mid = P.cell_material[c];
                const MaterialTables& T = P.mats[mid];
                const double Tc = cell_T[c];
                const double Tr = cfg.lifetime_temperature_is_local ? Tc : cfg.lifetime_temperature;
                std::vector<double> om, rn, rr, n;
                std::vector<std::array<double, 3>> kv;
                for (int i : members[c]) {
                    const int act = static_cast<int>(mode[i] & kActiveMask);
                    const auto r = mats[mid]->mode_callaway_rates(Tr, T.active_flat[act]);
                    om.push_back(T.omega[act]);
                    kv.push_back({T.col_k[3 * act], T.col_k[3 * act + 1], T.col_k[3 * act + 2]});
                    rn.push_back(r[0]);
                    rr.push_back(r[1]);
                    n.push_back(occ[i]);
                }
                const auto out = ncl::evolve(om, kv, rn, rr, n, Tc, dt);
                long double r = 0;
                for (size_t j = 0; j < out.size(); ++j) {
                    occ[members[c][j]] = out[j];
                    r += ncl::kHbarNcl * om[j] * (static_cast<long double>(out[j]) - n[j]);
                }
                sum += r * T.energy_weight;
            }
            return static_cast<double>(sum);
        }
        std::vector<double> om(alive.size(), 0.0), a(alive.size(), 0.0);
        for (size_t i = 0; i < alive.size(); ++i) {
            if (!alive[i]) continue;
            const int mid = static_cast<int>(mode[i] >> 28);
            const int act = static_cast<int>(mode[i] & kActiveMask);
            const int flat = P.mats[mid].active_flat[act];
            om[i] = P.mats[mid].omega[act];
            const double T = cfg.lifetime_temperature_is_local ? cell_T[cell[i]] : cfg.lifetime_temperature;
            a[i] = cfg.lifetime_temperature_is_local ? mats[mid]->mode_relaxation_weight(T, flat, dt)
                                                     : P.mats[mid].relax_fixed[act];
        }
        double res = 0.0;
        for (size_t c = 0; c < members.size(); ++c) {
            const MaterialTables& T = P.mats[P.cell_material[c]];
            res += rta_cell(members[c], om, a, occ, cell_T[c], T.energy_weight);
        }
        return res;
    }

    // src/solver/TemperatureGradientDrive.cpp:116-171
    void gradient_half() {
        if (!cfg.temperature_gradient) return;
        const double dt = 0.5 * cfg.time_step;
        const MaterialTables& T = P.mats[0];
        const auto members = members_by_cell();
        long double actual = 0;
        long long updates = 0;
        std::vector<double> next = occ;
        for (const auto& mem : members) {
            long double rs = 0, cs = 0;
            for (int i : mem) {
                const int m = static_cast<int>(mode[i] & kActiveMask);
                rs += T.grad_rate[m];
                cs += T.capacity_bg[m];
            }
            if (mem.empty()) continue;
            for (int i : mem) {
                const int m = static_cast<int>(mode[i] & kActiveMask);
                const long double e = dt * (T.grad_rate[m] - rs * T.capacity_bg[m] / cs);
                next[i] += static_cast<double>(e / T.hw[m]);
                actual += T.hw[m] * (static_cast<long double>(next[i]) - occ[i]);
                if (e != 0) ++updates;
            }
        }
        occ = next;
        energy.record_drive(updates, static_cast<double>(actual * P.gradient_energy_weight));
    }

    // src/solver/GridStatistics.cpp:269-347 + src/solver/Observables.cpp:38-144
    void update_flux() {
        const int nc = domain->grid_count();
        std::vector<Vec3> q(nc, {0, 0, 0});
        for (size_t i = 0; i < alive.size(); ++i) {
            if (!alive[i]) continue;
            const MaterialTables& T = P.mats[mode[i] >> 28];
            const int a = static_cast<int>(mode[i] & kActiveMask);
            const double e = T.hw[a] * (occ[i] - T.nbg[a]);
            q[cell[i]] = add3(q[cell[i]], mul3(velocity_of(i), e * T.energy_weight));
        }
        double phi = 0, vol = 0;
        const int axis = P.kappa_axis;
        for (int c = 0; c < nc; ++c) {
            cell_q[c] = mul3(mul3(q[c], 1.0 / domain->grid_volumes()[c]), 1.602176634e13);
            phi += cell_q[c][axis] * domain->grid_volumes()[c];
            vol += domain->grid_volumes()[c];
        }
        avg_flux = phi / vol;
        kappa_fit = kappa_end = 0;
        if (!cfg.compute_kappa) return;
        if (cfg.temperature_gradient) {
            kappa_end = -avg_flux / *cfg.temperature_gradient;
            return;
        }
        double Tl = cell_T.front(), Tr = cell_T.back();
        const auto& rf = domain->reservoir_facets();
        if (rf.size() >= 2) {
            int fl = rf.front(), fr = rf.front();
            for (int f : rf) {
                if (domain->facets()[f].centroid[axis] < domain->facets()[fl].centroid[axis]) fl = f;
                if (domain->facets()[f].centroid[axis] > domain->facets()[fr].centroid[axis]) fr = f;
            }
            Tl = domain->facets()[fl].value;
            Tr = domain->facets()[fr].value;
        }
        const double L = std::abs(domain->bounds_max()[axis] - domain->bounds_min()[axis]) * 1e-10;
        const double ge = std::abs(L) > 1e-24 ? (Tr - Tl) / L : 0.0;
        kappa_end = std::abs(ge) > 1e-18 ? -avg_flux / ge : 0.0;
        double sx = 0, st = 0, sxx = 0, sxt = 0;
        for (int c = 0; c < nc; ++c) {
            const double xx = domain->grid_centers()[c][axis] * 1e-10;
            sx += xx; st += cell_T[c]; sxx += xx * xx; sxt += xx * cell_T[c];
        }
        double gf = 0;
        const double dTw = std::abs(cell_T.back() - cell_T.front());
        if (nc >= 2) {
            const double den = nc * sxx - sx * sx;
            if (std::abs(den) > 1e-30 && dTw > 1e-6) gf = (nc * sxt - sx * st) / den;
        }
        kappa_fit = std::abs(gf) > 1e-18 ? -avg_flux / gf : 0.0;
    }

    // src/MonteCarloSolver.cpp:348-398
    // ------------------------------------------------------ heat source
    std::vector<double> src_pending, src_prescribed, src_deposited;

    // src/solver/PrescribedHeatSource.cpp:218-240
    void source_accrue(double factor) {
        if (!std::isfinite(factor) || factor < 0.0)
            throw std::invalid_argument("Integrated heat-source time must be finite and nonnegative.");
        for (size_t c = 0; c < P.source.rates.size(); ++c) {
            const double e = P.source.rates[c] * factor;
            src_prescribed[c] += e;
            src_pending[c] += e;
        }
    }

    void source_apply(long long& updates, double& deposited) {
        source_apply_cells(P.source, mats, P.mats, P.cell_material, cfg.background_temperature, members_by_cell(),
                           mode, occ, cell_T, src_pending, src_deposited, updates, deposited);
    }

    // src/solver/HeatSourceDriving.cpp:46-80
    void apply_heat_source(double begin, double end) {
        if (!P.source.enabled) return;
        const double factor = heat_source_time_factor(cfg, begin, end);
        double pending_total = 0.0;
        for (double e : src_pending) pending_total += e;
        if (factor <= 0.0 && pending_total <= 0.0) return;
        source_accrue(factor);
        long long updates = 0;
        double e = 0.0;
        source_apply(updates, e);
        energy.record_source(updates, e);
    }

    // Stable reordering of the carrier slots by (active mode, cell), by (cell,
    // active mode) in mesh domains, dead slots last -- the device's periodic
    // carrier sort (resolved_sort_interval). Slots key the counter-based
    // draws, so the oracle reorders its slots at the same steps.
    void sort_carriers() {
        const size_t n = alive.size();
        const bool cell_major = domain->is_mesh();
        auto key = [&](size_t i) -> uint64_t {
            if (!alive[i]) return std::numeric_limits<uint64_t>::max();
            const uint64_t a = mode[i] & kActiveMask, c = static_cast<uint32_t>(cell[i]);
            return cell_major ? (c << 32) | a : (a << 32) | c;
        };
        std::vector<uint64_t> k(n);
        for (size_t i = 0; i < n; ++i) k[i] = key(i);
        std::vector<size_t> perm(n);
        std::iota(perm.begin(), perm.end(), size_t{0});
        std::stable_sort(perm.begin(), perm.end(), [&](size_t a, size_t b) { return k[a] < k[b]; });
        auto apply = [&](auto& v) {
            if (v.size() != n) return;
            auto w = v;
            for (size_t i = 0; i < n; ++i) w[i] = v[perm[i]];
            v.swap(w);
        };
        apply(x), apply(y), apply(z), apply(occ), apply(mode), apply(cell), apply(alive);
        apply(mirror), apply(hit_t), apply(hit_p), apply(hit_f);
    }

    void run_timestep() {
        if (failed) throw std::runtime_error("Cannot resume a failed timestep; construct a new solver after fixing its cause.");
        failed = true;
        const int sort_every = resolved_sort_interval(cfg, false); // the plain FP64 state's schedule
        if (sort_every > 0 && step % sort_every == 0) sort_carriers();
        energy.begin_step();
        step_b = {};
        const double midpoint = elapsed + 0.5 * cfg.time_step;
        const double end = elapsed + cfg.time_step;
        apply_heat_source(elapsed, midpoint);
        if (energy.step().source_energy_ev > 0.0) refresh();
        gradient_half();
        transport();
        refresh();
        energy.set_lifetime_residual(collide());
        apply_heat_source(midpoint, end);
        gradient_half();
        refresh();
        energy.finish_step(total_thermal(), step_b);
        total_b.absorbed += step_b.absorbed;
        total_b.injected += step_b.injected;
        total_b.absorbed_energy_ev += step_b.absorbed_energy_ev;
        total_b.injected_energy_ev += step_b.injected_energy_ev;
        ++step;
        elapsed += cfg.time_step;
        if (step == 1 || step % cfg.convergence_write_interval == 0) update_flux();
        failed = false;
    }
};

struct OracleMaterial {
    std::unique_ptr<PhononMaterial> m;
};

template <class F> int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 1;
    }
}
} // namespace

extern "C" {
const char* orc_last_error() { return g_error.c_str(); }

int orc_material_create(const phmc_material_data* d, double dt, int stationary, int complete_bz, void** out) {
    return guard([&] {
        auto* m = new OracleMaterial;
        m->m = std::make_unique<PhononMaterial>(material_from_pod(*d), dt, stationary != 0, complete_bz != 0);
        *out = m;
    });
}
void orc_material_destroy(void* m) { delete static_cast<OracleMaterial*>(m); }

int orc_solver_create(const phmc_config* c, void* const* mats, int n, void** out) {
    return guard([&] {
        auto* s = new OracleSolver;
        s->cfg = config_from_pod(*c);
        std::vector<const PhononMaterial*> ms;
        for (int i = 0; i < n; ++i) ms.push_back(static_cast<OracleMaterial*>(mats[i])->m.get());
        try {
            s->init(ms);
        } catch (...) {
            delete s;
            throw;
        }
        *out = s;
    });
}
void orc_solver_destroy(void* s) { delete static_cast<OracleSolver*>(s); }
int orc_solver_run(void* sp, int steps) {
    return guard([&] {
        auto* s = static_cast<OracleSolver*>(sp);
        for (int k = 0; k < steps; ++k) s->run_timestep();
    });
}
int orc_solver_stats(void* sp, phmc_stats* o) {
    return guard([&] {
        auto* s = static_cast<OracleSolver*>(sp);
        std::memset(o, 0, sizeof *o);
        o->current_timestep = s->step;
        long long n = 0;
        for (auto a : s->alive) n += a;
        o->particle_count = n;
        o->absorbed_total = s->total_b.absorbed;
        o->injected_total = s->total_b.injected;
        o->step_absorbed = s->step_b.absorbed;
        o->step_injected = s->step_b.injected;
        o->step_absorbed_energy_ev = s->step_b.absorbed_energy_ev;
        o->step_injected_energy_ev = s->step_b.injected_energy_ev;
        o->total_thermal_energy_ev = s->energy.thermal_energy_ev();
        o->total_lifetime_energy_residual_ev = s->energy.total().lifetime_residual_ev;
        o->step_lifetime_energy_residual_ev = s->energy.step().lifetime_residual_ev;
        o->total_energy_balance_residual_ev = s->energy.total().balance_residual_ev;
        o->step_energy_balance_residual_ev = s->energy.step().balance_residual_ev;
        o->total_gradient_energy_ev = s->energy.total().drive_energy_ev;
        o->step_gradient_energy_ev = s->energy.step().drive_energy_ev;
        o->step_gradient_updates = s->energy.step().drive_updates;
        o->average_heat_flux_along_axis = s->avg_flux;
        o->kappa_fit = s->kappa_fit;
        o->kappa_endpoints = s->kappa_end;
        o->total_heat_source_energy_ev = s->energy.total().source_energy_ev;
        o->step_heat_source_energy_ev = s->energy.step().source_energy_ev;
        o->step_heat_source_updates = s->energy.step().source_updates;
        for (double e : s->src_prescribed) o->prescribed_heat_source_energy_ev += e;
        for (double e : s->src_pending) o->pending_heat_source_energy_ev += e;
        o->interface_events = s->iface_events;
        o->interface_transmitted = s->iface_transmitted;
        o->interface_reflected = s->iface_reflected;
        for (int k = 0; k < 8; ++k) o->rough_counts[k] = s->rough_counts[k];
        o->collision_cache_corrections = s->cache_corrections;
    });
}
int orc_solver_cell_count(void* sp, int* n) {
    *n = static_cast<OracleSolver*>(sp)->domain->grid_count();
    return 0;
}
int orc_solver_cells(void* sp, double* T, double* E, double* q3) {
    auto* s = static_cast<OracleSolver*>(sp);
    for (size_t c = 0; c < s->cell_T.size(); ++c) {
        if (T) T[c] = s->cell_T[c];
        if (E) E[c] = s->cell_E[c];
        if (q3)
            for (int k = 0; k < 3; ++k) q3[3 * c + k] = s->cell_q[c][k];
    }
    return 0;
}
int orc_solver_slot_count(void* sp, int64_t* n) {
    *n = static_cast<int64_t>(static_cast<OracleSolver*>(sp)->alive.size());
    return 0;
}
int orc_solver_get_carriers(void* sp, double* x, double* y, double* z, double* occ, uint32_t* mode, int32_t* cell,
                            uint8_t* alive) {
    auto* s = static_cast<OracleSolver*>(sp);
    const size_t n = s->alive.size();
    std::copy(s->x.begin(), s->x.end(), x);
    std::copy(s->y.begin(), s->y.end(), y);
    std::copy(s->z.begin(), s->z.end(), z);
    std::copy(s->occ.begin(), s->occ.end(), occ);
    std::copy(s->mode.begin(), s->mode.end(), mode);
    std::copy(s->cell.begin(), s->cell.end(), cell);
    std::copy(s->alive.begin(), s->alive.end(), alive);
    (void)n;
    return 0;
}
int orc_solver_set_carriers(void* sp, int64_t n, const double* x, const double* y, const double* z, const double* occ,
                            const uint32_t* mode, const uint8_t* alive) {
    return guard([&] {
        auto* s = static_cast<OracleSolver*>(sp);
        s->x.assign(x, x + n); s->y.assign(y, y + n); s->z.assign(z, z + n);
        s->occ.assign(occ, occ + n); s->mode.assign(mode, mode + n); s->alive.assign(alive, alive + n);
        if (s->domain->is_mesh()) s->reset_mesh_state();
        s->cell.resize(n);
        for (int64_t i = 0; i < n; ++i) s->cell[i] = s->domain->fast_grid_index({x[i], y[i], z[i]});
        s->refresh();
        s->energy.initialize(s->total_thermal());
        for (size_t r = 0; r < s->P.reservoirs.size(); ++r) s->prev_absorbed[r] = s->P.reservoirs[r].initial_count;
        s->step = 0;
        s->elapsed = 0;
    });
}

// ---- deterministic sub-steps (same signatures as the phmc_dev_* entry points)
int orc_trace_box(const double lo[3], const double hi[3], int64_t n, const double* p3, const double* v3, double* hit3,
                  double* t, int32_t* facet) {
    return guard([&] {
        SimulationConfig c;
        c.sizes = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
        c.face_condition = {'R', 'R', 'R', 'R', 'R', 'R'};
        SimulationDomain d(c);
        for (int64_t i = 0; i < n; ++i) {
            // Domain is anchored at the origin; shift in and out.
            Vec3 p{p3[3 * i] - lo[0], p3[3 * i + 1] - lo[1], p3[3 * i + 2] - lo[2]};
            Vec3 v{v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]};
            Vec3 cp;
            int f;
            d.trace(p, v, cp, t[i], f);
            facet[i] = f;
            for (int k = 0; k < 3; ++k) hit3[3 * i + k] = f >= 0 ? cp[k] + lo[k] : p3[3 * i + k];
        }
    });
}

int orc_temperature_from_energy(void* m, int64_t n, const double* E, double* T) {
    auto* M = static_cast<OracleMaterial*>(m)->m.get();
    for (int64_t i = 0; i < n; ++i) T[i] = M->temperature_from_energy_density(E[i]);
    return 0;
}

int orc_rta_collide(void* m, int64_t n, const int32_t* flat, const int32_t* cell, double* occ, int cells,
                    const double* cell_T, double dt, double vol, int local, double Tlife, double* residual) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        std::vector<double> om(n), a(n), o(occ, occ + n);
        std::vector<std::vector<int>> members(cells);
        for (int64_t i = 0; i < n; ++i) {
            om[i] = M->omega(flat[i]);
            a[i] = M->mode_relaxation_weight(local ? cell_T[cell[i]] : Tlife, flat[i], dt);
            members[cell[i]].push_back(static_cast<int>(i));
        }
        const double w = M->active_mode_count() * vol / M->energy_density_normalization();
        double r = 0;
        for (int c = 0; c < cells; ++c) r += rta_cell(members[c], om, a, o, cell_T[c], w);
        std::copy(o.begin(), o.end(), occ);
        *residual = r;
    });
}

// One cell of nonlinear Callaway: carriers with modes into the per-mode tables.
int orc_ncallaway_evolve(int32_t n_modes, const double* omega, const double* k3, const double* rn, const double* rr,
                         int64_t n, const int32_t* mode, double* occ, double T, double dt) {
    return guard([&] {
        std::vector<double> om(n), a(n), b(n), o(occ, occ + n);
        std::vector<std::array<double, 3>> k(n);
        for (int64_t i = 0; i < n; ++i) {
            const int m = mode[i];
            if (m < 0 || m >= n_modes) throw std::invalid_argument("Invalid nonlinear Callaway mode");
            om[i] = omega[m];
            k[i] = {k3[3 * m], k3[3 * m + 1], k3[3 * m + 2]};
            a[i] = rn[m];
            b[i] = rr[m];
        }
        const auto out = ncl::evolve(om, k, a, b, o, T, dt);
        std::copy(out.begin(), out.end(), occ);
    });
}

int orc_linear_collide(void* m, int model, double Tref, int64_t n, const int32_t* flat, const int32_t* cell, double* occ,
                       int cells, double dt, double vol, double* residual) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        const CallawayData d = model == 1 ? M->callaway_data(Tref) : M->linearized_rta_data(Tref);
        MaterialTables T;
        T.n_active = M->active_mode_count();
        T.omega = d.omega;
        T.col_capacity = d.capacity;
        T.col_normal = d.normal_rate;
        T.col_resistive = d.resistive_rate;
        for (const auto& k : d.wavevector) T.col_k.insert(T.col_k.end(), k.begin(), k.end());
        for (int a = 0; a < T.n_active; ++a) T.nbg.push_back(M->bose_occupation(Tref, M->active_flat()[a]));
        std::vector<int> act(n);
        std::vector<std::vector<int>> members(cells);
        std::vector<double> o(occ, occ + n);
        for (int64_t i = 0; i < n; ++i) {
            act[i] = M->active_index_for_flat(flat[i]);
            if (act[i] < 0) throw std::invalid_argument("Invalid existing collision carrier.");
            members[cell[i]].push_back(static_cast<int>(i));
        }
        long double sum = 0;
        const double w = M->active_mode_count() * vol / M->energy_density_normalization();
        for (int c = 0; c < cells; ++c) sum += linear_cell(members[c], T, act, o, dt, w);
        std::copy(o.begin(), o.end(), occ);
        *residual = static_cast<double>(sum);
    });
}

int orc_rough_reflect(void* m, int conservative, double Tref, const double nout[3], double rough_a, int64_t n,
                      const int32_t* flat_in, const double* occ_in, const double* u3, int32_t* flat_out, double* occ_out) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        RoughTables rt;
        rt.build({M}, {{nout[0], nout[1], nout[2]}}, {rough_a}, {1}, conservative != 0, conservative ? Tref : 0.0);
        MaterialTables T;
        T.n_active = M->active_mode_count();
        for (int a = 0; a < T.n_active; ++a) {
            T.omega.push_back(M->omega(M->active_flat()[a]));
            T.nbg.push_back(M->bose_occupation(Tref, M->active_flat()[a]));
        }
        for (int64_t i = 0; i < n; ++i) {
            const int ai = M->active_index_for_flat(flat_in[i]);
            double o;
            const int out = rough_sample(rt.tables[0], T, ai, occ_in[i], conservative != 0,
                                         RoughDraws{{u3[3 * i], u3[3 * i + 1], u3[3 * i + 2]}}, o);
            flat_out[i] = M->active_flat()[out];
            occ_out[i] = o;
        }
    });
}

// Interface interactions between two materials with explicit weights and draws
// (src/solver/InterfaceInteraction.cpp:46-153); signs are the carrier's three
// velocity sign bits relative to the table velocity.
int orc_interface(void* ma, void* mb, double wa, double wb, int axis, double bin_thz, double Tref, int linearized,
                  int64_t n, const int32_t* src, const int32_t* flat_in, const int32_t* signs_in, const double* occ_in,
                  const double* u3, int32_t* action, int32_t* material_out, int32_t* flat_out, int32_t* signs_out,
                  double* occ_out) {
    return guard([&] {
        const PhononMaterial* M[2] = {static_cast<OracleMaterial*>(ma)->m.get(), static_cast<OracleMaterial*>(mb)->m.get()};
        InterfaceTables I;
        I.enabled = true;
        I.linearized = linearized != 0;
        I.reference_temperature = Tref;
        I.band_width = 2.0 * std::acos(-1.0) * bin_thz;
        I.build({M[0], M[1]}, axis);
        std::vector<MaterialTables> T(2);
        const double w[2] = {wa, wb};
        for (int k = 0; k < 2; ++k) {
            T[k].n_active = M[k]->active_mode_count();
            T[k].energy_weight = w[k];
            for (int a = 0; a < T[k].n_active; ++a) {
                const int f = M[k]->active_flat()[a];
                T[k].omega.push_back(M[k]->omega(f));
                T[k].nbg.push_back(M[k]->bose_occupation(Tref, f));
                for (int c = 0; c < 3; ++c) T[k].vel.push_back(M[k]->velocity(f)[c]);
            }
        }
        for (int64_t i = 0; i < n; ++i) {
            const int m = src[i];
            const int a = M[m]->active_index_for_flat(flat_in[i]);
            const double u[4] = {u3[3 * i], u3[3 * i + 1], u3[3 * i + 2], 0.0};
            const InterfaceOutcome r = interface_interact(I, T, m, a, static_cast<uint32_t>(signs_in[i]), occ_in[i], 1 - m,
                                                          u);
            action[i] = r.action;
            material_out[i] = r.material;
            flat_out[i] = M[r.material]->active_flat()[r.active];
            signs_out[i] = static_cast<int32_t>(r.signs);
            occ_out[i] = r.occ;
        }
    });
}

// Acoustic-mismatch rows of one side of the a|b interface normal to z
// (AcousticInterfaceSampler::configure / row): reflected partner and the
// transmitted entries [start[a], start[a+1]) of every active mode; dest / prob
// may be NULL to read the sizes first (start has n_active + 1 entries).
int orc_amm_rows(void* ma, void* mb, double rho_a, double rho_b, double bin_thz, double bin_k, int side,
                 int32_t* reflected, int32_t* start, int32_t* dest, double* prob) {
    return guard([&] {
        const PhononMaterial* M[2] = {static_cast<OracleMaterial*>(ma)->m.get(), static_cast<OracleMaterial*>(mb)->m.get()};
        AmmTables A;
        A.build({M[0], M[1]}, 2, {rho_a, rho_b}, bin_thz, bin_k);
        const auto& rows = A.faces.at(0).rows[side];
        int at = 0;
        start[0] = 0;
        for (size_t a = 0; a < rows.size(); ++a) {
            reflected[a] = rows[a].reflected;
            for (const auto& e : rows[a].transmitted) {
                if (dest) dest[at] = e.first;
                if (prob) prob[at] = e.second;
                ++at;
            }
            start[a + 1] = at;
        }
    });
}

// Interface events with the acoustic (model 1) or mixed (model 2) mismatch
// model between materials a and b (z axis), uniforms u[4 i .. 4 i + 3] in the
// order InterfaceInteraction::interact consumes them.
int orc_interface_model(void* ma, void* mb, double wa, double wb, double bin_thz, double Tref, int linearized,
                        int model, double fraction, double rho_a, double rho_b, double bin_k, int64_t n,
                        const int32_t* src, const int32_t* flat_in, const double* occ_in, const double* u4,
                        int32_t* action, int32_t* material_out, int32_t* flat_out, double* occ_out) {
    return guard([&] {
        const PhononMaterial* M[2] = {static_cast<OracleMaterial*>(ma)->m.get(), static_cast<OracleMaterial*>(mb)->m.get()};
        InterfaceTables I;
        I.enabled = true;
        I.linearized = linearized != 0;
        I.reference_temperature = Tref;
        I.band_width = 2.0 * std::acos(-1.0) * bin_thz;
        I.build({M[0], M[1]}, 2);
        I.model = model;
        I.amm_fraction = model == 1 ? 1.0 : fraction;
        I.amm.build({M[0], M[1]}, 2, {rho_a, rho_b}, bin_thz, bin_k);
        std::vector<MaterialTables> T(2);
        const double w[2] = {wa, wb};
        for (int k = 0; k < 2; ++k) {
            T[k].n_active = M[k]->active_mode_count();
            T[k].energy_weight = w[k];
            for (int a = 0; a < T[k].n_active; ++a) {
                const int f = M[k]->active_flat()[a];
                T[k].omega.push_back(M[k]->omega(f));
                T[k].nbg.push_back(M[k]->bose_occupation(Tref, f));
                for (int c = 0; c < 3; ++c) T[k].vel.push_back(M[k]->velocity(f)[c]);
            }
        }
        for (int64_t i = 0; i < n; ++i) {
            const int m = src[i];
            const int a = M[m]->active_index_for_flat(flat_in[i]);
            const InterfaceOutcome r = interface_interact(I, T, m, a, 0u, occ_in[i], 1 - m, u4 + 4 * i);
            action[i] = r.action;
            material_out[i] = r.material;
            flat_out[i] = M[r.material]->active_flat()[r.active];
            occ_out[i] = r.occ;
        }
    });
}

// Ray traces through a triangle surface (src/SurfaceMesh.cpp:1164-1269) with the
// faces as given (oriented) and their facet ids.
int orc_trace_mesh(int nv, const double* vertices, int nf, const int32_t* faces, const int32_t* face_to_facet, int64_t n,
                   const double* p3, const double* v3, double* hit3, double* t, int32_t* facet) {
    return guard([&] {
        MeshTracer M;
        std::vector<Vec3> V(nv);
        for (int i = 0; i < nv; ++i) V[i] = {vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]};
        std::vector<std::array<int, 3>> F(nf);
        for (int i = 0; i < nf; ++i) F[i] = {faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]};
        M.build(std::move(V), std::move(F), std::vector<int>(face_to_facet, face_to_facet + nf));
        for (int64_t i = 0; i < n; ++i) {
            Vec3 h;
            int f;
            M.trace({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]}, {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]}, h, t[i], f);
            for (int a = 0; a < 3; ++a) hit3[3 * i + a] = h[a];
            facet[i] = f;
        }
    });
}

// PrescribedHeatSource cell powers (eV/ps) of a configuration
// (src/solver/PrescribedHeatSource.cpp:22-216); `rates` has one entry per cell.
int orc_source_rates(const phmc_config* cfg, double* rates, int* cells) {
    return guard([&] {
        const SimulationConfig c = config_from_pod(*cfg);
        SimulationDomain d(c);
        HeatSourceTables S;
        S.configure(c, d);
        *cells = d.grid_count();
        for (int k = 0; k < d.grid_count(); ++k) rates[k] = S.enabled ? S.rates[k] : 0.0;
    });
}

// PhononSourceOperator::apply on explicit carriers and cell budgets
// (src/solver/PhononSourceOperator.cpp:119-340); pending is updated in place.
int orc_source_apply(void* m, const phmc_heat_source* h, int linearized, double Tbg, double particle_volume,
                     int cells, const double* cell_T, double* pending, int64_t n, const int32_t* flat,
                     const int32_t* cell, double* occ, double* energy, int64_t* updates) {
    return guard([&] {
        const PhononMaterial* M = static_cast<OracleMaterial*>(m)->m.get();
        SimulationConfig c;
        heat_source_from_pod(*h, c);
        if (linearized) c.collision_model = CollisionModel::Callaway;
        validate_heat_source_config(c);
        HeatSourceTables S;
        S.set_spectrum(c);
        S.enabled = true;
        std::vector<MaterialTables> T(1);
        T[0].n_active = M->active_mode_count();
        T[0].active_flat = M->active_flat();
        T[0].energy_weight = T[0].n_active * particle_volume / M->energy_density_normalization();
        std::vector<uint32_t> mode(n);
        std::vector<double> o(occ, occ + n), cT(cell_T, cell_T + cells), pend(pending, pending + cells), dep(cells, 0.0);
        std::vector<std::vector<int>> members(cells);
        for (int64_t i = 0; i < n; ++i) {
            mode[i] = static_cast<uint32_t>(M->active_index_for_flat(flat[i]));
            members.at(cell[i]).push_back(static_cast<int>(i));
        }
        long long up = 0;
        double e = 0.0;
        source_apply_cells(S, {M}, T, std::vector<int>(cells, 0), Tbg, members, mode, o, cT, pend, dep, up, e);
        std::copy(o.begin(), o.end(), occ);
        std::copy(pend.begin(), pend.end(), pending);
        *energy = e;
        *updates = up;
    });
}

int orc_gradient_drive(void* m, int axis, double G, double Tref, int64_t n, const int32_t* flat, const int32_t* cell,
                       double* occ, int cells, double dt, double vol, double* energy) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        const int na = M->active_mode_count();
        std::vector<double> rate(na), cap(na), hw(na);
        long double sum = 0, tc = 0;
        for (int a = 0; a < na; ++a) {
            const int f = M->active_flat()[a];
            cap[a] = M->mode_heat_capacity(Tref, f);
            rate[a] = -cap[a] * M->velocity(f)[axis] * 1e-10 * G;
            hw[a] = kHbarEvPs * M->omega(f);
            sum += rate[a];
            tc += cap[a];
        }
        for (int a = 0; a < na; ++a) rate[a] -= static_cast<double>(sum * cap[a] / tc);
        std::vector<std::vector<int>> members(cells);
        for (int64_t i = 0; i < n; ++i) members[cell[i]].push_back(static_cast<int>(i));
        std::vector<double> next(occ, occ + n);
        long double actual = 0;
        for (const auto& mem : members) {
            long double rs = 0, cs = 0;
            for (int i : mem) {
                const int a = M->active_index_for_flat(flat[i]);
                rs += rate[a];
                cs += cap[a];
            }
            for (int i : mem) {
                const int a = M->active_index_for_flat(flat[i]);
                const long double e = dt * (rate[a] - rs * cap[a] / cs);
                next[i] += static_cast<double>(e / hw[a]);
                actual += hw[a] * (static_cast<long double>(next[i]) - occ[i]);
            }
        }
        std::copy(next.begin(), next.end(), occ);
        *energy = static_cast<double>(actual * (na * vol / M->energy_density_normalization()));
    });
}
// Material queries for the golden-vector tests: what = 0 bose(T), 1 capacity(T),
// 2 relaxation weight(T, dt=aux), 3 linearized bose(T, Tref=aux), 4 E(T) table,
// 5 T(E) table, 6 crystal E(T). in_flat may be NULL for table queries.
int orc_material_query(void* m, int what, int64_t n, const int32_t* flat, const double* x, double aux, double* out) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        for (int64_t i = 0; i < n; ++i) {
            switch (what) {
            case 0: out[i] = M->bose_occupation(x[i], flat[i]); break;
            case 1: out[i] = M->mode_heat_capacity(x[i], flat[i]); break;
            case 2: out[i] = M->mode_relaxation_weight(x[i], flat[i], aux); break;
            case 3: out[i] = M->linearized_bose_occupation(x[i], aux, flat[i]); break;
            case 4: out[i] = M->energy_density_from_temperature(x[i]); break;
            case 5: out[i] = M->temperature_from_energy_density(x[i]); break;
            case 6: out[i] = M->crystal_energy_density(x[i]); break;
            default: throw std::invalid_argument("unknown query");
            }
        }
    });
}

// Scalars: [active_count, normalization, zero_point, bg energy weight(vol=aux),
// bg energy density (table), bg energy density (exact), bg heat capacity density] at T=300.
int orc_material_scalars(void* m, double vol, double* out7, int32_t* active_flat) {
    auto* M = static_cast<OracleMaterial*>(m)->m.get();
    out7[0] = M->active_mode_count();
    out7[1] = M->energy_density_normalization();
    out7[2] = M->zero_point_energy_density();
    out7[3] = M->active_mode_count() * vol / M->energy_density_normalization();
    out7[4] = M->energy_density_from_temperature(300.0);
    out7[5] = M->crystal_energy_density(300.0);
    double c = 0;
    for (int f = 0; f < M->flat_count(); ++f) c += M->mode_heat_capacity(300.0, f) / M->energy_density_normalization();
    out7[6] = c;
    if (active_flat) std::copy(M->active_flat().begin(), M->active_flat().end(), active_flat);
    return 0;
}

int orc_grid_index(const double sizes[3], const int32_t grid[3], int64_t n, const double* p3, int32_t* out) {
    return guard([&] {
        SimulationConfig c;
        c.sizes = {sizes[0], sizes[1], sizes[2]};
        c.grid = {grid[0], grid[1], grid[2]};
        SimulationDomain d(c);
        for (int64_t i = 0; i < n; ++i) out[i] = d.fast_grid_index({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]});
    });
}

int orc_callaway_evolve(int64_t n, const double* omega, const double* cap, const double* k3, const double* rn,
                        const double* rr, const double* energy, double dt, double* out) {
    return guard([&] {
        std::vector<Vec3> k(n);
        for (int64_t i = 0; i < n; ++i) k[i] = {k3[3 * i], k3[3 * i + 1], k3[3 * i + 2]};
        const auto r = Callaway(std::vector<double>(omega, omega + n), std::vector<double>(cap, cap + n), k,
                                std::vector<double>(rn, rn + n), std::vector<double>(rr, rr + n))
                           .evolve(std::vector<double>(energy, energy + n), dt);
        std::copy(r.begin(), r.end(), out);
    });
}

// Incoming-flux CDF of one reservoir face (src/solver/ReservoirSampler.cpp:60-99).
int orc_reservoir_cdf(void* m, const double normal[3], double area, double density, double dt, double* cdf,
                      double* expected, int32_t* initial_count) {
    return guard([&] {
        auto* M = static_cast<OracleMaterial*>(m)->m.get();
        const auto& act = M->active_flat();
        const double thickness = M->active_mode_count() / (density * area);
        double e = 0;
        for (size_t i = 0; i < act.size(); ++i) {
            const auto& v = M->velocity(act[i]);
            const double par = -(normal[0] * v[0] + normal[1] * v[1] + normal[2] * v[2]);
            e += std::max(0.0, par * dt / thickness);
            cdf[i] = e;
        }
        if (e > 0)
            for (size_t i = 0; i < act.size(); ++i) cdf[i] /= e;
        *expected = e;
        *initial_count = static_cast<int32_t>(std::llround(e));
    });
}

// The solver's alias table of weights w (build_alias_table, shared with the
// device build) and the outcomes it gives for uniforms u (alias_draw).
int orc_alias_table(const double* w, int32_t n, double* prob, int32_t* alias, int32_t n_draws, const double* u,
                    int32_t* out) {
    return guard([&] {
        const std::vector<AliasCell> t = build_alias_table(std::vector<double>(w, w + n));
        for (int32_t k = 0; k < n; ++k) {
            prob[k] = t[k].prob;
            alias[k] = t[k].alias;
        }
        for (int32_t j = 0; j < n_draws; ++j) out[j] = alias_draw(t.data(), n, u[j]);
    });
}
} // extern "C"
