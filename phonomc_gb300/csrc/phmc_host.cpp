// Host-side tables for the carrier loop. See phmc_host.h for the map to the
// reference; each function cites the reference lines whose semantics it keeps.
#include "phmc_host.h"

#include "phmc_rng.h"
#include "phmc_tuning.h"

#include <algorithm>
#include <set>
#include <functional>
#include <cmath>
#include <cstdio>
#include <limits>
#include <numeric>
#include <sstream>

namespace phmc {
namespace {
double dot3(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double norm3(const Vec3& a) { return std::sqrt(dot3(a, a)); }
Vec3 sub3(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
Vec3 mul3(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
Vec3 q_to_k(const std::array<Vec3, 3>& R, const Vec3& q) {
    return {R[0][0] * q[0] + R[0][1] * q[1] + R[0][2] * q[2],
            R[1][0] * q[0] + R[1][1] * q[1] + R[1][2] * q[2],
            R[2][0] * q[0] + R[2][1] * q[1] + R[2][2] * q[2]};
}
} // namespace

// ------------------------------------------------------------- material
// Shape/finiteness checks of src/material/MaterialData.cpp:1-131.
void validate_material_data(const MaterialData& d) {
    const size_t nm = static_cast<size_t>(d.qpoints) * d.branches;
    if (!(d.volume_a3 > 0) || !std::isfinite(d.volume_a3))
        throw std::runtime_error("Unit-cell volume must be finite and positive");
    if (d.qpoints <= 0 || d.branches <= 0) throw std::runtime_error("empty phonon table");
    if (d.frequency_thz.size() != nm) throw std::runtime_error("frequency shape mismatch");
    if (d.qpoint_fractions.size() != static_cast<size_t>(d.qpoints))
        throw std::runtime_error("qpoint shape mismatch");
    if (d.group_velocity.size() != nm) throw std::runtime_error("group_velocity shape mismatch");
    size_t grid = 1;
    for (int m : d.mesh) {
        if (m <= 0) throw std::runtime_error("mesh entries must be positive integers");
        grid *= static_cast<size_t>(m);
    }
    if (grid != static_cast<size_t>(d.qpoints))
        throw std::runtime_error("Full Brillouin-zone grid required: qpoint count differs from "
                                 "mesh product. Expand reduced data first.");
    if (d.temperatures.empty() || d.temperatures.front() < 0 ||
        !std::is_sorted(d.temperatures.begin(), d.temperatures.end()) ||
        std::adjacent_find(d.temperatures.begin(), d.temperatures.end()) != d.temperatures.end())
        throw std::runtime_error("temperature must be nonempty, nonnegative and strictly increasing");
    if (d.gamma.size() != d.temperatures.size() * nm) throw std::runtime_error("gamma shape mismatch");
    for (double g : d.gamma)
        if (!std::isfinite(g) || g < 0) throw std::runtime_error("gamma must be nonnegative");
    if (d.gamma_normal.empty() != d.gamma_umklapp.empty())
        throw std::runtime_error("gamma_N and gamma_U must both be supplied or both omitted");
    if (!d.gamma_normal.empty() &&
        (d.gamma_normal.size() != d.gamma.size() || d.gamma_umklapp.size() != d.gamma.size()))
        throw std::runtime_error("N/U linewidth shape mismatch");
    for (const auto& [name, v] : d.gamma_resistive) {
        if (name != "gamma_isotope" && name != "gamma_impurity" && name != "gamma_defect")
            throw std::runtime_error("Unsupported resistive linewidth: " + name);
        if (v.size() != nm && v.size() != d.gamma.size()) throw std::runtime_error(name + " shape mismatch");
    }
}

// src/PhononMaterial.cpp:156-171, 216-291
// src/material/BzQuadrature.cpp:11-160: Callaway needs every q of the
// Gamma-centred mesh as its first-Brillouin-zone representative. A q with m
// equally short images q - G (zone-boundary points) is split into its images,
// and every q is repeated so all carry the same weight: the table grows by
// the least common multiple of the image counts (at most 96), q-major with
// the copies of one mesh point adjacent. Returns that factor.
unsigned complete_callaway_bz(MaterialData& d) {
    const auto& b = d.reciprocal;
    const double det = b[0][0] * (b[1][1] * b[2][2] - b[1][2] * b[2][1]) -
                       b[0][1] * (b[1][0] * b[2][2] - b[1][2] * b[2][0]) +
                       b[0][2] * (b[1][0] * b[2][1] - b[1][1] * b[2][0]);
    if (!std::isfinite(det) || det == 0) throw std::invalid_argument("Callaway reciprocal lattice is singular.");
    double inv[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            inv[i][j] = (b[(j + 1) % 3][(i + 1) % 3] * b[(j + 2) % 3][(i + 2) % 3] -
                         b[(j + 1) % 3][(i + 2) % 3] * b[(j + 2) % 3][(i + 1) % 3]) / det;
    auto len2 = [&](const Vec3& q) {
        double r = 0;
        for (int i = 0; i < 3; ++i) {
            double x = 0;
            for (int j = 0; j < 3; ++j) x += b[i][j] * q[j];
            r += x * x;
        }
        return r;
    };
    std::set<std::array<int, 3>> seen;
    std::vector<std::vector<Vec3>> images(d.qpoints);
    unsigned refinement = 1;
    for (int iq = 0; iq < d.qpoints; ++iq) {
        const Vec3& q = d.qpoint_fractions[iq];
        std::array<int, 3> key{};
        for (int a = 0; a < 3; ++a) {
            const double x = (q[a] - std::floor(q[a])) * d.mesh[a];
            const long idx = std::lround(x);
            if (std::abs(x - idx) > 2e-6 * d.mesh[a])
                throw std::invalid_argument("Callaway requires a complete Gamma-centred full q mesh.");
            key[a] = static_cast<int>(idx % d.mesh[a]);
        }
        if (!seen.insert(key).second)
            throw std::invalid_argument(
                "Callaway input q mesh contains duplicate points modulo reciprocal translations.");
        const double own = len2(q);
        int lo[3], hi[3];
        double count = 1;
        for (int a = 0; a < 3; ++a) {
            const double ext = std::sqrt(own * (inv[a][0] * inv[a][0] + inv[a][1] * inv[a][1] + inv[a][2] * inv[a][2]));
            if (!std::isfinite(ext) || ext > 100 || std::abs(q[a]) > 100)
                throw std::invalid_argument("Callaway first-BZ validation exceeds supported lattice conditioning.");
            lo[a] = static_cast<int>(std::ceil(q[a] - ext - 1e-10));
            hi[a] = static_cast<int>(std::floor(q[a] + ext + 1e-10));
            count *= hi[a] - lo[a] + 1;
        }
        if (count > 100000) throw std::invalid_argument("Callaway first-BZ validation work limit exceeded.");
        std::vector<std::pair<double, Vec3>> cand;
        double best = own;
        for (int i = lo[0]; i <= hi[0]; ++i)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int k = lo[2]; k <= hi[2]; ++k) {
                    const Vec3 p{q[0] - i, q[1] - j, q[2] - k};
                    const double r = len2(p);
                    best = std::min(best, r);
                    cand.push_back({r, p});
                }
        const double tol = 1e-10 * std::max(best, 1e-20);
        if (own > best + tol)
            throw std::invalid_argument("Callaway qpoint is outside the first Brillouin zone; supply first-BZ "
                                        "representatives.");
        for (const auto& c : cand)
            if (std::abs(c.first - best) <= tol) images[iq].push_back(c.second);
        if (images[iq].empty()) throw std::runtime_error("Empty Callaway BZ representative set.");
        const unsigned m = static_cast<unsigned>(images[iq].size());
        const unsigned long long next = static_cast<unsigned long long>(refinement / std::gcd(refinement, m)) * m;
        if (next > 96 || next * static_cast<unsigned long long>(d.qpoints) * d.branches >
                             static_cast<unsigned long long>(std::numeric_limits<int>::max()))
            throw std::length_error("Callaway equal-weight BZ refinement exceeds supported storage; use a smaller mesh.");
        refinement = static_cast<unsigned>(next);
    }
    if (refinement == 1) return 1;
    const size_t nm0 = d.frequency_thz.size();
    std::vector<size_t> src;
    std::vector<Vec3> qs;
    for (int iq = 0; iq < d.qpoints; ++iq)
        for (const Vec3& im : images[iq])
            for (unsigned c = 0; c < refinement / images[iq].size(); ++c) {
                qs.push_back(im);
                for (int br = 0; br < d.branches; ++br) src.push_back(static_cast<size_t>(iq) * d.branches + br);
            }
    auto expand = [&](const std::vector<double>& v) {
        if (v.empty()) return v;
        std::vector<double> out;
        out.reserve(v.size() * refinement);
        for (size_t t = 0; t < v.size() / nm0; ++t)
            for (size_t i : src) out.push_back(v[t * nm0 + i]);
        return out;
    };
    std::vector<Vec3> vel;
    vel.reserve(src.size());
    for (size_t i : src) vel.push_back(d.group_velocity[i]);
    d.frequency_thz = expand(d.frequency_thz);
    d.gamma = expand(d.gamma);
    d.gamma_normal = expand(d.gamma_normal);
    d.gamma_umklapp = expand(d.gamma_umklapp);
    for (auto& e : d.gamma_resistive) e.second = expand(e.second);
    d.qpoints *= static_cast<int>(refinement);
    d.qpoint_fractions = std::move(qs);
    d.group_velocity = std::move(vel);
    return refinement;
}

PhononMaterial::PhononMaterial(MaterialData d, double lookup_dt, bool stationary, bool complete_bz)
    : dT_(lookup_dt), stationary_(stationary) {
    if (!std::isfinite(lookup_dt) || lookup_dt <= 0)
        throw std::invalid_argument("Temperature lookup spacing must be finite and positive");
    validate_material_data(d);
    if (complete_bz && !d.gamma_normal.empty()) refinement_ = complete_callaway_bz(d);
    volume_ = d.volume_a3;
    nq_ = d.qpoints;
    nb_ = d.branches;
    reciprocal_ = d.reciprocal;
    mesh_ = d.mesh;
    const int nm = nq_ * nb_;
    omega_.resize(nm);
    knorm_.assign(nm, 0.0);
    window_.assign(nm, 0.0);
    kvec_.resize(nm);
    for (int i = 0; i < nm; ++i) omega_[i] = std::max(0.0, d.frequency_thz[i]) * 2.0 * kPi;
    vel_ = std::move(d.group_velocity);
    temps_ = std::move(d.temperatures);
    gamma_normal_ = std::move(d.gamma_normal);
    gamma_umklapp_ = std::move(d.gamma_umklapp);
    gamma_extra_.assign(d.gamma.size(), 0.0);
    for (const auto& [name, values] : d.gamma_resistive) {
        (void)name;
        for (size_t i = 0; i < gamma_extra_.size(); ++i)
            gamma_extra_[i] += values[values.size() == static_cast<size_t>(nm) ? i % nm : i];
    }
    gamma_total_ = d.gamma;
    for (size_t i = 0; i < gamma_total_.size(); ++i) gamma_total_[i] += gamma_extra_[i];
    qfrac_ = d.qpoint_fractions;
    const Vec3 mesh_q{1.0 / (2.0 * mesh_[0]), 1.0 / (2.0 * mesh_[1]), 1.0 / (2.0 * mesh_[2])};
    const Vec3 kg = q_to_k(reciprocal_, mesh_q);
    for (int q = 0; q < nq_; ++q) {
        const Vec3 k = q_to_k(reciprocal_, qfrac_[q]);
        const double kn = norm3(k);
        for (int b = 0; b < nb_; ++b) {
            const int f = q * nb_ + b;
            const Vec3& v = vel_[f];
            knorm_[f] = kn;
            kvec_[f] = k;
            window_[f] = std::sqrt((v[0] * kg[0]) * (v[0] * kg[0]) + (v[1] * kg[1]) * (v[1] * kg[1]) +
                                   (v[2] * kg[2]) * (v[2] * kg[2]));
        }
    }
    active_.clear();
    for (int base = 0; base < nq_; base += static_cast<int>(refinement_)) {
        for (int b = 0; b < nb_; ++b) {
            for (unsigned c = 0; c < refinement_; ++c) {
                const int f = (base + static_cast<int>(c)) * nb_ + b;
                const double vn = norm3(vel_[f]);
                if (stationary_ ? omega_[f] > 0.0 : vn > 1e-12) active_.push_back(f);
            }
        }
    }
    if (active_.empty()) throw std::runtime_error("No active modes found in material data.");
    flat_to_active_.assign(nm, -1);
    for (size_t a = 0; a < active_.size(); ++a) flat_to_active_[active_[a]] = static_cast<int>(a);
    build_lookup();
}

// src/material/Thermodynamics.cpp:71-82
double PhononMaterial::bose_occupation(double T, int flat) const {
    const double w = omega_[flat];
    if (T <= 0.0 || w <= 0.0) return 0.0;
    const double x = kHbarEvPs * w / (kBoltzmannEvK * T);
    if (x > 700.0) return 0.0;
    return 1.0 / std::max(std::exp(x) - 1.0, 1e-12);
}

// src/material/Thermodynamics.cpp:11-25
double PhononMaterial::mode_heat_capacity(double T, int flat) const {
    const double hw = kHbarEvPs * omega_[flat];
    if (!(T > 0.0) || !(hw > 0.0)) return 0.0;
    const double x = hw / (kBoltzmannEvK * T);
    if (x < 1e-6) return kBoltzmannEvK * (1.0 - x * x / 12.0);
    if (x > 700.0) return 0.0;
    const double den = -std::expm1(-x);
    return kBoltzmannEvK * x * x * std::exp(-x) / (den * den);
}

// src/material/Thermodynamics.cpp:27-37
double PhononMaterial::linearized_bose_occupation(double T, double Tref, int flat) const {
    const double hw = kHbarEvPs * omega_[flat];
    if (!(hw > 0.0)) return 0.0;
    return bose_occupation(Tref, flat) + mode_heat_capacity(Tref, flat) * (T - Tref) / hw;
}

// src/material/Thermodynamics.cpp:40-68
double PhononMaterial::interp_linear_clamped(const std::vector<double>& xs, const std::vector<double>& ys,
                                             double x) {
    if (xs.empty() || ys.empty()) return 0.0;
    if (xs.size() == 1 || ys.size() == 1) return ys.front();
    if (x <= xs.front()) return ys.front();
    if (x >= xs.back()) return ys.back();
    const size_t hi = static_cast<size_t>(std::upper_bound(xs.begin(), xs.end(), x) - xs.begin());
    const size_t lo = hi - 1;
    const double x0 = xs[lo], x1 = xs[hi], y0 = ys[lo], y1 = ys[hi];
    if (std::abs(x1 - x0) <= 1e-18) return y0;
    const double t = (x - x0) / (x1 - x0);
    return y0 * (1.0 - t) + y1 * t;
}

// src/material/Thermodynamics.cpp:108-132
double PhononMaterial::mode_gamma(double T, int flat) const {
    if (!std::isfinite(T) || T < 0.0)
        throw std::invalid_argument("Lifetime temperature must be finite and nonnegative");
    const size_t nm = static_cast<size_t>(nq_) * nb_;
    if (T <= temps_.front()) return gamma_total_[flat];
    if (T >= temps_.back()) return gamma_total_[(temps_.size() - 1) * nm + flat];
    const size_t hi = static_cast<size_t>(std::upper_bound(temps_.begin(), temps_.end(), T) - temps_.begin());
    const size_t lo = hi - 1;
    const double x0 = temps_[lo], x1 = temps_[hi];
    const double y0 = gamma_total_[lo * nm + flat], y1 = gamma_total_[hi * nm + flat];
    if (std::abs(x1 - x0) <= 1e-18) return y0;
    const double t = (T - x0) / (x1 - x0);
    return y0 * (1.0 - t) + y1 * t;
}

// src/material/Thermodynamics.cpp:96-105
double PhononMaterial::mode_relaxation_weight(double T, int flat, double dt) const {
    if (!std::isfinite(dt) || dt < 0.0)
        throw std::invalid_argument("Relaxation time step must be finite and nonnegative");
    const double g = mode_gamma(T, flat);
    if (g == 0.0 || dt == 0.0) return 0.0;
    return -std::expm1(-(g * dt) * (4.0 * kPi));
}

double PhononMaterial::energy_density_normalization() const {
    return std::max(1.0, static_cast<double>(nq_) * volume_);
}

// src/material/Thermodynamics.cpp:134-146
double PhononMaterial::crystal_energy_density(double T) const {
    double e = 0.0;
    for (int f : active_) {
        const double w = omega_[f];
        if (w <= 0.0) continue;
        e += kHbarEvPs * w * bose_occupation(T, f);
    }
    return e / energy_density_normalization() + zero_point_;
}

double PhononMaterial::energy_density_from_temperature(double T) const {
    if (table_T_.empty()) return crystal_energy_density(T);
    return interp_linear_clamped(table_T_, table_E_, T);
}

double PhononMaterial::temperature_from_energy_density(double E) const {
    return interp_linear_clamped(table_E_, table_T_, E);
}

// src/material/Thermodynamics.cpp:178-224
void PhononMaterial::build_lookup() {
    zero_point_ = 0.0;
    for (double w : omega_) zero_point_ += 0.5 * kHbarEvPs * std::max(0.0, w);
    zero_point_ /= energy_density_normalization();
    const double tmin = 0.0;
    const double tmax = temps_.empty() ? 1000.0 : std::max(1000.0, *std::max_element(temps_.begin(), temps_.end()));
    const double dT = std::max(1e-6, dT_);
    const double intervals = std::floor((tmax - tmin) / dT + 0.5);
    const int n = std::max(2, static_cast<int>(intervals) + 1);
    table_T_.assign(n, 0.0);
    table_E_.assign(n, 0.0);
    std::vector<double> raw(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) raw[i] = crystal_energy_density(tmin + static_cast<double>(i) * dT);
    for (int i = 0; i < n; ++i) {
        table_T_[i] = tmin + static_cast<double>(i) * dT;
        double E = raw[i];
        if (i > 0) E = std::max(E, std::nextafter(table_E_[i - 1], std::numeric_limits<double>::infinity()));
        table_E_[i] = E;
    }
}

// src/material/PhononMaterialCollisionData.cpp:8-23
CallawayData PhononMaterial::linearized_rta_data(double T) const {
    if (!std::isfinite(T) || T <= 0 || temps_.empty() || T < temps_.front() || T > temps_.back())
        throw std::invalid_argument("Linearized RTA reference temperature is outside the scattering data range.");
    CallawayData d;
    for (int f : active_) {
        d.omega.push_back(omega_[f]);
        d.capacity.push_back(mode_heat_capacity(T, f));
        d.wavevector.push_back({0, 0, 0});
        d.normal_rate.push_back(0);
        d.resistive_rate.push_back(4 * std::acos(-1.0) * mode_gamma(T, f));
    }
    return d;
}

// src/material/PhononMaterialCollisionData.cpp:32-166 (rates and data; the
// first-BZ validation of the reference is not repeated here).
CallawayData PhononMaterial::callaway_data(double T) const {
    if (gamma_normal_.empty() || gamma_umklapp_.empty())
        throw std::invalid_argument("Callaway requires gamma_N and gamma_U in kappa-fbz.hdf5; regenerate with "
                                    "phono3py --br --nu and expand consistently. No N/U split is inferred.");
    if (!std::isfinite(T) || T <= 0 || T < temps_.front() || T > temps_.back())
        throw std::invalid_argument("Callaway reference temperature is outside the N/U data range.");
    const size_t hi = static_cast<size_t>(std::lower_bound(temps_.begin(), temps_.end(), T) - temps_.begin());
    const size_t lo = hi > 0 ? hi - 1 : hi;
    const double fr = hi == lo ? 0 : (T - temps_[lo]) / (temps_[hi] - temps_[lo]);
    const size_t nm = static_cast<size_t>(nq_) * nb_;
    CallawayData d;
    for (int f : active_) {
        d.omega.push_back(omega_[f]);
        d.capacity.push_back(mode_heat_capacity(T, f));
        d.wavevector.push_back(kvec_[f]);
        auto rate = [&](const std::vector<double>& t) {
            return 4 * std::acos(-1.0) * ((1 - fr) * t[lo * nm + f] + fr * t[hi * nm + f]);
        };
        d.normal_rate.push_back(rate(gamma_normal_));
        d.resistive_rate.push_back(rate(gamma_umklapp_) + rate(gamma_extra_));
    }
    return d;
}

// src/material/PhononMaterialCollisionData.cpp:168-193: normal and resistive
// (umklapp + extra) rates of one mode at T, linear in the temperature samples.
std::array<double, 2> PhononMaterial::mode_callaway_rates(double T, int f) const {
    if (gamma_normal_.empty() || gamma_umklapp_.empty() || !std::isfinite(T) || T <= 0 || T < temps_.front() ||
        T > temps_.back())
        throw std::invalid_argument("Nonlinear Callaway temperature " + std::to_string(T) +
                                    " K is outside the supplied N/U table");
    const size_t hi = static_cast<size_t>(std::lower_bound(temps_.begin(), temps_.end(), T) - temps_.begin());
    const size_t lo = hi ? hi - 1 : hi;
    const double fr = lo == hi ? 0 : (T - temps_[lo]) / (temps_[hi] - temps_[lo]);
    const size_t nm = static_cast<size_t>(nq_) * nb_;
    auto rate = [&](const std::vector<double>& t) {
        return t.empty() ? 0.0 : 4 * std::acos(-1.) * ((1 - fr) * t[lo * nm + f] + fr * t[hi * nm + f]);
    };
    return {rate(gamma_normal_), rate(gamma_umklapp_) + rate(gamma_extra_)};
}

// ---------------------------------------------------------------- domain
// Box facets in the reference's order (plane 2*axis+side), boundary conditions,
// periodic pairs and the uniform grid (src/SimulationDomain.cpp:131-198, 408-611, 626-766).
SimulationDomain::~SimulationDomain() = default;

SimulationDomain::SimulationDomain(const SimulationConfig& cfg) {
    if (cfg.model != "box") {
        build_mesh_domain(cfg);
        return;
    }
    if (cfg.sizes.size() != 3) throw std::runtime_error("Box requires three finite positive sizes.");
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(cfg.sizes[a]) || cfg.sizes[a] <= 0)
            throw std::runtime_error("Box requires three finite positive sizes.");
        bmin_[a] = 0.0;
        bmax_[a] = cfg.sizes[a];
    }
    volume_ = cfg.sizes[0] * cfg.sizes[1] * cfg.sizes[2];
    facets_.resize(6);
    for (int f = 0; f < 6; ++f) {
        const int axis = f / 2, side = f % 2;
        Facet& F = facets_[f];
        F.normal = {0, 0, 0};
        F.normal[axis] = side ? 1.0 : -1.0;
        const int u = (axis + 1) % 3, v = (axis + 2) % 3;
        F.centroid[axis] = side ? bmax_[axis] : bmin_[axis];
        F.centroid[u] = 0.5 * (bmin_[u] + bmax_[u]);
        F.centroid[v] = 0.5 * (bmin_[v] + bmax_[v]);
        F.area = (bmax_[u] - bmin_[u]) * (bmax_[v] - bmin_[v]);
        Vec3 c00 = F.centroid, c10 = F.centroid, c11 = F.centroid, c01 = F.centroid;
        c00[u] = bmin_[u]; c00[v] = bmin_[v];
        c10[u] = bmax_[u]; c10[v] = bmin_[v];
        c11[u] = bmax_[u]; c11[v] = bmax_[v];
        c01[u] = bmin_[u]; c01[v] = bmax_[v];
        F.tris = {{c00, c10, c11}, {c00, c11, c01}};
        F.tri_area = {0.5 * F.area, 0.5 * F.area};
        const char cond = cfg.face_condition[f];
        if (cond != 'T' && cond != 'P' && cond != 'R') throw std::runtime_error("Unknown boundary condition.");
        const double value = cond == 'R' ? cfg.face_value[f] * 10.0 : cfg.face_value[f];
        if (!std::isfinite(value) || value < 0 || (cond == 'P' && value != 0))
            throw std::runtime_error("Boundary values must be finite, nonnegative, and zero for periodic boundaries.");
        F.condition = cond;
        F.value = value;
    }
    for (int axis = 0; axis < 3; ++axis) {
        Facet& a = facets_[2 * axis];
        Facet& b = facets_[2 * axis + 1];
        if (a.condition == 'P' && b.condition == 'P') {
            a.pair = 2 * axis + 1;
            b.pair = 2 * axis;
            a.shift = sub3(b.centroid, a.centroid);
            b.shift = sub3(a.centroid, b.centroid);
        } else if (a.condition == 'P' || b.condition == 'P') {
            throw std::runtime_error("Periodic boundary facet " + std::to_string(a.condition == 'P' ? 2 * axis : 2 * axis + 1) +
                                     " is not assigned to a periodic pair.");
        }
    }
    for (int f = 0; f < 6; ++f) {
        if (facets_[f].condition == 'T') {
            facets_[f].reservoir = static_cast<int>(reservoir_facets_.size());
            reservoir_facets_.push_back(f);
        }
    }
    const int nx = cfg.grid[0], ny = cfg.grid[1], nz = cfg.grid[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) throw std::runtime_error("Grid sizes must be positive.");
    shape_ = {nx, ny, nz};
    const Vec3 ext = sub3(bmax_, bmin_);
    inv_cell_ = {nx / ext[0], ny / ext[1], nz / ext[2]};
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz; ++iz)
                centers_.push_back({bmin_[0] + (ix + 0.5) * ext[0] / nx, bmin_[1] + (iy + 0.5) * ext[1] / ny,
                                    bmin_[2] + (iz + 0.5) * ext[2] / nz});
    volumes_.assign(centers_.size(), volume_ / static_cast<double>(centers_.size()));
}

// src/SimulationDomain.cpp:92-126
int SimulationDomain::fast_grid_index(const Vec3& p) const {
    const int voxel = voxel_index(p);
    return mesh_ ? voxel_cell_[voxel] : voxel;
}

std::vector<int> SimulationDomain::cell_voxels() const {
    std::vector<int> home(centers_.size());
    for (size_t c = 0; c < centers_.size(); ++c) {
        home[c] = voxel_index(centers_[c]);
        if (mesh_ && voxel_cell_[home[c]] != static_cast<int>(c))
            throw std::runtime_error("cell centre outside its own voxel");
    }
    return home;
}

int SimulationDomain::voxel_index(const Vec3& p) const {
    int idx[3];
    for (int a = 0; a < 3; ++a) {
        const int n = shape_[a];
        if (n <= 1) {
            idx[a] = 0;
            continue;
        }
        int i = static_cast<int>(std::floor((p[a] - bmin_[a]) * inv_cell_[a]));
        idx[a] = i < 0 ? 0 : (i >= n ? n - 1 : i);
    }
    return (idx[0] * shape_[1] + idx[1]) * shape_[2] + idx[2];
}

// src/SimulationDomain.cpp:399-450 (analytic box branch)
void SimulationDomain::trace(const Vec3& p, const Vec3& v, Vec3& cp, double& t, int& facet) const {
    if (prism_) {
        prism_trace(p, v, cp, t, facet);
        return;
    }
    if (mesh_) {
        mesh_->trace(p, v, cp, t, facet);
        return;
    }
    constexpr double velocity_eps = 1e-18, time_eps = 1e-14;
    const Vec3 ext = sub3(bmax_, bmin_);
    const double scale = std::max({1.0, std::abs(ext[0]), std::abs(ext[1]), std::abs(ext[2])});
    const double tol = std::max(1e-9, 64.0 * std::numeric_limits<double>::epsilon() * scale);
    cp = p;
    t = std::numeric_limits<double>::infinity();
    facet = -1;
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(p[a]) || p[a] < bmin_[a] - tol || p[a] > bmax_[a] + tol) return;
    double best = std::numeric_limits<double>::infinity();
    int plane = -1;
    for (int a = 0; a < 3; ++a) {
        const double c = v[a];
        if (!std::isfinite(c) || std::abs(c) <= velocity_eps) continue;
        const int side = c > 0.0 ? 1 : 0;
        const double target = side ? bmax_[a] : bmin_[a];
        const double h = (target - p[a]) / c;
        if (std::isfinite(h) && h > time_eps && h < best) {
            best = h;
            plane = 2 * a + side;
        }
    }
    if (plane < 0) return;
    Vec3 c{p[0] + v[0] * best, p[1] + v[1] * best, p[2] + v[2] * best};
    const int ha = plane / 2;
    c[ha] = plane % 2 ? bmax_[ha] : bmin_[ha];
    for (int a = 0; a < 3; ++a) {
        if (!std::isfinite(c[a]) || c[a] < bmin_[a] - tol || c[a] > bmax_[a] + tol) return;
        c[a] = std::clamp(c[a], bmin_[a], bmax_[a]);
    }
    cp = c;
    t = best;
    facet = plane;
}

bool SimulationDomain::contains_point(const Vec3& p) const {
    // an extruded prism answers by the ray cast alone (include/SimulationDomain.h:43)
    if (mesh_) return prism_ ? mesh_->contains_point_ray_cast(p) : mesh_->contains_point(p);
    for (int a = 0; a < 3; ++a)
        if (!(p[a] >= bmin_[a] && p[a] <= bmax_[a])) return false;
    return true;
}

int SimulationDomain::nearest_facet(const Vec3& p) const {
    if (mesh_) return mesh_->nearest_facet(p);
    int best = -1;
    double bd = std::numeric_limits<double>::infinity();
    for (int f = 0; f < 6; ++f) {
        const int a = f / 2;
        const double d = std::abs(p[a] - (f % 2 ? bmax_[a] : bmin_[a]));
        if (d < bd) {
            bd = d;
            best = f;
        }
    }
    return best;
}

// ----------------------------------------------------------- rough tables
// src/solver/RoughBoundarySampler.cpp:77-368
// Specular match of every incoming mode of every job: the first outgoing
// mode of its window in frequency order that minimises
// |v_try - v_out| / max(1e-12, |v_try|, |v_out|), v_try the incoming velocity
// mirrored in the facet plane (src/solver/RoughBoundarySampler.cpp:286-310).
void spec_match_host(const std::vector<Vec3>& va, std::vector<SpecMatchJob>& jobs) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < static_cast<int>(jobs.size()); ++k) {
        const SpecMatchJob& J = jobs[k];
        for (int ai : *J.incoming) {
            const int ib = (*J.begin)[ai], ie = (*J.end)[ai];
            if (ib < 0 || ie <= ib) continue;
            const Vec3 vin = va[ai];
            const double vdn = dot3(vin, J.n_in);
            const Vec3 vtry = sub3(vin, mul3(J.n_in, 2.0 * vdn));
            int best = -1;
            double bm = std::numeric_limits<double>::infinity();
            for (int pos = ib; pos < ie; ++pos) {
                const int ao = (*J.sorted)[pos];
                const Vec3 dv = sub3(vtry, va[ao]);
                const double ref = std::max({1e-12, norm3(vtry), norm3(va[ao])});
                const double metric = norm3(dv) / ref;
                if (metric < bm) {
                    bm = metric;
                    best = ao;
                }
            }
            if (best >= 0) (*J.match)[ai] = best;
        }
    }
}

void RoughTables::build(const std::vector<const PhononMaterial*>& mats, const std::vector<Vec3>& normals,
                        const std::vector<double>& roughness, const std::vector<char>& enabled,
                        bool require_discrete, double Teq, const SpecMatchScan* scan) {
    // one facet's table between the preparation and the specular-match scan
    struct FacetWork {
        RoughTable rd;
        std::vector<int> incoming, outgoing;
        std::vector<double> destr, creat;
        Vec3 n_in{};
    };
    const int nf = static_cast<int>(normals.size());
    tables.clear();
    facet_table.assign(static_cast<size_t>(nf) * mats.size(), -1);
    int total = 0;
    for (char e : enabled) total += e ? 1 : 0;
    if (!total) return;
    for (size_t mid = 0; mid < mats.size(); ++mid) {
        const PhononMaterial& M = *mats[mid];
        const int na = M.active_mode_count();
        const auto& act = M.active_flat();
        std::vector<Vec3> va(na);
        std::vector<double> vn(na), wa(na), kn(na), dw(na);
        for (int i = 0; i < na; ++i) {
            va[i] = M.velocity(act[i]);
            vn[i] = norm3(va[i]);
            wa[i] = M.omega(act[i]);
            kn[i] = M.wavevector_norm(act[i]);
            dw[i] = M.frequency_window(act[i]);
        }
        std::vector<int> shell(na), order(na);
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int a, int b) { return wa[a] < wa[b]; });
        int shells = 0;
        double sf = -1;
        for (int ai : order) {
            if (sf < 0 || wa[ai] - sf > 1e-8 * std::max(sf, 1e-12)) {
                ++shells;
                sf = wa[ai];
            }
            shell[ai] = shells - 1;
        }
        auto prepare = [&](int f) {
            RoughTable rd;
            rd.facet = f;
            rd.material = static_cast<int>(mid);
            rd.strict_elastic = Teq > 0;
            rd.specularity.assign(na, 0.0);
            rd.spec_match.assign(na, -1);
            rd.diffuse_begin.assign(na, -1);
            rd.diffuse_end.assign(na, -1);
            const double eta = std::max(0.0, roughness[f]);
            const Vec3 nin = mul3(normals[f], -1.0);
            std::vector<int> incoming, outgoing;
            std::vector<double> destr(na, 0.0), creat(na, 0.0);
            for (int ai = 0; ai < na; ++ai) {
                const double v = dot3(va[ai], nin);
                if (v < 0.0) {
                    incoming.push_back(ai);
                    destr[ai] = -v;
                } else if (v > 0.0) {
                    outgoing.push_back(ai);
                    creat[ai] = v;
                }
                const double vnorm = std::max(1e-12, vn[ai]);
                const double cosi = std::abs(v) / vnorm;
                const double x = rd.strict_elastic ? 2 * eta * std::abs(dot3(M.wavevector(act[ai]), nin))
                                                   : 2.0 * eta * cosi * kn[ai];
                double p = std::exp(-(x * x));
                if (!std::isfinite(p)) p = 0.0;
                rd.specularity[ai] = v < 0.0 ? std::clamp(p, 0.0, 1.0) : 0.0;
                if (rd.strict_elastic) {
                    const double c = M.mode_heat_capacity(Teq, act[ai]);
                    destr[ai] *= c;
                    creat[ai] *= c;
                }
            }
            if (require_discrete && !incoming.empty() && outgoing.empty())
                throw std::invalid_argument("Full-matrix reflecting facet " + std::to_string(f) +
                                            " has incoming modes but no inward outgoing material mode for material " +
                                            std::to_string(mid) + ". Supply a complete full-Brillouin-zone mode bank.");
            rd.outgoing_active = outgoing;
            rd.outgoing_sorted = outgoing;
            std::sort(rd.outgoing_sorted.begin(), rd.outgoing_sorted.end(),
                      [&](int a, int b) { return wa[a] < wa[b]; });
            rd.outgoing_sorted_omega.resize(rd.outgoing_sorted.size());
            for (size_t k = 0; k < rd.outgoing_sorted.size(); ++k) rd.outgoing_sorted_omega[k] = wa[rd.outgoing_sorted[k]];
            std::vector<int> sb(shells, -1), se(shells, -1);
            if (rd.strict_elastic) {
                std::vector<double> inf(shells, 0), outf(shells, 0);
                for (int ai : incoming) inf[shell[ai]] += destr[ai];
                for (int ao : outgoing) outf[shell[ao]] += creat[ao];
                const double resolved = std::max(*std::max_element(inf.begin(), inf.end()),
                                                 *std::max_element(outf.begin(), outf.end()));
                const double roundoff = 64 * std::numeric_limits<double>::epsilon() * resolved;
                for (int s = 0; s < shells; ++s)
                    if (std::abs(inf[s] - outf[s]) > 1e-7 * std::max(inf[s], outf[s]) + roundoff)
                        throw std::invalid_argument("Callaway reflecting boundary lacks balanced equal-frequency "
                                                    "incoming/outgoing flux. Check full-BZ material symmetry and velocities.");
                for (int pos = 0; pos < static_cast<int>(rd.outgoing_sorted.size()); ++pos) {
                    const int s = shell[rd.outgoing_sorted[pos]];
                    if (sb[s] < 0) sb[s] = pos;
                    se[s] = pos + 1;
                }
            }
            for (int ai : incoming) {
                if (rd.outgoing_sorted.empty()) continue;
                const double win = wa[ai];
                const double tol = std::max(1e-12, dw[ai]);
                const auto lo = std::lower_bound(rd.outgoing_sorted_omega.begin(), rd.outgoing_sorted_omega.end(), win - tol);
                const auto hi = std::upper_bound(rd.outgoing_sorted_omega.begin(), rd.outgoing_sorted_omega.end(), win + tol);
                const int ib = rd.strict_elastic ? sb[shell[ai]] : static_cast<int>(lo - rd.outgoing_sorted_omega.begin());
                const int ie = rd.strict_elastic ? se[shell[ai]] : static_cast<int>(hi - rd.outgoing_sorted_omega.begin());
                if (ie <= ib) continue;
                rd.diffuse_begin[ai] = ib;
                rd.diffuse_end[ai] = ie;
            }
            return FacetWork{std::move(rd), std::move(incoming), std::move(outgoing), std::move(destr),
                             std::move(creat), nin};
        };
        // the rest of a table once its specular matches are known
        auto finish = [&](FacetWork& fw) {
            RoughTable& rd = fw.rd;
            const std::vector<int>& incoming = fw.incoming;
            const std::vector<int>& outgoing = fw.outgoing;
            const std::vector<double>& destr = fw.destr;
            const std::vector<double>& creat = fw.creat;
            for (int ai : incoming)
                if (rd.spec_match[ai] < 0) rd.specularity[ai] = 0.0;
            if (rd.strict_elastic) {
                std::vector<double> assigned(na, 0);
                for (int ai : incoming)
                    if (rd.spec_match[ai] >= 0) assigned[rd.spec_match[ai]] += destr[ai] * rd.specularity[ai];
                for (int ai : incoming) {
                    const int ao = rd.spec_match[ai];
                    if (ao >= 0 && assigned[ao] > creat[ao]) rd.specularity[ai] *= creat[ao] / assigned[ao];
                }
            }
            // residual diffuse creation rates (include/solver/BoundaryFluxSampling.h:16-42)
            std::vector<double> residual = creat;
            for (int in = 0; in < na; ++in) {
                const int out = rd.spec_match[in];
                if (out < 0 || out >= na) continue;
                const double flux = destr[in], prob = rd.specularity[in];
                if (!std::isfinite(flux) || !std::isfinite(prob) || flux <= 0.0 || prob <= 0.0) continue;
                residual[out] -= flux * std::clamp(prob, 0.0, 1.0);
            }
            for (double& r : residual)
                if (!std::isfinite(r) || r < 0.0) r = 0.0;
            double rate_sum = 0.0;
            for (int ao : outgoing) rate_sum += residual[ao];
            rd.residual_prefix.assign(rd.outgoing_sorted.size() + 1, 0.0);
            for (size_t i = 0; i < rd.outgoing_sorted.size(); ++i) {
                double w = residual[rd.outgoing_sorted[i]];
                if (!std::isfinite(w) || w < 0.0) w = 0.0;
                rd.residual_prefix[i + 1] = rd.residual_prefix[i] + w;
            }
            if (rate_sum > 0.0) {
                double cdf = 0.0;
                for (int ao : outgoing) {
                    const double r = residual[ao];
                    if (r <= 0.0) continue;
                    cdf += r;
                    rd.roulette_active.push_back(ao);
                    rd.roulette_cdf.push_back(cdf);
                }
            }
        };
        // Tables of different facets are independent: prepared in parallel,
        // their specular matches scanned (host loop, or the caller's scan),
        // finished in parallel and stored in facet order.
        std::vector<int> todo;
        for (int f = 0; f < nf; ++f)
            if (enabled[f]) todo.push_back(f);
        std::vector<FacetWork> work(todo.size());
        std::vector<std::string> errors(todo.size());
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k < static_cast<int>(todo.size()); ++k) {
            try {
                work[k] = prepare(todo[k]);
            } catch (const std::exception& e) {
                errors[k] = e.what();
            }
        }
        for (size_t k = 0; k < todo.size(); ++k)
            if (!errors[k].empty()) throw std::invalid_argument(errors[k]);
        std::vector<SpecMatchJob> jobs(work.size());
        for (size_t k = 0; k < work.size(); ++k)
            jobs[k] = SpecMatchJob{work[k].n_in, &work[k].incoming, &work[k].rd.diffuse_begin,
                                   &work[k].rd.diffuse_end, &work[k].rd.outgoing_sorted, &work[k].rd.spec_match};
        if (scan && *scan) (*scan)(va, jobs);
        else spec_match_host(va, jobs);
#pragma omp parallel for schedule(dynamic, 1)
        for (int k = 0; k < static_cast<int>(work.size()); ++k) finish(work[k]);
        for (size_t k = 0; k < todo.size(); ++k) {
            facet_table[mid * nf + todo[k]] = static_cast<int>(tables.size());
            tables.push_back(std::move(work[k].rd));
        }
    }
}

// ---------------------------------------------------------------- ledger
// src/solver/EnergyLedger.cpp:58-90 (same evaluation order of the residual).
void EnergyLedger::finish_step(double energy, const BoundaryBalance& b) {
    const double residual = energy - thermal_ - step_.source_energy_ev - step_.drive_energy_ev -
                            b.injected_energy_ev + b.absorbed_energy_ev - step_.lifetime_residual_ev;
    if (!std::isfinite(residual)) throw std::invalid_argument("Non-finite energy ledger input.");
    step_.balance_residual_ev = residual;
    total_.source_updates += step_.source_updates;
    total_.source_energy_ev += step_.source_energy_ev;
    total_.lifetime_residual_ev += step_.lifetime_residual_ev;
    total_.balance_residual_ev += step_.balance_residual_ev;
    total_.drive_updates += step_.drive_updates;
    total_.drive_energy_ev += step_.drive_energy_ev;
    thermal_ = energy;
}

// ---------------------------------------------------------------- problem
// ------------------------------------------------------- heat source
// src/config/ConfigValidation.cpp:196-290 (the rules the carrier loop relies on).
int resolved_sort_interval(const SimulationConfig& c, bool mixed) {
    if (c.carrier_sort_interval < 0) return 0;
    if (c.carrier_sort_interval > 0) return c.carrier_sort_interval;
    if (c.particle_count < tuning::kSortMinCarriers) return 0;
    return c.model != "box" ? tuning::kSortIntervalMesh[mixed ? 1 : 0] : tuning::kSortInterval[mixed ? 1 : 0];
}

void validate_heat_source_config(const SimulationConfig& c) {
    if (!c.heat_source_enabled) return;
    if (c.heat_source_total_power) {
        if (!std::isfinite(*c.heat_source_total_power) || !(*c.heat_source_total_power > 0.0))
            throw std::runtime_error("heat_source.total_power must be finite and positive (W).");
        if (c.heat_source_power_density != 0.0 || !c.heat_source_power_densities.empty())
            throw std::runtime_error("heat_source.total_power cannot be combined with power_density or power_densities.");
    } else if (!(c.heat_source_power_density > 0.0) || !std::isfinite(c.heat_source_power_density)) {
        throw std::runtime_error("enabled heat_source requires positive total_power or power_density.");
    }
    for (const auto* v : {&c.heat_source_min, &c.heat_source_max, &c.heat_source_center, &c.heat_source_centers,
                          &c.heat_source_sigma, &c.heat_source_half_width})
        for (double x : *v)
            if (!std::isfinite(x)) throw std::runtime_error("Heat-source spatial parameters must be finite.");
    std::vector<int> br = c.heat_source_branches;
    std::sort(br.begin(), br.end());
    if ((!br.empty() && br.front() < 0) || std::adjacent_find(br.begin(), br.end()) != br.end())
        throw std::runtime_error("heat_source.branches must contain unique nonnegative indices.");
    if (c.heat_source_spectrum == HeatSourceSpectrum::Gaussian) {
        if (!c.heat_source_frequency_center || !c.heat_source_frequency_sigma ||
            !std::isfinite(*c.heat_source_frequency_center) || *c.heat_source_frequency_center < 0 ||
            !std::isfinite(*c.heat_source_frequency_sigma) || *c.heat_source_frequency_sigma <= 0)
            throw std::runtime_error("Gaussian spectrum requires finite frequency_center >= 0 and frequency_sigma > 0, in THz.");
    } else if (c.heat_source_frequency_center || c.heat_source_frequency_sigma) {
        throw std::runtime_error("frequency_center/frequency_sigma require heat_source.spectrum='gaussian'.");
    }
    if (c.heat_source_spectrum != HeatSourceSpectrum::Weighted) {
        if (!c.heat_source_branch_weights.empty())
            throw std::runtime_error("branch_weights requires heat_source.spectrum='weighted'.");
    } else {
        bool positive = false;
        for (size_t b = 0; b < c.heat_source_branch_weights.size(); ++b) {
            const double w = c.heat_source_branch_weights[b];
            if (!std::isfinite(w) || w < 0.0) throw std::runtime_error("heat_source.branch_weights must be finite and nonnegative.");
            if (br.empty() || std::binary_search(br.begin(), br.end(), static_cast<int>(b))) positive = positive || w > 0.0;
        }
        if (!positive) throw std::runtime_error("weighted heat_source needs positive weights on selected branches.");
    }
    for (double q : c.heat_source_power_densities)
        if (!(q > 0.0) || !std::isfinite(q)) throw std::runtime_error("heat_source.power_densities values must be finite and positive.");
    for (double f : {c.heat_source_frequency_min, c.heat_source_frequency_max})
        if (!(f < 0.0) && !std::isfinite(f)) throw std::runtime_error("heat_source frequency cutoffs must be finite.");
    if (c.heat_source_time_profile == HeatSourceTimeProfile::Pulsed &&
        (!(c.heat_source_period > 0.0) || !std::isfinite(c.heat_source_period)))
        throw std::runtime_error("Pulsed heat source requires a positive period.");
    if (!std::isfinite(c.heat_source_amplitude) || c.heat_source_amplitude < 0.0)
        throw std::runtime_error("heat_source.amplitude must be finite and nonnegative.");
}

// src/solver/HeatSourceDriving.cpp:12-44
double heat_source_time_factor(const SimulationConfig& c, double begin_ps, double end_ps) {
    const double begin = std::max(begin_ps, c.heat_source_time_start);
    const double end = c.heat_source_time_end >= 0.0 ? std::min(end_ps, c.heat_source_time_end) : end_ps;
    if (end <= begin) return 0.0;
    if (c.heat_source_time_profile == HeatSourceTimeProfile::Constant) return c.heat_source_amplitude * (end - begin);
    const double period = c.heat_source_period;
    const double on = c.heat_source_on_duration < 0.0 ? c.heat_source_duty_cycle * period : c.heat_source_on_duration;
    if (on <= 0.0) return 0.0;
    auto on_time = [&](double rel) {
        if (!(rel > 0.0)) return 0.0;
        const double cycles = std::floor(rel / period);
        return cycles * on + std::min(rel - cycles * period, on);
    };
    const double rb = begin - c.heat_source_time_start, re = end - c.heat_source_time_start;
    return c.heat_source_amplitude * std::max(0.0, on_time(re) - on_time(rb));
}

// src/solver/PrescribedHeatSource.cpp:22-216: cell weights from the grid
// centres (uniform box, or Gaussian sources cut at 2 sigma per axis with an
// optional clip box and top-hat axes), then cell power from the density or the
// total power.
void HeatSourceTables::configure(const SimulationConfig& c, const SimulationDomain& domain) {
    *this = HeatSourceTables{};
    if (!c.heat_source_enabled) return;
    validate_heat_source_config(c);
    const double density = c.heat_source_total_power ? 1.0 : c.heat_source_power_density;
    const auto& centers = domain.grid_centers();
    std::vector<double> w(centers.size(), 0.0);
    int selected = 0;
    if (c.heat_source_profile == HeatSourceProfile::Uniform) {
        if (c.heat_source_min.size() != 3 || c.heat_source_max.size() != 3)
            throw std::runtime_error("uniform heat source requires min/max 3D vectors.");
        Vec3 lo{c.heat_source_min[0], c.heat_source_min[1], c.heat_source_min[2]};
        Vec3 hi{c.heat_source_max[0], c.heat_source_max[1], c.heat_source_max[2]};
        for (int k = 0; k < 3; ++k)
            if (lo[k] > hi[k]) std::swap(lo[k], hi[k]);
        for (size_t i = 0; i < centers.size(); ++i) {
            const Vec3& x = centers[i];
            if (x[0] >= lo[0] && x[0] <= hi[0] && x[1] >= lo[1] && x[1] <= hi[1] && x[2] >= lo[2] && x[2] <= hi[2]) {
                w[i] = 1.0;
                ++selected;
            }
        }
        if (!selected) throw std::runtime_error("uniform heat source region does not include any grid center.");
    } else {
        if ((c.heat_source_center.size() != 3 && c.heat_source_centers.empty()) || c.heat_source_sigma.size() != 3 ||
            (!c.heat_source_centers.empty() && c.heat_source_centers.size() % 3 != 0))
            throw std::runtime_error("gaussian heat source requires center=[x,y,z] or centers=[[x,y,z],...] and "
                                     "sigma=[sx,sy,sz].");
        std::vector<Vec3> src;
        if (!c.heat_source_centers.empty())
            for (size_t j = 0; j + 2 < c.heat_source_centers.size(); j += 3)
                src.push_back({c.heat_source_centers[j], c.heat_source_centers[j + 1], c.heat_source_centers[j + 2]});
        else
            src.push_back({c.heat_source_center[0], c.heat_source_center[1], c.heat_source_center[2]});
        std::vector<double> peak(src.size(), 1.0);
        if (!c.heat_source_power_densities.empty()) {
            if (c.heat_source_power_densities.size() != src.size())
                throw std::runtime_error("heat_source.power_densities size does not match heat_source.centers.");
            for (size_t j = 0; j < src.size(); ++j) peak[j] = c.heat_source_power_densities[j] / density;
        }
        const bool clip = c.heat_source_min.size() == 3 && c.heat_source_max.size() == 3;
        Vec3 lo{0, 0, 0}, hi{0, 0, 0}, sigma{1, 1, 1}, half{};
        std::array<bool, 3> gauss{true, true, true};
        for (int k = 0; k < 3; ++k) {
            if (clip) {
                lo[k] = std::min(c.heat_source_min[k], c.heat_source_max[k]);
                hi[k] = std::max(c.heat_source_min[k], c.heat_source_max[k]);
            }
            half[k] = std::numeric_limits<double>::infinity();
            if (c.heat_source_half_width.size() == 3 && std::isfinite(c.heat_source_half_width[k]) &&
                c.heat_source_half_width[k] > 0.0)
                half[k] = c.heat_source_half_width[k];
            else if (!c.heat_source_half_width.empty() && c.heat_source_half_width.size() != 3)
                throw std::runtime_error("heat_source.half_width must contain 3 values.");
            const double sk = c.heat_source_sigma[k];
            gauss[k] = std::isfinite(sk) && sk > 0.0;
            sigma[k] = gauss[k] ? std::max(1e-12, sk) : 1.0;
        }
        for (size_t i = 0; i < centers.size(); ++i) {
            const Vec3& x = centers[i];
            bool cut = false;
            if (clip)
                for (int k = 0; k < 3 && !cut; ++k) cut = x[k] < lo[k] || x[k] > hi[k];
            if (cut) continue;
            double sum = 0.0;
            for (size_t j = 0; j < src.size(); ++j) {
                double r2 = 0.0;
                bool outside = false;
                for (int k = 0; k < 3 && !outside; ++k) {
                    if (gauss[k]) {
                        const double u = std::abs(x[k] - src[j][k]) / sigma[k];
                        if (u > 2.0) outside = true;
                        else r2 += u * u;
                    } else if (std::isfinite(half[k]) && std::abs(x[k] - src[j][k]) > half[k]) {
                        outside = true;
                    }
                }
                if (!outside) sum += peak[j] * std::exp(-0.5 * r2);
            }
            if (sum > 0.0) {
                w[i] = sum;
                ++selected;
            }
        }
        if (!selected) throw std::runtime_error("gaussian heat source cannot be applied because grid is empty.");
    }
    const auto& vol = domain.grid_volumes();
    double weighted = 0.0;
    for (size_t i = 0; i < w.size(); ++i) weighted += w[i] * vol[i];
    if (!(weighted > 0.0) || !std::isfinite(weighted))
        throw std::runtime_error("Heat source has no finite positive sampled volume; refine the grid or source region.");
    rates.resize(w.size());
    for (size_t i = 0; i < w.size(); ++i) {
        rates[i] = c.heat_source_total_power ? *c.heat_source_total_power * 6.241509074e6 * (w[i] * vol[i] / weighted)
                                             : density * 6.241509074e-24 * w[i] * vol[i];
        if (!std::isfinite(rates[i]) || rates[i] < 0.0) throw std::runtime_error("Non-finite heat-source cell power.");
    }
    double total = 0.0;
    for (double r : rates) total += r;
    if (!std::isfinite(total) || !(total > 0.0))
        throw std::runtime_error("Total heat-source rate must be finite and representably positive.");
    set_spectrum(c);
    enabled = true;
}

// src/solver/PhononSourceOperator.cpp:20-40
void HeatSourceTables::set_spectrum(const SimulationConfig& c) {
    spectrum = c.heat_source_spectrum;
    linearized_thermal = uses_linearized_transport(c);
    frequency_min = c.heat_source_frequency_min;
    frequency_max = c.heat_source_frequency_max;
    branches = c.heat_source_branches;
    weights = c.heat_source_branch_weights;
    if (!weights.empty()) {
        const double top = *std::max_element(weights.begin(), weights.end());
        for (double& x : weights) x /= top;
    }
    gaussian_center = c.heat_source_frequency_center.value_or(0);
    gaussian_sigma = c.heat_source_frequency_sigma.value_or(1);
}

// src/solver/PhononSourceOperator.cpp:102-117
double HeatSourceTables::mode_weight(const PhononMaterial& m, int flat) const {
    constexpr double two_pi = 6.283185307179586476925286766559;
    const double f = m.omega(flat) / two_pi;
    if (!std::isfinite(f) || (frequency_min >= 0.0 && f < frequency_min) || (frequency_max >= 0.0 && f > frequency_max))
        return 0.0;
    const int branch = flat % m.branch_count();
    if (!branches.empty() && std::find(branches.begin(), branches.end(), branch) == branches.end()) return 0.0;
    return spectrum == HeatSourceSpectrum::Weighted ? weights.at(static_cast<size_t>(branch)) : 1.0;
}

// src/solver/InterfaceModeSampler.cpp:11-44
void InterfaceTables::build(const std::vector<const PhononMaterial*>& mats, int ax) {
    axis = ax;
    banks.assign(mats.size(), {});
    for (size_t mid = 0; mid < mats.size(); ++mid) {
        const PhononMaterial& M = *mats[mid];
        const auto& act = M.active_flat();
        for (int direction = 0; direction < 2; ++direction) {
            InterfaceBank& B = banks[mid][direction];
            std::vector<std::pair<double, int>> ordered;
            for (int a = 0; a < static_cast<int>(act.size()); ++a) {
                const double c = M.velocity(act[a])[axis];
                if ((direction == 0 && c < 0.0) || (direction == 1 && c > 0.0)) ordered.push_back({M.omega(act[a]), a});
            }
            std::sort(ordered.begin(), ordered.end());
            B.prefix.assign(ordered.size() + 1, 0.0);
            for (size_t i = 0; i < ordered.size(); ++i) {
                B.omega.push_back(ordered[i].first);
                B.active.push_back(ordered[i].second);
                const double flux = std::abs(M.velocity(act[ordered[i].second])[axis]) / M.energy_density_normalization();
                B.prefix[i + 1] = B.prefix[i] + flux;
            }
        }
    }
}

// src/solver/LayeredMaterialLayout.cpp:62-114: planes inside the box on cell
// boundaries, every layer with a cell, reservoirs normal to the layout axis,
// no periodic pair across it.
static void validate_layout(Problem& P, const SimulationConfig& cfg, const SimulationDomain& domain, int count) {
    const int axis = P.layout.axis;
    if (axis < 0 || axis > 2) throw std::invalid_argument("Invalid layered material count, axis or interface count.");
    for (size_t i = 0; i < P.layout.planes.size(); ++i)
        if (!std::isfinite(P.layout.planes[i]) || (i && P.layout.planes[i] <= P.layout.planes[i - 1]))
            throw std::invalid_argument("Material interface positions must be finite and strictly increasing.");
    const int cells = domain.grid_shape()[axis];
    const double lo = domain.bounds_min()[axis], hi = domain.bounds_max()[axis];
    const double width = (hi - lo) / cells;
    const double tol = std::max(1e-10, 1e-10 * std::abs(hi - lo));
    P.plane_cell.clear();
    for (double plane : P.layout.planes) {
        if (!std::isfinite(plane) || !(plane > lo) || !(plane < hi))
            throw std::runtime_error("Each material interface must lie strictly inside the loaded geometry bounds.");
        const double cc = (plane - lo) / width;
        if (std::abs(cc - std::round(cc)) > tol / width)
            throw std::runtime_error("Each materials.interface_positions value must coincide with a grid-cell boundary.");
        P.plane_cell.push_back(static_cast<int>(std::llround(cc)));
    }
    std::vector<bool> occupied(count, false);
    for (int id : P.cell_material) occupied.at(id) = true;
    for (bool o : occupied)
        if (!o) throw std::runtime_error("Every material layer must contain at least one active geometry cell.");
    for (const auto& F : domain.facets()) {
        if (F.condition == 'P' && std::abs(F.normal[axis]) > 0.99)
            throw std::runtime_error("Periodic boundaries normal to materials.interface_axis are not supported, "
                                     "because they would join different end materials.");
        if (F.condition == 'T' && std::abs(F.normal[axis]) < 0.99)
            throw std::runtime_error("In the layered-material model, thermal-reservoir facets must be normal to "
                                     "materials.interface_axis so each reservoir touches one material.");
    }
    if (!std::isfinite(cfg.material_interface_frequency_bin_thz) || cfg.material_interface_frequency_bin_thz <= 0)
        throw std::runtime_error("Interface frequency bin must be finite and positive.");
}

Problem build_problem(const SimulationConfig& cfg, SimulationDomain& domain,
                      const std::vector<const PhononMaterial*>& mats, const SpecMatchScan* scan) {
    if (mats.empty()) throw std::runtime_error("MonteCarloSolver requires at least one material.");
    if (!std::isfinite(cfg.time_step) || cfg.time_step <= 0) throw std::invalid_argument("time_step must be positive");
    Problem P;
    P.cfg = cfg;
    P.domain = &domain;
    // src/config/ConfigValidation.cpp:349-354
    if (cfg.callaway_nonlinear && (cfg.collision_model != CollisionModel::Callaway || cfg.temperature_gradient))
        throw std::runtime_error("Nonlinear Callaway requires model=callaway and finite-domain thermal driving");
    P.linearized = uses_linearized_transport(cfg);
    P.conservative = uses_conservative_transport(cfg);
    P.callaway_nonlinear = cfg.callaway_nonlinear;
    P.one_to_one = !(P.conservative || mats.size() > 1);
    P.initial_particles = static_cast<int>(std::llround(cfg.particle_count));
    if (P.initial_particles <= 0) throw std::invalid_argument("particle_count must be positive");
    P.push_eps = 1e-10 * std::max(cfg.time_step, 1.0);
    P.particle_volume = domain.volume() / static_cast<double>(P.initial_particles);
    const double Tbg = cfg.background_temperature;
    P.layout.axis = cfg.material_interface_axis;
    P.layout.planes = cfg.material_interface_positions;
    if (P.layout.planes.size() + 1 != mats.size())
        throw std::runtime_error("Layered materials require one interface plane fewer than materials.");
    P.cell_material.resize(domain.grid_count());
    for (int c = 0; c < domain.grid_count(); ++c) P.cell_material[c] = P.layout.material_at(domain.grid_centers()[c]);
    if (mats.size() > 1) validate_layout(P, cfg, domain, static_cast<int>(mats.size()));
    // Carrier volumes (src/MonteCarloSolver.cpp:80-100): one volume V/N for a
    // single material; layered crystals sample carriers in proportion to each
    // material's active-state density with one common state weight, so a
    // carrier of material m stands for common / density_m of space.
    P.material_spatial_volume.assign(mats.size(), P.particle_volume);
    if (mats.size() > 1) {
        std::vector<double> density(mats.size());
        for (size_t m = 0; m < mats.size(); ++m)
            density[m] = mats[m]->active_mode_count() / mats[m]->energy_density_normalization();
        double states = 0.0;
        for (int c = 0; c < domain.grid_count(); ++c) states += domain.grid_volumes()[c] * density[P.cell_material[c]];
        const double common = states / P.initial_particles;
        for (size_t m = 0; m < mats.size(); ++m) {
            if (!(density[m] > 0.0) || !std::isfinite(density[m]))
                throw std::runtime_error("Invalid material phase-space density.");
            P.material_spatial_volume[m] = common / density[m];
        }
    }

    int axis = 0;
    if (cfg.transport_axis >= 0) axis = cfg.transport_axis;
    else {
        const int nx = cfg.grid[0], ny = cfg.grid[1], nz = cfg.grid[2];
        if (ny > nx && ny >= nz) axis = 1;
        else if (nz > nx && nz > ny) axis = 2;
    }
    P.kappa_axis = axis;

    // Heat source (src/solver/HeatSourceDriving.cpp:8-11).
    P.source.configure(cfg, domain);
    if (P.source.enabled)
        for (const PhononMaterial* m : mats)
            for (int b : P.source.branches)
                if (b >= m->branch_count())
                    throw std::invalid_argument("heat_source.branches index exceeds a material's branch count.");
    if (P.source.enabled && P.source.spectrum == HeatSourceSpectrum::Weighted)
        for (const PhononMaterial* m : mats)
            if (P.source.weights.size() != static_cast<size_t>(m->branch_count()))
                throw std::invalid_argument("heat_source.branch_weights must match each material's branch count.");

    for (size_t mid = 0; mid < mats.size(); ++mid) {
        const PhononMaterial& M = *mats[mid];
        MaterialTables T;
        T.n_active = M.active_mode_count();
        T.active_flat = M.active_flat();
        const int na = T.n_active;
        T.omega.resize(na);
        T.hw.resize(na);
        T.vel.resize(3 * na);
        T.nbg.resize(na);
        T.capacity_bg.resize(na);
        for (int a = 0; a < na; ++a) {
            const int f = T.active_flat[a];
            T.omega[a] = M.omega(f);
            T.hw[a] = kHbarEvPs * M.omega(f);
            for (int k = 0; k < 3; ++k) T.vel[3 * a + k] = M.velocity(f)[k];
            T.nbg[a] = M.bose_occupation(Tbg, f);
            T.capacity_bg[a] = M.mode_heat_capacity(Tbg, f);
        }
        // BackgroundCache (include/solver/BackgroundCache.h:13-31)
        T.energy_weight = static_cast<double>(na) * P.material_spatial_volume[mid] / M.energy_density_normalization();
        T.energy_density_bg = P.linearized ? M.crystal_energy_density(Tbg) : M.energy_density_from_temperature(Tbg);
        T.heat_capacity_density_bg = 0.0;
        for (int f = 0; f < M.flat_count(); ++f)
            T.heat_capacity_density_bg += M.mode_heat_capacity(Tbg, f) / M.energy_density_normalization();
        T.zero_point = M.zero_point_energy_density();
        T.lookup_T = M.lookup_T();
        T.lookup_E = M.lookup_E();
        T.temperatures = M.temperature_samples();
        const size_t nT = T.temperatures.size();
        const size_t nm = static_cast<size_t>(M.flat_count());
        T.gamma_active.resize(nT * na);
        for (size_t it = 0; it < nT; ++it)
            for (int a = 0; a < na; ++a) T.gamma_active[it * na + a] = M.gamma_total()[it * nm + T.active_flat[a]];
        T.relax_fixed.resize(na);
        for (int a = 0; a < na; ++a)
            T.relax_fixed[a] = M.mode_relaxation_weight(cfg.lifetime_temperature, T.active_flat[a], cfg.time_step);
        if (P.callaway_nonlinear) {
            // src/solver/NonlinearCallawayCollision.cpp:250-263: the reference's
            // configure() validates the N/U data at the background temperature
            const CallawayData d = M.callaway_data(Tbg);
            T.col_k.resize(3 * na);
            for (int a = 0; a < na; ++a)
                for (int k = 0; k < 3; ++k) T.col_k[3 * a + k] = d.wavevector[a][k];
            auto active_rows = [&](const std::vector<double>& g) {
                std::vector<double> out(g.empty() ? 0 : nT * na);
                for (size_t it = 0; it < nT && !g.empty(); ++it)
                    for (int a = 0; a < na; ++a) out[it * na + a] = g[it * nm + T.active_flat[a]];
                return out;
            };
            T.ncl_gamma_n = active_rows(M.gamma_normal());
            T.ncl_gamma_u = active_rows(M.gamma_umklapp());
            T.ncl_gamma_x = active_rows(M.gamma_extra());
        }
        if (P.linearized) {
            const CallawayData d = cfg.collision_model == CollisionModel::Callaway ? M.callaway_data(Tbg)
                                                                                   : M.linearized_rta_data(Tbg);
            T.col_capacity = d.capacity;
            T.col_normal = d.normal_rate;
            T.col_resistive = d.resistive_rate;
            T.col_k.resize(3 * na);
            for (int a = 0; a < na; ++a)
                for (int k = 0; k < 3; ++k) T.col_k[3 * a + k] = d.wavevector[a][k];
        }
        // Mode classes: identical omega and identical linewidth row.
        std::vector<int> order(na);
        std::iota(order.begin(), order.end(), 0);
        // with a heat source, modes of one class must also share its spectral weight
        std::vector<double> sw(na, 0.0);
        if (P.source.enabled)
            for (int a = 0; a < na; ++a) sw[a] = P.source.mode_weight(M, T.active_flat[a]);
        auto key_less = [&](int a, int b) {
            if (T.omega[a] != T.omega[b]) return T.omega[a] < T.omega[b];
            if (sw[a] != sw[b]) return sw[a] < sw[b];
            for (size_t it = 0; it < nT; ++it) {
                const double ga = T.gamma_active[it * na + a], gb = T.gamma_active[it * na + b];
                if (ga != gb) return ga < gb;
            }
            return false;
        };
        std::stable_sort(order.begin(), order.end(), key_less);
        T.mode_class.assign(na, -1);
        for (size_t i = 0; i < order.size(); ++i) {
            const int a = order[i];
            if (i == 0 || key_less(order[i - 1], a)) {
                T.class_rep.push_back(a);
                T.class_omega.push_back(T.omega[a]);
                T.class_hw.push_back(T.hw[a]);
            }
            T.mode_class[a] = static_cast<int>(T.class_rep.size()) - 1;
        }
        T.n_classes = static_cast<int>(T.class_rep.size());
        P.mats.push_back(std::move(T));
    }

    // Gradient drive (src/solver/TemperatureGradientDrive.cpp:13-86).
    if (cfg.temperature_gradient) {
        if (mats.size() != 1) throw std::runtime_error("Gradient driving requires one material.");
        if (!domain.reservoir_facets().empty())
            throw std::invalid_argument("Temperature-gradient driving requires a periodic box without reservoirs.");
        int paired = 0;
        for (const auto& F : domain.facets()) {
            if (std::abs(F.normal[axis]) > 1e-8) {
                if (F.condition != 'P' || F.pair < 0)
                    throw std::invalid_argument("Temperature-gradient direction must have paired periodic boundaries.");
                ++paired;
            }
        }
        if (paired < 2) throw std::invalid_argument("Missing periodic boundaries along the imposed gradient.");
        const PhononMaterial& M = *mats[0];
        MaterialTables& T = P.mats[0];
        std::vector<double> cap(T.n_active);
        long double sum = 0, absolute = 0, total_c = 0;
        T.grad_rate.resize(T.n_active);
        for (int a = 0; a < T.n_active; ++a) {
            const double c = M.mode_heat_capacity(Tbg, T.active_flat[a]);
            const double rate = -c * M.velocity(T.active_flat[a])[axis] * 1e-10 * (*cfg.temperature_gradient);
            if (!(c > 0) || !std::isfinite(rate)) throw std::invalid_argument("Invalid gradient source mode.");
            cap[a] = c;
            T.grad_rate[a] = rate;
            sum += rate;
            absolute += std::abs(rate);
            total_c += c;
        }
        if (std::abs(sum) > 1e-8L * absolute)
            throw std::invalid_argument("Gradient source has nonzero net energy: supply a balanced full-BZ "
                                        "velocity/capacity bank.");
        for (int a = 0; a < T.n_active; ++a) T.grad_rate[a] -= static_cast<double>(sum * cap[a] / total_c);
        P.gradient_energy_weight = T.n_active * P.particle_volume / M.energy_density_normalization();
    }

    // Rough tables (src/solver/RoughBoundaryInitialization.cpp:1-26).
    std::vector<Vec3> normals;
    std::vector<double> rough;
    std::vector<char> enabled;
    for (const auto& F : domain.facets()) {
        normals.push_back(F.normal);
        rough.push_back(F.condition == 'R' ? std::max(0.0, F.value) : 0.0);
        const bool reflecting = F.condition != 'T' && !(F.condition == 'P' && F.pair >= 0);
        enabled.push_back(P.conservative ? reflecting : F.condition == 'R');
    }
    P.rough.build(mats, normals, rough, enabled, P.conservative, P.conservative ? Tbg : 0.0, scan);

    // Interface banks (src/solver/InterfaceInitialization.cpp:3-15, InterfaceInteraction.cpp:11-41).
    P.iface.enabled = mats.size() > 1;
    P.iface.linearized = P.linearized;
    P.iface.reference_temperature = Tbg;
    P.iface.band_width = 2.0 * std::acos(-1.0) * cfg.material_interface_frequency_bin_thz;
    // materials.interface_model checks of src/config/ConfigValidation.cpp:109-140
    const int model = cfg.material_interface_model;
    const double fraction = model == 1 ? 1.0 : cfg.material_interface_amm_fraction;
    if (model < 0 || model > 2) throw std::runtime_error("materials.interface_model must be dmm, amm or mmm.");
    if (!std::isfinite(cfg.material_interface_amm_fraction) || cfg.material_interface_amm_fraction < 0 ||
        cfg.material_interface_amm_fraction > 1)
        throw std::runtime_error("materials.interface_amm_fraction must be in [0,1].");
    if (!std::isfinite(cfg.material_interface_parallel_bin_inv_a) || cfg.material_interface_parallel_bin_inv_a <= 0)
        throw std::runtime_error("materials.interface_parallel_bin_inv_a must be finite and positive.");
    if (model == 0 && cfg.material_interface_amm_fraction != 0)
        throw std::runtime_error("DMM cannot have nonzero AMM fraction.");
    const bool acoustic = model == 1 || (model == 2 && fraction > 0);
    if (acoustic) {
        if (mats.size() < 2 || cfg.material_mass_densities_kg_m3.size() != mats.size())
            throw std::runtime_error("AMM/MMM requires one mass density per material layer.");
        for (double rho : cfg.material_mass_densities_kg_m3)
            if (!std::isfinite(rho) || rho <= 0) throw std::runtime_error("Material mass densities must be finite and positive.");
    }
    if (P.iface.enabled) {
        P.iface.build(mats, P.layout.axis);
        P.iface.model = model;
        P.iface.amm_fraction = model == 0 ? 0.0 : fraction;
        if (acoustic)
            P.iface.amm.build(mats, P.layout.axis, cfg.material_mass_densities_kg_m3,
                              cfg.material_interface_frequency_bin_thz, cfg.material_interface_parallel_bin_inv_a);
    }

    // Reservoirs (src/solver/ReservoirInitialization.cpp:1-45, ReservoirSampler.cpp:17-101).
    for (int f : domain.reservoir_facets()) {
        const Facet& F = domain.facets()[f];
        Reservoir R;
        R.facet = f;
        R.material = P.layout.material_at(F.centroid);
        // carriers per unit volume of the reservoir's material (src/solver/ReservoirInitialization.cpp:18-23)
        const double density = mats.size() > 1 ? 1.0 / P.material_spatial_volume[R.material]
                                               : static_cast<double>(P.initial_particles) / domain.volume();
        R.temperature = F.value;
        R.area = F.area;
        R.normal = F.normal;
        const PhononMaterial& M = *mats[R.material];
        const auto& act = M.active_flat();
        R.cdf.resize(act.size());
        std::vector<double> weight(act.size(), 0.0);
        const double n_active = static_cast<double>(M.active_mode_count());
        double expected = 0;
        if (density > 0.0 && cfg.time_step > 0.0) {
            const double thickness = n_active / (density * R.area);
            for (size_t m = 0; m < act.size(); ++m) {
                const double par = -dot3(R.normal, M.velocity(act[m]));
                weight[m] = std::max(0.0, par * cfg.time_step / thickness);
                expected += weight[m];
                R.cdf[m] = expected;
            }
        }
        if (expected > 0) {
            for (double& v : R.cdf) v /= expected;
            R.alias = build_alias_table(weight);
        }
        R.initial_count = static_cast<int>(std::llround(expected));
        R.expected = expected;
        std::vector<double> occ(act.size());
        for (size_t m = 0; m < act.size(); ++m)
            occ[m] = P.linearized ? M.linearized_bose_occupation(R.temperature, Tbg, act[m])
                                  : M.bose_occupation(R.temperature, act[m]);
        P.reservoir_occ.push_back(std::move(occ));
        P.reservoirs.push_back(std::move(R));
    }
    return P;
}

// src/solver/Initialization.cpp:32-137, 180-265 with Philox draws.
CarrierArrays initial_carriers(const Problem& p, const std::vector<const PhononMaterial*>& mats,
                               const double* preset_xyz) {
    const SimulationDomain& D = *p.domain;
    const int n = p.initial_particles;
    CarrierArrays c;
    c.x.resize(n);
    c.y.resize(n);
    c.z.resize(n);
    c.occ.resize(n);
    c.mode.resize(n);
    c.cell.resize(n);
    c.alive.assign(n, 1);
    // initial temperature profile
    double cold_t = std::numeric_limits<double>::infinity(), hot_t = -cold_t;
    int cold = -1, hot = -1;
    for (int f : D.reservoir_facets()) {
        const double T = D.facets()[f].value;
        if (T < cold_t) { cold_t = T; cold = f; }
        if (T > hot_t) { hot_t = T; hot = f; }
    }
    double tmin = 299.0, tmax = 301.0;
    if (!D.reservoir_facets().empty()) { tmin = cold_t; tmax = hot_t; }
    const bool linear = p.cfg.initial_temperature_mode == InitialTemperatureMode::Linear;
    const bool valid_pair = cold >= 0 && hot >= 0 && hot_t > cold_t + 1e-12;
    const double tmean = 0.5 * (tmin + tmax);
    Vec3 pc{}, axis{};
    double axis_len2 = 0;
    if (linear && valid_pair) {
        pc = D.facets()[cold].centroid;
        axis = sub3(D.facets()[hot].centroid, pc);
        axis_len2 = dot3(axis, axis);
    }
    const Vec3& lo = D.bounds_min();
    const Vec3& hi = D.bounds_max();
    const uint64_t seed = p.cfg.random_seed;
    // Mesh domains (src/geometry/SurfaceSampling.cpp:102-155): a simplex of the
    // volume decomposition by volume, then Dirichlet(1,1,1,1) weights from four
    // exponentials; without a valid decomposition, uniform box points kept
    // when the +x ray cast finds them inside (at most 200 trials per carrier).
    const SurfaceMesh* mesh = D.is_mesh() ? D.mesh() : nullptr;
    std::vector<double> simplex_cum;
    if (mesh) {
        double run = 0.0;
        for (const auto& sx : mesh->simplices()) simplex_cum.push_back(run += std::max(sx.volume, 0.0));
        if (!simplex_cum.empty() && !(run > 0.0)) simplex_cum.clear();
    }
    std::vector<double> prism_cum; // running doubled areas of the prism's top triangles
    if (D.is_prism()) {
        double run = 0.0;
        for (const auto& t : D.prism_top())
            prism_cum.push_back(run += std::abs((t[1][0] - t[0][0]) * (t[2][1] - t[0][1]) -
                                                (t[1][1] - t[0][1]) * (t[2][0] - t[0][0])));
    }
    int rejected = -1;
    const double smallest_volume = *std::min_element(p.material_spatial_volume.begin(), p.material_spatial_volume.end());
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const Uniform2 u0 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, 0, 0);
        const Uniform2 u1 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, 0, 1);
        Vec3 pos{lo[0] + (hi[0] - lo[0]) * u0.a, lo[1] + (hi[1] - lo[1]) * u0.b, lo[2] + (hi[2] - lo[2]) * u1.a};
        if (D.is_prism()) {
            // src/SimulationDomain.cpp:239-260: a top triangle by area, a
            // uniform point in it, a uniform height
            size_t k = static_cast<size_t>(std::upper_bound(prism_cum.begin(), prism_cum.end(),
                                                            u0.a * prism_cum.back()) - prism_cum.begin());
            if (k >= prism_cum.size()) k = prism_cum.size() - 1;
            const auto& t = D.prism_top()[k];
            const Uniform2 u2 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, 0, 2);
            const double a = std::sqrt(u0.b), b = u1.a;
            for (int j = 0; j < 2; ++j) pos[j] = (1 - a) * t[0][j] + a * (1 - b) * t[1][j] + a * b * t[2][j];
            pos[2] = lo[2] + u2.a * (hi[2] - lo[2]);
        } else if (mesh && !simplex_cum.empty()) {
            size_t k = static_cast<size_t>(std::upper_bound(simplex_cum.begin(), simplex_cum.end(),
                                                            u0.a * simplex_cum.back()) - simplex_cum.begin());
            if (k >= simplex_cum.size()) k = simplex_cum.size() - 1;
            const auto& sx = mesh->simplices()[k];
            const Uniform2 u2 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, 0, 2);
            double a[4] = {-std::log(std::max(u0.b, 1e-15)), -std::log(std::max(u1.a, 1e-15)),
                           -std::log(std::max(u2.a, 1e-15)), -std::log(std::max(u2.b, 1e-15))};
            const double sum = a[0] + a[1] + a[2] + a[3];
            for (double& w : a) w /= sum;
            for (int c = 0; c < 3; ++c)
                pos[c] = a[0] * sx.v[0][c] + a[1] * sx.v[1][c] + a[2] * sx.v[2][c] + a[3] * sx.v[3][c];
        } else if (mesh && preset_xyz && !std::isnan(preset_xyz[3 * static_cast<size_t>(i)])) {
            // accepted point of the same draws, found by the device ray cast
            const double* q = preset_xyz + 3 * static_cast<size_t>(i);
            if (std::isinf(q[0])) {
#pragma omp critical
                rejected = i;
            } else {
                pos = {q[0], q[1], q[2]};
            }
        } else if (mesh) {
            bool ok = mesh->contains_point_ray_cast(pos);
            for (uint32_t trial = 1; !ok && trial < 200; ++trial) {
                const Uniform2 r0 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial, 0);
                const Uniform2 r1 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial, 1);
                pos = {lo[0] + (hi[0] - lo[0]) * r0.a, lo[1] + (hi[1] - lo[1]) * r0.b, lo[2] + (hi[2] - lo[2]) * r1.a};
                ok = mesh->contains_point_ray_cast(pos);
            }
            if (!ok) {
#pragma omp critical
                rejected = i;
            }
        }
        double mode_u = u1.b;
        if (p.mats.size() > 1) {
            // keep a point of material m with probability smallest volume / volume_m
            // (src/solver/Initialization.cpp:48-65)
            for (uint32_t trial = 0;; ++trial) {
                const int m = p.layout.material_at(pos);
                const Uniform2 acc = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial, 3);
                if (acc.a < smallest_volume / p.material_spatial_volume[m]) break;
                if (trial + 1 >= 100000u) {
#pragma omp critical
                    rejected = i;
                    break;
                }
                const Uniform2 r0 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial + 1, 0);
                const Uniform2 r1 = uniform2(seed, static_cast<uint32_t>(i), 0xFFFFFFFFu, kDrawInit, trial + 1, 1);
                pos = {lo[0] + (hi[0] - lo[0]) * r0.a, lo[1] + (hi[1] - lo[1]) * r0.b, lo[2] + (hi[2] - lo[2]) * r1.a};
                mode_u = r1.b;
            }
        }
        const int mid = p.layout.material_at(pos);
        const MaterialTables& T = p.mats[mid];
        int a = static_cast<int>(mode_u * T.n_active);
        if (a >= T.n_active) a = T.n_active - 1;
        double temp = p.cfg.initial_temperature;
        if (linear) {
            if (valid_pair && axis_len2 > 1e-20) {
                const double s = std::clamp(dot3(sub3(pos, pc), axis) / axis_len2, 0.0, 1.0);
                temp = cold_t + s * (hot_t - cold_t);
            } else {
                temp = tmean;
            }
        }
        const int flat = T.active_flat[a];
        c.x[i] = pos[0];
        c.y[i] = pos[1];
        c.z[i] = pos[2];
        c.mode[i] = mode_word(static_cast<uint32_t>(a), 0u, static_cast<uint32_t>(mid));
        c.cell[i] = D.fast_grid_index(pos);
        c.occ[i] = p.linearized ? mats[mid]->linearized_bose_occupation(temp, p.cfg.background_temperature, flat)
                                : mats[mid]->bose_occupation(temp, flat);
    }
    if (rejected >= 0) throw std::runtime_error("Initial carrier sampling found no accepted position.");
    return c;
}

// ------------------------------------------------------------- writers
std::string format_convergence_header(size_t cells, bool gradient_driven) {
    std::ostringstream out;
    out << "# timestep time_ps";
    for (size_t i = 0; i < cells; ++i) out << " T_" << (i + 1);
    out << " heatflux kappa_int kappa_eff particle_count absorbed injected recovered net"
           " reservoir_absorbed_energy_ev reservoir_injected_energy_ev"
           " hs_occupation_updates hs_injected_energy_ev lifetime_energy_residual_ev"
           " energy_balance_residual_ev total_thermal_energy_ev"
           " hs_prescribed_total_ev hs_pending_total_ev hs_ledger_residual_ev";
    if (gradient_driven) out << " gradient_occupation_updates gradient_energy_ev";
    out << '\n';
    return out.str();
}

// src/solver/ResultWriter.cpp:100-119: default stream precision for the step,
// time and temperatures, then 12 significant digits.
std::string format_convergence_row(const ConvergenceRow& s) {
    std::ostringstream out;
    out << s.timestep << " " << s.time_ps;
    for (double t : s.temperatures) out << " " << t;
    out.precision(12);
    out << " " << s.heat_flux << " " << s.kappa_int << " " << s.kappa_eff << " " << s.particle_count << " "
        << s.absorbed << " " << s.injected << " " << 0 << " " << s.net << " " << s.absorbed_ev << " "
        << s.injected_ev << " " << s.source_updates << " " << s.source_ev << " " << s.lifetime_residual << " "
        << s.balance_residual << " " << s.thermal_energy << " " << s.source_prescribed << " " << s.source_pending << " "
        << (s.source_prescribed - s.source_deposited - s.source_pending);
    if (s.gradient) out << " " << s.gradient_updates << " " << s.gradient_energy;
    out << '\n';
    return out.str();
}

std::vector<AliasCell> build_alias_table(const std::vector<double>& weights) {
    const size_t n = weights.size();
    double sum = 0.0;
    for (double w : weights) {
        if (!(w >= 0.0) || !std::isfinite(w)) throw std::invalid_argument("alias table: weights must be finite and non-negative");
        sum += w;
    }
    if (n == 0 || !(sum > 0.0)) throw std::invalid_argument("alias table: weights must have a positive sum");
    std::vector<AliasCell> t(n, AliasCell{1.0, 0, 0});
    std::vector<double> p(n);
    std::vector<int32_t> small, large;
    int32_t heaviest = 0;
    for (size_t k = 0; k < n; ++k) {
        p[k] = weights[k] * static_cast<double>(n) / sum; // column mass in units of 1/n
        (p[k] < 1.0 ? small : large).push_back(static_cast<int32_t>(k));
        if (weights[k] > weights[heaviest]) heaviest = static_cast<int32_t>(k);
        t[k].alias = static_cast<int32_t>(k);
    }
    while (!small.empty() && !large.empty()) {
        const int32_t s = small.back(), l = large.back();
        small.pop_back();
        large.pop_back();
        t[s].prob = p[s];
        t[s].alias = l;
        p[l] = (p[l] + p[s]) - 1.0; // what is left of l after filling column s
        (p[l] < 1.0 ? small : large).push_back(l);
    }
    // columns left over hold mass 1 up to rounding; a weightless one (possible
    // only through rounding) hands its column to the heaviest outcome
    for (int32_t l : large) t[l] = AliasCell{1.0, l, 0};
    for (int32_t s : small) t[s] = weights[s] > 0.0 ? AliasCell{1.0, s, 0} : AliasCell{0.0, heaviest, 0};
    return t;
}

} // namespace phmc
