// Golden-vector harness around the reference's own C++ solver.
//
// Linked against oracle/_ref/libphonomc_ref.a, which is the reference's src/
// compiled unchanged (only the HDF5 readers are replaced). Every number this
// program prints comes from reference code: PhononMaterial, SimulationDomain,
// RtaCollisionOperator, CarrierCollisionOperator, CallawayOperator,
// RoughBoundarySampler, ReservoirSampler, TemperatureGradientDrive and
// MonteCarloSolver. Inputs that are not files are drawn here from
// std::mt19937_64 and printed beside the outputs, so the tests can replay them
// through the oracle and the CUDA path.
//
// Output is JSON on stdout (numbers with 17 significant digits).
#include "MonteCarloSolver.h"
#include <memory>
#include <sstream>
#include "PhononMaterial.h"
#include "material/MaterialDataReader.h"
#include "SimulationConfig.h"
#include "SimulationDomain.h"
#include "material/CallawayOperator.h"
#include "solver/BackgroundCache.h"
#include "solver/BoundaryInteraction.h"
#include "solver/CarrierCollisionOperator.h"
#include "solver/CellParticleIndex.h"
#include "solver/InterfaceInteraction.h"
#include "solver/AcousticInterfaceSampler.h"
#include "solver/PhononSourceOperator.h"
#include "SurfaceMesh.h"
#include "geometry/MeshReader.h"
#include "solver/PrescribedHeatSource.h"
#include "solver/NonlinearCallawayCollision.h"
#include "solver/ParticleStorage.h"
#include "solver/ReservoirSampler.h"
#include "solver/RoughBoundarySampler.h"
#include "solver/RtaCollisionOperator.h"
#include "solver/TemperatureGradientDrive.h"

#include <chrono>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {
using phonomc::MaterialData;

// ---------------------------------------------------------------- JSON out
struct Json {
    std::ostringstream s;
    bool first = true;
    Json() { s << "{"; }
    void key(const std::string& k) {
        if (!first) s << ",\n";
        first = false;
        s << '"' << k << "\":";
    }
    static std::string num(double x) {
        if (std::isnan(x)) return "NaN";
        if (std::isinf(x)) return x > 0 ? "Infinity" : "-Infinity";
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g", x);
        return buf;
    }
    void put(const std::string& k, double x) { key(k); s << num(x); }
    void put_i(const std::string& k, long long x) { key(k); s << x; }
    void put_s(const std::string& k, const std::string& v) { key(k); s << '"' << v << '"'; }
    template <class V> void arr(const std::string& k, const V& v) {
        key(k);
        s << "[";
        for (size_t i = 0; i < v.size(); ++i) s << (i ? "," : "") << num(static_cast<double>(v[i]));
        s << "]";
    }
    template <class V> void arr3(const std::string& k, const V& v) {
        key(k);
        s << "[";
        for (size_t i = 0; i < v.size(); ++i) {
            s << (i ? "," : "") << "[" << num(v[i][0]) << "," << num(v[i][1]) << "," << num(v[i][2]) << "]";
        }
        s << "]";
    }
    void raw(const std::string& k, const std::string& v) { key(k); s << v; }
    std::string str() const { return s.str() + "}"; }
};

// ------------------------------------------------------------ material input
MaterialData read_pmat(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("cannot open " + path);
    char magic[8];
    in.read(magic, 8);
    if (std::memcmp(magic, "PMAT0001", 8) != 0) throw std::runtime_error("bad magic");
    int32_t h[8];
    in.read(reinterpret_cast<char*>(h), sizeof h);
    MaterialData d;
    d.qpoints = h[0];
    d.branches = h[1];
    d.mesh = {h[2], h[3], h[4]};
    const int nT = h[5], has_nu = h[6], nres = h[7];
    in.read(reinterpret_cast<char*>(&d.lattice.volume_a3), 8);
    double R[9];
    in.read(reinterpret_cast<char*>(R), sizeof R);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) d.lattice.reciprocal[i][j] = R[3 * i + j];
    const size_t nm = static_cast<size_t>(d.qpoints) * d.branches;
    auto rd = [&](std::vector<double>& v, size_t n) {
        v.resize(n);
        in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * 8));
    };
    auto rd3 = [&](std::vector<phonomc::MaterialVec3>& v, size_t n) {
        v.resize(n);
        in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * 24));
    };
    rd(d.frequency_thz, nm);
    rd3(d.qpoint_fractions, d.qpoints);
    rd3(d.group_velocity, nm);
    rd(d.temperatures, nT);
    rd(d.gamma, nm * nT);
    if (has_nu) {
        rd(d.gamma_normal, nm * nT);
        rd(d.gamma_umklapp, nm * nT);
    }
    for (int r = 0; r < nres; ++r) {
        char name[17] = {0};
        in.read(name, 16);
        int64_t n;
        in.read(reinterpret_cast<char*>(&n), 8);
        std::vector<double> v;
        rd(v, static_cast<size_t>(n));
        d.gamma_resistive[name] = std::move(v);
    }
    if (!in) throw std::runtime_error("truncated pmat");
    return d;
}

// --------------------------------------------------------------- commands
// material <pmat> <stationary>: lookup tables and thermodynamic queries.
std::string cmd_material(const std::string& pmat, bool stationary, bool callaway) {
    PhononMaterial m(read_pmat(pmat), 0.1, stationary, callaway);
    Json j;
    j.put_i("active_mode_count", m.active_mode_count());
    std::vector<int> act;
    for (const auto& mode : m.active_mode_list()) act.push_back(mode[0] * m.branch_count() + mode[1]);
    j.arr("active_flat", act);
    j.put("energy_density_normalization", m.energy_density_normalization());
    j.put("zero_point_energy_density", m.zero_point_energy_density());
    std::vector<double> Ts, E;
    for (double T = 0; T <= 1000.0001; T += 7.3) {
        Ts.push_back(T);
        E.push_back(m.energy_density_from_temperature(T));
    }
    j.arr("table_T", Ts);
    j.arr("table_E", E);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(0, 1);
    const double e0 = m.energy_density_from_temperature(0.0), e1 = m.energy_density_from_temperature(1000.0);
    std::vector<double> qE, qT;
    for (int i = 0; i < 400; ++i) {
        double e = e0 + (e1 - e0) * (1.1 * U(rng) - 0.05);
        qE.push_back(e);
        qT.push_back(m.temperature_from_energy_density(e));
    }
    j.arr("inv_E", qE);
    j.arr("inv_T", qT);
    std::vector<double> cT, cE;
    for (double T : {0.0, 1.0, 50.0, 299.0, 300.0, 301.0, 777.7}) {
        cT.push_back(T);
        cE.push_back(m.crystal_energy_density(T));
    }
    j.arr("crystal_T", cT);
    j.arr("crystal_E", cE);
    // Per-mode queries on a sample of flat modes.
    std::vector<double> qm, qt, bose, cap, relax, lin;
    const int nm = m.qpoint_count() * m.branch_count();
    for (int i = 0; i < 300; ++i) {
        int flat = static_cast<int>(U(rng) * nm);
        double T = (i % 7 == 0) ? 300.0 : 1000.0 * U(rng);
        if (i % 11 == 0) T = 0.0;
        PhononMaterial::Mode mode{flat / m.branch_count(), flat % m.branch_count()};
        qm.push_back(flat);
        qt.push_back(T);
        bose.push_back(m.bose_occupation(T, mode));
        cap.push_back(m.mode_heat_capacity(T, mode));
        relax.push_back(m.mode_relaxation_weight(T, mode, 0.5));
        lin.push_back(m.linearized_bose_occupation(T, 300.0, mode));
    }
    j.arr("q_mode", qm);
    j.arr("q_T", qt);
    j.arr("q_bose", bose);
    j.arr("q_capacity", cap);
    j.arr("q_relax_dt0p5", relax);
    j.arr("q_linearized_300", lin);
    phonomc::BackgroundCache bg(m, 300.0, 1234.5, false), bgx(m, 300.0, 1234.5, true);
    j.put("bg_energy_weight", bg.energy_weight());
    j.put("bg_energy_density", bg.energy_density());
    j.put("bg_energy_density_exact", bgx.energy_density());
    j.put("bg_heat_capacity_density", bg.heat_capacity_density());
    const auto lr = m.linearized_rta_data(300.0);
    j.arr("lrta_omega", lr.omega);
    j.arr("lrta_capacity", lr.capacity);
    j.arr("lrta_rate", lr.resistive_rate);
    return j.str();
}

SimulationConfig box_config(double lx, double ly, double lz, int nx, int ny, int nz,
                            const std::vector<std::string>& bcs, const std::vector<double>& vals,
                            bool periodic_xy, bool periodic_x_only) {
    SimulationConfig a;
    a.model = "box";
    a.sizes = {lx, ly, lz};
    a.grid = {nx, ny, nz};
    const char* regions[6][6] = {{"-0.01", "0", "0", "0.01", "1", "1"}, {"0.99", "0", "0", "1.01", "1", "1"},
                                 {"0", "-0.01", "0", "1", "0.01", "1"}, {"0", "0.99", "0", "1", "1.01", "1"},
                                 {"0", "0", "-0.01", "1", "1", "0.01"}, {"0", "0", "0.99", "1", "1", "1.01"}};
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) a.boundary_position.push_back(regions[r][c]);
    for (const auto& b : bcs)
        a.boundary_conditions.push_back(b == "T" ? BoundaryCondition::ThermalReservoir
                                        : b == "P" ? BoundaryCondition::Periodic
                                                   : BoundaryCondition::Rough);
    a.boundary_values = vals;
    auto pair = [&](int r) {
        for (int c = 0; c < 6; ++c) a.periodic_pair.push_back(regions[r][c]);
    };
    if (periodic_x_only || periodic_xy) { pair(0); pair(1); }
    if (periodic_xy) { pair(2); pair(3); }
    return a;
}

// box: facet layout, boundary conditions, grid and ray traces of a reference box.
std::string cmd_box() {
    auto a = box_config(1000, 800, 600, 3, 2, 5, {"T", "T", "P", "P", "R", "R"}, {301, 299, 0, 0, 1, 0},
                        false, false);
    // Pair y only (regions 2,3).
    a.periodic_pair.clear();
    const char* yreg[2][6] = {{"0", "-0.01", "0", "1", "0.01", "1"}, {"0", "0.99", "0", "1", "1.01", "1"}};
    for (auto& r : yreg)
        for (auto* c : r) a.periodic_pair.push_back(c);
    SimulationDomain d(a);
    Json j;
    const auto& mesh = d.mesh();
    j.arr3("facet_normals", mesh.facet_normals());
    j.arr3("facet_centroids", mesh.facet_centroids());
    j.arr("facet_areas", mesh.facet_areas());
    std::vector<int> bc, pair;
    std::vector<std::array<double, 3>> shift;
    std::vector<double> rough;
    for (int f = 0; f < mesh.facet_count(); ++f) {
        bc.push_back(d.facet_boundary_condition(f));
        pair.push_back(d.periodic_pair_facet(f));
        shift.push_back(d.periodic_shift_for_facet(f));
        rough.push_back(d.roughness_for_facet(f, -1));
    }
    j.arr("facet_bc", bc);
    j.arr("facet_pair", pair);
    j.arr3("facet_shift", shift);
    j.arr("facet_roughness", rough);
    j.arr("reservoir_facets", d.reservoir_facets());
    j.arr("reservoir_values", d.reservoir_values());
    j.arr3("grid_centers", d.grid_centers());
    j.arr("grid_volumes", d.grid_volumes());
    j.put("volume", d.volume());
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> U(0, 1);
    std::normal_distribution<double> N(0, 1);
    std::vector<std::array<double, 3>> P, V, C;
    std::vector<double> T;
    std::vector<int> F, G;
    for (int i = 0; i < 2000; ++i) {
        std::array<double, 3> p{U(rng) * 1000, U(rng) * 800, U(rng) * 600};
        if (i % 13 == 0) p[i % 3] = (i % 2) ? (i % 3 == 0 ? 1000 : i % 3 == 1 ? 800 : 600) : 0.0;
        if (i % 17 == 0) p[0] = 1000 + 1e-10;  // just outside within tolerance
        if (i % 19 == 0) p[2] = -1e-6;         // outside beyond tolerance
        std::array<double, 3> v{N(rng) * 50, N(rng) * 50, N(rng) * 50};
        if (i % 5 == 0) v[i % 3] = 0.0;
        auto [cp, t, f] = d.trace_boundary_intersection(p, v);
        P.push_back(p);
        V.push_back(v);
        C.push_back(cp);
        T.push_back(t);
        F.push_back(f);
        G.push_back(d.fast_grid_index(p));
    }
    j.arr3("ray_p", P);
    j.arr3("ray_v", V);
    j.arr3("hit_p", C);
    j.arr("hit_t", T);
    j.arr("hit_f", F);
    j.arr("grid_index", G);
    return j.str();
}

struct CarrierSet {
    std::vector<int> flat, cell;
    std::vector<double> occ;
};

CarrierSet random_carriers(const PhononMaterial& m, int n, int cells, double dev, std::mt19937_64& rng,
                           double T0) {
    std::uniform_real_distribution<double> U(0, 1);
    CarrierSet c;
    for (int i = 0; i < n; ++i) {
        const int a = static_cast<int>(U(rng) * m.active_mode_count());
        const auto mode = m.active_mode_at(a);
        const int cell = static_cast<int>(U(rng) * cells);
        const double T = T0 + dev * (2 * U(rng) - 1) + 0.5 * cell;
        c.flat.push_back(mode[0] * m.branch_count() + mode[1]);
        c.cell.push_back(cell);
        c.occ.push_back(m.bose_occupation(T, mode) * (1 + 0.01 * (2 * U(rng) - 1)));
    }
    return c;
}

void fill_storage(phonomc::ParticleStorage& p, const PhononMaterial& m, const CarrierSet& c) {
    p.reset(static_cast<int>(c.flat.size()));
    for (size_t i = 0; i < c.flat.size(); ++i) {
        p.modes[i] = {c.flat[i] / m.branch_count(), c.flat[i] % m.branch_count()};
        p.material_ids[i] = 0;
        p.grid_ids[i] = c.cell[i];
        p.occupation[i] = c.occ[i];
        p.omega[i] = m.mode_angular_frequency(p.modes[i]);
    }
}

// rta <pmat> <local>: energy-conserving nonlinear RTA on random carriers.
std::string cmd_rta(const std::string& pmat, bool local) {
    PhononMaterial m(read_pmat(pmat), 0.1, false, false);
    std::mt19937_64 rng(23);
    const int cells = 6;
    auto c = random_carriers(m, 3000, cells, 3.0, rng, 300.0);
    // Two special cells: one empty, one far from equilibrium.
    for (size_t i = 0; i < c.cell.size(); ++i) {
        if (c.cell[i] == 4) c.cell[i] = 3;
        if (c.cell[i] == 5) c.occ[i] *= 3.0;
    }
    phonomc::ParticleStorage p;
    fill_storage(p, m, c);
    std::vector<double> cellT = {299.5, 300.0, 300.7, 301.2, 300.0, 320.0};
    for (size_t i = 0; i < c.cell.size(); ++i) p.temperatures[i] = cellT[c.cell[i]];
    std::vector<int> mats(cells, 0);
    phonomc::CellParticleIndex idx;
    idx.ensure(p, cells);
    phonomc::RtaCollisionOperator op;
    std::vector<const PhononMaterial*> ms{&m};
    const double vol = 17.25;
    const double res = op.apply(p, ms, {idx.counts(), mats, cellT, &idx}, {0.75, vol, local, 300.0});
    Json j;
    j.arr("flat", c.flat);
    j.arr("cell", c.cell);
    j.arr("occ_in", c.occ);
    j.arr("cell_T", cellT);
    j.put("dt", 0.75);
    j.put("particle_volume", vol);
    j.put_i("local", local);
    j.put("lifetime_T", 300.0);
    j.arr("occ_out", p.occupation);
    j.put("residual", res);
    return j.str();
}

// lincoll <pmat>: linearized-RTA carrier collision (CarrierCollisionOperator rta=true).
std::string cmd_lincoll(const std::string& pmat) {
    PhononMaterial m(read_pmat(pmat), 0.1, true, false);
    std::mt19937_64 rng(29);
    const int cells = 5;
    auto c = random_carriers(m, 2500, cells, 2.0, rng, 300.0);
    for (size_t i = 0; i < c.cell.size(); ++i) {
        const auto mode = PhononMaterial::Mode{c.flat[i] / m.branch_count(), c.flat[i] % m.branch_count()};
        // linearized occupations around 300 K
        const double T = 300.0 + 0.8 * c.cell[i] - 1.0;
        c.occ[i] = m.linearized_bose_occupation(T, 300.0, mode) + 1e-3 * std::sin(0.37 * i);
    }
    phonomc::ParticleStorage p;
    fill_storage(p, m, c);
    std::vector<int> mats(cells, 0);
    std::vector<double> cellT(cells, 300.0);
    phonomc::CellParticleIndex idx;
    idx.ensure(p, cells);
    phonomc::CarrierCollisionOperator op;
    std::vector<const PhononMaterial*> ms{&m};
    op.configure(ms, 300.0, true);
    const double vol = 9.5;
    const double res = op.apply(p, ms, {idx.counts(), mats, cellT, &idx}, 0.5, vol);
    Json j;
    j.arr("flat", c.flat);
    j.arr("cell", c.cell);
    j.arr("occ_in", c.occ);
    j.put("dt", 0.5);
    j.put("particle_volume", vol);
    j.arr("occ_out", p.occupation);
    j.put("residual", res);
    return j.str();
}

// callaway: CallawayOperator evolve on a random quadrature with N and R rates.
std::string cmd_callaway() {
    std::mt19937_64 rng(31);
    std::uniform_real_distribution<double> U(0, 1);
    Json j;
    std::ostringstream cases;
    cases << "[";
    for (int cs = 0; cs < 4; ++cs) {
        phonomc::CallawayData d;
        const int n = 40 + 60 * cs;
        std::vector<double> e;
        for (int i = 0; i < n; ++i) {
            d.omega.push_back(5 + 90 * U(rng));
            d.capacity.push_back(1e-5 + 8e-5 * U(rng));
            d.wavevector.push_back({2 * U(rng) - 1, 2 * U(rng) - 1, 2 * U(rng) - 1});
            d.normal_rate.push_back(cs == 3 ? 0.0 : (0.5 + cs) * U(rng));
            d.resistive_rate.push_back(0.05 + 0.3 * U(rng) * (cs + 1));
            e.push_back(1e-4 * (2 * U(rng) - 1));
        }
        const double dt = cs == 2 ? 7.0 : 0.5;
        phonomc::CallawayOperator op(d);
        const auto out = op.evolve(e, dt);
        const auto act = op.apply(e);
        Json c;
        c.arr("omega", d.omega);
        c.arr("capacity", d.capacity);
        c.arr3("wavevector", d.wavevector);
        c.arr("normal_rate", d.normal_rate);
        c.arr("resistive_rate", d.resistive_rate);
        c.arr("energy", e);
        c.put("dt", dt);
        c.arr("evolved", out);
        c.arr("action", act);
        c.put_i("normal_rank", static_cast<long long>(op.normal_constraint_rank()));
        cases << (cs ? "," : "") << c.str();
    }
    cases << "]";
    j.raw("cases", cases.str());
    return j.str();
}

// rough <pmat> <conservative>: rough-boundary tables for the two z walls of a box,
// plus reflections with the draws each one consumed.
std::string cmd_rough(const std::string& pmat, bool conservative) {
    PhononMaterial m(read_pmat(pmat), 0.1, conservative, false);
    std::vector<phonomc::RoughFacetSpec> facets;
    facets.push_back({true, {0, 0, -1}, 10.0});
    facets.push_back({true, {0, 0, 1}, 3.0});
    facets.push_back({false, {1, 0, 0}, 0.0});
    phonomc::RoughBoundarySampler s;
    std::vector<const PhononMaterial*> ms{&m};
    s.configure(facets, ms, nullptr, conservative, conservative ? 300.0 : 0.0);
    Json j;
    j.put_i("table0", s.table_index(0, 0));
    j.put_i("table1", s.table_index(0, 1));
    j.put_i("table2", s.table_index(0, 2));
    // Reflections: record draws by replaying a copy of the engine.
    std::mt19937_64 pick(41);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<int> in_flat, facet, out_flat, ndraw;
    std::vector<double> in_occ, out_occ, draws;
    for (int i = 0; i < 600; ++i) {
        const int f = i % 2;
        const int a = static_cast<int>(U(pick) * m.active_mode_count());
        const auto mode = m.active_mode_at(a);
        const auto v = m.mode_group_velocity(mode);
        const double vn = f == 0 ? -v[2] : v[2];
        if (!(vn > 0)) continue;  // incoming modes only
        const double occ = m.bose_occupation(300 + 5 * U(pick), mode);
        std::mt19937_64 eng(1000 + i), copy = eng;
        const auto r = s.sample(m, s.table_index(0, f), mode, occ, 300.0, eng, conservative);
        int used = 0;
        std::vector<double> u;
        while (!(copy == eng) && used < 8) {
            u.push_back(std::generate_canonical<double, 53>(copy));
            ++used;
        }
        in_flat.push_back(mode[0] * m.branch_count() + mode[1]);
        facet.push_back(f);
        in_occ.push_back(occ);
        out_flat.push_back(r.mode[0] * m.branch_count() + r.mode[1]);
        out_occ.push_back(r.occupation);
        ndraw.push_back(used);
        for (int k = 0; k < 3; ++k) draws.push_back(k < used ? u[k] : -1.0);
    }
    j.arr("in_flat", in_flat);
    j.arr("facet", facet);
    j.arr("in_occ", in_occ);
    j.arr("out_flat", out_flat);
    j.arr("out_occ", out_occ);
    j.arr("ndraw", ndraw);
    j.arr("draws", draws);
    return j.str();
}

// interface <pmat_a> <pmat_b> <linearized>: DMM interactions at a z-normal
// interface between two materials (InterfaceInteraction::interact), with the
// engine's draws recorded by replaying a copy of it.
std::string cmd_interface(const std::string& pa, const std::string& pb, bool linearized) {
    PhononMaterial ma(read_pmat(pa), 0.1, false, false), mb(read_pmat(pb), 0.1, false, false);
    const double wa = 1.375e-3, wb = 0.8125e-3;
    phonomc::InterfaceInteractionConfig cfg;
    cfg.axis = 2;
    cfg.enabled = true;
    cfg.linearized = linearized;
    cfg.model = InterfaceModel::DiffuseMismatch;
    cfg.frequency_bin_thz = 0.1;
    cfg.reference_temperature = 300.0;
    phonomc::InterfaceInteraction I;
    I.configure(cfg, {&ma, &mb}, {wa, wb});
    const PhononMaterial* mats[2] = {&ma, &mb};
    std::mt19937_64 pick(77);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<int> src, in_flat, in_signs, action, out_material, out_flat, ndraw, events, transmitted, reflected,
        error;
    std::vector<double> in_occ, out_occ, draws, out_v;
    for (int i = 0; i < 1200; ++i) {
        const int m = i % 2;
        const int next = 1 - m;
        const PhononMaterial& M = *mats[m];
        const int a = static_cast<int>(U(pick) * M.active_mode_count());
        const auto mode = M.active_mode_at(a);
        auto v = M.mode_group_velocity(mode);
        if (std::abs(v[2]) <= 1e-12) continue;
        // moving toward the other layer (material 0 below, material 1 above)
        int signs = 0;
        const bool want_up = m == 0;
        if ((v[2] > 0) != want_up) {
            v[2] = -v[2];
            signs |= 4;
        }
        for (int k = 0; k < 2; ++k)
            if (U(pick) < 0.5) {
                v[k] = -v[k];
                signs |= 1 << k;
            }
        const double Tn = 300.0 + 8.0 * (U(pick) - 0.5);
        const double occ = linearized ? M.bose_occupation(300.0, mode) + (U(pick) - 0.5) * 0.02
                                      : M.bose_occupation(Tn, mode);
        phonomc::BoundaryState st{mode, m, v, M.mode_angular_frequency(mode), occ};
        std::mt19937_64 eng(5000 + i), copy = eng;
        const auto r = I.interact(st, next, eng);
        int used = 0;
        std::vector<double> u;
        while (!(copy == eng) && used < 8) {
            u.push_back(std::generate_canonical<double, 53>(copy));
            ++used;
        }
        src.push_back(m);
        in_flat.push_back(mode[0] * M.branch_count() + mode[1]);
        in_signs.push_back(signs);
        in_occ.push_back(occ);
        action.push_back(static_cast<int>(r.action));
        error.push_back(static_cast<int>(r.error));
        out_material.push_back(r.state.material);
        const PhononMaterial& D = *mats[r.state.material];
        out_flat.push_back(r.state.mode[0] * D.branch_count() + r.state.mode[1]);
        out_occ.push_back(r.state.occupation);
        for (int k = 0; k < 3; ++k) out_v.push_back(r.state.velocity[k]);
        events.push_back(static_cast<int>(r.interface_events));
        transmitted.push_back(static_cast<int>(r.interface_transmitted));
        reflected.push_back(static_cast<int>(r.interface_reflected));
        ndraw.push_back(used);
        for (int k = 0; k < 3; ++k) draws.push_back(k < used ? u[k] : -1.0);
    }
    Json j;
    j.put("weight_a", wa);
    j.put("weight_b", wb);
    j.put("frequency_bin_thz", 0.1);
    j.put("reference_temperature", 300.0);
    j.put_i("axis", 2);
    j.arr("src", src);
    j.arr("in_flat", in_flat);
    j.arr("in_signs", in_signs);
    j.arr("in_occ", in_occ);
    j.arr("action", action);
    j.arr("error", error);
    j.arr("out_material", out_material);
    j.arr("out_flat", out_flat);
    j.arr("out_occ", out_occ);
    j.arr("out_v", out_v);
    j.arr("events", events);
    j.arr("transmitted", transmitted);
    j.arr("reflected", reflected);
    j.arr("ndraw", ndraw);
    j.arr("draws", draws);
    return j.str();
}

// amm <pmat a> <pmat b> <model 1 amm|2 mmm> <amm fraction> <linearized>:
// acoustic-mismatch rows of both sides of the a|b interface (AcousticInterfaceSampler::row
// for every active mode) and InterfaceInteraction::interact events with the
// uniforms each consumed (up to four), densities 2329 / 5323 kg/m^3, axis z.
std::string cmd_amm(const std::string& pa, const std::string& pb, int model, double fraction, bool linearized) {
    PhononMaterial ma(read_pmat(pa), 0.1, false, false), mb(read_pmat(pb), 0.1, false, false);
    const double wa = 1.375e-3, wb = 0.8125e-3;
    phonomc::InterfaceInteractionConfig cfg;
    cfg.axis = 2;
    cfg.enabled = true;
    cfg.linearized = linearized;
    cfg.model = model == 1 ? InterfaceModel::AcousticMismatch : InterfaceModel::MixedMismatch;
    cfg.amm_fraction = fraction;
    cfg.frequency_bin_thz = 0.1;
    cfg.parallel_bin_inv_a = 0.05;
    cfg.mass_densities_kg_m3 = {2329.0, 5323.0};
    cfg.reference_temperature = 300.0;
    phonomc::InterfaceInteraction I;
    I.configure(cfg, {&ma, &mb}, {wa, wb});
    phonomc::AcousticInterfaceSampler S;
    S.configure({&ma, &mb}, 2, cfg.mass_densities_kg_m3, cfg.frequency_bin_thz, cfg.parallel_bin_inv_a);
    Json j;
    const PhononMaterial* mats[2] = {&ma, &mb};
    for (int side = 0; side < 2; ++side) {
        std::vector<int> refl, start{0}, dest;
        std::vector<double> prob;
        for (int a = 0; a < mats[side]->active_mode_count(); ++a) {
            const auto& r = S.row(side, 1 - side, a);
            refl.push_back(r.reflected);
            for (const auto& e : r.transmitted) {
                dest.push_back(e.active);
                prob.push_back(e.probability);
            }
            start.push_back(static_cast<int>(dest.size()));
        }
        const std::string k = std::to_string(side);
        j.arr("reflected_" + k, refl);
        j.arr("start_" + k, start);
        j.arr("dest_" + k, dest);
        j.arr("prob_" + k, prob);
    }
    std::mt19937_64 pick(91);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<int> src, in_flat, in_signs, action, out_material, out_flat, ndraw, events, transmitted, reflected;
    std::vector<double> in_occ, out_occ, draws;
    for (int i = 0; i < 4000; ++i) {
        const int m = i % 2;
        const PhononMaterial& M = *mats[m];
        const int a = static_cast<int>(U(pick) * M.active_mode_count());
        const auto mode = M.active_mode_at(a);
        // the carrier moves with its mode's own velocity, toward the other layer
        // (acoustic rows exist only for those states)
        const auto v = M.mode_group_velocity(mode);
        if (std::abs(v[2]) <= 1e-12 || (v[2] > 0) != (m == 0)) continue;
        const int signs = 0;
        const double occ = linearized ? M.bose_occupation(300.0, mode) + (U(pick) - 0.5) * 0.02
                                      : M.bose_occupation(300.0 + 8.0 * (U(pick) - 0.5), mode);
        phonomc::BoundaryState st{mode, m, v, M.mode_angular_frequency(mode), occ};
        std::mt19937_64 eng(7000 + i), copy = eng;
        const auto r = I.interact(st, 1 - m, eng);
        int used = 0;
        std::vector<double> u;
        while (!(copy == eng) && used < 8) {
            u.push_back(std::generate_canonical<double, 53>(copy));
            ++used;
        }
        src.push_back(m);
        in_flat.push_back(mode[0] * M.branch_count() + mode[1]);
        in_signs.push_back(signs);
        in_occ.push_back(occ);
        action.push_back(static_cast<int>(r.action));
        out_material.push_back(r.state.material);
        const PhononMaterial& D = *mats[r.state.material];
        out_flat.push_back(r.state.mode[0] * D.branch_count() + r.state.mode[1]);
        out_occ.push_back(r.state.occupation);
        events.push_back(static_cast<int>(r.interface_events));
        transmitted.push_back(static_cast<int>(r.interface_transmitted));
        reflected.push_back(static_cast<int>(r.interface_reflected));
        ndraw.push_back(used);
        for (int k = 0; k < 4; ++k) draws.push_back(k < used ? u[k] : -1.0);
    }
    j.put("weight_a", wa);
    j.put("weight_b", wb);
    j.put("frequency_bin_thz", 0.1);
    j.put("parallel_bin_inv_a", 0.05);
    j.put("density_a", 2329.0);
    j.put("density_b", 5323.0);
    j.put("amm_fraction", fraction);
    j.put_i("model", model);
    j.put("reference_temperature", 300.0);
    j.put_i("axis", 2);
    j.arr("src", src);
    j.arr("in_flat", in_flat);
    j.arr("in_signs", in_signs);
    j.arr("in_occ", in_occ);
    j.arr("action", action);
    j.arr("out_material", out_material);
    j.arr("out_flat", out_flat);
    j.arr("out_occ", out_occ);
    j.arr("events", events);
    j.arr("transmitted", transmitted);
    j.arr("reflected", reflected);
    j.arr("ndraw", ndraw);
    j.arr("draws", draws);
    return j.str();
}

// source <pmat> <spectrum 0 thermal|1 weighted|2 gaussian> <linearized>:
// PrescribedHeatSource cell powers of a Gaussian source in a 2x2x3 box, one
// accrual, then PhononSourceOperator::apply on random carriers.
std::string cmd_source(const std::string& pmat, int spectrum, bool linearized) {
    PhononMaterial m(read_pmat(pmat), 0.1, true, false);
    auto a = box_config(500, 400, 300, 2, 2, 3, {"P", "P", "P", "P", "T", "T"}, {0, 0, 0, 0, 301, 299}, true, false);
    a.heat_source_enabled = true;
    a.heat_source_profile = HeatSourceProfile::Gaussian;
    a.heat_source_center = {180.0, 130.0, 90.0};
    a.heat_source_sigma = {160.0, 140.0, 70.0};
    a.heat_source_power_density = 3e19;
    if (linearized) a.collision_model = CollisionModel::Callaway;
    if (spectrum == 1) {
        a.heat_source_spectrum = HeatSourceSpectrum::Weighted;
        a.heat_source_branch_weights = {1.0, 2.0, 1.5, 0.5, 0.25, 0.0};
        a.heat_source_branches = {0, 1, 2, 3, 4};
    } else if (spectrum == 2) {
        a.heat_source_spectrum = HeatSourceSpectrum::Gaussian;
        a.heat_source_frequency_center = 6.0;
        a.heat_source_frequency_sigma = 2.5;
    }
    a.heat_source_frequency_max = 14.0;
    SimulationDomain d(a);
    phonomc::PrescribedHeatSource hs;
    hs.configure(a, d);
    const int cells = static_cast<int>(d.grid_centers().size());
    const double factor = 0.37;
    hs.accrue(factor);
    const std::vector<double> pending_before = hs.cell_pending_ev();
    phonomc::PhononSourceOperator op;
    std::vector<const PhononMaterial*> ms{&m};
    op.configure(a, ms);
    std::mt19937_64 rng(61);
    auto c = random_carriers(m, 4000, cells, 2.0, rng, 300.0);
    for (size_t i = 0; i < c.cell.size(); ++i)
        if (c.cell[i] == 1) c.cell[i] = 0; // cell 1 keeps its budget
    phonomc::ParticleStorage p;
    fill_storage(p, m, c);
    phonomc::CellParticleIndex idx;
    idx.ensure(p, cells);
    std::vector<int> mats(cells, 0);
    std::vector<double> cellT(cells);
    for (int k = 0; k < cells; ++k) cellT[k] = 298.5 + 0.4 * k;
    const double vol = 7.5;
    const auto r = op.apply(p, ms, {mats, cellT, &idx}, hs, vol, 300.0);
    Json j;
    j.arr("rates", hs.cell_rates_evps());
    j.put("factor", factor);
    j.arr("pending_before", pending_before);
    j.arr("pending_after", hs.cell_pending_ev());
    j.arr("cell_temperature", cellT);
    j.put("particle_volume", vol);
    j.arr("flat", c.flat);
    j.arr("cell", c.cell);
    j.arr("occ_in", c.occ);
    j.arr("occ_out", p.occupation);
    j.put("energy", r.energy_ev);
    j.put_i("updates", r.occupation_updates);
    j.arr3("centers", d.grid_centers());
    j.arr("volumes", d.grid_volumes());
    return j.str();
}

// mesh <stl>: a surface mesh as the box-free domain builds it (STL in nm scaled
// to Angstrom, coplanar facets merged, shifted to the origin), then ray traces
// through SurfaceMesh::trace_boundary_intersection from random interior
// points, and containment of random points.
std::string cmd_mesh(const std::string& stl) {
    auto loaded = phonomc::read_surface_mesh(stl);
    for (auto& v : loaded.vertices)
        for (double& x : v) x *= 10.0;
    SurfaceMesh mesh;
    mesh.set_merge_coplanar_facets(true);
    mesh.set_surface_mesh_data(std::move(loaded.vertices), std::move(loaded.faces));
    mesh.shift_to_origin();
    Json j;
    j.arr3("vertices", mesh.vertices());
    std::vector<int> faces;
    for (const auto& f : mesh.faces())
        for (int k = 0; k < 3; ++k) faces.push_back(f[k]);
    j.arr("faces", faces);
    std::vector<int> f2f;
    for (int i = 0; i < mesh.face_count(); ++i) f2f.push_back(mesh.facet_index_for_face(i));
    j.arr("face_to_facet", f2f);
    j.put_i("facet_count", mesh.facet_count());
    j.arr3("facet_normals", mesh.facet_normals());
    j.arr("bounds_max", std::vector<double>(mesh.bounds_max().begin(), mesh.bounds_max().end()));
    std::mt19937_64 rng(91);
    std::uniform_real_distribution<double> U(0, 1);
    std::normal_distribution<double> N(0, 1);
    const auto hi = mesh.bounds_max();
    std::vector<std::array<double, 3>> P, V, H;
    std::vector<double> T;
    std::vector<int> F;
    while (P.size() < 3000) {
        std::array<double, 3> p{U(rng) * hi[0], U(rng) * hi[1], U(rng) * hi[2]};
        if (!mesh.contains_point(p)) continue;
        std::array<double, 3> v{N(rng), N(rng), N(rng)};
        const double s = 60.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (double& c : v) c *= s;
        if (P.size() % 10 == 0) v[P.size() % 3] = 0.0; // axis-parallel in one component
        const auto [hit, t, facet] = mesh.trace_boundary_intersection(p, v);
        P.push_back(p);
        V.push_back(v);
        H.push_back(hit);
        T.push_back(t);
        F.push_back(facet);
    }
    j.arr3("origins", P);
    j.arr3("velocities", V);
    j.arr3("hits", H);
    j.arr("t", T);
    j.arr("facet", F);
    std::vector<std::array<double, 3>> Q;
    std::vector<int> inside;
    for (int i = 0; i < 3000; ++i) {
        std::array<double, 3> q{U(rng) * hi[0], U(rng) * hi[1], U(rng) * hi[2]};
        Q.push_back(q);
        inside.push_back(mesh.contains_point(q) ? 1 : 0);
    }
    j.arr3("points", Q);
    j.arr("inside", inside);
    j.put("volume", mesh.volume());
    return j.str();
}

// domain <toml>: SimulationDomain of a mesh TOML (facets, boundary assignment,
// periodic pairs, cells and the voxel map), membership / nearest-facet / cell
// queries at random points, and the domain summary file it writes.
// A text file as a JSON string body (quotes, backslashes, newlines, tabs escaped).
std::string escaped_file(const std::filesystem::path& path) {
    std::ifstream in(path);
    std::ostringstream text;
    text << in.rdbuf();
    std::string esc;
    for (char c : text.str()) {
        if (c == '"' || c == '\\') esc.push_back('\\');
        if (c == '\n') esc += "\\n";
        else if (c == '\t') esc += "\\t";
        else esc.push_back(c);
    }
    return esc;
}

std::string cmd_domain(const std::string& toml, int n_traces = 0) {
    SimulationConfig a = load_simulation_config(toml);
    SimulationDomain d(a);
    const SurfaceMesh& mesh = d.mesh();
    Json j;
    j.arr3("vertices", mesh.vertices());
    std::vector<int> faces, f2f;
    for (const auto& f : mesh.faces())
        for (int k = 0; k < 3; ++k) faces.push_back(f[k]);
    for (int i = 0; i < mesh.face_count(); ++i) f2f.push_back(mesh.facet_index_for_face(i));
    j.arr("faces", faces);
    j.arr("face_to_facet", f2f);
    j.arr3("facet_normals", mesh.facet_normals());
    j.arr3("facet_centroids", mesh.facet_centroids());
    j.arr("facet_areas", mesh.facet_areas());
    std::string cond;
    std::vector<double> value;
    std::vector<int> pair;
    std::vector<std::array<double, 3>> shift;
    for (int f = 0; f < mesh.facet_count(); ++f) {
        const char c = d.facet_boundary_condition(f);
        cond.push_back(c);
        value.push_back(c == 'T' ? d.reservoir_value_for_facet(f) : (c == 'R' ? d.roughness_for_facet(f) : 0.0));
        pair.push_back(d.periodic_pair_facet(f));
        shift.push_back(d.periodic_shift_for_facet(f));
    }
    j.put_s("conditions", cond);
    j.arr("values", value);
    j.arr("pair", pair);
    j.arr3("shift", shift);
    j.arr3("grid_centers", d.grid_centers());
    j.arr("grid_volumes", d.grid_volumes());
    j.put("volume", d.volume());
    std::vector<double> b(d.bounds_min().begin(), d.bounds_min().end());
    b.insert(b.end(), d.bounds_max().begin(), d.bounds_max().end());
    j.arr("bounds", b);
    const auto lo = d.bounds_min(), hi = d.bounds_max();
    std::vector<int> voxel;
    const int nx = a.grid.nx, ny = a.grid.ny, nz = a.grid.nz;
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy)
            for (int iz = 0; iz < nz; ++iz)
                voxel.push_back(d.fast_grid_index({lo[0] + (ix + 0.5) * (hi[0] - lo[0]) / nx,
                                                   lo[1] + (iy + 0.5) * (hi[1] - lo[1]) / ny,
                                                   lo[2] + (iz + 0.5) * (hi[2] - lo[2]) / nz}));
    j.arr("voxel_cell", voxel);
    std::mt19937_64 rng(17);
    std::uniform_real_distribution<double> U(0, 1);
    std::vector<std::array<double, 3>> P;
    std::vector<int> inside, nearest, cell;
    for (int i = 0; i < 2000; ++i) {
        std::array<double, 3> p{lo[0] + U(rng) * (hi[0] - lo[0]), lo[1] + U(rng) * (hi[1] - lo[1]),
                                lo[2] + U(rng) * (hi[2] - lo[2])};
        P.push_back(p);
        inside.push_back(d.contains_point(p) ? 1 : 0);
        nearest.push_back(mesh.nearest_facet(p));
        cell.push_back(d.fast_grid_index(p));
    }
    j.arr3("points", P);
    j.arr("inside", inside);
    j.arr("nearest_facet", nearest);
    j.arr("cell", cell);
    j.put_s("domain_summary", escaped_file(std::filesystem::path(a.output_folder) / "summary.txt"));
    // traces of the domain from inside points along random directions
    // (SimulationDomain::trace_boundary_intersection)
    std::vector<std::array<double, 3>> tp, tv, th;
    std::vector<double> tt;
    std::vector<int> tf;
    for (int i = 0; i < static_cast<int>(P.size()) && static_cast<int>(tp.size()) < n_traces; ++i) {
        if (!inside[i]) continue;
        const double c = 2 * U(rng) - 1, ph = 6.283185307179586 * U(rng), s = std::sqrt(1 - c * c);
        const double speed = 20 + 60 * U(rng);
        std::array<double, 3> v{speed * s * std::cos(ph), speed * s * std::sin(ph), speed * c};
        const auto [hit, t, f] = d.trace_boundary_intersection(P[i], v);
        tp.push_back(P[i]);
        tv.push_back(v);
        th.push_back(hit);
        tt.push_back(t);
        tf.push_back(f);
    }
    if (n_traces > 0) {
        j.arr3("trace_p", tp);
        j.arr3("trace_v", tv);
        j.arr3("trace_hit", th);
        j.arr("trace_t", tt);
        j.arr("trace_facet", tf);
    }
    return j.str();
}

// gradient <pmat>: TemperatureGradientDrive on random carriers in a periodic box.
std::string cmd_gradient(const std::string& pmat) {
    PhononMaterial m(read_pmat(pmat), 0.1, true, false);
    auto a = box_config(500, 400, 300, 1, 1, 4, {"P", "P", "P", "P", "R", "R"}, {0, 0, 0, 0, 1, 1}, true,
                        false);
    a.temperature_gradient = 1e7;
    a.transport_axis = 0;
    a.lifetime_temperature_is_local = false;
    SimulationDomain d(a);
    phonomc::TemperatureGradientDrive g;
    const double vol = 11.0;
    g.configure(a, d, m, vol);
    std::mt19937_64 rng(43);
    auto c = random_carriers(m, 2000, 4, 1.0, rng, 300.0);
    phonomc::ParticleStorage p;
    fill_storage(p, m, c);
    phonomc::CellParticleIndex idx;
    idx.ensure(p, 4);
    std::mt19937_64 unused(0);
    const auto r = g.apply(p, idx, 0.25, unused);
    Json j;
    j.arr("flat", c.flat);
    j.arr("cell", c.cell);
    j.arr("occ_in", c.occ);
    j.put("dt", 0.25);
    j.put("particle_volume", vol);
    j.put("gradient", 1e7);
    j.arr("occ_out", p.occupation);
    j.put("energy", r.energy_ev);
    j.put_i("updates", r.occupation_updates);
    return j.str();
}

// reservoir <pmat>: incoming-flux CDF draws for the two z faces of a box.
std::string cmd_reservoir(const std::string& pmat) {
    PhononMaterial m(read_pmat(pmat), 0.1, false, false);
    phonomc::ReservoirSampler s;
    std::vector<phonomc::ReservoirFacetSpec> f;
    f.push_back({4, 0, 301.0, 640000.0, {0, 0, -1}});
    f.push_back({5, 0, 299.0, 640000.0, {0, 0, 1}});
    std::vector<const PhononMaterial*> ms{&m};
    const double density = 1e-3, dt = 0.5;
    s.configure(f, ms, 6, density, dt);
    Json j;
    j.put("density", density);
    j.put("dt", dt);
    j.put("area", 640000.0);
    std::vector<int> init;
    for (int r = 0; r < 2; ++r) init.push_back(s.initial_emission_count(r));
    j.arr("initial_count", init);
    std::vector<int> mode;
    std::vector<double> draws, times;
    for (int r = 0; r < 2; ++r) {
        for (int i = 0; i < 300; ++i) {
            std::mt19937_64 eng(5000 + 1000 * r + i), copy = eng;
            const auto e = s.sample(r, 1, eng);
            draws.push_back(std::generate_canonical<double, 53>(copy));
            mode.push_back(static_cast<int>(e[0].active_index));
            times.push_back(e[0].time_ps);
        }
    }
    j.arr("draw", draws);
    j.arr("active_index", mode);
    j.arr("time", times);
    return j.str();
}

// run <pmat> <toml> <steps>: full reference solver; prints per-step observables.
// <pmat> may list several tables separated by commas (layered materials, in order).
// Seeded single-cell cases for nonlinear_callaway_evolve: n_modes modes with
// frequencies, wavevectors and N/R rates, n_carriers carriers drawn over the
// modes (unique = one carrier per mode) with occupations around Bose at T.
std::string cmd_ncallaway(int seed, int n_modes, int n_carriers, int unique) {
    std::mt19937_64 g(static_cast<uint64_t>(seed));
    std::uniform_real_distribution<double> u(0.0, 1.0);
    const double T = 150.0 + 300.0 * u(g), dt = 0.25 + u(g);
    std::vector<double> omega(n_modes), rn(n_modes), rr(n_modes);
    std::vector<std::array<double, 3>> k(n_modes);
    for (int m = 0; m < n_modes; ++m) {
        omega[m] = 2.0 + 90.0 * u(g);
        for (int a = 0; a < 3; ++a) k[m][a] = 2.0 * u(g) - 1.0;
        rn[m] = 1.5 * u(g);
        rr[m] = u(g) < 0.1 ? 0.0 : 0.8 * u(g);
    }
    std::vector<int> mode(n_carriers);
    std::vector<double> n(n_carriers);
    phonomc::CallawayData d;
    for (int i = 0; i < n_carriers; ++i) {
        mode[i] = unique ? i % n_modes : static_cast<int>(u(g) * n_modes) % n_modes;
        const double x = 6.582119569e-4 * omega[mode[i]] / (8.617333262145e-5 * T);
        n[i] = (1.0 / std::expm1(x)) * (0.5 + u(g));
        d.omega.push_back(omega[mode[i]]);
        d.wavevector.push_back(k[mode[i]]);
        d.normal_rate.push_back(rn[mode[i]]);
        d.resistive_rate.push_back(rr[mode[i]]);
    }
    const auto out = phonomc::nonlinear_callaway_evolve(d, n, T, dt);
    Json j;
    j.put("T", T);
    j.put("dt", dt);
    j.arr("omega", omega);
    j.arr3("k", k);
    j.arr("rn", rn);
    j.arr("rr", rr);
    j.arr("mode", mode);
    j.arr("n", n);
    j.arr("out", out);
    return j.str();
}

std::string cmd_run(const std::string& pmat, const std::string& toml, int steps) {
    SimulationConfig a = load_simulation_config(toml);
    const bool stationary = uses_conservative_transport(a);
    std::vector<std::unique_ptr<PhononMaterial>> owned;
    std::vector<std::reference_wrapper<const PhononMaterial>> mats;
    std::stringstream list(pmat);
    for (std::string item; std::getline(list, item, ',');) {
        // a material folder (POSCAR + HDF5) goes through the reference's own
        // read_material_data; a .pmat file through the flat-table reader above
        MaterialData md = std::filesystem::is_directory(item) ? phonomc::read_material_data(item) : read_pmat(item);
        owned.push_back(std::make_unique<PhononMaterial>(std::move(md), a.temperature_lookup_dt, stationary,
                                                         a.collision_model == CollisionModel::Callaway));
        mats.push_back(*owned.back());
    }
    SimulationDomain d(a);
    MonteCarloSolver s(a, d, mats);
    std::vector<double> pc, absorbed, injected, flux, energy, resid, source;
    while (s.current_timestep() < steps) {
        s.run_timestep();
        pc.push_back(s.particle_count());
        absorbed.push_back(static_cast<double>(s.absorbed_particle_count()));
        injected.push_back(static_cast<double>(s.injected_particle_count()));
        flux.push_back(s.average_heat_flux_along_axis());
        source.push_back(s.total_heat_source_energy_ev());
        energy.push_back(s.total_thermal_energy_ev());
        resid.push_back(s.total_energy_balance_residual_ev());
    }
    Json j;
    // convergence.txt rows written by the reference's ResultWriter
    if (!a.output_folder.empty()) {
        std::ifstream conv(std::filesystem::path(a.output_folder) / "convergence.txt");
        std::string line;
        std::ostringstream rows;
        rows << "[";
        bool first = true;
        while (std::getline(conv, line)) {
            if (line.empty() || line[0] == '#') continue;
            std::istringstream ls(line);
            std::string tok;
            rows << (first ? "" : ",") << "[";
            bool f2 = true;
            while (ls >> tok) {
                rows << (f2 ? "" : ",") << Json::num(std::stod(tok));
                f2 = false;
            }
            rows << "]";
            first = false;
        }
        rows << "]";
        j.raw("convergence", rows.str());
        const std::filesystem::path dir(a.output_folder);
        for (const char* f : {"convergence.txt", "grid_heat_flux.csv", "heat_source_ledger.txt"})
            if (std::filesystem::exists(dir / f)) j.put_s(std::string("file:") + f, escaped_file(dir / f));
    }
    j.arr3("grid_centers", d.grid_centers());
    j.arr("particle_count", pc);
    j.arr("absorbed_total", absorbed);
    j.arr("injected_total", injected);
    j.arr("heat_flux", flux);
    j.arr("thermal_energy", energy);
    j.arr("balance_residual_total", resid);
    j.arr("heat_source_total", source);
    j.put("lifetime_residual_total", s.total_lifetime_energy_residual_ev());
    j.put("gradient_energy_total", s.total_gradient_energy_ev());
    j.put_i("interface_events", s.interface_event_count());
    j.put_i("interface_transmitted", s.interface_transmitted_count());
    j.put_i("interface_reflected", s.interface_reflected_count());
    return j.str();
}
// Wall time of the reference's own step loop: `warm` steps, then `steps`
// timed steps of MonteCarloSolver::run_timestep; carrier-steps count the
// carriers present at the start of each timed step. Threads: OMP_NUM_THREADS.
std::string cmd_time(const std::string& pmat, const std::string& toml, int warm, int steps) {
    SimulationConfig a = load_simulation_config(toml);
    const bool stationary = uses_conservative_transport(a);
    MaterialData md = std::filesystem::is_directory(pmat) ? phonomc::read_material_data(pmat) : read_pmat(pmat);
    PhononMaterial m(std::move(md), a.temperature_lookup_dt, stationary, a.collision_model == CollisionModel::Callaway);
    std::vector<std::reference_wrapper<const PhononMaterial>> mats{m};
    SimulationDomain d(a);
    MonteCarloSolver s(a, d, mats);
    for (int k = 0; k < warm; ++k) s.run_timestep();
    double carrier_steps = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    for (int k = 0; k < steps; ++k) {
        carrier_steps += static_cast<double>(s.particle_count());
        s.run_timestep();
    }
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    Json j;
    j.put("carrier_steps", carrier_steps);
    j.put("seconds", sec);
    j.put("carrier_steps_per_s", carrier_steps / sec);
#ifdef _OPENMP
    j.put_i("threads", omp_get_max_threads());
#else
    j.put_i("threads", 1);
#endif
    return j.str();
}
} // namespace

int main(int argc, char** argv) {
    try {
        if (argc < 2) throw std::runtime_error("usage: ref_harness <command> ...");
        const std::string c = argv[1];
        std::string out;
        // Reference constructors log progress to stdout; keep stdout for JSON only.
        std::ostringstream sink;
        auto* saved = std::cout.rdbuf(sink.rdbuf());
        if (c == "material") out = cmd_material(argv[2], std::atoi(argv[3]) != 0, argc > 4 && std::atoi(argv[4]) != 0);
        else if (c == "box") out = cmd_box();
        else if (c == "rta") out = cmd_rta(argv[2], std::atoi(argv[3]) != 0);
        else if (c == "lincoll") out = cmd_lincoll(argv[2]);
        else if (c == "callaway") out = cmd_callaway();
        else if (c == "rough") out = cmd_rough(argv[2], std::atoi(argv[3]) != 0);
        else if (c == "gradient") out = cmd_gradient(argv[2]);
        else if (c == "mesh") out = cmd_mesh(argv[2]);
        else if (c == "domain") out = cmd_domain(argv[2], argc > 3 ? std::atoi(argv[3]) : 0);
        else if (c == "source") out = cmd_source(argv[2], std::atoi(argv[3]), std::atoi(argv[4]) != 0);
        else if (c == "interface") out = cmd_interface(argv[2], argv[3], std::atoi(argv[4]) != 0);
        else if (c == "reservoir") out = cmd_reservoir(argv[2]);
        else if (c == "amm")
            out = cmd_amm(argv[2], argv[3], std::atoi(argv[4]), std::atof(argv[5]), std::atoi(argv[6]) != 0);
        else if (c == "run") out = cmd_run(argv[2], argv[3], std::atoi(argv[4]));
        else if (c == "time") out = cmd_time(argv[2], argv[3], std::atoi(argv[4]), std::atoi(argv[5]));
        else if (c == "ncallaway")
            out = cmd_ncallaway(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]));
        else throw std::runtime_error("unknown command " + c);
        std::cout.rdbuf(saved);
        std::cout << out << std::endl;
    } catch (const std::exception& e) {
        std::cerr << "ref_harness: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
