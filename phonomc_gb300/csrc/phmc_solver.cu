// DeviceSolver: table upload, HBM allocation and the per-step kernel sequence.
#include "phmc_kernels.cuh"
#include "phmc_tuning.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <numeric>
#include <sstream>
#include <stdexcept>

namespace phmc {

#define PHMC_CUDA(x)                                                                                      \
    do {                                                                                                  \
        cudaError_t err_ = (x);                                                                           \
        if (err_ != cudaSuccess)                                                                          \
            throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(err_) + " at " #x); \
    } while (0)

template <class T> T* DeviceSolver::dalloc(size_t n) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(1, n) * sizeof(T);
    PHMC_CUDA(cudaMalloc(&p, bytes));
    PHMC_CUDA(cudaMemsetAsync(p, 0, bytes, stream_));
    allocations_.push_back(p);
    return static_cast<T*>(p);
}

template <class T> T* DeviceSolver::upload(const std::vector<T>& v) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) PHMC_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
    return p;
}

static const char* error_message(int code) {
    switch (code) {
    case kErrIntersection: return "Boundary intersection failed while advancing particles. Check that the STL is closed and manifold.";
    case kErrModeMapping: return "Full-matrix boundary mode mapping failed while advancing particles. An inward discrete material mode and finite signed energy weight are required; no velocity-only reflection was applied.";
    case kErrTooManyEvents: return "Particle exceeded 64 transport events in one timestep. Reduce simulation.time_step or inspect narrow STL features; no recovery was applied.";
    case kErrInvalidStatistics: return "Invalid particle in grid energy statistics.";
    case kErrEscaped: return "Particle escaped the domain. Refusing to relocate or rethermalize it; inspect the geometry and time step.";
    case kErrZeroFluxReservoir: return "Cannot sample positive emissions from a zero-flux reservoir.";
    case kErrCapacity: return "Carrier population exceeds the allocated device capacity.";
    case kErrOutwardReservoirMode: return "Full-matrix reservoir sampled an outward mode.";
    case kErrNonFinite: return "Non-finite grid energy reduction.";
    case kErrNoRoughTable: return "Rough facet without a sampling table.";
    case kErrCollision: return "Carrier collision occupation overflow.";
    // src/solver/NonlinearCallawayCollision.cpp:88-213, src/material/PhononMaterialCollisionData.cpp:172-174
    case kErrNclNoConstraint: return "Nonlinear Callaway has no representable energy constraint";
    case kErrNclSingular: return "Singular nonlinear Callaway moment Jacobian";
    case kErrNclLineSearch: return "Nonlinear Callaway moment line search failed";
    case kErrNclNoConverge: return "Nonlinear Callaway moment solve did not converge";
    case kErrNclInvalid: return "Nonlinear Callaway occupation is invalid";
    case kErrNclTemperature: return "Nonlinear Callaway temperature is outside the supplied N/U table";
    case kErrPipelineTimeout: return "Carrier tile copies did not complete within the wait limit.";
    // src/solver/AcousticInterfaceSampler.cpp:459-461
    case kErrAmmRow: return "AMM incoming state is tangent or unsupported.";
    default: return "Unknown device error.";
    }
}

const char* solver_error_message(int code) { return error_message(code); }

DeviceSolver::DeviceSolver(const SimulationConfig& cfg, const std::vector<const PhononMaterial*>& mats,
                           bool init_carriers, bool mixed)
    : cfg_(cfg), mats_(mats), mixed_(mixed) {
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count <= 0)
        throw std::runtime_error("No CUDA device is available for the GB300 carrier loop.");
    PHMC_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, 0);
    domain_ = std::make_unique<SimulationDomain>(cfg_);
    if (!cfg_.output_folder.empty()) {
        // written by the reference's SimulationDomain constructor (src/geometry/DomainOutput.cpp:12-241)
        std::filesystem::create_directories(cfg_.output_folder);
        std::ofstream(std::filesystem::path(cfg_.output_folder) / "summary.txt") << format_domain_summary(cfg_, *domain_);
        std::ofstream(std::filesystem::path(cfg_.output_folder) / "grid_centers.csv") << format_grid_centers(*domain_);
    }
    if (domain_->is_mesh() && mats_.size() != 1)
        throw std::runtime_error("Layered materials are built for box domains only.");
    // the specular-match scans of the rough tables run on the device
    const SpecMatchScan scan = [this](const std::vector<Vec3>& va, std::vector<SpecMatchJob>& jobs) {
        spec_match_device(va, jobs, stream_);
    };
    P_ = build_problem(cfg_, *domain_, mats_, &scan);
    ncells_ = domain_->grid_count();
    sort_interval_ = resolved_sort_interval(cfg_, mixed_);
    const int n0 = P_.initial_particles;
    const int margin = P_.reservoirs.empty() ? 1024 : std::max(65536, n0 / 4);
    allocate_state(n0 + margin);
    upload_tables();
    if (!init_carriers) return;
    // A mesh without a volume decomposition samples positions by ray-cast
    // rejection: that part runs on the device, with the host's draws.
    std::vector<double> preset;
    if (domain_->is_mesh() && !domain_->is_prism() && domain_->mesh()->simplices().empty() && n0 > 0) {
        double* d_xyz = nullptr;
        const size_t bytes = 3 * static_cast<size_t>(n0) * sizeof(double);
        PHMC_CUDA(cudaMalloc(&d_xyz, bytes));
        launch_mesh_initial_positions(ctx(), n0, cfg_.random_seed, domain_->bounds_min().data(),
                                      domain_->bounds_max().data(), d_xyz);
        preset.resize(3 * static_cast<size_t>(n0));
        const cudaError_t e = cudaMemcpyAsync(preset.data(), d_xyz, bytes, cudaMemcpyDeviceToHost, stream_);
        const cudaError_t e2 = cudaStreamSynchronize(stream_);
        cudaFree(d_xyz);
        PHMC_CUDA(e);
        PHMC_CUDA(e2);
    }
    const CarrierArrays c = initial_carriers(P_, mats_, preset.empty() ? nullptr : preset.data());
    set_carriers(n0, c.x.data(), c.y.data(), c.z.data(), c.occ.data(), c.mode.data(), c.alive.data());
    if (!cfg_.output_folder.empty()) {
        std::filesystem::create_directories(cfg_.output_folder);
        std::ofstream(std::filesystem::path(cfg_.output_folder) / "convergence.txt")
            << format_convergence_header(ncells_, cfg_.temperature_gradient.has_value());
        if (cfg_.temperature_gradient || cfg_.write_cell_heat_flux)
            std::ofstream(std::filesystem::path(cfg_.output_folder) / "grid_heat_flux.csv") << format_cell_flux_header();
    }
    flux_pass();
}

DeviceSolver::~DeviceSolver() {
    if (stream_) cudaStreamSynchronize(stream_);
    try {
        drain_observations(true);
    } catch (...) {
    }
    for (Observation* o : obs_pending_) obs_free_.push_back(o);
    for (Observation* o : obs_free_) {
        cudaFreeHost(o->T);
        cudaFreeHost(o->E);
        cudaFreeHost(o->q);
        cudaFreeHost(o->L);
        if (o->src) cudaFreeHost(o->src);
        cudaEventDestroy(o->done);
        delete o;
    }
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (void* p : allocations_) cudaFree(p);
    if (d_tables_) cudaFree(d_tables_);
    if (stream_) cudaStreamDestroy(stream_);
}

void DeviceSolver::allocate_state(int capacity) {
    state_.capacity = capacity;
    // streamed per-slot arrays get one tile (256 slots) of padding: the staged
    // carrier pass copies whole 16-byte units of the last tile
    const int padded = capacity + 256;
    state_.x = dalloc<double>(capacity);
    state_.y = dalloc<double>(capacity);
    state_.z = dalloc<double>(capacity);
    if (mixed_) {
        state_.ox = dalloc<float>(padded);
        state_.oy = dalloc<float>(padded);
        state_.oz = dalloc<float>(padded);
    }
    state_.deferred = dalloc<int4>(capacity); // wall-event queue of the carrier pass
    if (domain_->is_mesh()) {
        // per-carrier mesh state lives in the facet tables (tables_.fac), filled by upload_mesh
        mesh_mirror_ = dalloc<int32_t>(capacity);
        PHMC_CUDA(cudaMemsetAsync(mesh_mirror_, 0xFF, static_cast<size_t>(capacity) * sizeof(int32_t), stream_));
        mesh_hit_t_ = dalloc<double>(capacity);
        mesh_hit_x_ = dalloc<double>(capacity);
        mesh_hit_y_ = dalloc<double>(capacity);
        mesh_hit_z_ = dalloc<double>(capacity);
        mesh_hit_f_ = dalloc<int32_t>(capacity);
    }
    state_.occ = dalloc<double>(padded);
    state_.mode = dalloc<uint32_t>(padded);
    state_.cell = dalloc<int32_t>(padded);
    state_.alive = dalloc<uint8_t>(padded);
    d_holes_ = dalloc<int>(capacity);
    d_contain_count_ = dalloc<int>(1);
    n_dead_blocks_ = (capacity + 1023) / 1024;
    d_block_dead_ = dalloc<int>(n_dead_blocks_);
    d_ledger_ = dalloc<DevLedger>(1);
}

void DeviceSolver::upload_tables() {
    DevTables& T = tables_;
    std::memset(&T, 0, sizeof T);
    if (P_.mats.size() > static_cast<size_t>(kMaxMaterials)) throw std::runtime_error("too many materials");
    int hist_modes = 0;
    double r_max = 0.0;
    int max_src_classes = 0;
    for (size_t mi = 0; mi < P_.mats.size(); ++mi) {
        const MaterialTables& M = P_.mats[mi];
        DevMaterial& D = T.mat[mi];
        D.n_active = M.n_active;
        // RTA bins are the mode classes (every per-cell update is class-uniform);
        // linear response keeps one bin per mode (gain vectors and drive are per mode)
        if (!P_.linearized && !P_.callaway_nonlinear) {
            D.bin = upload(M.mode_class);
            D.bin_rep = upload(M.class_rep);
            D.n_bins = M.n_classes;
        } else {
            D.bin = nullptr;
            D.bin_rep = nullptr;
            D.n_bins = M.n_active;
        }
        hist_modes = std::max(hist_modes, D.n_bins);
        D.n_classes = M.n_classes;
        D.n_lookup = static_cast<int>(M.lookup_T.size());
        D.n_temps = static_cast<int>(M.temperatures.size());
        D.omega = upload(M.omega);
        D.hw = upload(M.hw);
        std::vector<double> inv(M.n_active);
        for (int a = 0; a < M.n_active; ++a) inv[a] = M.hw[a] > 0 ? 1.0 / M.hw[a] : 0.0;
        D.inv_hw = upload(inv);
        D.vel = upload(M.vel);
        std::vector<float> v32(4 * static_cast<size_t>(M.n_active));
        for (int a = 0; a < M.n_active; ++a) {
            const double vx = M.vel[3 * a], vy = M.vel[3 * a + 1], vz = M.vel[3 * a + 2];
            v32[4 * a] = static_cast<float>(vx);
            v32[4 * a + 1] = static_cast<float>(vy);
            v32[4 * a + 2] = static_cast<float>(vz);
            v32[4 * a + 3] = 0.0f;
        }
        D.vel32 = upload(v32);
        std::vector<float> iv32(4 * static_cast<size_t>(M.n_active), 0.0f);
        std::vector<double> speed(M.n_active), push(M.n_active);
        for (int a = 0; a < M.n_active; ++a) {
            for (int k = 0; k < 3; ++k) {
                const float c = v32[4 * a + k];
                iv32[4 * a + k] = c != 0.0f ? 1.0f / c : 0.0f;
            }
            const double vx = M.vel[3 * a], vy = M.vel[3 * a + 1], vz = M.vel[3 * a + 2];
            speed[a] = std::sqrt(vx * vx + vy * vy + vz * vz);
            push[a] = P_.push_eps / std::max(speed[a], 1e-12);
        }
        D.ivel32 = upload(iv32);
        D.speed = upload(speed);
        D.push = upload(push);
        if (P_.source.enabled) {
            // spectral weights, Gaussian log-weights and equal-frequency classes of eligible modes
            const PhononMaterial& Pm = *mats_[mi];
            std::vector<double> wgt(M.n_active, 0.0), logw(M.n_active, 0.0), cls_omega;
            std::vector<int> cls(M.n_active, -1);
            std::vector<std::pair<double, int>> order;
            for (int a = 0; a < M.n_active; ++a) {
                const int f = M.active_flat[a];
                const double hw = kHbarEvPs * Pm.omega(f);
                if (std::isfinite(hw) && hw > 1e-14) wgt[a] = P_.source.mode_weight(Pm, f);
                const double fr = Pm.omega(f) / 6.283185307179586476925286766559;
                const double z = (fr - P_.source.gaussian_center) / P_.source.gaussian_sigma;
                logw[a] = -0.5 * z * z;
                if (wgt[a] > 0.0) order.push_back({M.omega[a], a});
            }
            std::sort(order.begin(), order.end());
            for (size_t k = 0; k < order.size(); ++k) {
                if (k == 0 || order[k].first != order[k - 1].first) cls_omega.push_back(order[k].first);
                cls[order[k].second] = static_cast<int>(cls_omega.size()) - 1;
            }
            D.src_weight = upload(wgt);
            D.src_logw = upload(logw);
            D.src_class = upload(cls);
            D.src_class_omega = upload(cls_omega);
            D.n_src_classes = static_cast<int>(cls_omega.size());
            max_src_classes = std::max(max_src_classes, D.n_src_classes);
        }
        D.nbg = upload(M.nbg);
        D.cap_bg = upload(M.capacity_bg);
        D.mode_class = upload(M.mode_class);
        D.class_omega = upload(M.class_omega);
        D.class_hw = upload(M.class_hw);
        D.class_rep = upload(M.class_rep);
        D.relax_fixed = upload(M.relax_fixed);
        D.temps = upload(M.temperatures);
        D.gamma = upload(M.gamma_active);
        D.lookup_T = upload(M.lookup_T);
        D.lookup_E = upload(M.lookup_E);
        if (P_.callaway_nonlinear) {
            ncl_.gamma_n[mi] = upload(M.ncl_gamma_n);
            ncl_.gamma_u[mi] = upload(M.ncl_gamma_u);
            ncl_.gamma_x[mi] = M.ncl_gamma_x.empty() ? nullptr : upload(M.ncl_gamma_x);
            ncl_.k[mi] = upload(M.col_k);
            ncl_.lifetime_T = cfg_.lifetime_temperature;
            ncl_.local = cfg_.lifetime_temperature_is_local ? 1 : 0;
        }
        if (P_.linearized) {
            std::vector<double> rate(M.n_active);
            for (int a = 0; a < M.n_active; ++a) {
                rate[a] = M.col_normal[a] + M.col_resistive[a];
                r_max = std::max(r_max, rate[a]);
            }
            D.col_cap = upload(M.col_capacity);
            D.col_rate = upload(rate);
            D.col_rn = upload(M.col_normal);
            D.col_rr = upload(M.col_resistive);
            D.col_k = upload(M.col_k);
        }
        if (!M.grad_rate.empty()) {
            D.grad_rate = upload(M.grad_rate);
            std::vector<double> dr(M.n_active), dc(M.n_active);
            for (int a = 0; a < M.n_active; ++a) {
                dr[a] = 0.5 * cfg_.time_step * M.grad_rate[a] / M.hw[a];
                dc[a] = 0.5 * cfg_.time_step * M.capacity_bg[a] / M.hw[a];
            }
            D.drive_rate = upload(dr);
            D.drive_cap = upload(dc);
        }
        D.energy_weight = M.energy_weight;
        {
            std::vector<double> fv(3 * static_cast<size_t>(M.n_active));
            for (int a = 0; a < M.n_active; ++a)
                for (int k = 0; k < 3; ++k) fv[3 * a + k] = M.vel[3 * a + k] * (M.hw[a] * M.energy_weight);
            D.flux_vel = upload(fv);
        }
        D.energy_density_bg = M.energy_density_bg;
        D.heat_capacity_density_bg = M.heat_capacity_density_bg;
        D.zero_point = M.zero_point;
    }
    // rough tables: inline for the box, a device array for mesh domains
    const bool mesh = domain_->is_mesh();
    std::vector<DevRoughTable> mesh_rough(mesh ? P_.rough.tables.size() : 0);
    if (!mesh && P_.rough.tables.size() > static_cast<size_t>(kMaxRoughTables))
        throw std::runtime_error("too many rough tables");
    for (size_t t = 0; t < P_.rough.tables.size(); ++t) {
        const RoughTable& R = P_.rough.tables[t];
        DevRoughTable& D = mesh ? mesh_rough[t] : T.rough[t];
        D.strict = R.strict_elastic ? 1 : 0;
        D.n_sorted = static_cast<int>(R.outgoing_sorted.size());
        D.n_roulette = static_cast<int>(R.roulette_active.size());
        D.n_outgoing = static_cast<int>(R.outgoing_active.size());
        D.specularity = upload(R.specularity);
        D.spec_match = upload(R.spec_match);
        D.diffuse_begin = upload(R.diffuse_begin);
        D.diffuse_end = upload(R.diffuse_end);
        D.outgoing_sorted = upload(R.outgoing_sorted);
        D.prefix = upload(R.residual_prefix);
        D.coarse = upload(coarse_prefix(R.residual_prefix));
        D.roulette_active = upload(R.roulette_active);
        D.roulette_cdf = upload(R.roulette_cdf);
        D.outgoing_active = upload(R.outgoing_active);
    }
    // reservoirs
    if (P_.reservoirs.size() > static_cast<size_t>(kMaxReservoirs)) throw std::runtime_error("too many reservoirs");
    for (size_t r = 0; r < P_.reservoirs.size(); ++r) {
        const Reservoir& R = P_.reservoirs[r];
        DevReservoir& D = T.res[r];
        D.facet = R.facet;
        D.material = R.material;
        D.n_cdf = static_cast<int>(R.cdf.size());
        D.expected = R.expected;
        for (int k = 0; k < 3; ++k) D.normal[k] = R.normal[k];
        const Facet& F = domain_->facets()[R.facet];
        std::vector<double> tri, cum;
        double run = 0.0;
        for (size_t k = 0; k < F.tris.size(); ++k) {
            for (int v = 0; v < 3; ++v)
                for (int a = 0; a < 3; ++a) tri.push_back(F.tris[k][v][a]);
            run += std::max(F.tri_area[k], 0.0);
            cum.push_back(run);
        }
        if (cum.empty() || !(run > 0.0)) throw std::runtime_error("No faces available for surface sampling.");
        D.n_tri = static_cast<int>(cum.size());
        D.tri = upload(tri);
        D.tri_cum = upload(cum);
        D.cdf = upload(R.cdf);
        D.alias = R.alias.empty() ? nullptr : upload(R.alias);
        D.occ = upload(P_.reservoir_occ[r]);
    }
    // domain
    DevDomain& D = T.dom;
    const Vec3& lo = domain_->bounds_min();
    const Vec3& hi = domain_->bounds_max();
    double scale = 1.0;
    for (int a = 0; a < 3; ++a) {
        D.lo[a] = lo[a];
        D.hi[a] = hi[a];
        D.inv_cell[a] = domain_->inv_cell()[a];
        D.shape[a] = domain_->grid_shape()[a];
        D.cell_size[a] = (hi[a] - lo[a]) / D.shape[a];
        D.cell_size32[a] = static_cast<float>(D.cell_size[a]);
        D.inv_cell32[a] = 1.0f / D.cell_size32[a];
        scale = std::max(scale, std::abs(hi[a] - lo[a]));
    }
    D.scale = scale;
    D.tol = std::max(1e-9, 64.0 * std::numeric_limits<double>::epsilon() * scale);
    D.ncells = ncells_;
    {
        // multiply-high division constants, checked for every cell index
        auto magic = [](int d) -> unsigned long long {
            if (d <= 1) return 0ull;
            return static_cast<unsigned long long>((static_cast<unsigned __int128>(1) << 64) / d) + 1ull;
        };
        const int dyz = D.shape[1] * D.shape[2], dz = D.shape[2];
        D.div_yz = magic(dyz);
        D.div_z = magic(dz);
        auto q = [](long long n, unsigned long long m) -> long long {
            return m ? static_cast<long long>((static_cast<unsigned __int128>(n) * m) >> 64) : n;
        };
        // cell indices, and voxel indices of a mesh domain's grid
        const long long n_index = std::max<long long>(ncells_, static_cast<long long>(D.shape[0]) * dyz);
        for (long long c = 0; c < n_index; ++c) {
            const long long r = c % dyz;
            if (q(c, D.div_yz) != c / dyz || q(r, D.div_z) != r / dz)
                throw std::runtime_error("cell index division constants failed their check");
        }
    }
    if (mesh) upload_mesh(mesh_rough);
    for (int f = 0; f < 6 && !mesh; ++f) {
        const Facet& F = domain_->facets()[f];
        D.cond[f] = F.condition;
        D.pair[f] = F.pair;
        D.reservoir[f] = F.reservoir;
        for (int k = 0; k < 3; ++k) D.shift[f][k] = F.shift[k];
        for (size_t m = 0; m < P_.mats.size(); ++m) D.rough_table[m][f] = P_.rough.facet_table[m * 6 + f];
    }
    D.layout_axis = P_.layout.axis;
    D.n_planes = static_cast<int>(P_.layout.planes.size());
    for (int k = 0; k < D.n_planes; ++k) D.planes[k] = P_.layout.planes[k];
    for (size_t k = 0; k < P_.plane_cell.size(); ++k) D.plane_cell[k] = P_.plane_cell[k];
    // interface banks
    DevInterface& I = T.iface;
    I.enabled = P_.iface.enabled ? 1 : 0;
    I.linearized = P_.iface.linearized ? 1 : 0;
    I.axis = P_.iface.axis;
    I.band_width = P_.iface.band_width;
    for (size_t m = 0; m < P_.iface.banks.size(); ++m)
        for (int dir = 0; dir < 2; ++dir) {
            const InterfaceBank& B = P_.iface.banks[m][dir];
            for (double w : B.omega)
                if (!std::isfinite(w) || w < 0) throw std::invalid_argument("Invalid shared interface frequency band.");
            I.bank[m][dir].omega = upload(B.omega);
            I.bank[m][dir].active = upload(B.active);
            I.bank[m][dir].prefix = upload(B.prefix);
            I.bank[m][dir].n = static_cast<int>(B.omega.size());
        }
    I.model = P_.iface.model;
    I.amm_fraction = P_.iface.amm_fraction;
    for (size_t f = 0; f < P_.iface.amm.faces.size(); ++f)
        for (int side = 0; side < 2; ++side) {
            const auto& rows = P_.iface.amm.faces[f].rows[side];
            std::vector<int> refl, start{0}, dest;
            std::vector<double> prob;
            for (const AmmRow& r : rows) {
                refl.push_back(r.reflected);
                for (const auto& e : r.transmitted) {
                    dest.push_back(e.first);
                    prob.push_back(e.second);
                }
                start.push_back(static_cast<int>(dest.size()));
            }
            I.amm[f][side] = {upload(refl), upload(start), upload(dest), upload(prob)};
        }
    // params
    DevParams& p = T.par;
    p.dt = cfg_.time_step;
    p.dt32 = static_cast<float>(cfg_.time_step);
    p.push_eps = P_.push_eps;
    p.seed = cfg_.random_seed;
    p.conservative = P_.conservative;
    p.linearized = P_.linearized;
    p.one_to_one = P_.one_to_one;
    p.n_materials = static_cast<int>(P_.mats.size());
    p.n_reservoirs = static_cast<int>(P_.reservoirs.size());
    p.lifetime_local = cfg_.lifetime_temperature_is_local;
    p.lifetime_T = cfg_.lifetime_temperature;
    p.background_T = cfg_.background_temperature;
    p.gradient_axis = P_.kappa_axis;
    p.gradient_energy_weight = P_.gradient_energy_weight;
    p.source_enabled = P_.source.enabled ? 1 : 0;
    p.source_spectrum = P_.source.spectrum == HeatSourceSpectrum::Weighted ? 1
                        : P_.source.spectrum == HeatSourceSpectrum::Gaussian ? 2 : 0;
    p.source_linearized = P_.source.linearized_thermal ? 1 : 0;
    p.source_pulsed = cfg_.heat_source_time_profile == HeatSourceTimeProfile::Pulsed ? 1 : 0;
    p.source_time_start = cfg_.heat_source_time_start;
    p.source_time_end = cfg_.heat_source_time_end;
    p.source_period = cfg_.heat_source_period;
    p.source_on = cfg_.heat_source_on_duration < 0.0 ? cfg_.heat_source_duty_cycle * cfg_.heat_source_period
                                                      : cfg_.heat_source_on_duration;
    p.source_amplitude = cfg_.heat_source_amplitude;
    PHMC_CUDA(cudaMalloc(&d_tables_, sizeof(DevTables)));
    PHMC_CUDA(cudaMemcpyAsync(d_tables_, &tables_, sizeof(DevTables), cudaMemcpyHostToDevice, stream_));

    // cells
    CellArrays& C = cells_;
    C.ncells = ncells_;
    C.hist_modes = hist_modes;
    C.mixed = mixed_ ? 1 : 0;
    C.cell_material = upload(P_.cell_material);
    C.volume = upload(domain_->grid_volumes());
    const size_t hist = static_cast<size_t>(ncells_) * hist_modes;
    const bool rta = !P_.linearized && !P_.callaway_nonlinear;
    C.bins = dalloc<BinSum>(hist);
    C.ab = dalloc<double2>(hist);
    C.hM = rta ? dalloc<double>(hist) : nullptr;
    C.energy = dalloc<double>(ncells_);
    C.temperature = dalloc<double>(ncells_);
    C.energy_final = dalloc<double>(ncells_);
    C.temperature_final = dalloc<double>(ncells_);
    C.grad_ratio = dalloc<double>(ncells_);
    C.flux = dalloc<double>(3 * static_cast<size_t>(ncells_));
    C.cell_stats = dalloc<double>(4 * static_cast<size_t>(ncells_));
    if (P_.source.enabled) {
        C.src_rate = upload(P_.source.rates);
        // a cell of zero power never accrues a budget, so its halves only copy zeros
        std::vector<int> powered;
        for (int c = 0; c < ncells_; ++c)
            if (P_.source.rates[c] > 0.0) powered.push_back(c);
        C.n_src_cells = static_cast<int>(powered.size());
        C.src_cells = powered.empty() ? nullptr : upload(powered);
        C.src_pending = dalloc<double>(ncells_);
        C.src_prescribed = dalloc<double>(ncells_);
        C.src_deposited = dalloc<double>(ncells_);
        C.src_step_pending = dalloc<double>(ncells_);
        C.src_step_book = dalloc<double>(2 * static_cast<size_t>(ncells_));
        C.src_classes = std::max(1, max_src_classes);
        C.src_scratch = dalloc<double>(static_cast<size_t>(ncells_) * 2 * C.src_classes);
        C.src_next = dalloc<double>(hist);
    }
    C.cell_final = dalloc<double>(4 * static_cast<size_t>(ncells_));
    C.final_blocks = std::max(1, std::min(256, (ncells_ + 255) / 256));
    C.final_part = dalloc<double>(4 * static_cast<size_t>(C.final_blocks));
    C.final_done = dalloc<unsigned>(1);
    if (rta) {
        // per-cell class sums; the stride is the largest class count of the materials
        int max_classes = 0;
        for (const auto& M : P_.mats) max_classes = std::max(max_classes, M.n_classes);
        C.n_classes = max_classes; // == bins per cell
        C.rta_ab = dalloc<double2>(static_cast<size_t>(ncells_) * max_classes);
        C.rta_cell_cap = rta_cell_capacity(C, cfg_.rta_cell_update);
        if (C.rta_cell_cap) prepare_rta_cell(C);
    } else if (P_.callaway_nonlinear) {
        // composed (alpha, beta) per (cell, mode) and the moment-solve work space
        C.n_classes = hist_modes;
        C.rta_ab = dalloc<double2>(hist);
        ncl_.work = dalloc<double2>(hist);
    } else {
        C.lin_beta = dalloc<double>(hist);
        const int S = std::max(1, static_cast<int>(std::ceil(cfg_.time_step * r_max)));
        const double h = cfg_.time_step / S;
        const double x = h * r_max;
        // smallest K with x^(K+1)/(K+1)! <= 1e-17 (x = h * max rate <= 1)
        int K = 1;
        double bound = x;
        while (K < 40) {
            bound = bound * x / (K + 1);
            if (bound <= 1e-17) break;
            ++K;
        }
        C.lin_substeps = S;
        C.lin_h = h;
        C.lin_terms = std::max(1, K);
        // per-mode constants of every material at offset material * hist_modes
        const size_t nmat = P_.mats.size(), hm = static_cast<size_t>(hist_modes);
        std::vector<double> decay(nmat * hm, 1.0), sc(nmat * hm, 0.0), srn(nmat * hm, 0.0), srr(nmat * hm, 0.0);
        std::vector<float> inv_s(nmat * hm, 0.0f), rate(nmat * hm, 0.0f), dec(nmat * hm, 1.0f), soh(nmat * hm, 0.0f),
            basis(nmat * 5 * hm, 0.0f), rn(nmat * hm, 0.0f), rr(nmat * hm, 0.0f);
        std::vector<double> omd(nmat * hm, 0.0), bg(nmat * hm, 0.0);
        bool has_normal = false;
        for (size_t mi = 0; mi < nmat; ++mi) {
            const MaterialTables& Mt = P_.mats[mi];
            const size_t o = mi * hm;
            for (int a = 0; a < Mt.n_active; ++a) {
                decay[o + a] = std::exp(-(Mt.col_normal[a] + Mt.col_resistive[a]) * cfg_.time_step);
                sc[o + a] = std::sqrt(Mt.col_capacity[a]);
                srn[o + a] = std::sqrt(Mt.col_normal[a]);
                srr[o + a] = std::sqrt(Mt.col_resistive[a]);
                has_normal = has_normal || Mt.col_normal[a] > 0.0;
                const double hw = Mt.hw[a];
                inv_s[o + a] = sc[o + a] > 0.0 ? static_cast<float>(1.0 / sc[o + a]) : 0.0f;
                rate[o + a] = static_cast<float>(Mt.col_normal[a] + Mt.col_resistive[a]);
                dec[o + a] = static_cast<float>(decay[o + a]);
                soh[o + a] = hw > 0.0 ? static_cast<float>(sc[o + a] / hw) : 0.0f;
                basis[(mi * 5) * hm + a] = static_cast<float>(sc[o + a] * srr[o + a]);
                for (int b = 0; b < 4; ++b) {
                    const double kb = b == 0 ? 1.0 : (Mt.omega[a] != 0.0 ? Mt.col_k[3 * a + b - 1] / Mt.omega[a] : 0.0);
                    basis[(mi * 5 + 1 + b) * hm + a] = static_cast<float>(sc[o + a] * kb * srn[o + a]);
                }
                rn[o + a] = static_cast<float>(srn[o + a]);
                rr[o + a] = static_cast<float>(srr[o + a]);
                omd[o + a] = 1.0 - decay[o + a];
                bg[o + a] = omd[o + a] * Mt.nbg[a];
            }
        }
        C.lin_decay = upload(decay);
        C.lin_s = upload(sc);
        C.lin_sqrt_rn = upload(srn);
        C.lin_sqrt_rr = upload(srr);
        C.lin_has_normal = has_normal ? 1 : 0;
        C.lin32_inv_s = upload(inv_s);
        C.lin32_rate = upload(rate);
        C.lin32_decay = upload(dec);
        C.lin32_s_over_hw = upload(soh);
        C.lin32_basis = upload(basis);
        C.lin32_sqrt_rn = upload(rn);
        C.lin32_sqrt_rr = upload(rr);
        C.lin_omd = upload(omd);
        C.lin_bg = upload(bg);
        C.lin_cluster = linear_cluster_size(C, mixed_);
        if (C.lin_cluster == 0) {
            // a cell's modes exceed the shared memory of a 16-CTA cluster: the
            // per-mode vectors live in a global work area, 16 CTAs per cell
            C.lin_cluster = 16;
            lin_slice_ = linear_global_slice(C, mixed_);
            lin_work_ = dalloc<unsigned char>(static_cast<size_t>(ncells_) * 16 * lin_slice_);
        }
        prepare_linear_solve(C, lin_work_ != nullptr);
    }
}

// Facet arrays, rough tables, voxel map, face BVH and star simplices of a mesh domain.
void DeviceSolver::upload_mesh(const std::vector<DevRoughTable>& rough) {
    DevFacets& G = tables_.fac;
    fill_dev_facets(*domain_, tables_.dom.scale, G, [&](const auto& v) { return upload(v); });
    G.rough_table = upload(P_.rough.facet_table);
    G.rough = upload(rough);
    G.mirror = mesh_mirror_;
    G.hit_t = mesh_hit_t_;
    G.hit_x = mesh_hit_x_;
    G.hit_y = mesh_hit_y_;
    G.hit_z = mesh_hit_z_;
    G.hit_f = mesh_hit_f_;
}

LaunchCtx DeviceSolver::ctx() const {
    LaunchCtx x;
    x.T = d_tables_;
    x.Th = &tables_;
    x.S = state_;
    x.C = cells_;
    x.L = d_ledger_;
    x.stream = stream_;
    // grid-stride carrier kernels: 8 CTAs of 256 per SM, fewer for small
    // populations (about four carriers per thread), so small instances of a
    // batch do not launch idle CTAs
    const long long want = (static_cast<long long>(state_.capacity) + 1023) / 1024;
    x.grid_blocks = static_cast<int>(std::max<long long>(8, std::min<long long>(sm_count_ * 8, want)));
    // event kernels: the CTAs resident in one wave (their queues are short)
    x.event_grid = static_cast<int>(std::max<long long>(1, std::min<long long>(sm_count_, want)));
    // the box carrier pass: tuned threads per CTA and resident CTAs per SM, at
    // least about four carriers per thread for small populations
    const int tk = mixed_ ? 1 : 0;
    x.transport_block = cfg_.transport_block > 0 ? cfg_.transport_block : tuning::kTransportBlock[tk];
    const int per_sm = cfg_.transport_blocks_per_sm > 0 ? std::min(cfg_.transport_blocks_per_sm, 16)
                                                        : tuning::kTransportBlocksPerSm[tk];
    const long long want_pass = (static_cast<long long>(state_.capacity) + 4LL * x.transport_block - 1) /
                                (4LL * x.transport_block);
    x.transport_grid = static_cast<int>(std::max<long long>(8, std::min<long long>(sm_count_ * per_sm, want_pass)));
    x.tally_agg = cfg_.tally_aggregation > 0 || (cfg_.tally_aggregation == 0 && tuning::kTallyAggregation[tk] > 0);
    // TMA-staged tiles of 256 carriers (mixed state), one CTA per tile slot
    x.transport_pipe = mixed_ && (cfg_.transport_pipeline > 0 ||
                                  (cfg_.transport_pipeline == 0 && tuning::kTransportPipeline > 0));
    const long long tiles = (static_cast<long long>(state_.capacity) + 255) / 256;
    x.pipe_grid = static_cast<int>(std::max<long long>(1, std::min<long long>(sm_count_ * per_sm, tiles)));
    x.mesh = domain_->is_mesh();
    x.ncl = P_.callaway_nonlinear ? &ncl_ : nullptr;
    x.lin_work = lin_work_;
    x.lin_slice = lin_slice_;
    return x;
}

int DeviceSolver::collision_kind() const {
    return P_.callaway_nonlinear ? kCollideNonlinear : P_.linearized ? kCollideLinear : kCollideRta;
}

void DeviceSolver::initial_statistics() {
    const LaunchCtx x = ctx();
    launch_histogram(x, collision_kind() == kCollideRta);
    counters_.launches += 2 + launch_cell_solve(x, 0, collision_kind());
    launch_cells_final(x, 0);
    if (P_.source.enabled) {
        // first heat-source half of the coming step (src/MonteCarloSolver.cpp:364-370)
        launch_source(x, true, true);
        counters_.launches += 1;
    }
    materialized_ = true;
}

// Device address of registered (pinned or mapped) host memory, or null.
static const void* mapped_host(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void DeviceSolver::set_carriers(long long n, const double* x, const double* y, const double* z, const double* occ,
                                const uint32_t* mode, const uint8_t* alive, bool keep_clock) {
    if (n < 0 || n > state_.capacity) throw std::invalid_argument("carrier count exceeds device capacity");
    const LaunchCtx c = ctx();
    if (keep_clock) {
        launch_ledger_replace(c, static_cast<int>(n));
        counters_.launches += 1;
    } else {
        DevLedger L{};
        L.n_slots = static_cast<int>(n);
        for (size_t r = 0; r < P_.reservoirs.size(); ++r) L.previous_res[r] = P_.reservoirs[r].initial_count;
        PHMC_CUDA(cudaMemcpyAsync(d_ledger_, &L, sizeof L, cudaMemcpyHostToDevice, stream_));
        step_ = 0;
        elapsed_ = 0;
    }
    failed_ = false;
    HostCarriers h{};
    h.x = static_cast<const double*>(mapped_host(x));
    h.y = static_cast<const double*>(mapped_host(y));
    h.z = static_cast<const double*>(mapped_host(z));
    h.occ = static_cast<const double*>(mapped_host(occ));
    h.mode = static_cast<const uint32_t*>(mapped_host(mode));
    h.alive = static_cast<const uint8_t*>(mapped_host(alive));
    if (h.x && h.y && h.z && h.occ && h.mode && (h.alive || !alive)) {
        // registered host arrays: one kernel reads them over the link
        launch_ingest(c, mixed_, h);
    } else {
        PHMC_CUDA(cudaMemcpyAsync(state_.x, x, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
        PHMC_CUDA(cudaMemcpyAsync(state_.y, y, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
        PHMC_CUDA(cudaMemcpyAsync(state_.z, z, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
        PHMC_CUDA(cudaMemcpyAsync(state_.occ, occ, n * sizeof(double), cudaMemcpyHostToDevice, stream_));
        PHMC_CUDA(cudaMemcpyAsync(state_.mode, mode, n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_));
        if (alive) PHMC_CUDA(cudaMemcpyAsync(state_.alive, alive, n * sizeof(uint8_t), cudaMemcpyHostToDevice, stream_));
        else PHMC_CUDA(cudaMemsetAsync(state_.alive, 1, n * sizeof(uint8_t), stream_));
        launch_init_cells(c, mixed_);
    }
    counters_.launches += 1 + launch_mesh_cache_init(c, mixed_);
    initial_statistics();
    if (!keep_clock) synchronize();
}

// The launches of one timestep (src/MonteCarloSolver.cpp:348-398): transport,
// injection, cell solve, heat-source halves, ledger. Step-dependent values
// (draw counter, time windows) are read on the device, so the same sequence is
// captured once into a graph and replayed.
void DeviceSolver::enqueue_step(bool profile) {
    const LaunchCtx x = ctx();
    const int coll = collision_kind();
    launch_step_begin(x);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profile) {
        PHMC_CUDA(cudaEventCreate(&e0));
        PHMC_CUDA(cudaEventCreate(&e1));
        PHMC_CUDA(cudaEventRecord(e0, stream_));
    }
    counters_.launches += 1 + launch_transport(x, mixed_, coll == kCollideRta);
    if (profile) {
        PHMC_CUDA(cudaEventRecord(e1, stream_));
        pass_a_events_.push_back({e0, e1});
    }
    if (!P_.reservoirs.empty())
        counters_.launches += launch_inject(x, mixed_, coll == kCollideRta, d_holes_, d_block_dead_, state_.capacity);
    counters_.launches += 1 + launch_cell_solve(x, 1, coll);
    if (P_.source.enabled) {
        // second heat-source half of this step, after the collision (src/MonteCarloSolver.cpp:376)
        launch_source(x, false, false);
        counters_.launches += 1;
    }
    launch_cells_final(x, 1);
    if (P_.source.enabled) {
        // first half of the next step, folded into the pending update
        launch_source(x, true, true);
        counters_.launches += 1;
    }
}

void DeviceSolver::capture_step_graph() {
    const long long l0 = counters_.launches;
    PHMC_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    try {
        enqueue_step(false);
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        counters_.launches = l0;
        throw;
    }
    PHMC_CUDA(cudaStreamEndCapture(stream_, &graph_));
    PHMC_CUDA(cudaGraphInstantiate(&graph_exec_, graph_, 0));
    graph_launches_ = counters_.launches - l0;
    counters_.launches = l0;
}

bool DeviceSolver::fusable() const {
    // fused batch steps run no carrier sorts: instances that sort step on their own graphs
    return !domain_->is_mesh() && P_.mats.size() == 1 && !P_.linearized && !P_.source.enabled &&
           !cfg_.temperature_gradient.has_value() && collision_kind() == kCollideRta && sort_interval_ == 0;
}

int DeviceSolver::carrier_blocks() const { return ctx().grid_blocks; }

bool DeviceSolver::batch_extras_due() const {
    const int next = step_ + 1;
    return step_ % 100 == 0 || next == 1 || next % cfg_.convergence_write_interval == 0;
}

void DeviceSolver::finish_batched_step(long long launches) {
    if (failed_) throw std::runtime_error("Cannot resume a failed timestep; construct a new solver after fixing its cause.");
    counters_.launches += launches;
    if (step_ % 100 == 0) counters_.launches += launch_containment(ctx(), mixed_, d_holes_, d_contain_count_);
    materialized_ = false;
    ++step_;
    elapsed_ += cfg_.time_step;
    if (step_ == 1 || step_ % cfg_.convergence_write_interval == 0) flux_pass();
}

void DeviceSolver::set_schedule(int sort_interval, int transport_block, int blocks_per_sm, int tally_aggregation,
                                int transport_pipeline) {
    if (transport_block != 0 && transport_block != 128 && transport_block != 256 && transport_block != 512)
        throw std::invalid_argument("transport_block must be 0 (tuned), 128, 256 or 512 threads");
    if (blocks_per_sm < 0 || blocks_per_sm > 16) throw std::invalid_argument("transport_blocks_per_sm must be in [0, 16]");
    synchronize();
    cfg_.carrier_sort_interval = sort_interval;
    cfg_.transport_block = transport_block;
    cfg_.transport_blocks_per_sm = blocks_per_sm;
    cfg_.tally_aggregation = tally_aggregation;
    cfg_.transport_pipeline = transport_pipeline;
    sort_interval_ = resolved_sort_interval(cfg_, mixed_);
    // the captured step bakes in the launch shapes: capture again at the next step
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    graph_exec_ = nullptr;
    graph_ = nullptr;
}

void DeviceSolver::sort_carriers() {
    if (sort_.capacity != state_.capacity) {
        const int slot_bytes = carrier_slot_bytes(ctx(), mixed_);
        void* p = nullptr;
        PHMC_CUDA(cudaMalloc(&p, SortScratch::bytes_for(state_.capacity, slot_bytes)));
        allocations_.push_back(p);
        sort_.carve(p, state_.capacity, slot_bytes);
    }
    int modes = 1;
    for (const PhononMaterial* m : mats_) modes = std::max(modes, m->active_mode_count());
    counters_.launches += launch_carrier_sort(ctx(), sort_, ncells_, modes, domain_->is_mesh(), mixed_);
}

void DeviceSolver::run_timestep() {
    if (failed_) throw std::runtime_error("Cannot resume a failed timestep; construct a new solver after fixing its cause.");
    failed_ = true;
    // stable carrier sort at the start of every sort_interval_-th step (resolved_sort_interval)
    if (sort_interval_ > 0 && step_ % sort_interval_ == 0) sort_carriers();
    if (use_graphs_ && !profile_pass_a_) {
        if (!graph_exec_) capture_step_graph();
        PHMC_CUDA(cudaGraphLaunch(graph_exec_, stream_));
        counters_.launches += graph_launches_;
    } else {
        enqueue_step(profile_pass_a_);
    }
    // src/solver/TransportOperator.cpp:364-402, every 100 steps (the free-slot
    // list of the injection is the queue: it is rebuilt before its next use)
    if (step_ % 100 == 0) counters_.launches += launch_containment(ctx(), mixed_, d_holes_, d_contain_count_);
    materialized_ = false;
    ++step_;
    elapsed_ += cfg_.time_step;
    if (step_ == 1 || step_ % cfg_.convergence_write_interval == 0) flux_pass();
    failed_ = false;
}

void DeviceSolver::materialize() {
    if (materialized_) return;
    launch_apply_pending(ctx(), true);
    counters_.launches += 2;
    materialized_ = true;
}

double DeviceSolver::collide_only(const double* cell_temperature) {
    const LaunchCtx x = ctx();
    launch_step_begin(x);
    launch_histogram(x, collision_kind() == kCollideRta);
    int phase = 1;
    if (cell_temperature) {
        PHMC_CUDA(cudaMemcpyAsync(cells_.temperature, cell_temperature, ncells_ * sizeof(double),
                                  cudaMemcpyHostToDevice, stream_));
        phase = 2;
    }
    counters_.launches += 5 + launch_cell_solve(x, phase, collision_kind());
    launch_cells_final(x, phase);
    launch_apply_pending(x, false);
    synchronize();
    double r = 0;
    PHMC_CUDA(cudaMemcpy(&r, &d_ledger_->step_lifetime_residual, sizeof(double), cudaMemcpyDeviceToHost));
    materialized_ = true;
    return r;
}

double DeviceSolver::drive_only() {
    const LaunchCtx x = ctx();
    double r = 0;
    synchronize();
    PHMC_CUDA(cudaMemcpy(&r, &d_ledger_->next_drive_ev, sizeof(double), cudaMemcpyDeviceToHost));
    launch_apply_pending(x, false);
    counters_.launches += 2;
    synchronize();
    materialized_ = true;
    return r;
}

void DeviceSolver::timed_run(int steps, double& total_ms, double& kernel_ms, long long& launches,
                             long long& live_before, long long& live_after) {
    // carrier-pass duration from a few eager steps with events around it
    const int profiled = std::max(1, std::min(steps, 3));
    profile_pass_a_ = true;
    run(profiled);
    profile_pass_a_ = false;
    synchronize();
    kernel_ms = 0;
    for (auto& ev : pass_a_events_) {
        float k = 0;
        PHMC_CUDA(cudaEventElapsedTime(&k, ev.first, ev.second));
        kernel_ms += k;
        cudaEventDestroy(ev.first);
        cudaEventDestroy(ev.second);
    }
    kernel_ms /= static_cast<double>(pass_a_events_.size() ? pass_a_events_.size() : 1);
    pass_a_events_.clear();
    // the timed region: `steps` steps (graph replays), events on the solver stream
    DevLedger L;
    PHMC_CUDA(cudaMemcpy(&L, d_ledger_, sizeof L, cudaMemcpyDeviceToHost));
    live_before = L.particle_count;
    cudaEvent_t a, b;
    PHMC_CUDA(cudaEventCreate(&a));
    PHMC_CUDA(cudaEventCreate(&b));
    const long long l0 = counters_.launches;
    PHMC_CUDA(cudaEventRecord(a, stream_));
    run(steps);
    PHMC_CUDA(cudaEventRecord(b, stream_));
    synchronize();
    float ms = 0;
    PHMC_CUDA(cudaEventElapsedTime(&ms, a, b));
    total_ms = ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    launches = counters_.launches - l0;
    PHMC_CUDA(cudaMemcpy(&L, d_ledger_, sizeof L, cudaMemcpyDeviceToHost));
    live_after = L.particle_count;
}

void DeviceSolver::run(int steps) {
    for (int k = 0; k < steps; ++k) run_timestep();
}

void DeviceSolver::synchronize() {
    PHMC_CUDA(cudaStreamSynchronize(stream_));
    drain_observations(true);
    check_error();
}

// Stored position of one carrier slot (FP64 positions, or cell corner plus the
// FP32 offset in the mixed path) and its cached wall facet (mesh domains, else -1).
void DeviceSolver::carrier_position(int slot, double p[3], int& facet) {
    facet = -1;
    if (mixed_) {
        int c = 0;
        float o[3];
        PHMC_CUDA(cudaMemcpy(&c, state_.cell + slot, sizeof(int), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&o[0], state_.ox + slot, sizeof(float), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&o[1], state_.oy + slot, sizeof(float), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&o[2], state_.oz + slot, sizeof(float), cudaMemcpyDeviceToHost));
        const DevDomain& D = tables_.dom;
        if (mesh_hit_f_) {
            // offsets of a mesh carrier are measured from its cell's home voxel
            if (cell_voxel_host_.empty()) cell_voxel_host_ = domain_->cell_voxels();
            if (c >= 0 && c < static_cast<int>(cell_voxel_host_.size())) c = cell_voxel_host_[c];
            PHMC_CUDA(cudaMemcpy(&facet, mesh_hit_f_ + slot, sizeof(int), cudaMemcpyDeviceToHost));
        }
        const int idx[3] = {c / (D.shape[1] * D.shape[2]), (c / D.shape[2]) % D.shape[1], c % D.shape[2]};
        for (int a = 0; a < 3; ++a) p[a] = D.lo[a] + idx[a] * D.cell_size[a] + static_cast<double>(o[a]);
        return;
    }
    PHMC_CUDA(cudaMemcpy(&p[0], state_.x + slot, sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(&p[1], state_.y + slot, sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(&p[2], state_.z + slot, sizeof(double), cudaMemcpyDeviceToHost));
    if (mesh_hit_f_) PHMC_CUDA(cudaMemcpy(&facet, mesh_hit_f_ + slot, sizeof(int), cudaMemcpyDeviceToHost));
}

void DeviceSolver::carrier_state(long long slot, double out[13]) {
    if (slot < 0 || slot >= state_.capacity) throw std::invalid_argument("carrier slot out of range");
    PHMC_CUDA(cudaStreamSynchronize(stream_));
    const int i = static_cast<int>(slot);
    int facet = -1;
    double p[3];
    carrier_position(i, p, facet);
    double occ = 0;
    uint32_t w = 0;
    int32_t c = 0;
    uint8_t a = 0;
    PHMC_CUDA(cudaMemcpy(&occ, state_.occ + i, sizeof occ, cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(&w, state_.mode + i, sizeof w, cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(&c, state_.cell + i, sizeof c, cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(&a, state_.alive + i, sizeof a, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 3; ++k) out[k] = p[k];
    out[3] = occ;
    out[4] = static_cast<double>(w);
    out[5] = c;
    out[6] = a;
    for (int k = 7; k < 13; ++k) out[k] = k == 11 || k == 12 ? -1.0 : 0.0;
    if (mesh_hit_t_) {
        double t = 0, h[3] = {0, 0, 0};
        int32_t mir = -1;
        PHMC_CUDA(cudaMemcpy(&t, mesh_hit_t_ + i, sizeof t, cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&h[0], mesh_hit_x_ + i, sizeof(double), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&h[1], mesh_hit_y_ + i, sizeof(double), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&h[2], mesh_hit_z_ + i, sizeof(double), cudaMemcpyDeviceToHost));
        PHMC_CUDA(cudaMemcpy(&mir, mesh_mirror_ + i, sizeof mir, cudaMemcpyDeviceToHost));
        out[7] = t;
        for (int k = 0; k < 3; ++k) out[8 + k] = h[k];
        out[11] = facet;
        out[12] = mir;
    }
}

// Device errors surface at the next host synchronisation with the text of the
// reference's exceptions; carrier errors name the slot and its position as
// src/solver/TransportOperator.cpp:252-284 and :364-402 name the particle.
void DeviceSolver::check_error() {
    int code = 0, slot = 0;
    PHMC_CUDA(cudaMemcpy(&code, &d_ledger_->error_code, sizeof(int), cudaMemcpyDeviceToHost));
    if (!code) return;
    PHMC_CUDA(cudaMemcpy(&slot, &d_ledger_->error_slot, sizeof(int), cudaMemcpyDeviceToHost));
    failed_ = true;
    if ((code == kErrTooManyEvents || code == kErrEscaped || code == kErrIntersection) && slot >= 0 &&
        slot < state_.capacity) {
        double p[3];
        int facet = -1;
        carrier_position(slot, p, facet);
        const std::string at = "(" + std::to_string(p[0]) + ", " + std::to_string(p[1]) + ", " +
                               std::to_string(p[2]) + ")";
        const std::string cached = facet >= 0 ? ", cached facet=" + std::to_string(facet) : std::string();
        if (code == kErrTooManyEvents)
            throw std::runtime_error("Particle " + std::to_string(slot) + " exceeded 64 transport events in one timestep at " +
                                     at + cached + ". Reduce simulation.time_step or inspect narrow STL features; no "
                                     "recovery was applied.");
        if (code == kErrEscaped)
            throw std::runtime_error("Particle " + std::to_string(slot) + " escaped the domain at " + at + cached +
                                     ". Refusing to relocate or rethermalize it; inspect the geometry and time step.");
        throw std::runtime_error("Boundary intersection failed while advancing particles for particle " +
                                 std::to_string(slot) + " at " + at + ". Check that the STL is closed and manifold.");
    }
    throw std::runtime_error(std::string(error_message(code)) + " (carrier slot or cell " + std::to_string(slot) + ")");
}

// Heat flux tally at step 1 and every convergence_write_interval steps. The
// device results and the ledger are copied into a pinned slot; the host part
// (flux average, kappa, convergence.txt row) runs when the slot's event has
// completed, so stepping never waits on it.
void DeviceSolver::flux_pass() {
    drain_observations(false);
    Observation* o;
    if (!obs_free_.empty()) {
        o = obs_free_.back();
        obs_free_.pop_back();
    } else if (obs_pending_.size() >= 8) {
        drain_observations(true);
        o = obs_free_.back();
        obs_free_.pop_back();
    } else {
        o = new Observation;
        PHMC_CUDA(cudaMallocHost(&o->T, ncells_ * sizeof(double)));
        PHMC_CUDA(cudaMallocHost(&o->E, ncells_ * sizeof(double)));
        PHMC_CUDA(cudaMallocHost(&o->q, 3 * ncells_ * sizeof(double)));
        PHMC_CUDA(cudaMallocHost(&o->L, sizeof(DevLedger)));
        if (P_.source.enabled) PHMC_CUDA(cudaMallocHost(&o->src, 3 * ncells_ * sizeof(double)));
        PHMC_CUDA(cudaEventCreateWithFlags(&o->done, cudaEventDisableTiming));
    }
    o->step = step_;
    o->elapsed = elapsed_;
    const LaunchCtx x = ctx();
    PHMC_CUDA(cudaMemsetAsync(cells_.flux, 0, 3 * sizeof(double) * ncells_, stream_));
    launch_flux(x, mixed_);
    counters_.launches += 1;
    PHMC_CUDA(cudaMemcpyAsync(o->T, cells_.temperature_final, ncells_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    PHMC_CUDA(cudaMemcpyAsync(o->E, cells_.energy_final, ncells_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    PHMC_CUDA(cudaMemcpyAsync(o->q, cells_.flux, 3 * ncells_ * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    PHMC_CUDA(cudaMemcpyAsync(o->L, d_ledger_, sizeof(DevLedger), cudaMemcpyDeviceToHost, stream_));
    if (o->src) {
        const size_t b = ncells_ * sizeof(double);
        PHMC_CUDA(cudaMemcpyAsync(o->src, cells_.src_step_book, 2 * b, cudaMemcpyDeviceToHost, stream_));
        PHMC_CUDA(cudaMemcpyAsync(o->src + 2 * ncells_, cells_.src_step_pending, b, cudaMemcpyDeviceToHost, stream_));
    }
    PHMC_CUDA(cudaEventRecord(o->done, stream_));
    obs_pending_.push_back(o);
}

void DeviceSolver::drain_observations(bool wait) {
    while (!obs_pending_.empty()) {
        Observation* o = obs_pending_.front();
        if (wait) PHMC_CUDA(cudaEventSynchronize(o->done));
        else {
            const cudaError_t q = cudaEventQuery(o->done);
            if (q == cudaErrorNotReady) return;
            PHMC_CUDA(q);
        }
        obs_pending_.erase(obs_pending_.begin());
        process_observation(*o);
        obs_free_.push_back(o);
    }
}

void DeviceSolver::process_observation(Observation& o) {
    host_T_.assign(o.T, o.T + ncells_);
    host_E_.assign(o.E, o.E + ncells_);
    host_q_.assign(o.q, o.q + 3 * static_cast<size_t>(ncells_));
    // src/solver/GridStatistics.cpp:334-343 and src/solver/Observables.cpp:38-144
    const auto& vol = domain_->grid_volumes();
    const int axis = P_.kappa_axis;
    double phi = 0, tv = 0;
    for (int c = 0; c < ncells_; ++c) {
        for (int k = 0; k < 3; ++k) host_q_[3 * c + k] = host_q_[3 * c + k] * (1.0 / vol[c]) * 1.602176634e13;
        phi += host_q_[3 * c + axis] * vol[c];
        tv += vol[c];
    }
    avg_flux_ = phi / tv;
    update_kappa();
    if (!cfg_.output_folder.empty()) {
        phmc_stats s;
        stats_from_ledger(*o.L, s);
        append_convergence_row(o, s);
    }
}

// kappa_eff from the reservoir temperatures (or the imposed gradient) and
// kappa_int from the fitted cell-temperature slope (src/solver/Observables.cpp:38-144).
void DeviceSolver::update_kappa() {
    const int axis = P_.kappa_axis;
    kappa_fit_ = kappa_end_ = 0;
    if (!cfg_.compute_kappa) return;
    if (cfg_.temperature_gradient) {
        kappa_end_ = -avg_flux_ / *cfg_.temperature_gradient;
        return;
    }
    double Tl = host_T_.front(), Tr = host_T_.back();
    const auto& rf = domain_->reservoir_facets();
    if (rf.size() >= 2) {
        int fl = rf.front(), fr = rf.front();
        for (int f : rf) {
            if (domain_->facets()[f].centroid[axis] < domain_->facets()[fl].centroid[axis]) fl = f;
            if (domain_->facets()[f].centroid[axis] > domain_->facets()[fr].centroid[axis]) fr = f;
        }
        Tl = domain_->facets()[fl].value;
        Tr = domain_->facets()[fr].value;
    }
    const double L = std::abs(domain_->bounds_max()[axis] - domain_->bounds_min()[axis]) * 1e-10;
    const double ge = std::abs(L) > 1e-24 ? (Tr - Tl) / L : 0.0;
    kappa_end_ = std::abs(ge) > 1e-18 ? -avg_flux_ / ge : 0.0;
    double sx = 0, st = 0, sxx = 0, sxt = 0;
    for (int c = 0; c < ncells_; ++c) {
        const double xx = domain_->grid_centers()[c][axis] * 1e-10;
        sx += xx;
        st += host_T_[c];
        sxx += xx * xx;
        sxt += xx * host_T_[c];
    }
    double gf = 0;
    if (ncells_ >= 2) {
        const double den = ncells_ * sxx - sx * sx;
        if (std::abs(den) > 1e-30 && std::abs(host_T_.back() - host_T_.front()) > 1e-6) gf = (ncells_ * sxt - sx * st) / den;
    }
    kappa_fit_ = std::abs(gf) > 1e-18 ? -avg_flux_ / gf : 0.0;
}

// Ledger-derived fields of phmc_stats.
void stats_from_ledger(const DevLedger& L, phmc_stats& o) {
    std::memset(&o, 0, sizeof o);
    o.particle_count = L.particle_count;
    o.absorbed_total = static_cast<int64_t>(L.total_absorbed);
    o.injected_total = static_cast<int64_t>(L.total_injected);
    o.step_absorbed = static_cast<int64_t>(L.step_absorbed);
    o.step_injected = static_cast<int64_t>(L.step_injected);
    o.step_absorbed_energy_ev = L.step_absorbed_ev;
    o.step_injected_energy_ev = L.step_injected_ev;
    o.total_thermal_energy_ev = L.thermal_energy;
    o.total_lifetime_energy_residual_ev = L.total_lifetime_residual;
    o.step_lifetime_energy_residual_ev = L.step_lifetime_residual;
    o.total_energy_balance_residual_ev = L.total_balance_residual;
    o.step_energy_balance_residual_ev = L.step_balance_residual;
    o.total_gradient_energy_ev = L.total_drive_ev;
    o.step_gradient_energy_ev = L.step_drive_ev;
    o.step_gradient_updates = static_cast<int64_t>(L.step_drive_updates);
    o.total_heat_source_energy_ev = L.total_source_ev;
    o.step_heat_source_energy_ev = L.step_source_ev;
    o.step_heat_source_updates = static_cast<int64_t>(L.step_source_updates);
    o.interface_events = static_cast<int64_t>(L.total_iface_events);
    o.interface_transmitted = static_cast<int64_t>(L.total_iface_transmitted);
    o.interface_reflected = static_cast<int64_t>(L.total_iface_reflected);
    for (int k = 0; k < kRoughCounters; ++k) o.rough_counts[k] = static_cast<int64_t>(L.total_rough[k]);
    o.collision_cache_corrections = static_cast<int64_t>(L.total_cache_corrections);
}

void DeviceSolver::read_stats(phmc_stats& o) {
    synchronize();
    DevLedger L;
    PHMC_CUDA(cudaMemcpy(&L, d_ledger_, sizeof L, cudaMemcpyDeviceToHost));
    stats_from_ledger(L, o);
    o.current_timestep = step_;
    o.average_heat_flux_along_axis = avg_flux_;
    o.kappa_fit = kappa_fit_;
    o.kappa_endpoints = kappa_end_;
    if (P_.source.enabled) {
        // budgets at the step boundary: the next step's first half is already accrued here
        std::vector<double> h(3 * static_cast<size_t>(ncells_));
        read_source_book(h.data());
        for (int c = 0; c < ncells_; ++c) {
            o.prescribed_heat_source_energy_ev += h[c];
            o.pending_heat_source_energy_ev += h[2 * ncells_ + c];
        }
    }
    o.device_launches = counters_.launches;
}

void DeviceSolver::read_cells(double* T, double* E, double* q3) {
    synchronize();
    if (T) PHMC_CUDA(cudaMemcpy(T, cells_.temperature_final, ncells_ * sizeof(double), cudaMemcpyDeviceToHost));
    if (E) PHMC_CUDA(cudaMemcpy(E, cells_.energy_final, ncells_ * sizeof(double), cudaMemcpyDeviceToHost));
    if (q3) std::copy(host_q_.begin(), host_q_.end(), q3);
}

long long DeviceSolver::slot_count() {
    synchronize();
    int n = 0;
    PHMC_CUDA(cudaMemcpy(&n, &d_ledger_->n_slots, sizeof(int), cudaMemcpyDeviceToHost));
    return n;
}

void DeviceSolver::get_carriers(double* x, double* y, double* z, double* occ, uint32_t* mode, int32_t* cell,
                                uint8_t* alive) {
    const long long n = slot_count();
    materialize();
    if (mixed_) {
        launch_positions_out(ctx());
        counters_.launches += 1;
    }
    synchronize();
    PHMC_CUDA(cudaMemcpy(x, state_.x, n * sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(y, state_.y, n * sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(z, state_.z, n * sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(occ, state_.occ, n * sizeof(double), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(mode, state_.mode, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(cell, state_.cell, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(alive, state_.alive, n * sizeof(uint8_t), cudaMemcpyDeviceToHost));
}

void DeviceSolver::append_convergence_row(const Observation& o, const phmc_stats& s) {
    if (cfg_.output_folder.empty()) return;
    ConvergenceRow r;
    r.timestep = o.step;
    r.time_ps = o.elapsed;
    r.temperatures = host_T_;
    r.heat_flux = avg_flux_;
    r.kappa_int = kappa_fit_;
    r.kappa_eff = kappa_end_;
    r.particle_count = s.particle_count;
    r.absorbed = s.step_absorbed;
    r.injected = s.step_injected;
    r.net = s.step_injected - s.step_absorbed;
    r.absorbed_ev = s.step_absorbed_energy_ev;
    r.injected_ev = s.step_injected_energy_ev;
    r.lifetime_residual = s.step_lifetime_energy_residual_ev;
    r.balance_residual = s.step_energy_balance_residual_ev;
    r.thermal_energy = s.total_thermal_energy_ev;
    r.gradient = cfg_.temperature_gradient.has_value();
    r.gradient_updates = s.step_gradient_updates;
    r.gradient_energy = s.step_gradient_energy_ev;
    r.source_updates = s.step_heat_source_updates;
    r.source_ev = s.step_heat_source_energy_ev;
    if (o.src) {
        // src/solver/PrescribedHeatSource.cpp:265-275: sums in cell order
        for (int c = 0; c < ncells_; ++c) {
            r.source_prescribed += o.src[c];
            r.source_deposited += o.src[ncells_ + c];
            r.source_pending += o.src[2 * ncells_ + c];
        }
    }
    const std::filesystem::path dir(cfg_.output_folder);
    std::ofstream(dir / "convergence.txt", std::ios::app) << format_convergence_row(r);
    if (cfg_.temperature_gradient || cfg_.write_cell_heat_flux)
        std::ofstream(dir / "grid_heat_flux.csv", std::ios::app) << format_cell_flux_rows(o.step, o.elapsed, host_T_, host_q_);
    if (o.src) write_source_ledger(o.src, o.src + ncells_, o.src + 2 * ncells_);
}

// Per-cell prescribed, deposited and pending heat-source energy at the step
// boundary (the device has already accrued, and maybe deposited, the next
// step's first half): [3 ncells].
void DeviceSolver::read_source_book(double* h) {
    synchronize();
    const size_t b = ncells_ * sizeof(double);
    PHMC_CUDA(cudaMemcpy(h, cells_.src_step_book, 2 * b, cudaMemcpyDeviceToHost));
    PHMC_CUDA(cudaMemcpy(h + 2 * ncells_, cells_.src_step_pending, b, cudaMemcpyDeviceToHost));
}

// heat_source_ledger.txt, rewritten with every convergence row and at the
// end of the run (src/solver/Diagnostics.cpp:206-224).
void DeviceSolver::write_source_ledger(const double* prescribed, const double* deposited, const double* pending) const {
    std::ofstream(std::filesystem::path(cfg_.output_folder) / "heat_source_ledger.txt")
        << format_source_ledger(cfg_, *domain_, P_.cell_material, P_.source.rates, prescribed, deposited, pending);
}

void DeviceSolver::write_outputs() {
    if (cfg_.output_folder.empty()) return;
    std::ofstream(std::filesystem::path(cfg_.output_folder) / "grid_centers.csv") << format_grid_centers(*domain_);
}

// The end of summary.txt (src/main.cpp:117-131, src/solver/Diagnostics.cpp:216-224):
// run time, then the run diagnostics.
void DeviceSolver::append_summary(long long total_seconds) {
    if (cfg_.output_folder.empty()) return;
    phmc_stats st;
    read_stats(st);
    RunSummary r;
    r.cfg = cfg_;
    r.random_seed = cfg_.random_seed;
    r.cache_corrections = st.collision_cache_corrections;
    // per step: one (cell, class) binning pass; cell temperatures at the
    // start (from the bins) and at the end of the step
    r.cell_index_rebuilds = step_ + 1;
    r.temperature_refreshes = 2LL * step_ + 1;
    for (int k = 0; k < 8; ++k) r.rough[k] = st.rough_counts[k];
    r.material_count = static_cast<int>(P_.mats.size());
    r.interface_frequency_bin_thz = cfg_.material_interface_frequency_bin_thz;
    r.conservative = P_.conservative;
    r.fixed_flux_reservoirs = !P_.one_to_one;
    if (P_.mats.size() > 1) r.material_carrier_volumes_a3 = P_.material_spatial_volume;
    r.interface_events = st.interface_events;
    r.interface_transmitted = st.interface_transmitted;
    r.interface_reflected = st.interface_reflected;
    r.absorbed_total = st.absorbed_total;
    r.injected_total = st.injected_total;
    DevLedger L;
    PHMC_CUDA(cudaMemcpy(&L, d_ledger_, sizeof L, cudaMemcpyDeviceToHost));
    r.absorbed_energy_ev = L.total_absorbed_ev;
    r.injected_energy_ev = L.total_injected_ev;
    r.initial_particle_count = P_.initial_particles;
    r.particle_count = st.particle_count;
    r.particle_spatial_weight_a3 = P_.particle_volume;
    r.background_temperature = cfg_.background_temperature;
    r.total_thermal_energy_ev = st.total_thermal_energy_ev;
    r.lifetime_residual_ev = st.total_lifetime_energy_residual_ev;
    r.balance_residual_ev = st.total_energy_balance_residual_ev;
    r.gradient_driven = cfg_.temperature_gradient.has_value();
    r.gradient_updates = static_cast<long long>(L.total_drive_updates);
    r.gradient_energy_ev = st.total_gradient_energy_ev;
    if (P_.source.enabled) {
        double rate = 0.0;
        for (double x : P_.source.rates) rate += x;
        r.source_base_power = rate / 6.241509074e6; // eV/ps per W
        r.source_prescribed = st.prescribed_heat_source_energy_ev;
        r.source_pending = st.pending_heat_source_energy_ev;
        r.source_deposited = st.total_heat_source_energy_ev;
    }
    r.source_updates_total = static_cast<long long>(L.total_source_updates);
    r.source_energy_total_ev = st.total_heat_source_energy_ev;
    r.source_updates_step = st.step_heat_source_updates;
    r.source_energy_step_ev = st.step_heat_source_energy_ev;
    std::ofstream out(std::filesystem::path(cfg_.output_folder) / "summary.txt", std::ios::app);
    out << format_runtime(total_seconds) << format_run_summary(r);
    if (!out) throw std::runtime_error("Cannot append runtime summary.txt.");
    if (P_.source.enabled) {
        std::vector<double> h(3 * static_cast<size_t>(ncells_));
        read_source_book(h.data());
        write_source_ledger(h.data(), h.data() + ncells_, h.data() + 2 * ncells_);
    }
}

} // namespace phmc
