// Text outputs of a run: the domain summary that opens summary.txt and
// grid_centers.csv (src/geometry/DomainOutput.cpp:12-241), and the run summary
// appended at the end (src/solver/ResultWriter.cpp:120-341, src/main.cpp:117-131).
// Streams keep their default formatting (6 significant digits) where the
// reference's do, and 17 digits where it sets them.
#include "phmc_host.h"

#include <algorithm>
#include <cmath>
#include <iomanip>
#include <sstream>

namespace phmc {
namespace {
std::string join_numbers(const std::vector<double>& v, double scale = 1.0) {
    std::ostringstream o;
    o << "[";
    for (size_t i = 0; i < v.size(); ++i) o << (i ? ", " : "") << v[i] * scale;
    o << "]";
    return o.str();
}

// selector coordinates as the reference's configuration parser keeps them:
// 17 significant digits (src/config/ConfigParsing.cpp:280-285)
std::string token(double x) {
    std::ostringstream o;
    o << std::setprecision(17) << x;
    return o.str();
}

std::string join_tokens(const std::vector<std::string>& v) {
    if (v.empty()) return "[]";
    std::ostringstream o;
    o << "[";
    for (size_t i = 0; i < v.size(); ++i) o << (i ? ", " : "") << v[i];
    o << "]";
    return o.str();
}

// Box configurations name their walls per face; the equivalent selectors are
// the six relative face regions in facet order.
const std::array<std::array<double, 6>, 6> kBoxFaceRegions{{{-0.01, 0, 0, 0.01, 1, 1},
                                                            {0.99, 0, 0, 1.01, 1, 1},
                                                            {0, -0.01, 0, 1, 0.01, 1},
                                                            {0, 0.99, 0, 1, 1.01, 1},
                                                            {0, 0, -0.01, 1, 1, 0.01},
                                                            {0, 0, 0.99, 1, 1, 1.01}}};
} // namespace

std::string format_domain_summary(const SimulationConfig& a, const SimulationDomain& d) {
    std::ostringstream out;
    const bool box = !d.is_mesh();
    std::vector<char> conds;
    std::vector<double> values;
    std::vector<std::array<double, 6>> regions, pairs;
    if (box) {
        for (int f = 0; f < 6; ++f) {
            conds.push_back(a.face_condition[f]);
            values.push_back(a.face_value[f]);
            regions.push_back(kBoxFaceRegions[f]);
        }
        for (int axis = 0; axis < 3; ++axis)
            if (a.face_condition[2 * axis] == 'P') {
                pairs.push_back(kBoxFaceRegions[2 * axis]);
                pairs.push_back(kBoxFaceRegions[2 * axis + 1]);
            }
    } else {
        conds = a.boundary_conditions;
        values = a.boundary_values;
        regions = a.boundary_position;
        pairs = a.periodic_pair;
    }
    auto tokens = [](const std::vector<std::array<double, 6>>& r) {
        std::vector<std::string> t;
        if (r.empty()) return t;
        t.push_back("relative_box");
        for (const auto& b : r)
            for (double x : b) t.push_back(token(x));
        return t;
    };
    int npairs = 0;
    for (size_t f = 0; f < d.facets().size(); ++f)
        if (d.facets()[f].pair > static_cast<int>(f)) ++npairs;
    const bool conservative = a.conservative_boundaries || a.collision_model == CollisionModel::Callaway;

    out << "[input]\n";
    out << "model = " << a.model << '\n';
    const std::vector<double> sz = box ? a.sizes : std::vector<double>{200.0, 200.0, 200.0};
    out << "sizes_nm = [" << sz[0] / 10.0 << ", " << sz[1] / 10.0 << ", " << sz[2] / 10.0 << "]\n";
    out << "sizes_angstrom = [" << sz[0] << ", " << sz[1] << ", " << sz[2] << "]\n";
    out << "particle_count = " << a.particle_count << '\n';
    out << "time_step = " << a.time_step << '\n';
    out << "iterations = " << a.iterations << '\n';
    out << "convergence_write_interval = " << a.convergence_write_interval << '\n';
    out << "random_seed = " << a.random_seed << '\n';
    out << "temperature_lookup_dt = " << a.temperature_lookup_dt << '\n';
    out << "background_temperature = " << a.background_temperature << '\n';
    out << "callaway_formulation = linearized\n";
    out << "conservative_boundaries = " << (conservative ? "true" : "false") << '\n';
    if (conservative) {
        out << "collision_model = " << (a.collision_model == CollisionModel::Callaway ? "callaway" : "rta") << '\n';
        out << "collision_reference_temperature = " << a.background_temperature << '\n';
        out << "reservoir_generation = fixed_incoming_flux\n";
    }
    out << "lifetime_temperature = ";
    if (a.lifetime_temperature_is_local) out << "local";
    else out << a.lifetime_temperature;
    out << '\n';
    if (a.transport_axis >= 0) out << "transport_axis = " << "xyz"[a.transport_axis] << '\n';
    if (a.temperature_gradient) {
        out << "temperature_gradient_K_per_m = " << *a.temperature_gradient << '\n';
        out << "conductivity_definition = -mean_heatflux/imposed_gradient\n";
        out << "temperature_output = T0_plus_periodic_correction\n";
        out << "kappa_int_applicable = false\n";
    }
    out << "compute_kappa = " << (a.compute_kappa ? "true" : "false") << '\n';
    out << "profile_timers = false\n";
    out << "progress_temperature_summary_only = false\n";
    out << "merge_coplanar_facets = " << (a.merge_coplanar_facets ? "true" : "false") << '\n';
    out << "initial_temperature = ";
    if (a.initial_temperature_mode == InitialTemperatureMode::Uniform) out << a.initial_temperature;
    else out << "linear";
    out << '\n';
    out << "grid_xyz = [" << a.grid[0] << ", " << a.grid[1] << ", " << a.grid[2] << "]\n";
    out << "boundary_conditions = ";
    for (size_t i = 0; i < conds.size(); ++i) out << (i ? " " : "") << conds[i];
    out << '\n';
    out << "boundary_values = " << join_numbers(values) << '\n';
    out << "boundary_position_selector_mode = " << (regions.empty() ? "none" : "region") << '\n';
    out << "boundary_position_selector_count = " << regions.size() << '\n';
    out << "boundary_position_tokens = " << join_tokens(tokens(regions)) << '\n';
    out << "periodic_pair_region_count = " << pairs.size() << '\n';
    out << "periodic_pair_tokens = " << join_tokens(tokens(pairs)) << '\n';
    out << "material_folder = " << a.material_folder << '\n';
    out << "material_folders = []\n";
    out << "material_interface_axis = " << "xyz"[a.material_interface_axis] << '\n';
    out << "material_interface_positions_nm = " << join_numbers(a.material_interface_positions, 0.1) << '\n';
    out << "material_interface_model = diffuse_mismatch\n";
    out << "material_interface_amm_fraction = 0\n";
    out << "material_interface_parallel_bin_inv_a = 0.05\n";
    out << "output_folder = " << a.output_folder << '\n';
    out << "heat_source_enabled = " << (a.heat_source_enabled ? "true" : "false") << '\n';
    out << "heat_source_profile = " << (a.heat_source_profile == HeatSourceProfile::Gaussian ? "gaussian" : "uniform")
        << '\n';
    out << "heat_source_min_nm = " << join_numbers(a.heat_source_min, 0.1) << '\n';
    out << "heat_source_max_nm = " << join_numbers(a.heat_source_max, 0.1) << '\n';
    out << "heat_source_center_nm = " << join_numbers(a.heat_source_center, 0.1) << '\n';
    out << "heat_source_centers_nm = " << join_numbers(a.heat_source_centers, 0.1) << '\n';
    out << "heat_source_sigma_nm = " << join_numbers(a.heat_source_sigma, 0.1) << '\n';
    out << "heat_source_half_width_nm = " << join_numbers(a.heat_source_half_width, 0.1) << '\n';
    out << "heat_source_min_angstrom = " << join_numbers(a.heat_source_min) << '\n';
    out << "heat_source_max_angstrom = " << join_numbers(a.heat_source_max) << '\n';
    out << "heat_source_center_angstrom = " << join_numbers(a.heat_source_center) << '\n';
    out << "heat_source_centers_angstrom = " << join_numbers(a.heat_source_centers) << '\n';
    out << "heat_source_sigma_angstrom = " << join_numbers(a.heat_source_sigma) << '\n';
    out << "heat_source_half_width_angstrom = " << join_numbers(a.heat_source_half_width) << '\n';
    out << "heat_source_power_density = " << a.heat_source_power_density << '\n';
    out << "heat_source_power_densities = " << join_numbers(a.heat_source_power_densities) << '\n';
    out << "heat_source_frequency_min_THz = " << a.heat_source_frequency_min << '\n';
    out << "heat_source_frequency_max_THz = " << a.heat_source_frequency_max << '\n';
    out << "heat_source_time_profile = "
        << (a.heat_source_time_profile == HeatSourceTimeProfile::Pulsed ? "square" : "constant") << '\n';
    out << "mode_excitation_enabled = false\n";
    out << "mode_excitation_frequency_min_THz = -1\n";
    out << "mode_excitation_frequency_max_THz = -1\n";
    out << "mode_excitation_occupation_multiplier = 1\n";
    out << '\n';

    out << "[geometry]\n";
    out << "volume = " << d.volume() << '\n';
    const Vec3& lo = d.bounds_min();
    const Vec3& hi = d.bounds_max();
    out << "bounds_min = [" << lo[0] << ", " << lo[1] << ", " << lo[2] << "]\n";
    out << "bounds_max = [" << hi[0] << ", " << hi[1] << ", " << hi[2] << "]\n";
    // the analytic box is the reference's 12-triangle box mesh, whose star
    // decomposition from the centre is exact
    out << "n_faces = " << (box ? 12 : d.mesh()->faces().size()) << '\n';
    out << "n_facets = " << d.facets().size() << '\n';
    out << "n_simplices = " << (box ? 12 : d.mesh()->simplices().size()) << '\n';
    out << '\n';

    out << "[grid]\n";
    out << "count = " << d.grid_count() << '\n';
    out << "lookup = voxel_to_active_grid_o1\n";
    out << '\n';

    int rough = 0;
    for (const auto& F : d.facets()) rough += F.condition == 'R' ? 1 : 0;
    out << "[boundary]\n";
    out << "reservoir_facets = " << d.reservoir_facets().size() << '\n';
    out << "rough_facets = " << rough << '\n';
    out << "periodic_pairs = " << npairs << '\n';
    out << '\n';

    out << "[files]\n";
    std::string folder = a.output_folder;
    if (!folder.empty() && folder.back() != '/') folder += '/';
    out << "grid_centers_csv = " << folder << "grid_centers.csv" << '\n';
    return out.str();
}

std::string format_grid_centers(const SimulationDomain& d) {
    std::ostringstream out;
    out << "index,x_nm,y_nm,z_nm,volume_nm3\n";
    for (int i = 0; i < d.grid_count(); ++i) {
        const Vec3& c = d.grid_centers()[i];
        out << i << "," << (c[0] / 10.0) << "," << (c[1] / 10.0) << "," << (c[2] / 10.0) << ","
            << (d.grid_volumes()[i] / 1000.0) << "\n";
    }
    return out.str();
}

std::string format_run_summary(const RunSummary& s) {
    std::ostringstream out;
    if (s.gradient_driven)
        out << "\n[temperature_gradient_accounting]\noccupation_updates = " << s.gradient_updates
            << "\nnet_energy_ev = " << s.gradient_energy_ev << "\n";
    out << std::setprecision(17);
    out << "\n[performance]\n";
    out << "openmp_enabled = false\n";
    out << "openmp_thread_count = 1\n";
    out << "random_seed = " << s.random_seed << '\n';
    out << "profile_timers_enabled = false\n";
    out << "collision_cache_corrections_total = " << s.cache_corrections << '\n';
    out << "collision_cache_failures_total = 0\n";
    out << "transport_failure_policy = strict\n";
    out << "excessive_collision_recoveries_total = 0\n";
    out << "cell_index_rebuilds = " << s.cell_index_rebuilds << '\n';
    out << "temperature_refreshes = " << s.temperature_refreshes << '\n';
    const long long* r = s.rough;
    const long long total = r[7];
    const double den = std::max(1.0, static_cast<double>(total));
    out << "\n[rough_boundary_diagnostics]\n";
    out << "events_total = " << total << '\n';
    out << "specular_selected = " << r[0] << '\n';
    out << "diffuse_selected = " << r[4] << '\n';
    out << "specular_ratio = " << (static_cast<double>(r[0]) / den) << '\n';
    out << "diffuse_ratio = " << (static_cast<double>(r[4]) / den) << '\n';
    out << "residual_flux_frequency_window_selected = " << r[2] << '\n';
    out << "residual_flux_frequency_window_fallback = " << r[3] << '\n';
    out << "fallback_missing_rough_data = 0\n";
    out << "fallback_missing_spec_match = " << r[1] << '\n';
    out << "fallback_outgoing_pool = " << r[5] << '\n';
    out << "fallback_global_random = " << r[6] << '\n';
    out << "fallback_total = " << (r[3] + r[1] + r[5] + r[6]) << '\n';
    out << "mode_map_csv = disabled\n";
    const double iden = std::max(1.0, static_cast<double>(s.interface_events));
    out << "\n[material_interface_diagnostics]\n";
    out << "material_count = " << s.material_count << '\n';
    out << "model = diffuse_mismatch\n";
    if (s.material_count > 1) {
        out << "frequency_bin_thz = " << s.interface_frequency_bin_thz << '\n';
        out << "amm_fraction = 0\n";
        out << "carrier_sampling = equal_physical_state_weight\n";
        out << "fixed_flux_reservoirs = " << (s.fixed_flux_reservoirs ? "true" : "false") << '\n';
        for (size_t m = 0; m < s.material_carrier_volumes_a3.size(); ++m)
            out << "material_" << m << "_carrier_volume_a3 = " << s.material_carrier_volumes_a3[m] << '\n';
    }
    out << "events_total = " << s.interface_events << '\n';
    out << "transmitted_total = " << s.interface_transmitted << '\n';
    out << "reflected_total = " << s.interface_reflected << '\n';
    out << "transmission_ratio = " << (static_cast<double>(s.interface_transmitted) / iden) << '\n';
    out << "reflection_ratio = " << (static_cast<double>(s.interface_reflected) / iden) << '\n';
    out << "\n[escaped_particle_recovery]\n";
    out << "check_interval = 100\n";
    out << "policy = strict\n";
    out << "recovery_events = 0\n";
    out << "recovered_particles_total = 0\n";
    out << "\n[reservoir_balance_diagnostics]\n";
    out << "reservoir_gen = " << (s.conservative ? "fixed_incoming_flux" : "one_to_one") << '\n';
    out << "absorbed_particles_total = " << s.absorbed_total << '\n';
    out << "injected_particles_total = " << s.injected_total << '\n';
    out << "recovered_particles_total = 0\n";
    out << "net_particles_total = " << (s.injected_total - s.absorbed_total) << '\n';
    out << "absorbed_deviational_energy_total_ev = " << s.absorbed_energy_ev << '\n';
    out << "injected_deviational_energy_total_ev = " << s.injected_energy_ev << '\n';
    out << "\n[energy_weighting]\n";
    out << "initial_particle_count = " << s.initial_particle_count << '\n';
    out << "current_particle_count = " << s.particle_count << '\n';
    out << "particle_spatial_weight_a3 = " << s.particle_spatial_weight_a3 << '\n';
    out << "background_reference_temperature_k = " << s.background_temperature << '\n';
    out << "total_thermal_energy_ev = " << s.total_thermal_energy_ev << '\n';
    out << "lifetime_energy_residual_total_ev = " << s.lifetime_residual_ev << '\n';
    out << "energy_balance_residual_total_ev = " << s.balance_residual_ev << '\n';
    // src/solver/ResultWriter.cpp:120-170
    const SimulationConfig& c = s.cfg;
    out << "\n[local_heat_source_occupation_injection]\n";
    out << "enabled = " << (c.heat_source_enabled ? "true" : "false") << '\n';
    out << "profile = " << (c.heat_source_profile == HeatSourceProfile::Gaussian ? "gaussian" : "uniform") << '\n';
    if (c.heat_source_total_power) out << "specified_total_power_w = " << *c.heat_source_total_power << '\n';
    else out << "power_density_wm3 = " << c.heat_source_power_density << '\n';
    out << "model = prescribed_lattice_power\n";
    out << "electron_transport = false\n";
    out << "empty_cell_policy = " << s.empty_cell_policy << '\n';
    const char* spectrum = c.heat_source_spectrum == HeatSourceSpectrum::Gaussian  ? "gaussian"
                           : c.heat_source_spectrum == HeatSourceSpectrum::Weighted ? "weighted"
                                                                                    : "thermal";
    out << "spectrum = " << spectrum << '\n';
    if (c.heat_source_spectrum == HeatSourceSpectrum::Gaussian) {
        out << "frequency_center_thz = " << c.heat_source_frequency_center.value_or(0) << '\n';
        out << "frequency_sigma_thz = " << c.heat_source_frequency_sigma.value_or(0) << '\n';
        out << "spectral_normalization = existing_carrier_weights_within_each_cell\n";
        out << "spectral_weight = exp(-0.5*((f-f_center)/sigma_f)^2); energy_per_mode\n";
    }
    out << "power_input = " << (c.heat_source_total_power ? "total_power" : "power_density") << '\n';
    out << "base_total_power_w = " << s.source_base_power << '\n';
    out << "frequency_min_thz = " << c.heat_source_frequency_min << '\n';
    out << "frequency_max_thz = " << c.heat_source_frequency_max << '\n';
    out << "branches_zero_based = [";
    for (size_t i = 0; i < c.heat_source_branches.size(); ++i) out << (i ? ", " : "") << c.heat_source_branches[i];
    out << "]\nbranch_weights_per_sampled_mode = [";
    for (size_t i = 0; i < c.heat_source_branch_weights.size(); ++i)
        out << (i ? ", " : "") << c.heat_source_branch_weights[i];
    out << "]\n";
    out << "prescribed_energy_total_ev = " << s.source_prescribed << '\n';
    out << "pending_energy_total_ev = " << s.source_pending << '\n';
    out << "deposition_complete = " << (s.source_pending == 0.0 ? "true" : "false") << '\n';
    out << "source_ledger_residual_ev = " << s.source_prescribed - s.source_deposited - s.source_pending << '\n';
    out << "time_profile = " << (c.heat_source_time_profile == HeatSourceTimeProfile::Pulsed ? "square" : "constant")
        << '\n';
    out << "time_start_ps = " << c.heat_source_time_start << '\n';
    out << "time_end_ps = " << c.heat_source_time_end << '\n';
    out << "period_ps = " << c.heat_source_period << '\n';
    out << "on_duration_ps = " << c.heat_source_on_duration << '\n';
    out << "duty_cycle = " << c.heat_source_duty_cycle << '\n';
    out << "amplitude = " << c.heat_source_amplitude << '\n';
    out << "occupation_updates_total = " << s.source_updates_total << '\n';
    out << "injected_energy_total_ev = " << s.source_energy_total_ev << '\n';
    out << "occupation_updates_last_step = " << s.source_updates_step << '\n';
    out << "injected_energy_last_step_ev = " << s.source_energy_step_ev << '\n';
    return out.str();
}

// grid_heat_flux.csv (src/solver/ResultWriter.cpp:35-42, 52-65): the header
// when the run starts, then per observation one row per cell at 17 digits.
std::string format_cell_flux_header() { return "timestep,time_ps,cell_index,temperature_K,qx_W_m2,qy_W_m2,qz_W_m2\n"; }

std::string format_cell_flux_rows(int timestep, double time_ps, const std::vector<double>& temperatures,
                                  const std::vector<double>& q) {
    std::ostringstream out;
    out << std::setprecision(17);
    for (size_t c = 0; c < temperatures.size(); ++c)
        out << timestep << ',' << time_ps << ',' << c << ',' << temperatures[c] << ',' << q[3 * c] << ','
            << q[3 * c + 1] << ',' << q[3 * c + 2] << '\n';
    return out.str();
}

// heat_source_ledger.txt (src/solver/ResultWriter.cpp:343-354): per cell its
// centre (Angstrom), material, base power (W) and prescribed / deposited /
// pending energies (eV).
std::string format_source_ledger(const SimulationConfig& c, const SimulationDomain& d, const std::vector<int>& material,
                                 const std::vector<double>& rate_evps, const double* prescribed,
                                 const double* deposited, const double* pending) {
    const char* spectrum = c.heat_source_spectrum == HeatSourceSpectrum::Gaussian  ? "gaussian"
                           : c.heat_source_spectrum == HeatSourceSpectrum::Weighted ? "weighted"
                                                                                    : "thermal";
    std::ostringstream out;
    out << std::setprecision(17) << "# prescribed_lattice_power; not an electron-phonon calculation\n"
        << "# spectrum=" << spectrum << "; pending energy is not yet represented by phonons\n"
        << "# cell x_A y_A z_A material base_power_W prescribed_eV deposited_eV pending_eV\n";
    const auto& centers = d.grid_centers();
    for (size_t k = 0; k < rate_evps.size(); ++k)
        out << k << " " << centers[k][0] << " " << centers[k][1] << " " << centers[k][2] << " " << material[k] << " "
            << rate_evps[k] / 6.241509074e6 << " " << prescribed[k] << " " << deposited[k] << " " << pending[k]
            << '\n';
    return out.str();
}

std::string format_runtime(long long sec) {
    const long long days = sec / (24 * 3600), hours = (sec % (24 * 3600)) / 3600, minutes = (sec % 3600) / 60,
                    seconds = sec % 60;
    std::ostringstream out;
    out << "\n[runtime]\n";
    out << "total_seconds = " << sec << '\n';
    out << "total_days = " << days << '\n';
    out << "total_hours = " << hours << '\n';
    out << "total_minutes = " << minutes << '\n';
    out << "total_seconds_remainder = " << seconds << '\n';
    out << "total_human_readable = " << days << " days " << hours << " h " << minutes << " min " << seconds << " s\n";
    return out.str();
}

} // namespace phmc
