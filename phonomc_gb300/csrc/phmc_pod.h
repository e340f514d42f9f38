// Conversions from the C-ABI plain structs (include/phonomc_gb300.h) to the
// host model types. Header-only so the CUDA library and the CPU oracle build
// their inputs identically.
#pragma once
#include "../../include/phonomc_gb300.h"
#include "phmc_host.h"

namespace phmc {

inline MaterialData material_from_pod(const phmc_material_data& p) {
    MaterialData d;
    d.qpoints = p.qpoints;
    d.branches = p.branches;
    d.mesh = {p.mesh[0], p.mesh[1], p.mesh[2]};
    d.volume_a3 = p.volume_a3;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) d.reciprocal[i][j] = p.reciprocal[3 * i + j];
    const size_t nm = static_cast<size_t>(p.qpoints) * p.branches;
    const size_t nT = static_cast<size_t>(p.ntemps);
    if (!p.frequency_thz || !p.qpoint_fractions || !p.group_velocity || !p.temperatures || !p.gamma)
        throw std::invalid_argument("material data requires frequency, qpoint, group_velocity, temperature and gamma");
    d.frequency_thz.assign(p.frequency_thz, p.frequency_thz + nm);
    d.qpoint_fractions.resize(p.qpoints);
    for (int q = 0; q < p.qpoints; ++q)
        d.qpoint_fractions[q] = {p.qpoint_fractions[3 * q], p.qpoint_fractions[3 * q + 1], p.qpoint_fractions[3 * q + 2]};
    d.group_velocity.resize(nm);
    for (size_t i = 0; i < nm; ++i)
        d.group_velocity[i] = {p.group_velocity[3 * i], p.group_velocity[3 * i + 1], p.group_velocity[3 * i + 2]};
    d.temperatures.assign(p.temperatures, p.temperatures + nT);
    d.gamma.assign(p.gamma, p.gamma + nT * nm);
    if (p.gamma_normal) d.gamma_normal.assign(p.gamma_normal, p.gamma_normal + nT * nm);
    if (p.gamma_umklapp) d.gamma_umklapp.assign(p.gamma_umklapp, p.gamma_umklapp + nT * nm);
    if (p.gamma_isotope && p.gamma_isotope_len > 0)
        d.gamma_resistive["gamma_isotope"].assign(p.gamma_isotope, p.gamma_isotope + p.gamma_isotope_len);
    return d;
}

inline SimulationConfig config_from_pod(const phmc_config& c) {
    SimulationConfig s;
    s.sizes = {c.sizes[0], c.sizes[1], c.sizes[2]};
    s.particle_count = c.particle_count;
    s.time_step = c.time_step;
    s.iterations = c.iterations;
    s.convergence_write_interval = c.convergence_write_interval > 0 ? c.convergence_write_interval : 10;
    s.random_seed = c.random_seed;
    s.compute_kappa = c.compute_kappa != 0;
    s.transport_axis = c.transport_axis;
    if (c.has_temperature_gradient) s.temperature_gradient = c.temperature_gradient;
    s.temperature_lookup_dt = c.temperature_lookup_dt > 0 ? c.temperature_lookup_dt : 0.1;
    s.background_temperature = c.background_temperature;
    s.lifetime_temperature_is_local = c.lifetime_temperature_is_local != 0;
    s.lifetime_temperature = c.lifetime_temperature;
    s.collision_model = c.collision_model == 1 ? CollisionModel::Callaway : CollisionModel::Rta;
    s.conservative_boundaries = c.conservative_boundaries != 0;
    s.grid = {c.grid[0], c.grid[1], c.grid[2]};
    s.initial_temperature_mode = c.initial_temperature_linear ? InitialTemperatureMode::Linear
                                                              : InitialTemperatureMode::Uniform;
    s.initial_temperature = c.initial_temperature;
    for (int f = 0; f < 6; ++f) {
        s.face_condition[f] = c.face_condition[f];
        s.face_value[f] = c.face_value[f];
    }
    if (c.output_folder) s.output_folder = c.output_folder;
    s.material_interface_axis = c.material_interface_axis;
    if (c.n_interfaces > 0 && c.material_interface_positions)
        s.material_interface_positions.assign(c.material_interface_positions,
                                              c.material_interface_positions + c.n_interfaces);
    if (c.interface_frequency_bin_thz > 0) s.material_interface_frequency_bin_thz = c.interface_frequency_bin_thz;
    // Validation of src/config/ConfigValidation.cpp:403-408: gradient driving
    // requires fixed lifetimes.
    if (s.temperature_gradient && s.lifetime_temperature_is_local)
        throw std::invalid_argument("driving.temperature_gradient requires a fixed numeric lifetime_temperature.");
    return s;
}

} // namespace phmc
