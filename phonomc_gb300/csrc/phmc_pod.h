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

// [heat_source] fields of phmc_config (include/SimulationConfig.h:103-139).
inline void heat_source_from_pod(const phmc_heat_source& h, SimulationConfig& s) {
    s.heat_source_enabled = true;
    s.heat_source_profile = h.profile == 1 ? HeatSourceProfile::Gaussian : HeatSourceProfile::Uniform;
    if (h.has_box) {
        s.heat_source_min.assign(h.min, h.min + 3);
        s.heat_source_max.assign(h.max, h.max + 3);
    }
    if (h.profile == 1) {
        if (h.n_centers == 1 && h.centers) s.heat_source_center.assign(h.centers, h.centers + 3);
        else if (h.n_centers > 1 && h.centers) s.heat_source_centers.assign(h.centers, h.centers + 3 * h.n_centers);
        s.heat_source_sigma.assign(h.sigma, h.sigma + 3);
        if (h.half_width[0] > 0 || h.half_width[1] > 0 || h.half_width[2] > 0)
            s.heat_source_half_width.assign(h.half_width, h.half_width + 3);
    }
    s.heat_source_power_density = h.power_density;
    if (h.has_total_power) s.heat_source_total_power = h.total_power;
    if (h.n_power_densities > 0 && h.power_densities)
        s.heat_source_power_densities.assign(h.power_densities, h.power_densities + h.n_power_densities);
    s.heat_source_spectrum = h.spectrum == 1 ? HeatSourceSpectrum::Weighted
                           : h.spectrum == 2 ? HeatSourceSpectrum::Gaussian
                                             : HeatSourceSpectrum::Thermal;
    if (h.has_frequency_gaussian) {
        s.heat_source_frequency_center = h.frequency_center;
        s.heat_source_frequency_sigma = h.frequency_sigma;
    }
    s.heat_source_frequency_min = h.frequency_min;
    s.heat_source_frequency_max = h.frequency_max;
    if (h.n_branches > 0 && h.branches) s.heat_source_branches.assign(h.branches, h.branches + h.n_branches);
    if (h.n_branch_weights > 0 && h.branch_weights)
        s.heat_source_branch_weights.assign(h.branch_weights, h.branch_weights + h.n_branch_weights);
    s.heat_source_time_profile = h.time_profile == 1 ? HeatSourceTimeProfile::Pulsed : HeatSourceTimeProfile::Constant;
    s.heat_source_time_start = h.time_start;
    s.heat_source_time_end = h.time_end;
    s.heat_source_period = h.period;
    s.heat_source_on_duration = h.on_duration;
    s.heat_source_duty_cycle = h.duty_cycle;
    s.heat_source_amplitude = h.amplitude;
    }

// [geometry] model and [boundary] regions of a mesh domain.
inline void mesh_domain_from_pod(const phmc_mesh_domain& m, SimulationConfig& s) {
    if (m.model && m.model[0]) {
        s.model = m.model;
        if (s.model == "box" || s.model == "mesh") throw std::invalid_argument("mesh model must be a file path");
    } else {
        if (m.n_vertices <= 0 || m.n_faces <= 0 || !m.vertices || !m.faces)
            throw std::invalid_argument("mesh domain requires a model path or vertices and faces");
        s.model = "mesh";
        s.mesh_vertices.resize(static_cast<size_t>(m.n_vertices));
        for (int64_t i = 0; i < m.n_vertices; ++i)
            s.mesh_vertices[i] = {m.vertices[3 * i], m.vertices[3 * i + 1], m.vertices[3 * i + 2]};
        s.mesh_faces.resize(static_cast<size_t>(m.n_faces));
        for (int64_t i = 0; i < m.n_faces; ++i) s.mesh_faces[i] = {m.faces[3 * i], m.faces[3 * i + 1], m.faces[3 * i + 2]};
    }
    s.merge_coplanar_facets = m.merge_coplanar_facets != 0;
    s.extruded_z = m.extruded_z != 0;
    if (m.n_regions < 0 || m.n_periodic_regions < 0) throw std::invalid_argument("negative region count");
    if (m.n_regions > 0 && (!m.boundary_position || !m.boundary_conditions || !m.boundary_values))
        throw std::invalid_argument("boundary regions require positions, conditions and values");
    for (int i = 0; i < m.n_regions; ++i) {
        std::array<double, 6> b;
        for (int k = 0; k < 6; ++k) b[k] = m.boundary_position[6 * i + k];
        s.boundary_position.push_back(b);
        s.boundary_conditions.push_back(m.boundary_conditions[i]);
        s.boundary_values.push_back(m.boundary_values[i]);
    }
    if (m.n_periodic_regions > 0 && !m.periodic_pair) throw std::invalid_argument("periodic_pair regions missing");
    for (int i = 0; i < m.n_periodic_regions; ++i) {
        std::array<double, 6> b;
        for (int k = 0; k < 6; ++k) b[k] = m.periodic_pair[6 * i + k];
        s.periodic_pair.push_back(b);
    }
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
    s.write_cell_heat_flux = c.write_cell_heat_flux != 0;
    s.callaway_nonlinear = c.callaway_nonlinear != 0;
    s.carrier_sort_interval = c.carrier_sort_interval;
    s.transport_block = c.transport_block;
    s.transport_blocks_per_sm = c.transport_blocks_per_sm;
    s.tally_aggregation = c.tally_aggregation;
    s.transport_pipeline = c.transport_pipeline;
    s.rta_cell_update = c.rta_cell_update;
    s.material_interface_model = c.interface_model;
    s.material_interface_amm_fraction = c.interface_amm_fraction;
    if (c.interface_parallel_bin_inv_a != 0) s.material_interface_parallel_bin_inv_a = c.interface_parallel_bin_inv_a;
    if (c.n_mass_densities > 0 && c.mass_densities_kg_m3)
        s.material_mass_densities_kg_m3.assign(c.mass_densities_kg_m3, c.mass_densities_kg_m3 + c.n_mass_densities);
    if (c.material_folder) s.material_folder = c.material_folder;
    s.material_interface_axis = c.material_interface_axis;
    if (c.n_interfaces > 0 && c.material_interface_positions)
        s.material_interface_positions.assign(c.material_interface_positions,
                                              c.material_interface_positions + c.n_interfaces);
    if (c.interface_frequency_bin_thz > 0) s.material_interface_frequency_bin_thz = c.interface_frequency_bin_thz;
    if (c.heat_source) heat_source_from_pod(*c.heat_source, s);
    if (c.mesh) mesh_domain_from_pod(*c.mesh, s);
    // Validation of src/config/ConfigValidation.cpp:403-408: gradient driving
    // requires fixed lifetimes.
    if (s.temperature_gradient && s.lifetime_temperature_is_local)
        throw std::invalid_argument("driving.temperature_gradient requires a fixed numeric lifetime_temperature.");
    return s;
}

} // namespace phmc
