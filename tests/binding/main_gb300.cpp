// PhonoMC's main program with the GB300 carrier loop dropped in: the binding a
// maintainer adds to src/main.cpp (reference src/main.cpp:61-141), compiled
// by tests/test_binding.py against the reference's headers and its own build
// (oracle/_ref/libphonomc_ref.a, whose read_material_data reads HDF5 folders)
// and linked with libphonomc_gb300.so.
//
//   main_gb300 check <input.toml>   host only: parse the TOML with the
//       reference's loader, read the material folder with the reference's
//       reader, fill phmc_material_data / phmc_config, build the library's
//       host domain and material, and compare them with the reference's
//       SimulationDomain and PhononMaterial (prints one JSON line)
//   main_gb300 run <input.toml>     the main.cpp step loop on the device
#include "PhononMaterial.h"
#include "SimulationConfig.h"
#include "SimulationDomain.h"
#include "material/MaterialDataReader.h"

#include "phonomc_gb300.h"

#include <cmath>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

void check(int rc) {
    if (rc != 0) throw std::runtime_error(phmc_last_error());
}

// MaterialData -> phmc_material_data (pointers into `data`, which must outlive the call)
phmc_material_data material_pod(const phonomc::MaterialData& data) {
    phmc_material_data md{};
    md.qpoints = data.qpoints;
    md.branches = data.branches;
    for (int a = 0; a < 3; ++a) md.mesh[a] = data.mesh[a];
    md.ntemps = static_cast<int32_t>(data.temperatures.size());
    md.volume_a3 = data.lattice.volume_a3;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) md.reciprocal[3 * i + j] = data.lattice.reciprocal[i][j];
    md.frequency_thz = data.frequency_thz.data();
    md.qpoint_fractions = &data.qpoint_fractions[0][0];
    md.group_velocity = &data.group_velocity[0][0];
    md.temperatures = data.temperatures.data();
    md.gamma = data.gamma.data();
    md.gamma_normal = data.gamma_normal.empty() ? nullptr : data.gamma_normal.data();
    md.gamma_umklapp = data.gamma_umklapp.empty() ? nullptr : data.gamma_umklapp.data();
    auto iso = data.gamma_resistive.find("gamma_isotope");
    if (iso != data.gamma_resistive.end()) {
        md.gamma_isotope = iso->second.data();
        md.gamma_isotope_len = static_cast<int64_t>(iso->second.size());
    }
    return md;
}

// SimulationConfig (+ its SimulationDomain for the box face conditions) -> phmc_config
phmc_config config_pod(const SimulationConfig& args, const SimulationDomain& geo) {
    phmc_config c{};
    for (int a = 0; a < 3; ++a) c.sizes[a] = args.sizes[a];
    c.particle_count = args.particle_count;
    c.time_step = args.time_step;
    c.iterations = args.iterations;
    c.convergence_write_interval = args.convergence_write_interval;
    c.random_seed = args.random_seed;
    c.compute_kappa = args.compute_kappa;
    c.transport_axis = args.transport_axis;
    c.has_temperature_gradient = args.temperature_gradient.has_value();
    c.temperature_gradient = args.temperature_gradient.value_or(0.0);
    c.temperature_lookup_dt = args.temperature_lookup_dt;
    c.background_temperature = args.background_temperature;
    c.lifetime_temperature_is_local = args.lifetime_temperature_is_local;
    c.lifetime_temperature = args.lifetime_temperature;
    c.collision_model = args.collision_model == CollisionModel::Callaway;
    c.conservative_boundaries = args.conservative_boundaries;
    c.grid[0] = args.grid.nx;
    c.grid[1] = args.grid.ny;
    c.grid[2] = args.grid.nz;
    c.initial_temperature_linear = args.initial_temperature.mode == InitialTemperatureMode::Linear;
    c.initial_temperature = args.initial_temperature.uniform_temperature;
    // box faces in the reference's facet order (xmin, xmax, ymin, ymax, zmin,
    // zmax): condition and value as the reference's domain assigned them from
    // the boundary_position selectors; roughness back from Angstrom to nm
    for (int f = 0; f < 6; ++f) {
        const char code = geo.facet_boundary_condition(f);
        c.face_condition[f] = code;
        c.face_value[f] = code == 'T' ? geo.reservoir_value_for_facet(f) : code == 'R' ? geo.roughness_for_facet(f) / 10.0 : 0.0;
    }
    c.output_folder = args.output_folder.empty() ? nullptr : args.output_folder.c_str();
    c.material_interface_axis = args.material_interface_axis;
    c.n_interfaces = static_cast<int32_t>(args.material_interface_positions.size());
    c.material_interface_positions = args.material_interface_positions.empty() ? nullptr : args.material_interface_positions.data();
    c.interface_frequency_bin_thz = args.material_interface_frequency_bin_thz;
    c.write_cell_heat_flux = args.write_cell_heat_flux;
    c.callaway_nonlinear = args.callaway_nonlinear;
    c.precision = 1; // mixed: FP32 flight, FP64 tallies (0: plain FP64)
    return c;
}

std::string material_folder(const SimulationConfig& args) {
    namespace fs = std::filesystem;
    fs::path p(args.material_folder);
    if (!p.is_absolute()) p = fs::path(args.input_directory) / p;
    return p.lexically_normal().string();
}

} // namespace

int main(int argc, char** argv) {
    try {
        if (argc < 3) throw std::runtime_error("usage: main_gb300 check|run <input.toml>");
        const std::string mode = argv[1];
        SimulationConfig args = load_simulation_config(argv[2]);
        if (mode == "check") args.output_folder.clear();
        SimulationDomain geo(args);
        const phonomc::MaterialData data = phonomc::read_material_data(material_folder(args));
        const bool stationary = uses_conservative_transport(args);
        const bool callaway = args.collision_model == CollisionModel::Callaway;

        phmc_material_data md = material_pod(data);
        phmc_material* mat = nullptr;
        check(phmc_material_create(&md, args.temperature_lookup_dt, stationary, callaway, &mat));
        phmc_config c = config_pod(args, geo);

        if (mode == "check") {
            // the library's host domain and material against the reference's
            phmc_domain* dom = nullptr;
            check(phmc_domain_create(&c, &dom));
            int32_t nf = 0, nc = 0, nfaces = 0, shape[3];
            double volume = 0, bounds[6];
            check(phmc_domain_info(dom, &nf, &nc, &nfaces, shape, &volume, bounds));
            std::vector<double> vols(nc), centers(3 * static_cast<size_t>(nc)), value(nf);
            std::vector<char> cond(nf);
            check(phmc_domain_cells(dom, centers.data(), vols.data(), nullptr));
            check(phmc_domain_facets(dom, nullptr, nullptr, nullptr, cond.data(), value.data(), nullptr, nullptr));
            double vol_err = 0, ctr_err = 0;
            for (int k = 0; k < nc && k < geo.grid_count(); ++k) {
                vol_err = std::fmax(vol_err, std::abs(vols[k] - geo.grid_volumes()[k]) / geo.grid_volumes()[k]);
                for (int a = 0; a < 3; ++a)
                    ctr_err = std::fmax(ctr_err, std::abs(centers[3 * k + a] - geo.grid_centers()[k][a]));
            }
            int face_mismatch = 0;
            for (int f = 0; f < nf && f < 6; ++f) {
                const char code = geo.facet_boundary_condition(f);
                const double ref = code == 'T' ? geo.reservoir_value_for_facet(f) : code == 'R' ? geo.roughness_for_facet(f) : 0.0;
                if (cond[f] != code || std::abs(value[f] - ref) > 1e-12 * std::max(1.0, std::abs(ref))) ++face_mismatch;
            }
            int active = 0;
            check(phmc_material_active_count(mat, &active));
            const PhononMaterial ref_mat(data, args.temperature_lookup_dt, stationary, callaway);
            std::printf("{\"cells\": %d, \"ref_cells\": %d, \"facets\": %d, \"volume_rel_err\": %.3e, "
                        "\"center_err\": %.3e, \"face_mismatch\": %d, \"active\": %d, \"ref_active\": %d, "
                        "\"qpoints\": %d, \"face_condition\": \"%.6s\", \"face_value\": [%g, %g, %g, %g, %g, %g], "
                        "\"precision\": %d, \"gradient\": %g}\n",
                        nc, geo.grid_count(), nf, vol_err, ctr_err, face_mismatch, active,
                        ref_mat.active_mode_count(), data.qpoints, c.face_condition, c.face_value[0],
                        c.face_value[1], c.face_value[2], c.face_value[3], c.face_value[4], c.face_value[5],
                        c.precision, c.temperature_gradient);
            phmc_domain_destroy(dom);
            phmc_material_destroy(mat);
            return 0;
        }

        // the main.cpp step loop on the device
        phmc_solver* pop = nullptr;
        check(phmc_solver_create(&c, &mat, 1, &pop));
        for (int step = 0; step < args.iterations; ++step) check(phmc_solver_run_timestep(pop));
        phmc_stats st{};
        check(phmc_solver_stats(pop, &st));
        check(phmc_solver_write_outputs(pop));
        std::printf("{\"steps\": %d, \"particles\": %lld, \"kappa_eff\": %.9g, \"balance_residual_ev\": %.3e}\n",
                    st.current_timestep, static_cast<long long>(st.particle_count), st.kappa_endpoints,
                    st.total_energy_balance_residual_ev);
        phmc_solver_destroy(pop);
        phmc_material_destroy(mat);
        return 0;
    } catch (const std::exception& e) {
        std::cerr << "Fatal error: " << e.what() << '\n';
        return 1;
    }
}
