/*
 * C ABI of the GB300 carrier-loop library (libphonomc_gb300.so).
 *
 * Plain structs, pointers and sizes; no C++ or torch types cross this
 * boundary. Every entry point returns 0 on success and a nonzero status on
 * failure; phmc_last_error() then holds the message the reference would have
 * thrown (std::runtime_error / std::invalid_argument text).
 *
 * Reference interfaces each entry point replaces (paths inside the PhonoMC
 * project):
 *   phmc_material_create      PhononMaterial::PhononMaterial(MaterialData, double, bool, bool)
 *                             include/PhononMaterial.h:23-26
 *   phmc_solver_create        MonteCarloSolver::MonteCarloSolver(args, geometry, materials)
 *                             include/MonteCarloSolver.h:44-49 (with SimulationDomain(args),
 *                             include/SimulationDomain.h:16)
 *   phmc_solver_run_timestep  MonteCarloSolver::run_timestep()  include/MonteCarloSolver.h:57
 *   phmc_solver_run           the main.cpp:100-102 step loop
 *   phmc_solver_stats         the getters of include/MonteCarloSolver.h:59-101
 *   phmc_solver_cells         GridState temperatures / energy density / heat flux
 *                             (include/solver/GridState.h:8-14)
 *   phmc_solver_get_carriers  ParticleStorage SoA fields (include/solver/ParticleStorage.h:57-71)
 *   phmc_solver_destroy       ~MonteCarloSolver
 *   phmc_dev_trace_box        SimulationDomain::trace_boundary_intersection (box branch)
 *                             src/SimulationDomain.cpp:341-450
 *   phmc_dev_temperature_from_energy  PhononMaterial::temperature_from_energy_density
 *                             src/material/Thermodynamics.cpp:173-175
 *   phmc_dev_rta_collide      RtaCollisionOperator::apply  src/solver/RtaCollisionOperator.cpp:13-189
 *   phmc_dev_linear_collide   CarrierCollisionOperator::apply src/solver/CarrierCollisionOperator.cpp:38-141
 *   phmc_dev_ncallaway_evolve nonlinear_callaway_evolve src/solver/NonlinearCallawayCollision.cpp:216-248
 *   phmc_dev_rough_reflect    RoughBoundarySampler::sample src/solver/RoughBoundarySampler.cpp:459-533
 *   phmc_dev_rough_spec_match RoughBoundarySampler::build (specular matches) src/solver/RoughBoundarySampler.cpp:286-310
 *   phmc_dev_gradient_drive   TemperatureGradientDrive::apply src/solver/TemperatureGradientDrive.cpp:116-171
 */
#ifndef PHONOMC_GB300_H
#define PHONOMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct phmc_material phmc_material;
typedef struct phmc_solver phmc_solver;

/* phonomc::MaterialData (include/material/MaterialData.h:17-31). Arrays are
 * q-major/branch-minor; gamma tables are (temperature, q, branch). Optional
 * pointers may be NULL. */
typedef struct phmc_material_data {
    int32_t qpoints, branches, mesh[3], ntemps;
    double volume_a3;
    double reciprocal[9]; /* row-major: reciprocal[3*i+j] = component i of b_j */
    const double* frequency_thz;    /* [qpoints*branches] */
    const double* qpoint_fractions; /* [qpoints*3] */
    const double* group_velocity;   /* [qpoints*branches*3], Angstrom/ps */
    const double* temperatures;     /* [ntemps] */
    const double* gamma;            /* [ntemps*qpoints*branches], THz */
    const double* gamma_normal;     /* optional, same shape as gamma */
    const double* gamma_umklapp;    /* optional, same shape as gamma */
    const double* gamma_isotope;    /* optional, length gamma_isotope_len */
    int64_t gamma_isotope_len;
} phmc_material_data;

/* Prescribed lattice heat source (include/SimulationConfig.h:103-139; the
 * [heat_source] table of the reference's TOML), lengths in Angstrom. */
typedef struct phmc_heat_source {
    int32_t profile;                 /* 0 uniform region, 1 gaussian */
    int32_t has_box;                 /* min/max given: uniform region or gaussian clip box */
    double min[3], max[3];
    int32_t n_centers;               /* gaussian sources; centers[3*n_centers] */
    const double* centers;
    double sigma[3];                 /* <= 0: that axis is uniform */
    double half_width[3];            /* <= 0: none */
    double power_density;            /* W/m^3 (0 when total_power is used) */
    int32_t has_total_power;
    double total_power;              /* W */
    int32_t n_power_densities;       /* per-source peak values, W/m^3 */
    const double* power_densities;
    int32_t spectrum;                /* 0 thermal, 1 weighted, 2 gaussian */
    int32_t has_frequency_gaussian;
    double frequency_center, frequency_sigma; /* THz */
    double frequency_min, frequency_max;      /* THz, < 0: no cut */
    int32_t n_branches;
    const int32_t* branches;
    int32_t n_branch_weights;
    const double* branch_weights;
    int32_t time_profile;            /* 0 constant, 1 pulsed */
    double time_start, time_end;     /* ps; time_end < 0: no end */
    double period, on_duration, duty_cycle, amplitude;
} phmc_heat_source;

/* Surface-mesh domain (include/SimulationConfig.h:43-86): the closed surface
 * and the boundary regions. Regions are relative boxes
 * [xmin,ymin,zmin,xmax,ymax,zmax] over the mesh bounding box that select
 * facets by centroid; later regions override earlier ones and unselected
 * facets are smooth rough walls. */
typedef struct phmc_mesh_domain {
    const char* model;               /* STL (nm) or OBJ path; NULL: the triangles below */
    int64_t n_vertices;
    const double* vertices;          /* [n_vertices][3], Angstrom */
    int64_t n_faces;
    const int32_t* faces;            /* [n_faces][3] vertex indices */
    int32_t merge_coplanar_facets;   /* reference default 1 */
    int32_t n_regions;
    const double* boundary_position; /* [n_regions][6] */
    const char* boundary_conditions; /* [n_regions] 'T', 'P' or 'R' */
    const double* boundary_values;   /* [n_regions] K, roughness nm, 0 for periodic */
    int32_t n_periodic_regions;      /* even: region 2k pairs with 2k+1 */
    const double* periodic_pair;     /* [n_periodic_regions][6] */
    int32_t extruded_z;              /* geometry.extruded_z: constant-height prism, exact cut cells */
} phmc_mesh_domain;

/* SimulationConfig fields read by the carrier loop (include/SimulationConfig.h:42-146),
 * in internal units (Angstrom, ps, K). Box faces are in facet order
 * xmin,xmax,ymin,ymax,zmin,zmax with condition 'T','P' or 'R'. */
typedef struct phmc_config {
    double sizes[3];
    double particle_count;
    double time_step;
    int32_t iterations;
    int32_t convergence_write_interval;
    uint64_t random_seed;
    int32_t compute_kappa;
    int32_t transport_axis;          /* -1 legacy grid-based choice, else 0/1/2 */
    int32_t has_temperature_gradient;
    double temperature_gradient;     /* K/m */
    double temperature_lookup_dt;
    double background_temperature;
    int32_t lifetime_temperature_is_local;
    double lifetime_temperature;
    int32_t collision_model;         /* 0 = RTA, 1 = Callaway */
    int32_t conservative_boundaries;
    int32_t grid[3];
    int32_t initial_temperature_linear;
    double initial_temperature;
    char face_condition[6];
    double face_value[6];            /* reservoir K, roughness nm, 0 for periodic */
    const char* output_folder;       /* NULL or "" disables file output */
    int32_t material_interface_axis;
    int32_t n_interfaces;
    const double* material_interface_positions; /* Angstrom */
    double interface_frequency_bin_thz;
    int32_t precision;               /* 0 = plain FP64 state, 1 = mixed (FP32 transport) */
    const phmc_heat_source* heat_source; /* NULL: no heat source */
    const phmc_mesh_domain* mesh;    /* NULL: the analytic box of sizes / face_condition */
    const char* material_folder;     /* NULL or a label reported in summary.txt */
    int32_t write_cell_heat_flux;    /* simulation.write_cell_heat_flux: grid_heat_flux.csv rows */
    int32_t callaway_nonlinear;      /* collision.callaway_formulation: 0 linearized, 1 nonlinear */
    /* Device scheduling (no counterpart in the reference's SimulationConfig;
     * 0 selects the library's tuned default, phonomc_gb300/csrc/phmc_tuning.h).
     * The sort permutes carrier slots and so which counter-based draws a
     * carrier receives (the statistics are unchanged); the others change no
     * result beyond the order of floating-point tally sums. */
    int32_t carrier_sort_interval;   /* steps between stable carrier sorts by (mode, cell), (cell, mode)
                                        for mesh domains; < 0 never */
    int32_t transport_block;         /* threads per CTA of the carrier pass: 128, 256 or 512 */
    int32_t transport_blocks_per_sm; /* resident CTAs per SM of the carrier kernels (1..16) */
    int32_t tally_aggregation;       /* 1: warp-summed bin tallies, < 0: one atomic per carrier */
    int32_t transport_pipeline;      /* mixed state: 1 carrier tiles staged in shared memory by bulk
                                        asynchronous copies, < 0 direct loads */
    /* [materials] interface model (include/SimulationConfig.h:93-99):
     * 0 diffuse mismatch (dmm), 1 acoustic mismatch (amm), 2 mixed (mmm) */
    int32_t interface_model;
    double interface_amm_fraction;        /* mmm: acoustic-model probability per event */
    double interface_parallel_bin_inv_a;  /* amm search bins in k parallel, 1/Angstrom (0: 0.05) */
    int32_t n_mass_densities;
    const double* mass_densities_kg_m3;   /* one per material (amm, mmm) */
    /* RTA cell update: 1 one warp per cell for the bin sums, cell state,
     * pseudo-temperature and pending update together, < 0 separate kernels,
     * 0 automatic (fused on grids of 1024 cells or more with at most 512
     * mode classes per cell). */
    int32_t rta_cell_update;
} phmc_config;

/* Getters of include/MonteCarloSolver.h:59-101 plus the last step's ledger. */
typedef struct phmc_stats {
    int32_t current_timestep;
    int64_t particle_count;
    int64_t absorbed_total, injected_total;
    int64_t step_absorbed, step_injected;
    double step_absorbed_energy_ev, step_injected_energy_ev;
    double total_thermal_energy_ev;
    double total_lifetime_energy_residual_ev, step_lifetime_energy_residual_ev;
    double total_energy_balance_residual_ev, step_energy_balance_residual_ev;
    double total_gradient_energy_ev, step_gradient_energy_ev;
    int64_t step_gradient_updates;
    double average_heat_flux_along_axis;
    double kappa_fit, kappa_endpoints;
    int64_t interface_events, interface_transmitted, interface_reflected;
    int64_t device_launches;          /* CUDA kernels launched by this solver so far */
    /* heat source: total_/step_ ledger source energy, prescribed and pending budgets (eV) */
    double total_heat_source_energy_ev, step_heat_source_energy_ev;
    double prescribed_heat_source_energy_ev, pending_heat_source_energy_ev;
    int64_t step_heat_source_updates;
    /* rough reflections since the start (src/solver/RoughBoundarySampler.cpp:371-533):
     * specular, missing specular partner, residual window, window without flux,
     * diffuse, outgoing-pool fallback, uniform fallback, then all events */
    int64_t rough_counts[8];
    int64_t collision_cache_corrections; /* wall caches found from a nudged position */
} phmc_stats;

const char* phmc_last_error(void);
int phmc_device_count(int* count);

int phmc_material_create(const phmc_material_data* data, double temperature_lookup_dt,
                         int include_stationary_modes, int complete_callaway_bz, phmc_material** out);
void phmc_material_destroy(phmc_material* m);
int phmc_material_active_count(const phmc_material* m, int* n_active);
/* A material from a folder in the reference's layout: POSCAR plus
 * kappa-fbz.hdf5, kappa.hdf5 or a single *.hdf5 (read_material_data,
 * src/material/MaterialDataReader.cpp:150-302, then the PhononMaterial
 * constructor, include/PhononMaterial.h:23-26). libhdf5 is not required. */
int phmc_material_load(const char* folder, double temperature_lookup_dt, int include_stationary_modes,
                       int complete_callaway_bz, phmc_material** out);
/* Writes `data` as a material folder in the reference's layout (POSCAR and
 * kappa-fbz.hdf5 with unit weights). No counterpart in the reference, whose
 * tables come from phono3py. */
int phmc_material_save(const phmc_material_data* data, const char* folder);
/* One numeric dataset of an HDF5 file's root group, as doubles: its rank and
 * dims (up to 8), then its values (row-major). No counterpart in the
 * reference, which links libhdf5. */
int phmc_h5_shape(const char* path, const char* name, int32_t* rank, int64_t* dims);
int phmc_h5_read(const char* path, const char* name, double* values);

int phmc_solver_create(const phmc_config* cfg, phmc_material* const* materials, int n_materials,
                       phmc_solver** out);
int phmc_solver_run_timestep(phmc_solver* s);
int phmc_solver_run(phmc_solver* s, int steps);
int phmc_solver_synchronize(phmc_solver* s);
int phmc_solver_stats(phmc_solver* s, phmc_stats* out);
int phmc_solver_cell_count(const phmc_solver* s, int* cells);
int phmc_solver_cells(phmc_solver* s, double* temperature, double* energy_density, double* heat_flux3);
/* Carrier slots [0, n_slots): dead slots have alive == 0. */
int phmc_solver_slot_count(phmc_solver* s, int64_t* n_slots);
int phmc_solver_get_carriers(phmc_solver* s, double* x, double* y, double* z, double* occupation,
                             uint32_t* mode_word, int32_t* cell, uint8_t* alive);
/* State of one carrier slot for diagnostics: out[0..2] position, [3]
 * occupation, [4] mode word, [5] cell, [6] alive, and in mesh domains the
 * wall cache [7] time to the wall in units of dt, [8..10] hit point, [11]
 * cached facet, [12] mirror facet (-1 elsewhere). */
int phmc_solver_carrier_state(phmc_solver* s, int64_t slot, double out[13]);
/* Replace the carrier population (same SoA layout; mode_word = active | signs<<24 | material<<28). */
int phmc_solver_set_carriers(phmc_solver* s, int64_t n, const double* x, const double* y, const double* z,
                             const double* occupation, const uint32_t* mode_word, const uint8_t* alive);
/* End-to-end stepping from host memory: replaces the carrier population with
 * the host arrays (all alive), advances `steps` timesteps from the solver's
 * current time (step counter, elapsed time and ledger totals continue) and
 * reads the cell temperatures back. Registered host arrays
 * (phmc_host_register) are read by the device directly over the host link. */
int phmc_solver_run_from_host(phmc_solver* s, int64_t n, const double* x, const double* y, const double* z,
                              const double* occupation, const uint32_t* mode_word, int steps,
                              double* cell_temperature_out);
/* Measurement helper (no counterpart in the reference): first up to three
 * steps with CUDA events around the carrier pass (kernel_ms = its mean duration
 * per launch), then `steps` timesteps bracketed by CUDA events on the solver's
 * stream (total_ms; replayed from the captured step graph unless disabled);
 * launches counts the kernels of the timed region, live_before/live_after the
 * live carriers at its ends (either may be NULL). */
int phmc_solver_timed_run(phmc_solver* s, int steps, double* total_ms, double* kernel_ms, int64_t* launches,
                          int64_t* live_before, int64_t* live_after);
/* Timesteps are captured once into a CUDA graph and replayed (default 1);
 * 0 launches every kernel of every step from the host. No counterpart in the
 * reference. */
int phmc_solver_set_graphs(phmc_solver* s, int on);
/* Steps between the solver's carrier sorts, 0 for never (the configured
 * carrier_sort_interval or its tuned default). No counterpart in the reference. */
int phmc_solver_sort_interval(const phmc_solver* s, int* steps);
/* Changes the scheduling fields of the configuration (carrier_sort_interval,
 * transport_block, transport_blocks_per_sm, tally_aggregation,
 * transport_pipeline; 0 = tuned
 * default) between steps, e.g. for a tuning sweep on one population. No
 * counterpart in the reference. */
int phmc_solver_set_schedule(phmc_solver* s, int sort_interval, int transport_block, int blocks_per_sm,
                             int tally_aggregation, int transport_pipeline);
/* Page-lock / release caller-owned host buffers used for end-to-end stepping. */
int phmc_host_register(void* ptr, int64_t bytes);
int phmc_host_unregister(void* ptr);
/* grid_centers.csv again (summary.txt's domain part and grid_centers.csv are
 * written when the solver is created with an output folder). */
int phmc_solver_write_outputs(phmc_solver* s);
/* Appends the [runtime] block and the run diagnostics to summary.txt, as the
 * reference's main does after the step loop (src/main.cpp:117-131,
 * MonteCarloSolver::append_profile_summary). */
int phmc_solver_append_summary(phmc_solver* s, int64_t total_seconds);
void phmc_solver_destroy(phmc_solver* s);

/* ---- batched instances (no counterpart in the reference's API; the
 * reference runs one instance per process) ----
 * A batch holds independent solvers, one per configuration (films of
 * different thickness, grid, carrier count and seed) sharing the materials;
 * each advances on its own stream by replaying its captured step graph, so
 * the instances' kernels overlap on the device. */
typedef struct phmc_batch phmc_batch;

/* Host geometry of a configuration (SimulationDomain, include/SimulationDomain.h:14-99):
 * facets, boundary assignment, cells and the voxel -> cell map, with point
 * membership and cell lookup. No device work. */
typedef struct phmc_domain phmc_domain;
/* With cfg->output_folder set, writes summary.txt (domain part) and
 * grid_centers.csv there, as SimulationDomain's constructor does. */
int phmc_domain_create(const phmc_config* cfg, phmc_domain** out);
void phmc_domain_destroy(phmc_domain* d);
/* counts; shape3 = voxel grid, bounds6 = min xyz, max xyz; volume in A^3 */
int phmc_domain_info(const phmc_domain* d, int32_t* n_facets, int32_t* n_cells, int32_t* n_faces, int32_t* shape3,
                     double* volume, double* bounds6);
/* per facet: outward normal, centroid, area, condition, value (K or Angstrom),
 * periodic partner (-1) and shift to it; any pointer may be NULL */
int phmc_domain_facets(const phmc_domain* d, double* normal3, double* centroid3, double* area, char* condition,
                       double* value, int32_t* pair, double* shift3);
/* cell centres and volumes [n_cells], voxel -> cell map [nx*ny*nz]; any may be NULL */
int phmc_domain_cells(const phmc_domain* d, double* centers3, double* volumes, int32_t* voxel_cell);
/* mesh domains: oriented faces [n_faces][3], vertices [n_faces*3][3] as a
 * triangle soup, and the facet of each face; any may be NULL */
int phmc_domain_faces(const phmc_domain* d, int32_t* face_to_facet, double* triangles9);
int phmc_domain_contains(const phmc_domain* d, int64_t n, const double* p3, uint8_t* inside);
/* voxel [nx*ny*nz] -> 1 when every point of its box lies inside the mesh (no
 * face's bounding box reaches it, its centre inside): the containment check
 * of the carrier loop skips the ray cast of carriers in such voxels. Mesh
 * domains other than extruded prisms; 0 elsewhere. */
int phmc_domain_voxel_interior(const phmc_domain* d, uint8_t* interior);
int phmc_domain_grid_index(const phmc_domain* d, int64_t n, const double* p3, int32_t* cell);
/* closest facet of each point (-1 for none), src/SurfaceMesh.cpp:996-1003 */
/* Wall trace of rays from p (velocity v): hit point, time, facet (-1 and
 * infinite time on a miss), by the host domain (SimulationDomain::
 * trace_boundary_intersection, src/SimulationDomain.cpp:341-450). */
int phmc_domain_trace(const phmc_domain* d, int64_t n, const double* p3, const double* v3, double* hit3, double* t,
                      int32_t* facet);
int phmc_domain_nearest_facet(const phmc_domain* d, int64_t n, const double* p3, int32_t* facet);
/* The same traces by the device code of a mesh domain (face BVH, or the
 * facet scan of an extruded prism). */
int phmc_dev_domain_trace(const phmc_domain* d, int64_t n, const double* p3, const double* v3, double* hit3,
                          double* t, int32_t* facet);
/* The same membership / nearest-facet / cell queries evaluated by the device
 * code of the carrier loop on a device copy of a mesh domain (nearest may be NULL). */
int phmc_dev_domain_query(const phmc_domain* d, int64_t n, const double* p3, uint8_t* inside, int32_t* nearest,
                          int32_t* cell);
int phmc_batch_create(const phmc_config* cfgs, int n, phmc_material* const* materials, int n_materials,
                      phmc_batch** out);
int phmc_batch_size(const phmc_batch* b, int* n);
int phmc_batch_run(phmc_batch* b, int steps);
/* `steps` steps of every instance bracketed by CUDA events: device time of the
 * whole batch, carrier-steps summed over instances, kernels launched. */
int phmc_batch_timed_run(phmc_batch* b, int steps, double* total_ms, double* carrier_steps, int64_t* launches);
int phmc_batch_stats(phmc_batch* b, int i, phmc_stats* out);
int phmc_batch_cells(phmc_batch* b, int i, double* temperature, double* energy_density, double* heat_flux3);
int phmc_batch_cell_count(const phmc_batch* b, int i, int* cells);
void phmc_batch_destroy(phmc_batch* b);

/* ---- deterministic sub-steps on the device (parity entry points) ---- */
/* Box ray trace for n rays; returns hit point, time and facet (-1 on miss). */
int phmc_dev_trace_box(const double lo[3], const double hi[3], int64_t n, const double* p3, const double* v3,
                       double* hit3, double* t, int32_t* facet);
/* No counterpart in the reference: phmc_dev_trace_box without any device
 * allocation, for callers that cannot allocate device memory at call time (a
 * process whose device memory is held by another allocator or pool, or a
 * caller that must not hit the device-wide synchronization of cudaFree while
 * a solver steps on another stream). Rays are staged in one static device
 * block of PHMC_NOALLOC_MAX_RAYS rays: larger n returns 1 before any device
 * work. Calls on one device share that block and are serialized by a
 * process-wide lock. The first call per device resolves the block's address
 * and creates a non-blocking stream (n = 0 performs only this setup); make it
 * before any phase in which the device must not allocate, such as a stream
 * capture. `misses` (may be null) receives the number of rays without a
 * facet. */
#define PHMC_NOALLOC_MAX_RAYS 65536
int phmc_dev_trace_box_noalloc(const double lo[3], const double hi[3], int64_t n, const double* p3, const double* v3,
                               double* hit3, double* t, int32_t* facet, int64_t* misses);
/* Ray traces through a closed triangle surface (faces oriented, facet id per
 * face) with the face BVH: hit point, time (infinity on a miss) and facet (-1
 * on a miss). Replaces SurfaceMesh::trace_boundary_intersection
 * (src/SurfaceMesh.cpp:1164-1269). */
int phmc_dev_trace_mesh(int nv, const double* vertices, int nf, const int32_t* faces, const int32_t* face_to_facet,
                        int64_t n, const double* p3, const double* v3, double* hit3, double* t, int32_t* facet);
/* Diffuse-mismatch interface events between material a (0) and b (1) with
 * explicit energy weights and uniforms u[3*i..3*i+2]; the interface is normal to
 * `axis`, each event goes from src[i] to the other material. Replaces
 * InterfaceInteraction::interact (src/solver/InterfaceInteraction.cpp:46-153).
 * action: 3 reflect, 4 transmit, 5 invalid outgoing mode (linearized). */
int phmc_dev_interface(const phmc_material* a, const phmc_material* b, double weight_a, double weight_b, int axis,
                       double frequency_bin_thz, double reference_temperature, int linearized, int64_t n,
                       const int32_t* src, const int32_t* flat_in, const int32_t* signs_in, const double* occ_in,
                       const double* u3, int32_t* action, int32_t* material_out, int32_t* flat_out,
                       int32_t* signs_out, double* occ_out);
/* Piecewise-linear E -> T inversion on a material's lookup table. */
int phmc_dev_temperature_from_energy(const phmc_material* m, int64_t n, const double* energy, double* temperature);
/* Energy-conserving RTA on carriers grouped by cell (flat modes, one material). */
int phmc_dev_rta_collide(const phmc_material* m, int64_t n, const int32_t* flat_mode, const int32_t* cell,
                         double* occupation, int cells, const double* cell_temperature, double dt,
                         double particle_volume, int local_lifetime, double lifetime_temperature,
                         double* residual_ev);
/* One cell of nonlinear Callaway (N(dt/2), R(dt), N(dt/2) moment-matched Bose BGK
 * substeps): n_modes modes (omega rad/ps, wavevector[3*n_modes], normal and
 * resistive rates 1/ps), n carriers with their mode index and occupation
 * (updated in place) at cell temperature T (K) over dt (ps). */
int phmc_dev_ncallaway_evolve(int32_t n_modes, const double* omega, const double* wavevector,
                              const double* normal_rate, const double* resistive_rate, int64_t n,
                              const int32_t* mode, double* occupation, double temperature, double dt);
/* Linearized RTA (model 0) or Callaway (model 1) collision at reference temperature Tref. */
int phmc_dev_linear_collide(const phmc_material* m, int model, double Tref, int64_t n, const int32_t* flat_mode,
                            const int32_t* cell, double* occupation, int cells, double dt, double particle_volume,
                            double* residual_ev);
/* Rough reflection with explicit uniforms u[3*i..3*i+2] for n incoming carriers. */
int phmc_dev_rough_reflect(const phmc_material* m, int conservative, double Tref, const double normal_out[3],
                           double roughness_a, int64_t n, const int32_t* flat_in, const double* occ_in,
                           const double* u3, int32_t* flat_out, double* occ_out);
/* Specular matches of the rough tables of nf facets (outward normals[3*f..],
 * roughness in Angstrom) built with the device scan (device = 1) or the host
 * loop (device = 0): match[f * active + ai] = matched outgoing active mode or -1
 * (RoughBoundarySampler::build, src/solver/RoughBoundarySampler.cpp:286-310). */
int phmc_dev_rough_spec_match(const phmc_material* m, int conservative, double Tref, int32_t nf,
                              const double* normals_out, const double* roughness_a, int device, int32_t* match);
/* Periodic-gradient drive on carriers grouped by cell. */
int phmc_dev_gradient_drive(const phmc_material* m, int axis, double gradient, double Tref, int64_t n,
                            const int32_t* flat_mode, const int32_t* cell, double* occupation, int cells,
                            double dt, double particle_volume, double* energy_ev);

#ifdef __cplusplus
}
#endif
#endif
