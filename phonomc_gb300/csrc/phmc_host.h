// Host-side model of PhonoMC's per-timestep carrier loop: configuration,
// phonon material, box domain and the immutable sampling tables that the CUDA
// kernels (and the CPU oracle used by the tests) read every step.
//
// The classes keep the reference's names and query semantics:
//   SimulationConfig   include/SimulationConfig.h:42-156 (the fields this path reads)
//   PhononMaterial     include/PhononMaterial.h:14-125, src/PhononMaterial.cpp,
//                      src/material/Thermodynamics.cpp
//   SimulationDomain   include/SimulationDomain.h:14-99 (analytic box geometry)
//   RoughTables        src/solver/RoughBoundarySampler.cpp:77-368
//   ReservoirTables    src/solver/ReservoirSampler.cpp:17-101
// Everything is flattened into `Problem`, the one structure uploaded to HBM.
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "phmc_rng.h"

namespace phmc {

constexpr double kHbarEvPs = 6.582119569e-4;
constexpr double kBoltzmannEvK = 8.617333262145e-5;
constexpr double kPi = 3.14159265358979323846;

using Vec3 = std::array<double, 3>;

// ------------------------------------------------------------------ config
enum class CollisionModel { Rta, Callaway };
enum class BoundaryCondition : char { ThermalReservoir = 'T', Periodic = 'P', Rough = 'R' };
enum class InitialTemperatureMode { Uniform, Linear };

// Subset of the reference's SimulationConfig read by the carrier loop, with the
// same names, units (lengths in Angstrom internally, as after parsing) and
// defaults (include/SimulationConfig.h:42-146).
enum class HeatSourceProfile { Uniform, Gaussian };
enum class HeatSourceSpectrum { Thermal, Weighted, Gaussian };
enum class HeatSourceTimeProfile { Constant, Pulsed };

struct SimulationConfig {
    std::string model = "box";
    std::vector<double> sizes{200.0, 200.0, 200.0}; // Angstrom
    double particle_count = 1e4;
    double time_step = 1.0;
    int iterations = 10000;
    int convergence_write_interval = 10;
    uint64_t random_seed = 12345;
    bool compute_kappa = false;
    int transport_axis = -1;
    std::optional<double> temperature_gradient;
    double temperature_lookup_dt = 0.1;
    double background_temperature = 300.0;
    bool lifetime_temperature_is_local = true;
    double lifetime_temperature = 300.0;
    CollisionModel collision_model = CollisionModel::Rta;
    bool conservative_boundaries = false;
    std::array<int, 3> grid{1, 1, 1};
    InitialTemperatureMode initial_temperature_mode = InitialTemperatureMode::Uniform;
    double initial_temperature = 300.0;
    // Per box face in facet order xmin,xmax,ymin,ymax,zmin,zmax: condition and value
    // (reservoir K, roughness in nm as in TOML; zero for periodic). Periodic faces
    // are paired with the opposite face of the same axis.
    std::array<char, 6> face_condition{'R', 'R', 'R', 'R', 'R', 'R'};
    std::array<double, 6> face_value{0, 0, 0, 0, 0, 0};
    // Surface-mesh domains (include/SimulationConfig.h:43-86): `model` is the
    // path of an STL (nm, scaled to Angstrom) or OBJ file, or "mesh" with the
    // triangles given in mesh_vertices (Angstrom) / mesh_faces. Boundary
    // regions are relative boxes [xmin,ymin,zmin,xmax,ymax,zmax] over the
    // bounding box that select facets by centroid; later regions override.
    std::vector<Vec3> mesh_vertices;
    std::vector<std::array<int, 3>> mesh_faces;
    bool merge_coplanar_facets = true;
    // geometry.extruded_z: a constant-height prism (vertical side walls, flat
    // top and bottom), traced by its facets and gridded with exact cut-cell
    // volumes (src/SimulationDomain.cpp:206-260, 344-396, 650-740)
    bool extruded_z = false;
    std::vector<std::array<double, 6>> boundary_position;
    std::vector<char> boundary_conditions;
    std::vector<double> boundary_values;   // K for 'T', roughness in nm for 'R', 0 for 'P'
    std::vector<std::array<double, 6>> periodic_pair; // region pairs, matched facet by facet
    std::string output_folder;
    bool write_cell_heat_flux = false; // grid_heat_flux.csv also without a gradient drive
    bool callaway_nonlinear = false;   // collision.callaway_formulation = "nonlinear"
    // Device scheduling, no counterpart in the reference (0: tuned default,
    // see phmc_tuning.h): carrier sort interval (< 0 never), threads per CTA
    // and resident CTAs per SM of the carrier pass, bin-tally aggregation,
    // shared-memory staging of the mixed carrier pass.
    int carrier_sort_interval = 0;
    int transport_block = 0;
    int transport_blocks_per_sm = 0;
    int tally_aggregation = 0;
    int transport_pipeline = 0;
    int rta_cell_update = 0; // 1 fused warp-per-cell RTA cell kernel, < 0 separate kernels, 0 by grid size
    std::string material_folder; // reported in summary.txt; tables enter as arrays
    // Layered materials (include/SimulationConfig.h:93-99): N materials, N-1 planes.
    int material_interface_axis = 0;
    std::vector<double> material_interface_positions; // Angstrom
    double material_interface_frequency_bin_thz = 0.1;
    int material_interface_model = 0; // 0 = diffuse mismatch (dmm), 1 = acoustic (amm), 2 = mixed (mmm)
    double material_interface_amm_fraction = 0.0;      // mmm: acoustic-model probability per event
    double material_interface_parallel_bin_inv_a = 0.05; // amm search bins in k parallel
    std::vector<double> material_mass_densities_kg_m3; // one per material (amm / mmm)
    // Prescribed lattice heat source (include/SimulationConfig.h:103-139), lengths in Angstrom.
    bool heat_source_enabled = false;
    std::vector<double> heat_source_min, heat_source_max;
    double heat_source_power_density = 0.0; // W/m^3
    std::optional<double> heat_source_total_power; // W
    HeatSourceSpectrum heat_source_spectrum = HeatSourceSpectrum::Thermal;
    std::optional<double> heat_source_frequency_center, heat_source_frequency_sigma; // THz
    std::vector<int> heat_source_branches;
    std::vector<double> heat_source_branch_weights;
    double heat_source_frequency_min = -1.0, heat_source_frequency_max = -1.0; // THz, <0: no cut
    HeatSourceProfile heat_source_profile = HeatSourceProfile::Uniform;
    std::vector<double> heat_source_center, heat_source_centers, heat_source_sigma, heat_source_half_width;
    std::vector<double> heat_source_power_densities;
    HeatSourceTimeProfile heat_source_time_profile = HeatSourceTimeProfile::Constant;
    double heat_source_time_start = 0.0, heat_source_time_end = -1.0, heat_source_period = 0.0;
    double heat_source_on_duration = -1.0, heat_source_duty_cycle = 0.5, heat_source_amplitude = 1.0;
};

void validate_heat_source_config(const SimulationConfig& c);
// Steps between carrier sorts, 0 for never: the configured interval, else the
// tuned default of the carrier state (plain FP64 or mixed) for populations of
// at least tuning::kSortMinCarriers. A sort is
// a stable reordering of the carrier slots by (active mode, cell) -- by (cell,
// active mode) in mesh domains -- with dead slots last, at the start of every
// step whose index (steps completed, 0 included) is a multiple of the interval.
int resolved_sort_interval(const SimulationConfig& c, bool mixed);
// Source energy factor (ps) of [begin, end] under the time profile
// (src/solver/HeatSourceDriving.cpp:12-44).
double heat_source_time_factor(const SimulationConfig& c, double begin_ps, double end_ps);

// include/SimulationConfig.h:148-156
inline bool uses_linearized_transport(const SimulationConfig& c) {
    return (c.collision_model == CollisionModel::Callaway && !c.callaway_nonlinear) || c.temperature_gradient.has_value();
}
inline bool uses_conservative_transport(const SimulationConfig& c) {
    return uses_linearized_transport(c) || c.callaway_nonlinear || c.conservative_boundaries;
}

// ------------------------------------------------------------- material
// include/material/MaterialData.h:17-31
struct MaterialData {
    double volume_a3 = 0;
    std::array<Vec3, 3> reciprocal{}; // row i = Cartesian component i of (b1,b2,b3)
    int qpoints = 0, branches = 0;
    std::array<int, 3> mesh{};
    std::vector<double> frequency_thz;
    std::vector<Vec3> qpoint_fractions, group_velocity;
    std::vector<double> temperatures, gamma;
    std::vector<double> gamma_normal, gamma_umklapp;
    std::map<std::string, std::vector<double>> gamma_resistive;
};

void validate_material_data(const MaterialData& d);

// Linear-response (Callaway) modal data on the active bank
// (include/material/CallawayOperator.h:17-24 of the reference).
struct CallawayData {
    std::vector<double> omega, capacity, normal_rate, resistive_rate;
    std::vector<Vec3> wavevector;
};

class PhononMaterial {
public:
    PhononMaterial(MaterialData data, double temperature_lookup_dt = 0.1,
                   bool include_stationary_modes = false, bool complete_callaway_bz = true);

    int active_mode_count() const { return static_cast<int>(active_.size()); }
    int qpoint_count() const { return nq_; }
    int branch_count() const { return nb_; }
    int flat_count() const { return nq_ * nb_; }
    const std::vector<int>& active_flat() const { return active_; }
    int active_index_for_flat(int flat) const {
        return flat >= 0 && flat < flat_count() ? flat_to_active_[flat] : -1;
    }
    double omega(int flat) const { return omega_[flat]; }
    const Vec3& velocity(int flat) const { return vel_[flat]; }
    const Vec3& wavevector(int flat) const { return kvec_[flat]; }
    double wavevector_norm(int flat) const { return knorm_[flat]; }
    double frequency_window(int flat) const { return window_[flat]; }

    double bose_occupation(double T, int flat) const;
    double mode_heat_capacity(double T, int flat) const;
    double linearized_bose_occupation(double T, double Tref, int flat) const;
    double mode_gamma(double T, int flat) const;
    double mode_relaxation_weight(double T, int flat, double dt) const;
    double crystal_energy_density(double T) const;
    double energy_density_from_temperature(double T) const;
    double temperature_from_energy_density(double E) const;
    double energy_density_normalization() const;
    double zero_point_energy_density() const { return zero_point_; }
    CallawayData linearized_rta_data(double T) const;
    CallawayData callaway_data(double T) const;
    bool has_callaway_rates() const { return !gamma_normal_.empty(); }
    const std::vector<double>& gamma_normal() const { return gamma_normal_; }
    const std::vector<double>& gamma_umklapp() const { return gamma_umklapp_; }
    const std::vector<double>& gamma_extra() const { return gamma_extra_; }
    std::array<double, 2> mode_callaway_rates(double T, int flat) const;

    const std::vector<double>& lookup_T() const { return table_T_; }
    const std::vector<double>& lookup_E() const { return table_E_; }
    const std::vector<double>& temperature_samples() const { return temps_; }
    const std::vector<double>& gamma_total() const { return gamma_total_; }
    const std::array<int, 3>& q_mesh() const { return mesh_; }
    const std::array<Vec3, 3>& reciprocal_lattice() const { return reciprocal_; }

    static double interp_linear_clamped(const std::vector<double>& xs, const std::vector<double>& ys,
                                        double x);

private:
    void build_lookup();
    int nq_ = 0, nb_ = 0;
    double volume_ = 1.0, dT_ = 0.1, zero_point_ = 0.0;
    bool stationary_ = false;
    unsigned refinement_ = 1;
    std::vector<double> omega_, knorm_, window_;
    std::vector<Vec3> vel_, kvec_, qfrac_;
    std::vector<int> active_, flat_to_active_;
    std::vector<double> temps_, gamma_total_, gamma_normal_, gamma_umklapp_, gamma_extra_;
    std::vector<double> table_T_, table_E_;
    std::array<Vec3, 3> reciprocal_{};
    std::array<int, 3> mesh_{};
};

// ---------------------------------------------------------------- domain
struct Facet {
    Vec3 normal{}, centroid{};
    double area = 0;
    char condition = 'R';
    double value = 0;      // reservoir temperature (K) or roughness (Angstrom)
    int pair = -1;         // periodic partner facet
    Vec3 shift{};          // periodic translation a -> pair
    int reservoir = -1;    // reservoir index for 'T'
    // Triangles of the facet and their areas (area-weighted injection points,
    // src/geometry/SurfaceSampling.cpp:20-73); a box face has two.
    std::vector<std::array<Vec3, 3>> tris;
    std::vector<double> tri_area;
};

// ------------------------------------------------------ mesh tracing
// Triangle-surface ray trace of the reference's SurfaceMesh: face planes,
// centroids and bounds (src/SurfaceMesh.cpp:455-477), the face BVH (median
// split on the largest centroid extent, leaves of <= 8 faces, none below 65
// faces; :479-553) and the near-first traversal with the plane/closest-point
// face test (:1164-1269). Faces are taken as oriented and grouped by the
// caller (face_to_facet).
struct MeshTracer {
    struct Node {
        Vec3 bmin{}, bmax{};
        int left = -1, right = -1, begin = 0, end = 0;
    };
    std::vector<Vec3> vertices;
    std::vector<std::array<int, 3>> faces;
    std::vector<int> face_to_facet;
    std::vector<Vec3> normals, centroids;
    std::vector<double> k;
    std::vector<std::array<Vec3, 2>> bounds;
    std::vector<Node> nodes;
    std::vector<int> order; // BVH leaf order of the faces
    int root = -1;
    void build(std::vector<Vec3> v, std::vector<std::array<int, 3>> f, std::vector<int> f2f);
    // hit point, time (infinity and the origin on a miss) and facet (-1 on a miss)
    void trace(const Vec3& x, const Vec3& v, Vec3& hit, double& t, int& facet) const;
};

// ------------------------------------------------------- surface mesh
// Closed triangle surface of a mesh domain, restating the reference's
// SurfaceMesh (src/SurfaceMesh.cpp:227-1160): edge list in first-encounter
// order, winding made consistent (BFS over shared edges, each shell with a
// positive signed volume; T-junction surfaces by ray-cast side tests), face
// metrics, the face BVH, coplanar connected faces merged into facets
// (plane keys llround(1e6 n), llround(1e6 d)), the enclosed volume, the
// star tetrahedra used by contains_point and volume sampling (the Delaunay
// path needs the external qdelaunay program; without it the reference uses
// this same star fallback), +x ray-cast membership and nearest-facet queries.
class SurfaceMesh {
public:
    struct Simplex {
        std::array<Vec3, 4> v;
        double volume = 0;
        std::array<Vec3, 2> bounds;
        std::array<std::array<double, 3>, 3> inv;
    };
    void set_merge_coplanar_facets(bool on) { merge_coplanar_ = on; }
    void set_data(std::vector<Vec3> vertices, std::vector<std::array<int, 3>> faces);
    void shift_to_origin();

    const std::vector<Vec3>& vertices() const { return vertices_; }
    const std::vector<std::array<int, 3>>& faces() const { return faces_; }
    const std::vector<Vec3>& face_normals() const { return face_normals_; }
    const std::vector<double>& face_areas() const { return face_areas_; }
    const std::vector<int>& face_to_facet() const { return face_to_facet_; }
    int facet_count() const { return static_cast<int>(facet_faces_.size()); }
    const std::vector<std::vector<int>>& facet_faces() const { return facet_faces_; }
    const std::vector<Vec3>& facet_normals() const { return facet_normals_; }
    const std::vector<Vec3>& facet_centroids() const { return facet_centroids_; }
    const std::vector<double>& facet_areas() const { return facet_areas_; }
    // sorted lengths of the edges used by exactly one face of the facet
    std::vector<double> facet_boundary_edge_lengths(int facet) const;
    const Vec3& bounds_min() const { return bmin_; }
    const Vec3& bounds_max() const { return bmax_; }
    double volume() const { return volume_; }
    const MeshTracer& tracer() const { return tracer_; }
    const std::vector<Simplex>& simplices() const; // empty: no valid decomposition

    bool contains_point(const Vec3& p) const;
    bool contains_point_ray_cast(const Vec3& p) const;
    int nearest_facet(const Vec3& p) const;
    void trace(const Vec3& x, const Vec3& v, Vec3& hit, double& t, int& facet) const { tracer_.trace(x, v, hit, t, facet); }

private:
    void rebuild();
    void compute_edges();
    void orient();
    void compute_face_metrics();
    void compute_facets();
    void build_simplices() const;

    bool merge_coplanar_ = true;
    std::vector<Vec3> vertices_;
    std::vector<std::array<int, 3>> faces_;
    Vec3 bmin_{}, bmax_{};
    double volume_ = 0;
    std::vector<std::array<int, 2>> edges_;
    std::vector<std::vector<int>> edge_faces_;
    std::vector<std::array<int, 3>> face_edges_;
    std::vector<Vec3> face_normals_, face_centroids_;
    std::vector<double> face_areas_;
    std::vector<std::array<int, 2>> face_adjacency_;
    std::vector<int> face_to_facet_;
    std::vector<std::vector<int>> facet_faces_;
    std::vector<std::vector<int>> facet_boundary_edges_;
    std::vector<Vec3> facet_normals_, facet_centroids_;
    std::vector<double> facet_areas_;
    MeshTracer tracer_;
    mutable bool simplices_ready_ = false;
    mutable std::vector<Simplex> simplices_;
};

// STL (binary or ASCII, vertices merged on a 1e-10 lattice) and OBJ readers
// (src/geometry/MeshReader.cpp:60-243). Coordinates as stored in the file.
void read_surface_mesh(const std::string& path, std::vector<Vec3>& vertices, std::vector<std::array<int, 3>>& faces);

// Analytic axis-aligned box (src/SimulationDomain.cpp:73-126, 292-450, 626-766),
// facet f = 2*axis + side, which is the reference's box facet order; or a
// closed surface mesh (model = file path or "mesh"): facets of the merged
// mesh with boundary regions and periodic pairs assigned by facet centroid
// (:452-626), cells at the voxel centres inside the mesh and every voxel
// mapped to an active cell by a breadth-first fill (:626-766).
class SimulationDomain {
public:
    explicit SimulationDomain(const SimulationConfig& cfg);
    ~SimulationDomain();
    bool is_mesh() const { return mesh_ != nullptr; }
    // extruded prism (geometry.extruded_z): its top triangles and the z extent
    bool is_prism() const { return prism_; }
    const std::vector<std::array<Vec3, 3>>& prism_top() const { return prism_top_; }
    const SurfaceMesh* mesh() const { return mesh_.get(); }
    // voxel (ix*ny + iy)*nz + iz -> active cell (mesh domains; identity for boxes)
    const std::vector<int>& voxel_cells() const { return voxel_cell_; }
    // active cell -> its home voxel, the voxel whose centre made the cell
    // (mesh domains; the identity for boxes)
    std::vector<int> cell_voxels() const;
    // voxel -> 1 when every point of its box (widened by 1e-6 of the domain
    // scale) lies inside the mesh: no face's bounding box reaches the widened
    // box and the voxel centre is inside (mesh domains other than prisms)
    const std::vector<unsigned char>& voxel_interior() const { return voxel_interior_; }
    const Vec3& bounds_min() const { return bmin_; }
    const Vec3& bounds_max() const { return bmax_; }
    double volume() const { return volume_; }
    int grid_count() const { return static_cast<int>(centers_.size()); }
    const std::array<int, 3>& grid_shape() const { return shape_; }
    const Vec3& inv_cell() const { return inv_cell_; }
    const std::vector<Vec3>& grid_centers() const { return centers_; }
    const std::vector<double>& grid_volumes() const { return volumes_; }
    const std::vector<Facet>& facets() const { return facets_; }
    const std::vector<int>& reservoir_facets() const { return reservoir_facets_; }
    int fast_grid_index(const Vec3& p) const;
    // Returns (collision point, time, facet); facet -1 and infinite time on a miss.
    void trace(const Vec3& p, const Vec3& v, Vec3& cp, double& t, int& facet) const;
    bool contains_point(const Vec3& p) const;
    int nearest_facet(const Vec3& p) const;

private:
    void build_mesh_domain(const SimulationConfig& cfg);
    int voxel_index(const Vec3& p) const;

    Vec3 bmin_{}, bmax_{}, inv_cell_{};
    double volume_ = 0;
    std::array<int, 3> shape_{1, 1, 1};
    std::vector<Vec3> centers_;
    std::vector<double> volumes_;
    std::vector<Facet> facets_;
    std::vector<int> reservoir_facets_;
    std::unique_ptr<SurfaceMesh> mesh_;
    std::vector<int> voxel_cell_;
    std::vector<unsigned char> voxel_interior_;
    bool prism_ = false;
    std::vector<std::array<Vec3, 3>> prism_top_;
    void build_prism_cells(int nx, int ny, int nz);
    void prism_trace(const Vec3& p, const Vec3& v, Vec3& cp, double& t, int& facet) const;
};

// Layered materials along one axis (src/solver/LayeredMaterialLayout.cpp:24-115).
struct LayeredLayout {
    int axis = 0;
    std::vector<double> planes; // ascending
    int material_at(const Vec3& p) const {
        int m = 0;
        while (m < static_cast<int>(planes.size()) && p[axis] >= planes[m]) ++m;
        return m;
    }
};

// ------------------------------------------------------- heat source
// PrescribedHeatSource (src/solver/PrescribedHeatSource.cpp:22-216): per-cell
// power in eV/ps; PhononSourceOperator's spectral filter
// (src/solver/PhononSourceOperator.cpp:20-130).
struct HeatSourceTables {
    bool enabled = false;
    bool linearized_thermal = false;
    HeatSourceSpectrum spectrum = HeatSourceSpectrum::Thermal;
    std::vector<double> rates;            // [cells] eV/ps
    double frequency_min = -1, frequency_max = -1;
    std::vector<int> branches;
    std::vector<double> weights;          // branch weights scaled by their maximum
    double gaussian_center = 0, gaussian_sigma = 1;
    void configure(const SimulationConfig& c, const SimulationDomain& domain);
    void set_spectrum(const SimulationConfig& c); // the PhononSourceOperator part of configure()
    double mode_weight(const PhononMaterial& m, int flat) const;
};

// ---------------------------------------------------- interface banks
// Diffuse-mismatch mode banks (src/solver/InterfaceModeSampler.cpp:11-44): per
// material and direction (0: v_axis < 0, 1: v_axis > 0) the active modes sorted
// by (omega, active index), with the running sum of |v_axis| / energy-density
// normalization.
struct InterfaceBank {
    std::vector<double> omega;
    std::vector<int> active;
    std::vector<double> prefix; // size + 1
};

// Acoustic-mismatch rows (src/solver/AcousticInterfaceSampler.cpp:18-472): for
// each incoming active mode of one side of an interface, its mirror partner
// (the specular reflection) and the transmitted (destination active mode,
// probability) entries; rows of modes that do not move into the interface
// stay empty (reflected = -1).
struct AmmRow {
    int reflected = -1;
    double flux = 0;
    std::vector<std::pair<int, double>> transmitted;
};
struct AmmFace {
    std::array<std::vector<AmmRow>, 2> rows; // [0]: lower material moving +axis, [1]: upper moving -axis
};
struct AmmTables {
    std::vector<AmmFace> faces; // between material f and f + 1
    // densities kg/m^3 per material; df in THz, dk in 1/Angstrom (search bins only)
    void build(const std::vector<const PhononMaterial*>& mats, int axis, const std::vector<double>& densities,
               double df, double dk);
    static double transmission(double z1, double z2, double c1, double c2);
};

struct InterfaceTables {
    bool enabled = false;
    bool linearized = false;
    int axis = 0;
    double band_width = 0;            // 2 pi * frequency bin (rad/ps)
    double reference_temperature = 300;
    std::vector<std::array<InterfaceBank, 2>> banks; // [material][direction]
    // materials.interface_model: 0 diffuse (dmm), 1 acoustic (amm), 2 mixed (mmm)
    int model = 0;
    double amm_fraction = 0;  // probability of the acoustic model per event (1 for amm)
    AmmTables amm;
    void build(const std::vector<const PhononMaterial*>& mats, int axis);
};

// Outcome of one interface event (src/solver/InterfaceInteraction.cpp:46-153).
enum InterfaceAction { kInterfaceReflect = 3, kInterfaceTransmit = 4, kInterfaceFail = 5, kInterfaceAmmRow = 6 };

// -------------------------------------------------------- rough tables
struct RoughTable {
    int material = 0, facet = -1;
    bool strict_elastic = false;
    std::vector<double> specularity;                    // [active]
    std::vector<int> spec_match, diffuse_begin, diffuse_end; // [active]
    std::vector<int> outgoing_active, outgoing_sorted;
    std::vector<double> outgoing_sorted_omega, residual_prefix; // prefix: size sorted+1
    std::vector<int> roulette_active;
    std::vector<double> roulette_cdf;
};

// The specular-match scan of one facet's table (the O(modes x window) part
// of RoughBoundarySampler::build, src/solver/RoughBoundarySampler.cpp:286-310):
// for every incoming active mode ai with a window [begin[ai], end[ai]) of the
// frequency-sorted outgoing modes `sorted`, match[ai] = the first mode of the
// window that minimises |v_try - v_out| / max(1e-12, |v_try|, |v_out|), with
// v_try = v_ai - 2 (v_ai . n_in) n_in; match[ai] stays -1 when none compares.
struct SpecMatchJob {
    Vec3 n_in;
    const std::vector<int>* incoming;
    const std::vector<int>* begin;
    const std::vector<int>* end;
    const std::vector<int>* sorted;
    std::vector<int>* match;
};
// A scan over all jobs of one material (velocities of its active modes).
using SpecMatchScan = std::function<void(const std::vector<Vec3>& velocities, std::vector<SpecMatchJob>& jobs)>;
// The host scan (OpenMP over facets), in the reference's operation order.
void spec_match_host(const std::vector<Vec3>& velocities, std::vector<SpecMatchJob>& jobs);

// Builds one table per (material, enabled facet) exactly as the reference's
// RoughBoundarySampler::build; facet_table[material * facets + facet] -> table.
// `scan` replaces the host specular-match scan (the device solver passes the
// GPU scan; the results are the same modes).
struct RoughTables {
    std::vector<RoughTable> tables;
    std::vector<int> facet_table;
    void build(const std::vector<const PhononMaterial*>& mats, const std::vector<Vec3>& normals,
               const std::vector<double>& roughness, const std::vector<char>& enabled,
               bool require_discrete, double equilibrium_temperature, const SpecMatchScan* scan = nullptr);
};

// ----------------------------------------------------- reservoir tables
struct Reservoir {
    int facet = -1, material = 0;
    double temperature = 300, area = 0;
    Vec3 normal{};
    std::vector<double> cdf; // over the material's active modes
    // the same emission distribution as an alias table over the active modes:
    // one uniform per draw, O(1), in place of a search of `cdf`
    std::vector<AliasCell> alias;
    double expected = 0;
    int initial_count = 0;
};

// Alias table of a discrete distribution with non-negative weights (positive
// sum), built by Vose's two-worklist method (M. D. Vose, IEEE TSE
// 17(9):972-975, 1991). Outcome k is drawn with probability w_k / sum(w) up
// to rounding; an outcome of weight zero is never drawn.
std::vector<AliasCell> build_alias_table(const std::vector<double>& weights);

// ---------------------------------------------------------------- ledgers
// src/solver/BoundaryLedger.cpp and src/solver/EnergyLedger.cpp, single writer.
struct BoundaryBalance {
    long long absorbed = 0, injected = 0;
    double absorbed_energy_ev = 0, injected_energy_ev = 0;
    long long net() const { return injected - absorbed; }
};
struct EnergyBalance {
    long long source_updates = 0;
    double source_energy_ev = 0, lifetime_residual_ev = 0, balance_residual_ev = 0;
    long long drive_updates = 0;
    double drive_energy_ev = 0;
};
class EnergyLedger {
public:
    void initialize(double e) { thermal_ = e; step_ = {}; total_ = {}; }
    void begin_step() { step_ = {}; }
    void record_drive(long long updates, double e) { step_.drive_updates += updates; step_.drive_energy_ev += e; }
    void record_source(long long updates, double e) { step_.source_updates += updates; step_.source_energy_ev += e; }
    void set_lifetime_residual(double e) { step_.lifetime_residual_ev = e; }
    void finish_step(double energy, const BoundaryBalance& b);
    double thermal_energy_ev() const { return thermal_; }
    const EnergyBalance& step() const { return step_; }
    const EnergyBalance& total() const { return total_; }

private:
    double thermal_ = 0;
    EnergyBalance step_, total_;
};

// ---------------------------------------------------------------- problem
// Flattened per-material tables in active-mode order.
struct MaterialTables {
    int n_active = 0;
    std::vector<int> active_flat;
    std::vector<double> omega, hw, vel; // vel: [active*3]
    std::vector<double> nbg;            // Bose occupation at the background temperature
    std::vector<double> capacity_bg;    // modal heat capacity at the background temperature
    double energy_weight = 0;           // active * particle volume / normalization
    double energy_density_bg = 0;
    double heat_capacity_density_bg = 0;
    double zero_point = 0;
    std::vector<double> lookup_T, lookup_E;
    std::vector<double> temperatures;   // linewidth temperature axis
    std::vector<double> gamma_active;   // [nT * active], total linewidth (THz)
    std::vector<double> relax_fixed;    // RTA weight at the fixed lifetime temperature
    // Linear-response collision data (linearized RTA or Callaway) at T_bg.
    std::vector<double> col_capacity, col_normal, col_resistive, col_k; // col_k: [active*3]
    // nonlinear Callaway: N, U and extra resistive linewidths [nT * active] (THz HWHM)
    std::vector<double> ncl_gamma_n, ncl_gamma_u, ncl_gamma_x;
    // Mode classes: active modes sharing (omega, linewidth row) share the Bose
    // function and RTA weight; per-cell RTA sums aggregate over them.
    int n_classes = 0;
    std::vector<int> mode_class;        // [active]
    std::vector<double> class_omega, class_hw;
    std::vector<int> class_rep;         // representative active mode
    std::vector<double> grad_rate;      // gradient source rate per active mode (eV/ps)
    std::vector<double> occ_reservoir;  // filled per reservoir: [reservoir][active]
};

struct Problem {
    SimulationConfig cfg;
    bool linearized = false, conservative = false;
    bool callaway_nonlinear = false;
    bool one_to_one = true;
    double push_eps = 1e-10;
    double particle_volume = 0;
    std::vector<double> material_spatial_volume; // per material, layered domains (common state weight)
    int initial_particles = 0;
    std::vector<MaterialTables> mats;
    SimulationDomain* domain = nullptr;
    LayeredLayout layout;
    std::vector<int> cell_material;      // [cells]
    RoughTables rough;
    InterfaceTables iface;
    HeatSourceTables source;
    std::vector<int> plane_cell;         // cell boundary index of each interface plane along the layout axis
    std::vector<Reservoir> reservoirs;
    std::vector<std::vector<double>> reservoir_occ; // [reservoir][active of its material]
    double gradient_energy_weight = 0;
    int kappa_axis = 2;
};

// Builds every table. Materials must outlive the problem.
Problem build_problem(const SimulationConfig& cfg, SimulationDomain& domain,
                      const std::vector<const PhononMaterial*>& mats, const SpecMatchScan* scan = nullptr);

// Initial carriers exactly as src/solver/Initialization.cpp:32-137 samples them,
// with Philox draws: positions uniform in the box, modes uniform over the active
// bank, temperatures uniform or linear between the reservoirs, occupations
// Bose or linearized. SoA output; mode word = active | signs<<24 | material<<28.
struct CarrierArrays {
    std::vector<double> x, y, z, occ;
    std::vector<uint32_t> mode;
    std::vector<int32_t> cell;
    std::vector<uint8_t> alive;
};
// preset_xyz: accepted ray-cast positions of a mesh domain without a volume
// decomposition, computed elsewhere from the same draws ([3n]; x NaN: sample
// that carrier here, x +inf: rejected).
CarrierArrays initial_carriers(const Problem& p, const std::vector<const PhononMaterial*>& mats,
                               const double* preset_xyz = nullptr);

// Mode-word helpers shared with the kernels.
constexpr uint32_t kActiveMask = 0x00FFFFFFu;
inline uint32_t mode_word(uint32_t active, uint32_t signs, uint32_t material) {
    return active | (signs << 24) | (material << 28);
}

// Convergence output (src/solver/ResultWriter.cpp:82-119): header and one row.
struct ConvergenceRow {
    int timestep = 0;
    double time_ps = 0;
    std::vector<double> temperatures;
    double heat_flux = 0, kappa_int = 0, kappa_eff = 0;
    long long particle_count = 0, absorbed = 0, injected = 0, net = 0;
    double absorbed_ev = 0, injected_ev = 0;
    long long source_updates = 0;
    double source_ev = 0, lifetime_residual = 0, balance_residual = 0, thermal_energy = 0;
    double source_prescribed = 0, source_pending = 0, source_deposited = 0;
    bool gradient = false;
    long long gradient_updates = 0;
    double gradient_energy = 0;
};
std::string format_convergence_header(size_t cells, bool gradient_driven);
std::string format_convergence_row(const ConvergenceRow& r);

// summary.txt and grid_centers.csv (phmc_output.cpp).
struct RunSummary {
    SimulationConfig cfg;
    uint64_t random_seed = 0;
    long long cache_corrections = 0, cell_index_rebuilds = 0, temperature_refreshes = 0;
    long long rough[8] = {0, 0, 0, 0, 0, 0, 0, 0}; // outcome flags of rough reflections, then events
    int material_count = 1;
    double interface_frequency_bin_thz = 0.1;
    bool conservative = false, fixed_flux_reservoirs = false;
    std::vector<double> material_carrier_volumes_a3;
    long long interface_events = 0, interface_transmitted = 0, interface_reflected = 0;
    long long absorbed_total = 0, injected_total = 0;
    double absorbed_energy_ev = 0, injected_energy_ev = 0;
    long long initial_particle_count = 0, particle_count = 0;
    double particle_spatial_weight_a3 = 0, background_temperature = 300;
    double total_thermal_energy_ev = 0, lifetime_residual_ev = 0, balance_residual_ev = 0;
    bool gradient_driven = false;
    long long gradient_updates = 0;
    double gradient_energy_ev = 0;
    std::string empty_cell_policy = "defer_locally";
    double source_base_power = 0, source_prescribed = 0, source_pending = 0, source_deposited = 0;
    long long source_updates_total = 0, source_updates_step = 0;
    double source_energy_total_ev = 0, source_energy_step_ev = 0;
};
std::string format_domain_summary(const SimulationConfig& cfg, const SimulationDomain& domain);
std::string format_grid_centers(const SimulationDomain& domain);
std::string format_run_summary(const RunSummary& s);
std::string format_cell_flux_header();
std::string format_cell_flux_rows(int timestep, double time_ps, const std::vector<double>& temperatures,
                                  const std::vector<double>& q);
std::string format_source_ledger(const SimulationConfig& c, const SimulationDomain& d, const std::vector<int>& material,
                                 const std::vector<double>& rate_evps, const double* prescribed,
                                 const double* deposited, const double* pending);
std::string format_runtime(long long total_seconds);

} // namespace phmc
