// Device solver: owns the HBM carrier arrays, the uploaded tables and the
// per-step kernel sequence of MonteCarloSolver::run_timestep
// (src/MonteCarloSolver.cpp:348-398), mirrored as
//
//   pass A  k_transport  gradient half-step, free flight + wall events, new cell,
//                        (cell x mode) histogram of counts and energies
//   inject  hole scan + k_inject (reservoir emissions, advanced from emission time)
//   cells   k_cell_solve per cell: energy density and temperature, gradient
//           sums, RTA pseudo-temperature Newton / linearized-RTA coefficients
//   pass B  k_update     collision update, gradient half-step, energy tally
//   ledger  k_cells_final + k_ledger_finish
//
// Every sum that the reference forms over the carriers of one cell is formed
// here from the (cell, mode) histogram: carriers of one mode in one cell share
// frequency, velocity magnitude, rates and equilibrium occupation, so the
// per-cell solves only need the mode multiplicities and summed energies.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include "../../include/phonomc_gb300.h"
#include "phmc_device.cuh"
#include "phmc_host.h"
#include "phmc_sort.cuh"

namespace phmc {


// Per-cell data of the single-pass timestep.
//
// The transport pass bins the post-transport population by (cell, mode):
// multiplicity, summed occupation and summed max(1, n). The cell solve turns
// the bins into the cell energy and temperature and into a pending affine
// update n <- alpha n + beta per (cell, mode) that holds this step's collision
// and both gradient half-steps around the next transport; the next transport
// pass applies it when it loads the carrier. Every collision and drive update
// of the reference is affine in the occupation with coefficients that depend
// only on the carrier's cell and mode, so this reproduces them exactly.
// Population sums of one (cell, mode) bin, accumulated by the transport pass:
// sum of occupations and multiplicity share one 16-byte record, so the two
// atomics of a carrier touch one L2 sector.
// Nonlinear Callaway tables of every material (linewidths in the layout of
// DevMaterial::gamma) and the per-(cell, mode) work space of the moment solve.
struct DevNcl {
    const double* gamma_n[kMaxMaterials]; // [n_temps * active] normal linewidth
    const double* gamma_u[kMaxMaterials]; // umklapp
    const double* gamma_x[kMaxMaterials]; // extra resistive (isotope, boundary)
    const double* k[kMaxMaterials];       // [3 * active] wavevector
    double2* work;                        // [ncells * hist_modes] (sum of occupations, relaxation weight)
    double lifetime_T;
    int local;                            // rates at the cell temperature (else lifetime_T)
};

struct __align__(16) BinSum {
    double N;
    unsigned int cnt;
    unsigned int pad;
};

struct CellArrays {
    int ncells;
    int hist_modes;          // modes per cell in the bins (max active count over materials)
    const int* cell_material;
    const double* volume;
    BinSum* bins;            // [ncells * hist_modes] bin sums (sum of n, multiplicity)
    double2* ab;             // [ncells * hist_modes] pending (alpha, beta)
    double* hM;              // [ncells * hist_modes] summed max(1, n) (RTA only)
    double* energy;          // energy density after transport
    double* temperature;     // temperature after transport
    double* energy_final;    // energy density at the end of the step
    double* temperature_final;
    double* grad_ratio;      // sum of gradient rates / sum of capacities, per cell
    double* flux;            // [ncells*3]
    double* cell_stats;      // [ncells*4] energy deviation, gradient rate sum, capacity sum
    double* cell_final;      // [ncells*4] lifetime residual, drive energy, drive updates, final energy deviation
    int mixed;               // FP32 linear-response exponential with FP64 energy rescale
    // RTA: per (cell, class) (a, n_eq(T*)); the class sums are the bins
    double2* rta_ab;
    // linear response: beta of the pending update per (cell, mode)
    double* lin_beta;
    int lin_cluster;         // CTAs per cell of the cluster exponential
    // linear-response collision (one material): per-mode constants
    const double* lin_decay; // exp(-r dt)
    const double* lin_s;     // sqrt(capacity)
    const double* lin_sqrt_rn;
    const double* lin_sqrt_rr;
    int lin_has_normal;
    // FP32 exponential (mixed precision): per-mode constants without divisions
    const float* lin32_inv_s;     // 1 / sqrt(capacity)
    const float* lin32_rate;      // total collision rate
    const float* lin32_decay;     // exp(-r dt)
    const float* lin32_s_over_hw; // sqrt(capacity) / (hbar omega)
    const float* lin32_basis;     // [5][modes]: s sqrt(r_R), s k_b/omega sqrt(r_N) (b = 0..3, k_0/omega = 1)
    const float* lin32_sqrt_rn;
    const float* lin32_sqrt_rr;
    const double* lin_omd;        // 1 - exp(-r dt)
    const double* lin_bg;         // (1 - exp(-r dt)) n_bg
    int lin_substeps;
    // heat source per cell: power (eV/ps), budgets (eV), Newton scratch [cells][2 * classes]
    const double* src_rate;
    double* src_pending;
    double* src_prescribed;
    double* src_deposited;
    double* src_step_pending;  // budget at the step boundary, before the next step's first accrual
    double* src_step_book;     // [2 ncells] prescribed, deposited at the step boundary, before the next step's first accrual
    double* src_scratch;
    double* src_next;        // [ncells * hist_modes] next step's first source half inside ab.y (null: no source)
    const int* src_cells;    // the cells of positive source power (the only ones a half changes)
    int n_src_cells;
    int src_classes;
    double lin_h;
    int lin_terms;
    // RTA classes of material 0
    const int* class_start;
    const int* class_modes;
    int n_classes;
    // end-of-step sums: one partial per CTA of k_cells_final, folded by the last CTA
    double* final_part;      // [final_blocks * 4]
    unsigned* final_done;    // CTAs finished (reset by the last one)
    int final_blocks;
    // RTA on grids of many cells: entries of the warp's occupied-class list in
    // shared memory (k_rta_cell); 0 runs the separate stats / solve / tables kernels
    int rta_cell_cap;
};

struct StepCounters {
    long long launches = 0;
};

struct LaunchCtx;

// One flux pass in flight: cell temperatures, energies, fluxes and the ledger
// copied into pinned host memory at the pass, processed in step order.
struct Observation {
    int step = 0;
    double elapsed = 0;
    double* T = nullptr;
    double* E = nullptr;
    double* q = nullptr;
    double* src = nullptr; // heat source: per-cell prescribed, deposited, pending (eV)
    DevLedger* L = nullptr;
    cudaEvent_t done = nullptr;
};

void stats_from_ledger(const DevLedger& L, phmc_stats& o);
const char* solver_error_message(int code); // message of a device error code

class DeviceSolver {
public:
    // init_carriers=false leaves the population empty (set_carriers fills it).
    DeviceSolver(const SimulationConfig& cfg, const std::vector<const PhononMaterial*>& mats,
                 bool init_carriers = true, bool mixed = false);
    ~DeviceSolver();
    DeviceSolver(const DeviceSolver&) = delete;
    DeviceSolver& operator=(const DeviceSolver&) = delete;

    void run_timestep();
    void run(int steps);
    void synchronize();
    void check_error();
    void carrier_position(int slot, double p[3], int& facet);
    void carrier_state(long long slot, double out[13]); // phmc_solver_carrier_state
    void read_stats(phmc_stats& out);
    int cell_count() const { return ncells_; }
    void read_cells(double* T, double* E, double* q3);
    long long slot_count();
    void get_carriers(double* x, double* y, double* z, double* occ, uint32_t* mode, int32_t* cell, uint8_t* alive);
    void set_carriers(long long n, const double* x, const double* y, const double* z, const double* occ,
                      const uint32_t* mode, const uint8_t* alive,
                      bool keep_clock = false);
    void write_outputs();
    void write_source_ledger(const double* prescribed, const double* deposited, const double* pending) const;
    void read_source_book(double* h);
    void append_summary(long long total_seconds);
    bool mixed() const { return mixed_; }
    // Deterministic sub-steps on the current population (parity entry points):
    // one collision with the given cell temperatures (or the tallied ones when
    // null), and one gradient half-step; both return the ledger energy.
    double collide_only(const double* cell_temperature);
    // `steps` steps bracketed by CUDA events on the solver stream (graph
    // replays when enabled), after a few event-profiled eager steps whose
    // carrier-pass duration gives kernel_ms (mean per launch). Live carrier
    // counts before and after the timed region are returned.
    void timed_run(int steps, double& total_ms, double& kernel_ms, long long& launches, long long& live_before,
                   long long& live_after);
    // Steps are replayed from a CUDA graph of one captured timestep (default on).
    void set_graphs(bool on) { use_graphs_ = on; }
    // Steps between carrier sorts (0 never).
    int sort_interval() const { return sort_interval_; }
    // Scheduling fields of the configuration (0: tuned default), changed
    // between steps; the step graph is captured again.
    void set_schedule(int sort_interval, int transport_block, int blocks_per_sm, int tally_aggregation,
                      int transport_pipeline);
    double drive_only();
    const Problem& problem() const { return P_; }
    long long launches() const { return counters_.launches; }
    cudaStream_t stream() const { return stream_; }
    // Instances that the fused batch kernels can advance together: box domain,
    // one material, nonlinear RTA, no heat source, no gradient drive, no sorts.
    bool fusable() const;
    // device state of this instance, read by the fused batch kernels
    const DevTables* device_tables() const { return d_tables_; }
    DevLedger* device_ledger() const { return d_ledger_; }
    const CarrierState& carrier_state() const { return state_; }
    const CellArrays& cell_arrays() const { return cells_; }
    int* hole_list() const { return d_holes_; }
    int rta_cell_update() const { return cfg_.rta_cell_update; }
    int* hole_blocks() const { return d_block_dead_; }
    bool has_reservoirs() const { return !P_.reservoirs.empty(); }
    int initial_particles() const { return P_.initial_particles; }
    int carrier_blocks() const;
    // Bookkeeping after a fused batch step: `extras` when the caller has ordered
    // this solver's stream after the step (containment, flux observation due).
    bool batch_extras_due() const;
    void finish_batched_step(long long launches);

private:
    void upload_tables();
    void upload_mesh(const std::vector<DevRoughTable>& rough);
    // mesh domains: per-carrier mirror facet and wall cache (device arrays)
    int32_t* mesh_mirror_ = nullptr;
    double *mesh_hit_t_ = nullptr, *mesh_hit_x_ = nullptr, *mesh_hit_y_ = nullptr, *mesh_hit_z_ = nullptr;
    int32_t* mesh_hit_f_ = nullptr;
    std::vector<int> cell_voxel_host_; // home voxels of a mesh domain's cells (error reports of the mixed state)
    void allocate_state(int capacity);
    void initial_statistics();
    void enqueue_step(bool profile);
    void capture_step_graph();
    void flux_pass();
    // stable reordering of the carrier slots (phmc_sort.cu), every sort_interval_ steps
    void sort_carriers();
    int sort_interval_ = 0;
    SortScratch sort_{};
    void drain_observations(bool wait);
    void process_observation(Observation& o);
    void update_kappa();
    void append_convergence_row(const Observation& o, const phmc_stats& s);

    SimulationConfig cfg_;
    std::vector<const PhononMaterial*> mats_;
    std::unique_ptr<SimulationDomain> domain_;
    Problem P_;
    int ncells_ = 0;
    int step_ = 0;
    double elapsed_ = 0;
    bool failed_ = false;
    bool mixed_ = false;
    cudaStream_t stream_ = nullptr;
    int sm_count_ = 152;
    StepCounters counters_;

    DevTables tables_{};
    DevTables* d_tables_ = nullptr;
    DevLedger* d_ledger_ = nullptr;
    CarrierState state_{};
    CellArrays cells_{};
    int* d_holes_ = nullptr;
    int* d_block_dead_ = nullptr;
    int* d_contain_count_ = nullptr; // carriers queued for the membership test of the containment check
    int n_dead_blocks_ = 0;
    std::vector<void*> allocations_;
    // host-side observables
    double avg_flux_ = 0, kappa_fit_ = 0, kappa_end_ = 0;
    std::vector<double> host_T_, host_E_, host_q_;
    // flux passes copied into pinned host slots and processed when their event completes
    std::vector<struct Observation*> obs_free_, obs_pending_;
    DevNcl ncl_{}; // nonlinear Callaway tables and work space
    unsigned char* lin_work_ = nullptr; // linear Callaway per-mode slices when a cell's modes exceed shared memory
    size_t lin_slice_ = 0;
    // graph of one timestep
    bool use_graphs_ = true;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    long long graph_launches_ = 0;

    bool profile_pass_a_ = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pass_a_events_;
    bool materialized_ = true;
    void materialize();
    struct LaunchCtx ctx() const;
    int collision_kind() const;

    template <class T> T* dalloc(size_t n);
    template <class T> T* upload(const std::vector<T>& v);
};

} // namespace phmc
