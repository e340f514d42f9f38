// extern "C" boundary of libphonomc_gb300.so (declared in include/phonomc_gb300.h).
// Exceptions never cross it: every entry point returns 0 or 1 and stores the
// message for phmc_last_error().
#include "phmc_kernels.cuh"
#include "phmc_pod.h"
#include "phmc_hdf5.h"

#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace phmc;

struct phmc_material {
    std::unique_ptr<PhononMaterial> m;
};

struct phmc_solver {
    std::unique_ptr<DeviceSolver> s;
};

struct phmc_domain {
    SimulationConfig cfg;
    std::unique_ptr<SimulationDomain> d;
};

// Independent instances (films of different thickness, cells, carriers and
// seeds) advancing together: each has its own stream and replays its own
// captured step graph, so the instances' kernels overlap on the device while
// the host only issues one graph launch per instance and step.
struct phmc_batch {
    std::vector<std::unique_ptr<DeviceSolver>> s;
    cudaStream_t master = nullptr;
    // Fused mode (every instance a nonlinear-RTA box with reservoirs, one
    // precision): each kernel of the timestep is one launch over all
    // instances, captured once into a graph on the master stream.
    // The instances split into kBranches ranges of about equal carrier count,
    // each its own chain of fused launches: the graph runs the chains side by
    // side, so one range's FP64 cell solve overlaps another's carrier pass.
    static constexpr int kBranches = 4;
    bool fused = false;
    std::vector<BatchDesc> desc;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> forks;
    std::vector<void*> dev;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<cudaEvent_t> joins;
    long long fused_launches = 0, launches = 0;
    ~phmc_batch() {
        if (master) cudaStreamSynchronize(master);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (done) cudaEventDestroy(done);
        for (cudaEvent_t e : joins) cudaEventDestroy(e);
        for (cudaEvent_t e : forks) cudaEventDestroy(e);
        for (cudaStream_t x : side) cudaStreamDestroy(x);
        for (void* p : dev) cudaFree(p);
        s.clear();
        if (master) cudaStreamDestroy(master);
    }
    template <class T> const T* put(const std::vector<T>& v);
    void build_fused();
    BatchDesc describe(int lo, int hi, int persist);
    void step();
    void sync_all();
};

namespace {
thread_local std::string g_error;

template <class F> int guard(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 1;
    } catch (...) {
        g_error = "unknown error";
        return 1;
    }
}

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

// Device copies that live until the end of one entry point.
struct DevHold {
    std::vector<void*> p;
    DevHold() = default;
    DevHold(const DevHold&) = delete;
    DevHold& operator=(const DevHold&) = delete;
    ~DevHold() {
        for (void* x : p) cudaFree(x);
    }
    template <class T> T* put(const std::vector<T>& v) {
        void* d = nullptr;
        cuda_check(cudaMalloc(&d, std::max<size_t>(1, v.size()) * sizeof(T)), "cudaMalloc");
        p.push_back(d);
        if (!v.empty()) cuda_check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
        return static_cast<T*>(d);
    }
    template <class T> T* put(const T* v, size_t n) {
        T* d = alloc<T>(n);
        if (n) cuda_check(cudaMemcpy(d, v, n * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
        return d;
    }
    template <class T> T* alloc(size_t n) {
        void* d = nullptr;
        cuda_check(cudaMalloc(&d, std::max<size_t>(1, n) * sizeof(T)), "cudaMalloc");
        p.push_back(d);
        cuda_check(cudaMemset(d, 0, std::max<size_t>(1, n) * sizeof(T)), "cudaMemset");
        return static_cast<T*>(d);
    }
};

// Membership, nearest facet and cell of points on the device copy of a mesh domain.
__global__ void k_domain_trace(const __grid_constant__ DevTables T, int n, const double* p3, const double* v3,
                               double* hit3, double* t, int32_t* facet) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p[3] = {p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]};
        const double v[3] = {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]};
        double h[3], tt;
        int f;
        domain_trace_dev(T.fac, p, v, h, tt, f);
        for (int k = 0; k < 3; ++k) hit3[3 * i + k] = h[k];
        t[i] = tt;
        facet[i] = f;
    }
}

__global__ void k_domain_query(const __grid_constant__ DevTables T, int n, const double* p3, uint8_t* inside,
                               int32_t* nearest, int32_t* cell, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p[3] = {p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]};
        const int in = mesh_contains(T.fac, p);
        if (in < 0) atomicExch(err, 1);
        inside[i] = in > 0 ? 1 : 0;
        if (nearest) nearest[i] = mesh_nearest_facet(T.fac, p);
        cell[i] = cell_at(T, p[0], p[1], p[2]);
    }
}

template <class T> struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    explicit DBuf(size_t count) : n(count) { cuda_check(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)), "cudaMalloc"); }
    DBuf(const T* host, size_t count) : DBuf(count) {
        if (count) cuda_check(cudaMemcpy(p, host, count * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    explicit DBuf(const std::vector<T>& v) : DBuf(v.data(), v.size()) {}
    void get(T* host) const {
        if (n) cuda_check(cudaMemcpy(host, p, n * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
    ~DBuf() { cudaFree(p); }
    DBuf(const DBuf&) = delete;
};

__global__ void k_trace_rays(DevDomain D, int64_t n, const double* p3, const double* v3, double* hit3, double* t,
                             int32_t* facet) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double p[3] = {p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]};
        const double v[3] = {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]};
        double cp[3], tt;
        int f;
        trace_box(D, p, v, cp, tt, f);
        for (int a = 0; a < 3; ++a) hit3[3 * i + a] = f >= 0 ? cp[a] : p[a];
        t[i] = tt;
        facet[i] = f;
    }
}

__global__ void k_trace_mesh_rays(DevMesh M, int64_t n, const double* p3, const double* v3, double* hit3, double* t,
                                  int32_t* facet) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double p[3] = {p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]};
        const double v[3] = {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]};
        double h[3], tt;
        int f;
        mesh_trace_dev(M, p, v, h, tt, f);
        for (int a = 0; a < 3; ++a) hit3[3 * i + a] = h[a];
        t[i] = tt;
        facet[i] = f;
    }
}

__global__ void k_interface_rays(const __grid_constant__ DevTables T, int64_t n, const int32_t* src,
                                 const int32_t* ain, const int32_t* signs, const double* occ, const double* u3,
                                 int32_t* action, int32_t* mat, int32_t* aout, int32_t* sout, double* oout) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const IfaceOut r = interface_dev(T, src[i], ain[i], static_cast<uint32_t>(signs[i]), occ[i], 1 - src[i],
                                         u3[3 * i], u3[3 * i + 1], u3[3 * i + 2], 0.0);
        action[i] = r.action;
        mat[i] = r.material;
        aout[i] = r.active;
        sout[i] = static_cast<int32_t>(r.signs);
        oout[i] = r.occ;
    }
}

__global__ void k_inverse_table(const double* E, const double* T, int nt, int64_t n, const double* e, double* out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = table_inverse(E, T, nt, e[i]);
}

__global__ void k_rough_rays(DevRoughTable R, DevMaterial M, int conservative, int64_t n, const int32_t* ain,
                             const double* occ, const double* u3, int32_t* aout, double* oout) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double o;
        unsigned diag;
        aout[i] = rough_sample_dev(R, M, ain[i], occ[i], conservative != 0, u3[3 * i], u3[3 * i + 1], u3[3 * i + 2], o,
                                   diag);
        oout[i] = o;
    }
}

// A one-material periodic column of `cells` cells whose particle volume is `vol`,
// used to run the solver's own collision/drive kernels on given carriers.
SimulationConfig column_config(int64_t n, int cells, double vol, double dt, double Tbg) {
    SimulationConfig c;
    c.sizes = {1.0, 1.0, vol * static_cast<double>(n)};
    c.particle_count = static_cast<double>(n);
    c.time_step = dt;
    c.grid = {1, 1, cells};
    c.face_condition = {'P', 'P', 'P', 'P', 'P', 'P'};
    c.face_value = {0, 0, 0, 0, 0, 0};
    c.background_temperature = Tbg;
    c.transport_axis = 0;
    return c;
}

void load_column(DeviceSolver& s, const PhononMaterial& M, const SimulationConfig& c, int64_t n, const int32_t* flat,
                 const int32_t* cell, const double* occ) {
    std::vector<double> x(n, 0.5), y(n, 0.5), z(n);
    std::vector<uint32_t> mode(n);
    std::vector<uint8_t> alive(n, 1);
    const double dz = c.sizes[2] / c.grid[2];
    for (int64_t i = 0; i < n; ++i) {
        if (cell[i] < 0 || cell[i] >= c.grid[2]) throw std::invalid_argument("carrier cell out of range");
        z[i] = (cell[i] + 0.5) * dz;
        const int a = M.active_index_for_flat(flat[i]);
        if (a < 0) throw std::invalid_argument("Invalid existing collision carrier.");
        mode[i] = static_cast<uint32_t>(a);
    }
    s.set_carriers(n, x.data(), y.data(), z.data(), occ, mode.data(), alive.data());
}

void read_occupations(DeviceSolver& s, int64_t n, double* occ) {
    std::vector<double> x(n), y(n), z(n);
    std::vector<uint32_t> mode(n);
    std::vector<int32_t> cell(n);
    std::vector<uint8_t> alive(n);
    s.get_carriers(x.data(), y.data(), z.data(), occ, mode.data(), cell.data(), alive.data());
}
} // namespace

template <class T> const T* phmc_batch::put(const std::vector<T>& v) {
    void* d = nullptr;
    cuda_check(cudaMalloc(&d, std::max<size_t>(1, v.size()) * sizeof(T)), "cudaMalloc");
    dev.push_back(d);
    cuda_check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy");
    return static_cast<const T*>(d);
}

BatchDesc phmc_batch::describe(int lo, int hi, int persist) {
    const int n = hi - lo;
    std::vector<const DevTables*> tables(n);
    std::vector<CarrierState> states(n);
    std::vector<CellArrays> cells(n);
    std::vector<DevLedger*> ledgers(n);
    std::vector<int*> holes(n), hole_counts(n);
    std::vector<int> capacity(n), carrier_block(n + 1, 0), hole_block(n + 1, 0), cell_begin(n + 1, 0),
        cell_block(n + 1, 0), inject_block(n + 1, 0);
    int chunks = 1;
    int rta_cap = 0;
    bool rta_fused = true;
    for (int i = 0; i < n; ++i) {
        const DeviceSolver& x = *s[lo + i];
        // the batch holds many cells in all: the fused RTA cell update where
        // every instance's classes fit it and none turned it off
        const int cap = x.rta_cell_update() < 0 ? 0 : rta_cell_capacity(x.cell_arrays(), 1);
        rta_fused = rta_fused && cap > 0;
        rta_cap = std::max(rta_cap, cap);
        tables[i] = x.device_tables();
        states[i] = x.carrier_state();
        cells[i] = x.cell_arrays();
        ledgers[i] = x.device_ledger();
        holes[i] = x.hole_list();
        hole_counts[i] = x.hole_blocks();
        capacity[i] = x.carrier_state().capacity;
        // virtual CTAs in proportion to the population (about eight carriers
        // per thread; the grid-stride bodies are correct for any count)
        const int n0 = x.initial_particles();
        carrier_block[i + 1] = carrier_block[i] + std::max(1, (n0 + n0 / 4 + 2047) / 2048);
        inject_block[i + 1] = inject_block[i] + std::max(1, (n0 + 32767) / 32768);
        hole_block[i + 1] = hole_block[i] + (capacity[i] + 1023) / 1024;
        cell_begin[i + 1] = cell_begin[i] + x.cell_arrays().ncells;
        cell_block[i + 1] = cell_block[i] + (x.cell_arrays().ncells + 255) / 256;
        chunks = std::max(chunks, (x.cell_arrays().hist_modes + kStatChunk - 1) / kStatChunk);
    }
    BatchDesc D{};
    D.n = n;
    D.tables = put(tables);
    D.states = put(states);
    D.cells = put(cells);
    D.ledgers = put(ledgers);
    D.holes = put(holes);
    D.hole_counts = put(hole_counts);
    D.capacity = put(capacity);
    D.carrier_block = put(carrier_block);
    D.hole_block = put(hole_block);
    D.cell_begin = put(cell_begin);
    D.cell_block = put(cell_block);
    D.inject_block = put(inject_block);
    D.total_carrier_blocks = carrier_block[n];
    D.total_inject_blocks = inject_block[n];
    D.total_hole_blocks = hole_block[n];
    D.total_cells = cell_begin[n];
    D.total_cell_blocks = cell_block[n];
    D.chunks = chunks;
    D.persist = persist;
    D.rta_cap = rta_fused ? rta_cap : 0;
    if (D.rta_cap) prepare_rta_cell(cells[0]);
    return D;
}

// Per-instance device state behind arrays and the CTA ranges of every fused
// launch; fused when all instances qualify (DeviceSolver::fusable).
void phmc_batch::build_fused() {
    fused = false;
    if (const char* e = std::getenv("PHMC_BATCH_FUSED"))
        if (e[0] == '0') return; // per-instance step graphs on the instance streams
    for (auto& x : s)
        if (!x->fusable() || !x->has_reservoirs() || x->mixed() != s[0]->mixed()) return;
    const int n = static_cast<int>(s.size());
    int dev = 0, sms = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    // contiguous instance ranges of about equal initial carrier count
    const int nb = std::min(kBranches, n);
    double total = 0.0;
    for (auto& x : s) total += x->initial_particles();
    std::vector<int> cut{0};
    double acc = 0.0;
    for (int i = 0; i < n && static_cast<int>(cut.size()) < nb; ++i) {
        acc += s[i]->initial_particles();
        if (acc >= total * static_cast<double>(cut.size()) / nb && i + 1 < n) cut.push_back(i + 1);
    }
    cut.push_back(n);
    const int branches = static_cast<int>(cut.size()) - 1;
    const int persist = std::max(1, sms * 8 / branches);
    desc.clear();
    for (int k = 0; k < branches; ++k) desc.push_back(describe(cut[k], cut[k + 1], persist));
    for (const BatchDesc& D : desc)
        if (D.total_cells > 65535) return; // the per-cell launches put cells on gridDim.y
    side.resize(branches);
    forks.resize(branches);
    for (int k = 0; k < branches; ++k) {
        cuda_check(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
        cuda_check(cudaEventCreateWithFlags(&forks[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    // work queued on the instance streams (uploads, first observations) precedes the graph
    for (auto& x : s) x->synchronize();
    cuda_check(cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
        fused_launches = 0;
        cuda_check(cudaEventRecord(forks[0], master), "cudaEventRecord");
        for (int k = 0; k < branches; ++k) {
            cuda_check(cudaStreamWaitEvent(side[k], forks[0], 0), "cudaStreamWaitEvent");
            fused_launches += launch_fused_step(desc[k], side[k], s[0]->mixed());
        }
        for (int k = 0; k < branches; ++k) {
            cuda_check(cudaEventRecord(forks[k], side[k]), "cudaEventRecord");
            cuda_check(cudaStreamWaitEvent(master, forks[k], 0), "cudaStreamWaitEvent");
        }
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(master, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cuda_check(cudaStreamEndCapture(master, &graph), "cudaStreamEndCapture");
    cuda_check(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    cuda_check(cudaEventCreateWithFlags(&done, cudaEventDisableTiming), "cudaEventCreate");
    joins.resize(s.size());
    for (auto& e : joins) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    fused = true;
}

// One timestep of every instance. Fused: one graph launch on the master
// stream; instances that observe or check containment this step order their
// own stream after it, and the master after their work.
void phmc_batch::step() {
    if (!fused) {
        for (auto& x : s) {
            const long long l0 = x->launches();
            x->run_timestep();
            launches += x->launches() - l0;
        }
        return;
    }
    cuda_check(cudaGraphLaunch(exec, master), "cudaGraphLaunch");
    launches += fused_launches;
    bool recorded = false;
    for (size_t i = 0; i < s.size(); ++i) {
        const bool extras = s[i]->batch_extras_due();
        if (extras) {
            if (!recorded) {
                cuda_check(cudaEventRecord(done, master), "cudaEventRecord");
                recorded = true;
            }
            cuda_check(cudaStreamWaitEvent(s[i]->stream(), done, 0), "cudaStreamWaitEvent");
        }
        const long long l0 = s[i]->launches();
        s[i]->finish_batched_step(0);
        launches += s[i]->launches() - l0;
        if (extras) {
            cuda_check(cudaEventRecord(joins[i], s[i]->stream()), "cudaEventRecord");
            cuda_check(cudaStreamWaitEvent(master, joins[i], 0), "cudaStreamWaitEvent");
        }
    }
}

void phmc_batch::sync_all() {
    cuda_check(cudaStreamSynchronize(master), "cudaStreamSynchronize");
    for (auto& x : s) x->synchronize();
}

extern "C" {

const char* phmc_last_error(void) { return g_error.c_str(); }

int phmc_device_count(int* count) {
    return guard([&] {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
        *count = n;
    });
}

int phmc_material_create(const phmc_material_data* data, double dt, int stationary, int complete_bz,
                         phmc_material** out) {
    return guard([&] {
        auto m = std::make_unique<phmc_material>();
        m->m = std::make_unique<PhononMaterial>(material_from_pod(*data), dt, stationary != 0, complete_bz != 0);
        *out = m.release();
    });
}

void phmc_material_destroy(phmc_material* m) { delete m; }

int phmc_material_load(const char* folder, double dt, int stationary, int complete_bz, phmc_material** out) {
    return guard([&] {
        if (!folder) throw std::invalid_argument("material folder path is null");
        const MaterialFolder f = read_material_folder(folder);
        MaterialData d;
        d.volume_a3 = f.volume_a3;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) d.reciprocal[i][j] = f.reciprocal[i][j];
        d.qpoints = f.qpoints;
        d.branches = f.branches;
        d.mesh = f.mesh;
        d.frequency_thz = f.frequency_thz;
        d.qpoint_fractions.assign(f.qpoint_fractions.begin(), f.qpoint_fractions.end());
        d.group_velocity.assign(f.group_velocity.begin(), f.group_velocity.end());
        d.temperatures = f.temperatures;
        d.gamma = f.gamma;
        d.gamma_normal = f.gamma_normal;
        d.gamma_umklapp = f.gamma_umklapp;
        d.gamma_resistive = f.gamma_resistive;
        auto m = std::make_unique<phmc_material>();
        m->m = std::make_unique<PhononMaterial>(std::move(d), dt, stationary != 0, complete_bz != 0);
        *out = m.release();
    });
}

int phmc_material_save(const phmc_material_data* p, const char* folder) {
    return guard([&] {
        if (!p || !folder) throw std::invalid_argument("material data or folder is null");
        const MaterialData d = material_from_pod(*p);
        MaterialFolder f;
        f.volume_a3 = d.volume_a3;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) f.reciprocal[i][j] = d.reciprocal[i][j];
        f.qpoints = d.qpoints;
        f.branches = d.branches;
        f.mesh = d.mesh;
        f.frequency_thz = d.frequency_thz;
        f.qpoint_fractions.assign(d.qpoint_fractions.begin(), d.qpoint_fractions.end());
        f.group_velocity.assign(d.group_velocity.begin(), d.group_velocity.end());
        f.temperatures = d.temperatures;
        f.gamma = d.gamma;
        f.gamma_normal = d.gamma_normal;
        f.gamma_umklapp = d.gamma_umklapp;
        f.gamma_resistive = d.gamma_resistive;
        write_material_folder(folder, f);
    });
}

int phmc_h5_shape(const char* path, const char* name, int32_t* rank, int64_t* dims) {
    return guard([&] {
        const h5::Dataset d = h5::Reader(path).read(name);
        if (d.dims.size() > 8) throw std::runtime_error("dataset rank above 8");
        *rank = static_cast<int32_t>(d.dims.size());
        for (size_t k = 0; k < d.dims.size(); ++k) dims[k] = static_cast<int64_t>(d.dims[k]);
    });
}

int phmc_h5_read(const char* path, const char* name, double* values) {
    return guard([&] {
        const h5::Dataset d = h5::Reader(path).read(name);
        std::copy(d.values.begin(), d.values.end(), values);
    });
}

int phmc_domain_create(const phmc_config* cfg, phmc_domain** out) {
    return guard([&] {
        if (!cfg || !out) throw std::invalid_argument("phmc_domain_create: null argument");
        auto d = std::make_unique<phmc_domain>();
        d->cfg = config_from_pod(*cfg);
        d->d = std::make_unique<SimulationDomain>(d->cfg);
        if (!d->cfg.output_folder.empty()) { // as the reference's SimulationDomain constructor does
            std::filesystem::create_directories(d->cfg.output_folder);
            std::ofstream(std::filesystem::path(d->cfg.output_folder) / "summary.txt")
                << format_domain_summary(d->cfg, *d->d);
            std::ofstream(std::filesystem::path(d->cfg.output_folder) / "grid_centers.csv")
                << format_grid_centers(*d->d);
        }
        *out = d.release();
    });
}

void phmc_domain_destroy(phmc_domain* d) { delete d; }

int phmc_domain_info(const phmc_domain* d, int32_t* n_facets, int32_t* n_cells, int32_t* n_faces, int32_t* shape3,
                     double* volume, double* bounds6) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        if (n_facets) *n_facets = static_cast<int32_t>(D.facets().size());
        if (n_cells) *n_cells = D.grid_count();
        if (n_faces) *n_faces = D.is_mesh() ? static_cast<int32_t>(D.mesh()->faces().size()) : 12;
        for (int a = 0; a < 3; ++a) {
            if (shape3) shape3[a] = D.grid_shape()[a];
            if (bounds6) {
                bounds6[a] = D.bounds_min()[a];
                bounds6[3 + a] = D.bounds_max()[a];
            }
        }
        if (volume) *volume = D.volume();
    });
}

int phmc_domain_facets(const phmc_domain* d, double* normal3, double* centroid3, double* area, char* condition,
                       double* value, int32_t* pair, double* shift3) {
    return guard([&] {
        const auto& F = d->d->facets();
        for (size_t f = 0; f < F.size(); ++f) {
            for (int a = 0; a < 3; ++a) {
                if (normal3) normal3[3 * f + a] = F[f].normal[a];
                if (centroid3) centroid3[3 * f + a] = F[f].centroid[a];
                if (shift3) shift3[3 * f + a] = F[f].shift[a];
            }
            if (area) area[f] = F[f].area;
            if (condition) condition[f] = F[f].condition;
            if (value) value[f] = F[f].value;
            if (pair) pair[f] = F[f].pair;
        }
    });
}

int phmc_domain_cells(const phmc_domain* d, double* centers3, double* volumes, int32_t* voxel_cell) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        for (int c = 0; c < D.grid_count(); ++c) {
            for (int a = 0; a < 3; ++a)
                if (centers3) centers3[3 * c + a] = D.grid_centers()[c][a];
            if (volumes) volumes[c] = D.grid_volumes()[c];
        }
        if (voxel_cell) {
            const auto& s = D.grid_shape();
            const size_t n = static_cast<size_t>(s[0]) * s[1] * s[2];
            for (size_t v = 0; v < n; ++v)
                voxel_cell[v] = D.is_mesh() ? D.voxel_cells()[v] : static_cast<int32_t>(v);
        }
    });
}

int phmc_domain_faces(const phmc_domain* d, int32_t* face_to_facet, double* triangles9) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        if (!D.is_mesh()) throw std::invalid_argument("phmc_domain_faces: the analytic box has no mesh faces");
        const SurfaceMesh& M = *D.mesh();
        for (size_t f = 0; f < M.faces().size(); ++f) {
            if (face_to_facet) face_to_facet[f] = M.face_to_facet()[f];
            if (triangles9)
                for (int k = 0; k < 3; ++k)
                    for (int a = 0; a < 3; ++a) triangles9[9 * f + 3 * k + a] = M.vertices()[M.faces()[f][k]][a];
        }
    });
}

int phmc_domain_contains(const phmc_domain* d, int64_t n, const double* p3, uint8_t* inside) {
    return guard([&] {
        for (int64_t i = 0; i < n; ++i)
            inside[i] = d->d->contains_point({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]}) ? 1 : 0;
    });
}

int phmc_domain_voxel_interior(const phmc_domain* d, uint8_t* interior) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        const auto& s = D.grid_shape();
        const size_t n = static_cast<size_t>(s[0]) * s[1] * s[2];
        const auto& f = D.voxel_interior();
        for (size_t v = 0; v < n; ++v) interior[v] = f.empty() ? 0 : f[v];
    });
}

int phmc_domain_grid_index(const phmc_domain* d, int64_t n, const double* p3, int32_t* cell) {
    return guard([&] {
        for (int64_t i = 0; i < n; ++i) cell[i] = d->d->fast_grid_index({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]});
    });
}

int phmc_domain_trace(const phmc_domain* d, int64_t n, const double* p3, const double* v3, double* hit3, double* t,
                      int32_t* facet) {
    return guard([&] {
        for (int64_t i = 0; i < n; ++i) {
            Vec3 cp;
            int f = -1;
            d->d->trace({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]}, {v3[3 * i], v3[3 * i + 1], v3[3 * i + 2]}, cp, t[i], f);
            facet[i] = f;
            for (int k = 0; k < 3; ++k) hit3[3 * i + k] = cp[k];
        }
    });
}

int phmc_domain_nearest_facet(const phmc_domain* d, int64_t n, const double* p3, int32_t* facet) {
    return guard([&] {
        for (int64_t i = 0; i < n; ++i) facet[i] = d->d->nearest_facet({p3[3 * i], p3[3 * i + 1], p3[3 * i + 2]});
    });
}

int phmc_material_active_count(const phmc_material* m, int* n) {
    return guard([&] { *n = m->m->active_mode_count(); });
}

int phmc_solver_create(const phmc_config* cfg, phmc_material* const* materials, int n_materials, phmc_solver** out) {
    return guard([&] {
        SimulationConfig c = config_from_pod(*cfg);
        std::vector<const PhononMaterial*> ms;
        for (int i = 0; i < n_materials; ++i) ms.push_back(materials[i]->m.get());
        auto s = std::make_unique<phmc_solver>();
        s->s = std::make_unique<DeviceSolver>(c, ms, true, cfg->precision == 1);
        *out = s.release();
    });
}

int phmc_solver_run_timestep(phmc_solver* s) {
    return guard([&] {
        s->s->run_timestep();
        s->s->synchronize();
    });
}

int phmc_solver_run(phmc_solver* s, int steps) {
    return guard([&] {
        s->s->run(steps);
        s->s->synchronize();
    });
}

int phmc_solver_synchronize(phmc_solver* s) { return guard([&] { s->s->synchronize(); }); }

int phmc_solver_stats(phmc_solver* s, phmc_stats* out) { return guard([&] { s->s->read_stats(*out); }); }

int phmc_solver_cell_count(const phmc_solver* s, int* cells) {
    return guard([&] { *cells = s->s->cell_count(); });
}

int phmc_solver_cells(phmc_solver* s, double* T, double* E, double* q3) {
    return guard([&] { s->s->read_cells(T, E, q3); });
}

int phmc_solver_slot_count(phmc_solver* s, int64_t* n) { return guard([&] { *n = s->s->slot_count(); }); }

int phmc_solver_get_carriers(phmc_solver* s, double* x, double* y, double* z, double* occ, uint32_t* mode,
                             int32_t* cell, uint8_t* alive) {
    return guard([&] { s->s->get_carriers(x, y, z, occ, mode, cell, alive); });
}

int phmc_solver_carrier_state(phmc_solver* s, int64_t slot, double out[13]) {
    return guard([&] { s->s->carrier_state(slot, out); });
}

int phmc_solver_set_carriers(phmc_solver* s, int64_t n, const double* x, const double* y, const double* z,
                             const double* occ, const uint32_t* mode, const uint8_t* alive) {
    return guard([&] { s->s->set_carriers(n, x, y, z, occ, mode, alive); });
}

int phmc_solver_run_from_host(phmc_solver* s, int64_t n, const double* x, const double* y, const double* z,
                              const double* occ, const uint32_t* mode, int steps, double* cell_T) {
    return guard([&] {
        s->s->set_carriers(n, x, y, z, occ, mode, nullptr, true);
        s->s->run(steps);
        s->s->read_cells(cell_T, nullptr, nullptr);
    });
}

int phmc_solver_timed_run(phmc_solver* s, int steps, double* total_ms, double* kernel_ms, int64_t* launches,
                          int64_t* live_before, int64_t* live_after) {
    return guard([&] {
        long long l = 0, n0 = 0, n1 = 0;
        s->s->timed_run(steps, *total_ms, *kernel_ms, l, n0, n1);
        *launches = l;
        if (live_before) *live_before = n0;
        if (live_after) *live_after = n1;
    });
}

int phmc_solver_set_graphs(phmc_solver* s, int on) {
    return guard([&] { s->s->set_graphs(on != 0); });
}

int phmc_solver_sort_interval(const phmc_solver* s, int* steps) {
    return guard([&] { *steps = s->s->sort_interval(); });
}

int phmc_solver_set_schedule(phmc_solver* s, int sort_interval, int transport_block, int blocks_per_sm,
                             int tally_aggregation, int transport_pipeline) {
    return guard([&] {
        s->s->set_schedule(sort_interval, transport_block, blocks_per_sm, tally_aggregation, transport_pipeline);
    });
}

// ---------------------------------------------------------------- batches
int phmc_batch_create(const phmc_config* cfgs, int n, phmc_material* const* materials, int n_materials,
                      phmc_batch** out) {
    return guard([&] {
        if (n <= 0) throw std::invalid_argument("a batch needs at least one instance");
        std::vector<const PhononMaterial*> ms;
        for (int i = 0; i < n_materials; ++i) ms.push_back(materials[i]->m.get());
        auto b = std::make_unique<phmc_batch>();
        for (int i = 0; i < n; ++i) {
            SimulationConfig c = config_from_pod(cfgs[i]);
            b->s.push_back(std::make_unique<DeviceSolver>(c, ms, true, cfgs[i].precision == 1));
        }
        cuda_check(cudaStreamCreateWithFlags(&b->master, cudaStreamNonBlocking), "cudaStreamCreateWithFlags");
        b->build_fused();
        *out = b.release();
    });
}

int phmc_batch_size(const phmc_batch* b, int* n) {
    *n = static_cast<int>(b->s.size());
    return 0;
}

int phmc_batch_run(phmc_batch* b, int steps) {
    return guard([&] {
        for (int k = 0; k < steps; ++k) b->step();
        b->sync_all();
    });
}

int phmc_batch_timed_run(phmc_batch* b, int steps, double* total_ms, double* carrier_steps, int64_t* launches) {
    return guard([&] {
        b->sync_all();
        std::vector<long long> n0(b->s.size());
        for (size_t i = 0; i < b->s.size(); ++i) {
            phmc_stats st;
            b->s[i]->read_stats(st);
            n0[i] = st.particle_count;
        }
        const long long l0 = b->launches;
        cudaEvent_t start, stop;
        cuda_check(cudaEventCreate(&start), "cudaEventCreate");
        cuda_check(cudaEventCreate(&stop), "cudaEventCreate");
        std::vector<cudaEvent_t> done(b->s.size());
        for (auto& e : done) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        // every instance stream starts after `start` and the master waits for all of them
        cuda_check(cudaEventRecord(start, b->master), "cudaEventRecord");
        for (auto& s : b->s) cuda_check(cudaStreamWaitEvent(s->stream(), start, 0), "cudaStreamWaitEvent");
        for (int k = 0; k < steps; ++k) b->step();
        for (size_t i = 0; i < b->s.size(); ++i) {
            cuda_check(cudaEventRecord(done[i], b->s[i]->stream()), "cudaEventRecord");
            cuda_check(cudaStreamWaitEvent(b->master, done[i], 0), "cudaStreamWaitEvent");
        }
        cuda_check(cudaEventRecord(stop, b->master), "cudaEventRecord");
        cuda_check(cudaEventSynchronize(stop), "cudaEventSynchronize");
        float ms = 0;
        cuda_check(cudaEventElapsedTime(&ms, start, stop), "cudaEventElapsedTime");
        *total_ms = ms;
        double cs = 0;
        for (size_t i = 0; i < b->s.size(); ++i) {
            phmc_stats st;
            b->s[i]->read_stats(st);
            cs += 0.5 * static_cast<double>(n0[i] + st.particle_count) * steps;
        }
        *carrier_steps = cs;
        *launches = b->launches - l0;
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        for (auto& e : done) cudaEventDestroy(e);
    });
}

int phmc_batch_stats(phmc_batch* b, int i, phmc_stats* out) {
    return guard([&] {
        b->sync_all();
        b->s.at(static_cast<size_t>(i))->read_stats(*out);
    });
}

int phmc_batch_cells(phmc_batch* b, int i, double* temperature, double* energy_density, double* heat_flux3) {
    return guard([&] {
        b->sync_all();
        b->s.at(static_cast<size_t>(i))->read_cells(temperature, energy_density, heat_flux3);
    });
}

int phmc_batch_cell_count(const phmc_batch* b, int i, int* cells) {
    return guard([&] { *cells = b->s.at(static_cast<size_t>(i))->cell_count(); });
}

void phmc_batch_destroy(phmc_batch* b) { delete b; }

int phmc_host_register(void* ptr, int64_t bytes) {
    return guard([&] { cuda_check(cudaHostRegister(ptr, static_cast<size_t>(bytes), cudaHostRegisterDefault), "cudaHostRegister"); });
}

int phmc_host_unregister(void* ptr) {
    return guard([&] { cuda_check(cudaHostUnregister(ptr), "cudaHostUnregister"); });
}

int phmc_solver_write_outputs(phmc_solver* s) { return guard([&] { s->s->write_outputs(); }); }

int phmc_solver_append_summary(phmc_solver* s, int64_t total_seconds) {
    return guard([&] { s->s->append_summary(static_cast<long long>(total_seconds)); });
}

void phmc_solver_destroy(phmc_solver* s) { delete s; }

// ------------------------------------------------------------- sub-steps
int phmc_dev_trace_box(const double lo[3], const double hi[3], int64_t n, const double* p3, const double* v3,
                       double* hit3, double* t, int32_t* facet) {
    return guard([&] {
        DevDomain D{};
        double scale = 1.0;
        for (int a = 0; a < 3; ++a) {
            D.lo[a] = lo[a];
            D.hi[a] = hi[a];
            scale = std::max(scale, std::abs(hi[a] - lo[a]));
        }
        D.scale = scale;
        D.tol = std::max(1e-9, 64.0 * std::numeric_limits<double>::epsilon() * scale);
        DBuf<double> dp(p3, 3 * n), dv(v3, 3 * n), dh(3 * n), dt(n);
        DBuf<int32_t> df(n);
        k_trace_rays<<<256, 256>>>(D, n, dp.p, dv.p, dh.p, dt.p, df.p);
        cuda_check(cudaDeviceSynchronize(), "k_trace_rays");
        dh.get(hit3);
        dt.get(t);
        df.get(facet);
    });
}

int phmc_dev_trace_mesh(int nv, const double* vertices, int nf, const int32_t* faces, const int32_t* face_to_facet,
                        int64_t n, const double* p3, const double* v3, double* hit3, double* t, int32_t* facet) {
    return guard([&] {
        MeshTracer T;
        std::vector<Vec3> V(nv);
        for (int i = 0; i < nv; ++i) V[i] = {vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]};
        std::vector<std::array<int, 3>> F(nf);
        for (int i = 0; i < nf; ++i) F[i] = {faces[3 * i], faces[3 * i + 1], faces[3 * i + 2]};
        T.build(std::move(V), std::move(F), std::vector<int>(face_to_facet, face_to_facet + nf));
        DevHold hold;
        DevMesh M;
        fill_dev_mesh(T, M, [&](const auto& v) { return hold.put(v); });
        DBuf<double> dp(p3, 3 * n), dvv(v3, 3 * n), dh(3 * n), dt(n);
        DBuf<int32_t> dfc(n);
        k_trace_mesh_rays<<<256, 128>>>(M, n, dp.p, dvv.p, dh.p, dt.p, dfc.p);
        cuda_check(cudaDeviceSynchronize(), "k_trace_mesh_rays");
        dh.get(hit3);
        dt.get(t);
        dfc.get(facet);
    });
}

int phmc_dev_domain_trace(const phmc_domain* d, int64_t n, const double* p3, const double* v3, double* hit3,
                          double* t, int32_t* facet) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        if (!D.is_mesh()) throw std::invalid_argument("phmc_dev_domain_trace: the analytic box has no mesh");
        if (n < 0 || n > (int64_t{1} << 31) - 1) throw std::invalid_argument("phmc_dev_domain_trace: bad ray count");
        DevHold hold;
        DevTables T;
        std::memset(&T, 0, sizeof T);
        double scale = 1.0;
        for (int a = 0; a < 3; ++a) scale = std::max(scale, std::abs(D.bounds_max()[a] - D.bounds_min()[a]));
        fill_dev_facets(D, scale, T.fac, [&](const auto& v) { return hold.put(v); });
        if (n == 0) return;
        DBuf<double> dp(p3, 3 * n), dv(v3, 3 * n), dh(3 * n), dt(n);
        DBuf<int32_t> df(n);
        k_domain_trace<<<256, 128>>>(T, static_cast<int>(n), dp.p, dv.p, dh.p, dt.p, df.p);
        cuda_check(cudaDeviceSynchronize(), "k_domain_trace");
        dh.get(hit3);
        dt.get(t);
        df.get(facet);
    });
}

int phmc_dev_domain_query(const phmc_domain* d, int64_t n, const double* p3, uint8_t* inside, int32_t* nearest,
                          int32_t* cell) {
    return guard([&] {
        const SimulationDomain& D = *d->d;
        if (!D.is_mesh()) throw std::invalid_argument("phmc_dev_domain_query: the analytic box has no mesh");
        if (n < 0 || n > (int64_t{1} << 31) - 1) throw std::invalid_argument("phmc_dev_domain_query: bad point count");
        DevHold hold;
        DevTables T;
        std::memset(&T, 0, sizeof T);
        double scale = 1.0;
        for (int a = 0; a < 3; ++a) {
            T.dom.lo[a] = D.bounds_min()[a];
            T.dom.hi[a] = D.bounds_max()[a];
            T.dom.inv_cell[a] = D.inv_cell()[a];
            T.dom.shape[a] = D.grid_shape()[a];
            scale = std::max(scale, std::abs(D.bounds_max()[a] - D.bounds_min()[a]));
        }
        T.dom.scale = scale;
        fill_dev_facets(D, scale, T.fac, [&](const auto& v) { return hold.put(v); });
        if (n == 0) return;
        DBuf<double> dp(p3, 3 * n);
        DBuf<uint8_t> din(n);
        DBuf<int32_t> dnear(n), dcell(n);
        DBuf<int> derr(1);
        cuda_check(cudaMemset(derr.p, 0, sizeof(int)), "cudaMemset");
        k_domain_query<<<256, 128>>>(T, static_cast<int>(n), dp.p, din.p, nearest ? dnear.p : nullptr, dcell.p,
                                     derr.p);
        cuda_check(cudaDeviceSynchronize(), "k_domain_query");
        int err = 0;
        derr.get(&err);
        if (err) throw std::runtime_error("phmc_dev_domain_query: membership ray cast hit-list overflow");
        din.get(inside);
        if (nearest) dnear.get(nearest);
        if (cell) dcell.get(cell);
    });
}

int phmc_dev_interface(const phmc_material* ma, const phmc_material* mb, double wa, double wb, int axis,
                       double bin_thz, double Tref, int linearized, int64_t n, const int32_t* src,
                       const int32_t* flat_in, const int32_t* signs_in, const double* occ_in, const double* u3,
                       int32_t* action, int32_t* material_out, int32_t* flat_out, int32_t* signs_out, double* occ_out) {
    return guard([&] {
        const PhononMaterial* M[2] = {ma->m.get(), mb->m.get()};
        InterfaceTables I;
        I.build({M[0], M[1]}, axis);
        DevTables T;
        std::memset(&T, 0, sizeof T);
        T.iface.enabled = 1;
        T.iface.linearized = linearized != 0;
        T.iface.axis = axis;
        T.iface.band_width = 2.0 * std::acos(-1.0) * bin_thz;
        std::vector<std::unique_ptr<DBuf<double>>> dbl;
        std::vector<std::unique_ptr<DBuf<int>>> ints;
        const double w[2] = {wa, wb};
        for (int k = 0; k < 2; ++k) {
            std::vector<double> om, vel, nbg;
            for (int a = 0; a < M[k]->active_mode_count(); ++a) {
                const int f = M[k]->active_flat()[a];
                om.push_back(M[k]->omega(f));
                nbg.push_back(M[k]->bose_occupation(Tref, f));
                for (int c = 0; c < 3; ++c) vel.push_back(M[k]->velocity(f)[c]);
            }
            dbl.emplace_back(new DBuf<double>(om));
            T.mat[k].omega = dbl.back()->p;
            dbl.emplace_back(new DBuf<double>(vel));
            T.mat[k].vel = dbl.back()->p;
            dbl.emplace_back(new DBuf<double>(nbg));
            T.mat[k].nbg = dbl.back()->p;
            T.mat[k].energy_weight = w[k];
            T.mat[k].n_active = M[k]->active_mode_count();
            for (int dir = 0; dir < 2; ++dir) {
                const InterfaceBank& B = I.banks[k][dir];
                dbl.emplace_back(new DBuf<double>(B.omega));
                T.iface.bank[k][dir].omega = dbl.back()->p;
                dbl.emplace_back(new DBuf<double>(B.prefix));
                T.iface.bank[k][dir].prefix = dbl.back()->p;
                ints.emplace_back(new DBuf<int>(B.active));
                T.iface.bank[k][dir].active = ints.back()->p;
                T.iface.bank[k][dir].n = static_cast<int>(B.omega.size());
            }
        }
        std::vector<int32_t> ain(n);
        for (int64_t i = 0; i < n; ++i) ain[i] = M[src[i]]->active_index_for_flat(flat_in[i]);
        DBuf<int32_t> dsrc(src, n), da(ain), dsg(signs_in, n), dact(n), dmat(n), dao(n), dso(n);
        DBuf<double> docc(occ_in, n), du(u3, 3 * n), doo(n);
        k_interface_rays<<<256, 256>>>(T, n, dsrc.p, da.p, dsg.p, docc.p, du.p, dact.p, dmat.p, dao.p, dso.p, doo.p);
        cuda_check(cudaDeviceSynchronize(), "k_interface_rays");
        std::vector<int32_t> ao(n), mo(n);
        dact.get(action);
        dmat.get(mo.data());
        dao.get(ao.data());
        dso.get(signs_out);
        doo.get(occ_out);
        for (int64_t i = 0; i < n; ++i) {
            material_out[i] = mo[i];
            flat_out[i] = M[mo[i]]->active_flat()[ao[i]];
        }
    });
}

int phmc_dev_temperature_from_energy(const phmc_material* m, int64_t n, const double* energy, double* temperature) {
    return guard([&] {
        DBuf<double> E(m->m->lookup_E()), T(m->m->lookup_T()), e(energy, n), out(n);
        k_inverse_table<<<256, 256>>>(E.p, T.p, static_cast<int>(E.n), n, e.p, out.p);
        cuda_check(cudaDeviceSynchronize(), "k_inverse_table");
        out.get(temperature);
    });
}

int phmc_dev_rta_collide(const phmc_material* m, int64_t n, const int32_t* flat, const int32_t* cell, double* occ,
                         int cells, const double* cell_T, double dt, double vol, int local, double Tlife,
                         double* residual) {
    return guard([&] {
        SimulationConfig c = column_config(n, cells, vol, dt, 300.0);
        c.lifetime_temperature_is_local = local != 0;
        c.lifetime_temperature = Tlife;
        DeviceSolver s(c, {m->m.get()}, false);
        load_column(s, *m->m, c, n, flat, cell, occ);
        *residual = s.collide_only(cell_T);
        read_occupations(s, n, occ);
    });
}

int phmc_dev_ncallaway_evolve(int32_t n_modes, const double* omega, const double* k3, const double* rn,
                              const double* rr, int64_t n, const int32_t* mode, double* occ, double T, double dt) {
    return guard([&] {
        // src/solver/NonlinearCallawayCollision.cpp:216-239: argument checks
        if (n <= 0 || n_modes <= 0 || !std::isfinite(T) || T <= 0 || !std::isfinite(dt) || dt < 0)
            throw std::invalid_argument("Invalid nonlinear Callaway state");
        for (int64_t i = 0; i < n; ++i) {
            const int m = mode[i];
            if (m < 0 || m >= n_modes || !std::isfinite(occ[i]) || occ[i] < 0 || !(omega[m] > 0) ||
                !std::isfinite(omega[m]) || !(rn[m] >= 0) || !(rr[m] >= 0) || !std::isfinite(rn[m]) ||
                !std::isfinite(rr[m]))
                throw std::invalid_argument("Invalid nonlinear Callaway mode");
            for (int k = 0; k < 3; ++k)
                if (!std::isfinite(k3[3 * m + k])) throw std::invalid_argument("Invalid nonlinear Callaway wavevector");
        }
        const size_t nm = static_cast<size_t>(n_modes), nc = static_cast<size_t>(n);
        DevHold h;
        double* d_om = h.put(omega, nm);
        double* d_k = h.put(k3, 3 * nm);
        double* d_rn = h.put(rn, nm);
        double* d_rr = h.put(rr, nm);
        int32_t* d_mode = h.put(mode, nc);
        double* d_occ = h.put(occ, nc);
        double* d_cnt = h.alloc<double>(nm);
        double2* d_ab = h.alloc<double2>(nm);
        double2* d_work = h.alloc<double2>(nm);
        int* d_status = h.alloc<int>(1);
        launch_ncl_cell(n_modes, d_om, d_k, d_rn, d_rr, d_cnt, d_ab, d_work, n, d_mode, d_occ, T, dt, d_status, nullptr);
        cuda_check(cudaGetLastError(), "k_ncl_cell launch");
        int status = 0;
        cuda_check(cudaMemcpy(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (status != 0) throw std::runtime_error(solver_error_message(status));
        cuda_check(cudaMemcpy(occ, d_occ, nc * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy");
    });
}

int phmc_dev_linear_collide(const phmc_material* m, int model, double Tref, int64_t n, const int32_t* flat,
                            const int32_t* cell, double* occ, int cells, double dt, double vol, double* residual) {
    return guard([&] {
        SimulationConfig c = column_config(n, cells, vol, dt, Tref);
        c.lifetime_temperature_is_local = false;
        c.lifetime_temperature = Tref;
        if (model == 1) c.collision_model = CollisionModel::Callaway;
        else c.temperature_gradient = 0.0; // linearized RTA, no drive
        DeviceSolver s(c, {m->m.get()}, false);
        load_column(s, *m->m, c, n, flat, cell, occ);
        *residual = s.collide_only(nullptr);
        read_occupations(s, n, occ);
    });
}

int phmc_dev_gradient_drive(const phmc_material* m, int axis, double G, double Tref, int64_t n, const int32_t* flat,
                            const int32_t* cell, double* occ, int cells, double dt, double vol, double* energy) {
    return guard([&] {
        SimulationConfig c = column_config(n, cells, vol, 2.0 * dt, Tref);
        c.lifetime_temperature_is_local = false;
        c.lifetime_temperature = Tref;
        c.temperature_gradient = G;
        c.transport_axis = axis;
        DeviceSolver s(c, {m->m.get()}, false);
        load_column(s, *m->m, c, n, flat, cell, occ);
        *energy = s.drive_only();
        read_occupations(s, n, occ);
    });
}

int phmc_dev_rough_spec_match(const phmc_material* m, int conservative, double Tref, int32_t nf,
                              const double* normals, const double* roughness, int device, int32_t* match) {
    return guard([&] {
        const PhononMaterial& M = *m->m;
        if (nf <= 0) throw std::invalid_argument("phmc_dev_rough_spec_match: no facets");
        std::vector<Vec3> nrm(nf);
        std::vector<double> rough(roughness, roughness + nf);
        for (int f = 0; f < nf; ++f) nrm[f] = {normals[3 * f], normals[3 * f + 1], normals[3 * f + 2]};
        RoughTables rt;
        const SpecMatchScan scan = [](const std::vector<Vec3>& va, std::vector<SpecMatchJob>& jobs) {
            spec_match_device(va, jobs, 0);
        };
        rt.build({&M}, nrm, rough, std::vector<char>(nf, 1), conservative != 0, conservative ? Tref : 0.0,
                 device ? &scan : nullptr);
        const size_t na = static_cast<size_t>(M.active_mode_count());
        for (int f = 0; f < nf; ++f) {
            const RoughTable& R = rt.tables.at(rt.facet_table.at(f));
            std::copy(R.spec_match.begin(), R.spec_match.end(), match + f * na);
        }
    });
}

int phmc_dev_rough_reflect(const phmc_material* m, int conservative, double Tref, const double nout[3],
                           double rough_a, int64_t n, const int32_t* flat_in, const double* occ_in, const double* u3,
                           int32_t* flat_out, double* occ_out) {
    return guard([&] {
        const PhononMaterial& M = *m->m;
        RoughTables rt;
        const SpecMatchScan scan = [](const std::vector<Vec3>& va, std::vector<SpecMatchJob>& jobs) {
            spec_match_device(va, jobs, 0);
        };
        rt.build({&M}, {{nout[0], nout[1], nout[2]}}, {rough_a}, {1}, conservative != 0, conservative ? Tref : 0.0,
                 &scan);
        const RoughTable& R = rt.tables.at(0);
        DBuf<double> spec(R.specularity), prefix(R.residual_prefix), rcdf(R.roulette_cdf),
            coarse(coarse_prefix(R.residual_prefix));
        DBuf<int> match(R.spec_match), db(R.diffuse_begin), de(R.diffuse_end), sorted(R.outgoing_sorted),
            ract(R.roulette_active), oact(R.outgoing_active);
        DevRoughTable D{};
        D.strict = R.strict_elastic;
        D.n_sorted = static_cast<int>(R.outgoing_sorted.size());
        D.n_roulette = static_cast<int>(R.roulette_active.size());
        D.n_outgoing = static_cast<int>(R.outgoing_active.size());
        D.specularity = spec.p;
        D.spec_match = match.p;
        D.diffuse_begin = db.p;
        D.diffuse_end = de.p;
        D.outgoing_sorted = sorted.p;
        D.prefix = prefix.p;
        D.coarse = coarse.p;
        D.roulette_active = ract.p;
        D.roulette_cdf = rcdf.p;
        D.outgoing_active = oact.p;
        std::vector<double> om(M.active_mode_count()), nb(M.active_mode_count());
        for (int a = 0; a < M.active_mode_count(); ++a) {
            om[a] = M.omega(M.active_flat()[a]);
            nb[a] = M.bose_occupation(Tref, M.active_flat()[a]);
        }
        DBuf<double> dom(om), dnb(nb);
        DevMaterial DM{};
        DM.n_active = M.active_mode_count();
        DM.omega = dom.p;
        DM.nbg = dnb.p;
        std::vector<int32_t> ain(n);
        for (int64_t i = 0; i < n; ++i) {
            ain[i] = M.active_index_for_flat(flat_in[i]);
            if (ain[i] < 0) throw std::invalid_argument("incoming mode is not active");
        }
        DBuf<int32_t> dain(ain), daout(n);
        DBuf<double> docc(occ_in, n), du(u3, 3 * n), dout(n);
        k_rough_rays<<<128, 256>>>(D, DM, conservative, n, dain.p, docc.p, du.p, daout.p, dout.p);
        cuda_check(cudaDeviceSynchronize(), "k_rough_rays");
        std::vector<int32_t> aout(n);
        daout.get(aout.data());
        dout.get(occ_out);
        for (int64_t i = 0; i < n; ++i) flat_out[i] = M.active_flat()[aout[i]];
    });
}

} // extern "C"

// ------------------------------------------------------ no-allocation variant
namespace phmc {
void trace_box_noalloc(const double lo[3], const double hi[3], long long n, const double* p3, const double* v3,
                       double* hit3, double* t, int32_t* facet, long long* misses);
}

int phmc_dev_trace_box_noalloc(const double lo[3], const double hi[3], int64_t n, const double* p3, const double* v3,
                               double* hit3, double* t, int32_t* facet, int64_t* misses) {
    return guard([&] {
        long long m = 0;
        phmc::trace_box_noalloc(lo, hi, n, p3, v3, hit3, t, facet, &m);
        if (misses) *misses = m;
    });
}
