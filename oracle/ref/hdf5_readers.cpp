// Replacement translation unit for the two HDF5-backed readers of the reference
// (src/material/MaterialDataReader.cpp and src/material/ScatteringMatrixReader.cpp).
// libhdf5 is not installed here: read_poscar_lattice and read_material_data
// delegate to this repository's HDF5 subset reader
// (phonomc_gb300/csrc/phmc_hdf5.cpp, the same file checks and messages), so the
// reference's own MaterialFactory and main.cpp flow read real material folders;
// the non-public full-matrix reader throws.
#include "material/MaterialDataReader.h"
#include "material/ScatteringMatrixReader.h"

#include "phmc_hdf5.h"

#include <stdexcept>

namespace phonomc {
namespace {
LatticeData lattice_of(const phmc::MaterialFolder& m) {
    LatticeData l;
    l.volume_a3 = m.volume_a3;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) l.reciprocal[i][j] = m.reciprocal[i][j];
    return l;
}
} // namespace

LatticeData read_poscar_lattice(const std::filesystem::path& path) {
    phmc::MaterialFolder m;
    phmc::read_poscar(path.string(), m);
    return lattice_of(m);
}

MaterialData read_material_data(const std::filesystem::path& folder, std::ostream* progress) {
    const phmc::MaterialFolder m = phmc::read_material_folder(folder.string());
    if (progress) *progress << "PhononMaterial HDF5 file: " << m.hdf5_path << '\n';
    MaterialData d;
    d.lattice = lattice_of(m);
    d.qpoints = m.qpoints;
    d.branches = m.branches;
    d.mesh = m.mesh;
    d.frequency_thz = m.frequency_thz;
    d.qpoint_fractions.assign(m.qpoint_fractions.begin(), m.qpoint_fractions.end());
    d.group_velocity.assign(m.group_velocity.begin(), m.group_velocity.end());
    d.temperatures = m.temperatures;
    d.gamma = m.gamma;
    d.gamma_normal = m.gamma_normal;
    d.gamma_umklapp = m.gamma_umklapp;
    for (const auto& kv : m.gamma_resistive) {
        d.gamma_resistive[kv.first] = kv.second;
        if (progress) *progress << "Including resistive linewidth " << kv.first << "\n";
    }
    validate_material_data(d);
    return d;
}

ScatteringMatrixData read_scattering_matrix(const std::filesystem::path&) {
    throw std::runtime_error("Full-matrix mode is not public and not built");
}
} // namespace phonomc
