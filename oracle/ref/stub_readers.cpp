// Replacement translation unit for the two HDF5-backed readers of the reference
// (src/material/MaterialDataReader.cpp and src/material/ScatteringMatrixReader.cpp).
// libhdf5 is not installed here, so these entry points throw; the reference
// harness constructs PhononMaterial from an in-memory MaterialData instead
// (include/PhononMaterial.h:23-26 of the reference).
#include "material/MaterialDataReader.h"
#include "material/ScatteringMatrixReader.h"

#include <stdexcept>

namespace phonomc {
LatticeData read_poscar_lattice(const std::filesystem::path&) {
    throw std::runtime_error("POSCAR reading is not built into the oracle harness");
}
MaterialData read_material_data(const std::filesystem::path&, std::ostream*) {
    throw std::runtime_error("HDF5 material reading is not built into the oracle harness");
}
ScatteringMatrixData read_scattering_matrix(const std::filesystem::path&) {
    throw std::runtime_error("Full-matrix mode is not public and not built");
}
} // namespace phonomc
