// Material tables in the reference's on-disk layout: a POSCAR beside a
// phono3py-style HDF5 file (kappa-fbz.hdf5, kappa.hdf5 or a single *.hdf5),
// read and written without libhdf5.
//
// The reader covers the part of the HDF5 file format that such tables use:
// superblock versions 0-3, version 1 and 2 object headers with continuation
// blocks, old-style groups (v1 B-tree of symbol-table nodes and a local heap)
// and compact link messages, contiguous, compact and chunked (v1 B-tree index)
// data layouts, deflate / shuffle / Fletcher-32 filters, and IEEE float or
// two's-complement integer elements of 1-8 bytes, returned as double (as the
// reference reads every dataset with H5::PredType::NATIVE_DOUBLE). Deflate is
// decoded by the inflate of RFC 1951 written here. The writer produces
// superblock version 0, an old-style root group and contiguous little-endian
// datasets.
//
// The datasets and checks follow the reference's read_material_data
// (src/material/MaterialDataReader.cpp:150-302) and read_poscar_lattice
// (:81-148): frequency [q, b] THz, qpoint [q, 3], mesh [3], optional weight
// [q] (all 1), group_velocity [q, b, 3], temperature [T], gamma [T, q, b] and
// optional gamma_N, gamma_U [T, q, b] and resistive gamma_isotope,
// gamma_impurity, gamma_defect ([q, b] or [T, q, b]).
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace phmc {
namespace h5 {

struct Dataset {
    std::vector<uint64_t> dims;
    std::vector<double> values;
};

// Numeric datasets of the root group of an HDF5 file.
class Reader {
public:
    explicit Reader(const std::string& path);
    bool has(const std::string& name) const { return objects_.count(name) != 0; }
    Dataset read(const std::string& name) const; // rank 0 (a scalar): empty dims, one value
    std::vector<std::string> names() const;

private:
    std::vector<uint8_t> f_;
    int so_ = 8, sl_ = 8; // sizes of offsets and lengths
    uint64_t base_ = 0;
    std::map<std::string, uint64_t> objects_; // name -> object header address
    uint64_t u(uint64_t at, int n) const;
    void need(uint64_t at, uint64_t n) const;
    void read_group(uint64_t header);
    void group_btree(uint64_t node, uint64_t heap_data);
    std::string heap_name(uint64_t heap_data, uint64_t offset) const;
    // messages of an object header: (type, absolute offset of the data, size)
    std::vector<std::array<uint64_t, 3>> messages(uint64_t header) const;
    void chunk_btree(uint64_t node, int rank, std::vector<std::array<uint64_t, 3>>& chunks,
                     std::vector<std::vector<uint64_t>>& offsets) const;
};

// A dataset to write: float64 values or int64 integers, row-major dims.
struct WriteSet {
    std::vector<uint64_t> dims;
    std::vector<double> values;
    bool integer = false;
};

// Writes a new HDF5 file whose root group holds `sets` (names sorted).
void write_file(const std::string& path, const std::map<std::string, WriteSet>& sets);

} // namespace h5

// The material of a folder in the reference's layout, in the field layout of
// phonomc::MaterialData (include/material/MaterialData.h of the reference).
struct MaterialFolder {
    std::array<std::array<double, 3>, 3> lattice{}; // POSCAR rows (scaled), Angstrom
    double volume_a3 = 0;
    std::array<std::array<double, 3>, 3> reciprocal{}; // 2 pi inv(lattice): row i = component i of b_j
    int qpoints = 0, branches = 0;
    std::array<int, 3> mesh{};
    std::vector<double> frequency_thz;
    std::vector<std::array<double, 3>> qpoint_fractions, group_velocity;
    std::vector<double> temperatures, gamma, gamma_normal, gamma_umklapp;
    std::map<std::string, std::vector<double>> gamma_resistive;
    std::string hdf5_path;
};

// read_poscar_lattice: lattice, volume and reciprocal lattice of a POSCAR.
void read_poscar(const std::string& path, MaterialFolder& m);
// read_material_data: POSCAR + the folder's HDF5 table, with the reference's
// file choice and shape checks (its exception texts).
MaterialFolder read_material_folder(const std::string& folder);
// POSCAR and kappa-fbz.hdf5 of `m` (lattice rows or, when absent, the lattice
// recovered from the reciprocal one), unit weights for a full-zone table.
void write_material_folder(const std::string& folder, const MaterialFolder& m);

} // namespace phmc
