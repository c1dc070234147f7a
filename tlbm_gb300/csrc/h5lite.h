// h5lite.h -- the subset of the HDF5 file format that tLBM's files use, without the HDF5 library.
//
// The reference reads its restart state from restart.h5 (TLBM_Partition::load_restart_data,
// src/TLBM_Partition.cpp:481-540: datasets density/rho and velocity/{x,y,z} read as
// NATIVE_FLOAT) and post-processing writes out{n}.h5 / timeAvg.h5 (python/hdf5Helper.py:4-56:
// groups velo_group, force_group, pres_group of float32 datasets).  Both are plain h5py files:
// groups and contiguous, unfiltered numeric datasets.
//
// Writer: superblock version 0, groups as symbol tables (a version-1 B-tree leaf, one symbol
// table node, a local heap), version-1 object headers, contiguous little-endian float32
// datasets -- the layout HDF5 writes with its default (earliest) format bounds.
// Reader: superblock versions 0-3; version-1 and version-2 object headers with continuation
// blocks; groups held as symbol tables (B-trees of any depth) or as link messages in the
// header; contiguous or compact datasets of little-endian IEEE float32 or float64, any rank.
// Chunked or filtered datasets, and groups with dense link storage, are reported as
// unsupported.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace tlbm {
namespace h5 {

struct Dataset {
  std::string path;             // "group/name" (groups are created as needed) or "name"
  std::vector<uint64_t> dims;   // row-major extents; their product is the value count
  const float* data = nullptr;  // little-endian float32 values
};

// Writes `file` (created or truncated) holding `sets`; false with *err on failure.
bool write_f32(const std::string& file, const std::vector<Dataset>& sets, std::string* err);

// Reads dataset `path` of `file` as float32 values (float64 data rounded to float32, as
// HDF5's conversion to NATIVE_FLOAT does); *dims gets its extents.  Returns "" on success, else
// the reason.
std::string read_f32(const std::string& file, const std::string& path, std::vector<float>* out,
                     std::vector<uint64_t>* dims);

}  // namespace h5
}  // namespace tlbm
