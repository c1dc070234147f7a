/*
 * Minimal stand-in for the HDF5 C++ API, used only to compile the CPU
 * reference solver into a test oracle where HDF5 is not installed.
 * The reference reads HDF5 only on its restart path; every read here throws,
 * so a restart run of the oracle fails loudly instead of reading garbage.
 *
 * Test infrastructure only: nothing in the product links this header.
 */
#ifndef TLBM_ORACLE_H5_STUB_H
#define TLBM_ORACLE_H5_STUB_H

#include <stdexcept>
#include <string>

typedef std::string H5std_string;
#define H5F_ACC_RDONLY 0

namespace H5 {
struct PredType {
  static const int NATIVE_FLOAT = 0;
};

struct DataSet {
  void read(void*, int) const {
    throw std::runtime_error("HDF5 is not available in the oracle build");
  }
};

struct H5File {
  H5File(const H5std_string&, unsigned) {}
  DataSet openDataSet(const H5std_string&) const { return DataSet(); }
};
}  // namespace H5

#endif
