// CPU harness of the engine's HDF5 subset (tlbm_gb300/csrc/h5lite.cpp) for tests/test_h5_cpu.py:
//   h5_harness write FILE N        the restart layout plus a 3-D and a root-level dataset,
//                                  value k of dataset d = d + k / 8 (exact in float32)
//   h5_harness read FILE PATH      dims, then every value as a hexadecimal float, one per line
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../tlbm_gb300/csrc/h5lite.h"

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  const std::string mode = argv[1], file = argv[2];
  if (mode == "write") {
    const uint64_t n = std::strtoull(argv[3], nullptr, 10);
    const char* names[] = {"velocity/x", "velocity/y", "velocity/z", "density/rho",
                           "pres_group/presmag", "top"};
    std::vector<std::vector<float>> vals(6);
    std::vector<tlbm::h5::Dataset> sets;
    for (int d = 0; d < 6; ++d) {
      vals[d].resize(n);
      for (uint64_t k = 0; k < n; ++k) vals[d][k] = static_cast<float>(d) + k / 8.0f;
      tlbm::h5::Dataset s;
      s.path = names[d];
      s.dims = d == 4 ? std::vector<uint64_t>{2, 2, n / 4} : std::vector<uint64_t>{n};
      s.data = vals[d].data();
      sets.push_back(s);
    }
    std::string err;
    if (!tlbm::h5::write_f32(file, sets, &err)) {
      std::printf("error: %s\n", err.c_str());
      return 1;
    }
    return 0;
  }
  std::vector<float> v;
  std::vector<uint64_t> dims;
  const std::string err = tlbm::h5::read_f32(file, argv[3], &v, &dims);
  if (!err.empty()) {
    std::printf("error: %s\n", err.c_str());
    return 1;
  }
  std::printf("dims");
  for (uint64_t e : dims) std::printf(" %llu", static_cast<unsigned long long>(e));
  std::printf("\n");
  for (float x : v) std::printf("%a\n", static_cast<double>(x));
  return 0;
}
