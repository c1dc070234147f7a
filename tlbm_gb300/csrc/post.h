// post.h -- post-processing of the solver's output (python/processTLBM.py) and sub-space output.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/tlbm.h"

namespace tlbm {

// planes of the processed output (the datasets of writeH5, python/hdf5Helper.py:4-31); the
// time-average output holds planes 0-3 then pressure
enum : int {
  kPostUx = 0,
  kPostUy = 1,
  kPostUz = 2,
  kPostVelmag = 3,
  kPostFx = 4,
  kPostFy = 5,
  kPostFz = 6,
  kPostPressure = 7,
  kPostFields = 8,
  kPostAvgFields = 5,
};

// float32 factors exactly as numpy applies them: the Python float rounded to float32
struct PostFactors {
  float u_conv = 1.0f;   // t_conv / l_conv (processTLBM.py:52)
  float p_conv = 1.0f;   // p_conv_fact
  float f_conv = 1.0f;   // l_conv / u_conv**2 (:101)
  float avg_div = 1.0f;  // Num_ts, divided first when `avg` (:150-153)
  int avg = 0;
  int p_plane = kPostPressure;  // kPostFz + 1 - 3 = 4 for the time-average layout
};

template <class E>
struct PostInputs {
  const E* ux = nullptr;
  const E* uy = nullptr;
  const E* uz = nullptr;
  const E* rho = nullptr;
  const E* fx = nullptr;  // null: no force planes (time averages)
  const E* fy = nullptr;
  const E* fz = nullptr;
};

// out: planes of n floats in global node order; order[i] = global node of input position i
// (null = inputs already in global order); p_ref_pos = input position of node pRef_idx
cudaError_t launch_post(const PostInputs<float>& in, const int32_t* order, int64_t n,
                        int64_t p_ref_pos, const PostFactors& k, float* out, cudaStream_t s);
cudaError_t launch_post(const PostInputs<double>& in, const int32_t* order, int64_t n,
                        int64_t p_ref_pos, const PostFactors& k, float* out, cudaStream_t s);

PostFactors post_factors(const tlbm_problem& p, bool time_avg);

// processTLBM.py's number of dumps: int((Num_ts - Warmup_ts) / plot_freq) (:65, :70)
int post_num_dumps(const tlbm_problem& p);

// writeXdmf / writeXdmf_time_avg (python/hdf5Helper.py:58-202): the XDMF text that describes
// the datasets of the HDF5 file `h5_name`
std::string post_xdmf(const tlbm_problem& p, const std::string& h5_name, bool time_avg);

// writeH5 / writeH5_time_avg (python/hdf5Helper.py:4-56): <dir>/<h5_name> with the planes above
// as the groups and datasets processTLBM.py stores, and <dir>/<xmf_name>; false with *err on
// failure
bool post_write(const std::string& dir, const std::string& h5_name, const std::string& xmf_name,
                const tlbm_problem& p, const float* planes, bool time_avg, std::string* err);

}  // namespace tlbm
