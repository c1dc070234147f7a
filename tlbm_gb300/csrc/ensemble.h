// ensemble.h -- a batch of independent channels stepped by one persistent launch per step.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tlbm.h"
#include "engine.h"
#include "kernels.h"

namespace tlbm {

// n / d for 0 <= n < 2^31 and a fixed d >= 1 as ((umulhi(m, n) + n) >> l), with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1 (Granlund and Montgomery's division by
// invariant integers; umulhi(m, n) <= n keeps the sum below 2^32)
struct FastDiv {
  uint32_t m;
  int l;
};

inline FastDiv make_fast_div(uint32_t d) {
  int l = 0;
  while ((uint64_t(1) << l) < d) ++l;
  const uint64_t m = ((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1;
  return {static_cast<uint32_t>(m), l};
}

struct EnsembleChannel {
  // step arguments for a step pulling from buffer 0 (fEven) and from buffer 1 (fOdd); the
  // kernel reads them in place, so a tile costs no copy of the problem description
  StepArgs step[2];
  int q;            // 15 or 19
  FastDiv div_nx;   // x, y of a cell from its index in the z-plane
  const DevProblem& pb() const { return step[0].pb; }
  void* f(int b) const { return b == 0 ? const_cast<void*>(step[0].src) : step[0].dst; }
};

// A tile: `cells` consecutive cells (threads x cells_per_thread) of one z-plane of one channel,
// in the plane's x-fastest order, starting at plane index r0.
struct alignas(16) EnsembleTile {  // one 16-byte load per tile
  int channel, z, r0, pad;
};

struct EnsembleArgs {
  const EnsembleChannel* channels;
  const EnsembleTile* tiles;
  int n_tiles;
  int src;  // buffer pulled from in this step (0 = fEven)
  int cells_per_thread;
};

int ensemble_resident_blocks(int store, int threads);
cudaError_t launch_ensemble_step(int store, const EnsembleArgs& a, int threads, int grid,
                                 cudaStream_t s);

class Ensemble {
 public:
  ~Ensemble();
  static Status create(int n, const tlbm_problem* probs, const int32_t* const* nd_types,
                       const tlbm_options& opt, Ensemble** out);
  Status set_tiles(int bx, int by, int cells_per_thread);
  Status autotune(int steps, int* bx, int* by, int* cpt);
  Status run(int first_ts, int nsteps);
  Status time_steps(int first_ts, int nsteps, float* ms);
  Status copy_macros(int channel, void* ux, void* uy, void* uz, void* rho);
  Status mass(int channel, double* out);
  int64_t cells() const { return cells_; }
  int64_t launches() const { return launches_; }
  int output_bytes() const { return ob_; }
  std::string last_error;

 private:
  Ensemble() = default;
  Status init(int n, const tlbm_problem* probs, const int32_t* const* nd_types);
  Status check(cudaError_t e, const char* what);
  Status enqueue(int is_even);
  Status reset_populations();
  void drop_graphs();

  tlbm_options opt_{};
  int store_ = kStoreF32, sb_ = 4, ob_ = 4;
  std::vector<EnsembleChannel> ch_;
  std::vector<tlbm_problem> prob_;
  int64_t cells_ = 0;
  void* arena_ = nullptr;
  EnsembleChannel* d_ch_ = nullptr;
  EnsembleTile* d_tiles_ = nullptr;
  int n_tiles_ = 0;
  int bx_ = 128, by_ = 1, cpt_ = 1, grid_ = 1;
  cudaStream_t stream_ = nullptr;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  double* d_partial_ = nullptr;
  double* d_mass_ = nullptr;
  int last_src_ = -1;
  int64_t launches_ = 0;
};

}  // namespace tlbm
