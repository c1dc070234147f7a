// engine.h -- the object behind a tlbm_handle: one lattice on one GPU.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tlbm.h"
#include "kernels.h"

namespace tlbm {

struct Status {
  tlbm_status code = TLBM_OK;
  std::string msg;
  static Status ok() { return Status(); }
  static Status err(tlbm_status c, std::string m) {
    Status s;
    s.code = c;
    s.msg = std::move(m);
    return s;
  }
  bool good() const { return code == TLBM_OK; }
};

// Problem::load_input semantics (src/Problem.cpp:5-32): 23 whitespace-separated tokens.
// Real values are parsed in the precision that will compute with them.
Status parse_params(const std::string& text, bool as_float, tlbm_problem* p);
// whitespace-separated integers of ndType.lbm / parts.lbm, exactly n of them (n < 0: any count)
Status parse_int_file(const std::string& path, int64_t n, std::vector<int32_t>* out);
Status read_text(const std::string& path, std::string* out);
Status apply_config_file(const std::string& path, tlbm_options* opt);
// processTLBM.py over a run directory (post.cpp): dumps 0 .. nDumps-1 and the time averages
Status post_process_dir(const std::string& dir, int device, int* dumps_done);

class Engine {
 public:
  ~Engine();
  static Status create(const tlbm_problem& prob, const int32_t* nd_type, const int32_t* parts,
                       int size, const std::string& workdir, const tlbm_options& opt,
                       Engine** out);

  Status step(int is_even);
  Status run(int first_ts, int nsteps);
  Status time_steps(int first_ts, int nsteps, float* ms);
  Status synchronize();
  const tlbm_options& options() const { return opt_; }
  Status write_data();
  Status write_time_avg_data();
  Status copy_macros(void* ux, void* uy, void* uz, void* rho);
  Status copy_force(void* fx, void* fy, void* fz);
  // ux, uy, uz, rho, fx, fy, fz (null entries skipped) of the last step, copied on a second
  // stream while later steps run; the host buffers hold them after synchronize()
  Status copy_outputs_async(void* const host[7]);
  Status copy_populations(int which, void* out);
  Status copy_adjacency(int32_t* out);
  Status mass(double* out);
  // both population buffers = feq(u, rho) of the given float fields (load_restart_data)
  Status load_restart(const float* ux, const float* uy, const float* uz, const float* rho);
  // per-(x, y) inlet velocity of the z = 0 plane (nx*ny values); null restores u_bc
  Status set_inlet_profile(const double* uz);
  // learned closure (mlp.cuh); params null removes it
  Status set_closure(const float* params, const float* scale, const float* shift,
                     float out_scale, float tau_min);
  // box filter by f of the last step's macroscopic fields: 10 coarse fields (mlp_kernels.h)
  Status filtered(int f, void* out);
  // processTLBM.py's fields of the last step (or of the time averages), planes of post.h
  Status processed(bool time_avg, float* out);
  // ... written as out{k}.bin + data{k}.xmf (k = 0, 1, ... per call) or timeAvg.bin/.xmf
  Status write_processed(bool time_avg);

  const tlbm_problem& problem() const { return prob_; }
  int output_bytes() const { return ob_; }
  int q() const { return q_; }
  int cut_size() const { return cut_size_; }
  int64_t launches() const { return launches_; }
  std::string last_error;

 private:
  Engine() = default;
  Status init(const int32_t* nd_type, const int32_t* parts, int size);
  // init's two halves, run concurrently: the host checks of the node types (narrowed into
  // `types`) and partitions, and the device setup that does not depend on them
  Status check_host_inputs(const int32_t* nd_type, const int32_t* parts, int size,
                           uint8_t* types);
  Status init_device();
  Status check(cudaError_t e, const char* what);
  Status enqueue_step(int is_even);
  // the output fields of the last step (no-op while fresh); macros_done, if given, is recorded
  // on the stream once ux..rho are ready
  Status compute_outputs(cudaEvent_t macros_done = nullptr);
  // one field in global order into host memory, on the stream (wait: synchronize it)
  Status fetch(const void* dev, void* host, bool wait = true);
  // the dump files names[0..k) of the fields dev[0..k), k <= 7, written in parallel
  Status write_fields(const std::string* names, const void* const* dev, int k);
  Status build_graph(int parity);

  tlbm_problem prob_{};
  tlbm_options opt_{};
  std::string workdir_;
  int q_ = 19;
  bool ref_arith_ = true;
  int sms_ = 0;  // multiprocessors of the device (set on first use)
  int store_ = kStoreF32;
  bool fx_ = false;  // FP64 fluid nodes collided in fixed point
  int sb_ = 4;  // bytes per stored population
  int ob_ = 4;  // bytes per output value
  int64_t n_ = 0;
  int cut_size_ = 0;
  bool has_type5_ = false;
  bool identity_order_ = true;
  std::vector<int32_t> order_;  // output position -> global node (partition-major)
  DevProblem pb_{};
  Launch launch_{};
  cudaStream_t stream_ = nullptr;
  // copy_outputs_async: copies on copy_stream_, ux..rho after macros_ready_ (while the force
  // kernel runs), Fx..Fz after outputs_ready_; the next recomputation of the output fields
  // waits for copies_done_
  cudaStream_t copy_stream_ = nullptr;
  cudaEvent_t outputs_ready_ = nullptr, copies_done_ = nullptr, macros_ready_ = nullptr;
  bool copies_pending_ = false;

  uint8_t* d_type_ = nullptr;
  void* d_f_[2] = {nullptr, nullptr};  // [0] = fEven, [1] = fOdd
  void* d_macro_[4] = {nullptr, nullptr, nullptr, nullptr};
  void* d_force_[3] = {nullptr, nullptr, nullptr};
  void* d_avg_[4] = {nullptr, nullptr, nullptr, nullptr};
  void* d_uyq_[2] = {nullptr, nullptr};
  void* d_stage_ = nullptr;
  int32_t* d_order_ = nullptr;
  double* d_partial_ = nullptr;
  double* d_mass_ = nullptr;
  void* h_pinned_ = nullptr;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  void drop_graphs();
  double* d_inlet_d_ = nullptr;
  float* d_inlet_f_ = nullptr;
  void* h_closure_ = nullptr;    // mlp::Closure (host: launches copy it by value)
  void* d_closure_w_ = nullptr;   // its weights (mlp::MmaWeights)

  // sub-space output (params.lbm line 23, ssNds.lbm): node list and gathered values
  std::vector<int32_t> ss_;
  int32_t* d_ss_ = nullptr;
  void* d_ss_stage_ = nullptr;
  Status load_subspace();
  Status write_subspace(const std::string& d);

  int last_src_ = -1, last_dst_ = -1;
  int proc_num_ = 0;
  bool outputs_fresh_ = false;
  int dump_num_ = 0;
  int64_t steps_ = 0;
  int64_t launches_ = 0;
};

}  // namespace tlbm
