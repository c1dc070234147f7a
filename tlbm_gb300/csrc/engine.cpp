// engine.cpp -- host side of the engine: inputs, device memory, step launches, dumps.
//
// It restates TLBM_Partition's initialisation and output pipeline (src/TLBM_Partition.cpp)
// for a lattice that lives whole on one GPU:
//   * load_input / load_ndType / load_parts      -> parse_* below (same files, same order)
//   * create_adj_matrix / compute_halo_data       -> no tables: neighbours are computed in the
//     kernels; the halo exchange vanishes (one global array); get_cut_size is still reported
//   * allocate_arrays / initialize_data_arrays    -> two SoA population buffers on the device
//   * write_node_ordering / write_data            -> partition-major order (writeOffset), the
//     same file names and raw layout, MPI_File_write_at semantics (create, no truncation)
#include "engine.h"

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <system_error>
#include <thread>

#include "h5lite.h"
#include "mlp.cuh"
#include "mlp_kernels.h"
#include "post.h"
#include "trace.h"

namespace tlbm {

namespace {

// Splits [0, n) into contiguous chunks of at least 2^20 items, one per host thread (at most 8),
// and runs fn(begin, end, &state) on each; states come back in chunk order, so the first chunk
// that reports something holds the lowest index.
template <class State, class Fn>
void for_chunks(int64_t n, std::vector<State>* states, Fn fn) {
  const int64_t kMinChunk = int64_t{1} << 20;
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t t = std::max<int64_t>(1, std::min<int64_t>({8, hw, n / kMinChunk}));
  states->assign(static_cast<size_t>(t), State{});
  const int64_t per = (n + t - 1) / t;
  std::vector<std::thread> pool;
  for (int64_t k = 1; k < t; ++k) {
    auto chunk = [&, k] { fn(k * per, std::min(n, (k + 1) * per), &(*states)[k]); };
    try {
      pool.emplace_back(chunk);
    } catch (const std::system_error&) {
      chunk();  // no thread to be had: this chunk in turn
    }
  }
  fn(0, std::min(n, per), &(*states)[0]);
  for (auto& th : pool) th.join();
}

}  // namespace

// ----------------------------------------------------------------------------- input parsing

Status read_text(const std::string& path, std::string* out) {
  std::ifstream in(path, std::ios::in | std::ios::binary);
  if (!in.is_open()) return Status::err(TLBM_ERR_IO, "Could not open " + path + "!");
  std::ostringstream ss;
  ss << in.rdbuf();
  *out = ss.str();
  return Status::ok();
}

namespace {

template <class T>
bool parse_token(const std::string& tok, T* v) {
  std::istringstream is(tok);
  T x;
  is >> x;
  if (is.fail()) return false;
  // accept the token only if it was consumed entirely
  char rest;
  if (is >> rest) return false;
  *v = x;
  return true;
}

bool parse_real(const std::string& tok, bool as_float, double* v) {
  if (as_float) {
    float f;
    if (!parse_token(tok, &f)) return false;
    *v = static_cast<double>(f);
    return true;
  }
  return parse_token(tok, v);
}

}  // namespace

Status parse_params(const std::string& text, bool as_float, tlbm_problem* p) {
  std::istringstream is(text);
  std::vector<std::string> tok;
  std::string t;
  while (tok.size() < 23 && (is >> t)) tok.push_back(t);
  // the solver needs the first 15 tokens; the rest only feed post-processing
  if (tok.size() < 15)
    return Status::err(TLBM_ERR_FORMAT, "params.lbm has " + std::to_string(tok.size()) +
                                            " values; at least 15 are required");
  std::memset(p, 0, sizeof(*p));
  if (tok[0].size() >= sizeof(p->lattice))
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "Invalid Lattice Structure!");
  std::snprintf(p->lattice, sizeof(p->lattice), "%s", tok[0].c_str());
  bool ok = true;
  int* ints[] = {&p->dynamics, &p->num_ts, &p->ts_rep_freq, &p->warmup_ts, &p->plot_freq};
  for (int k = 0; k < 5; ++k) ok = ok && parse_token(tok[1 + k], ints[k]);
  double* reals[] = {&p->cs, &p->rho_lbm, &p->u_lbm, &p->omega};
  for (int k = 0; k < 4; ++k) ok = ok && parse_real(tok[6 + k], as_float, reals[k]);
  int* dims[] = {&p->nx, &p->ny, &p->nz, &p->restart_flag, &p->time_avg_flag};
  for (int k = 0; k < 5; ++k) ok = ok && parse_token(tok[10 + k], dims[k]);
  if (!ok) return Status::err(TLBM_ERR_FORMAT, "params.lbm: malformed value in lines 2-15");
  // the conversion factors only feed post-processing, which reads them as Python floats
  // (python/processTLBM.py:42-47): always parsed in double
  double* phys[] = {&p->lx_p, &p->ly_p, &p->lz_p, &p->t_conv, &p->l_conv, &p->p_conv};
  for (int k = 0; k < 6 && 15 + k < (int)tok.size(); ++k)
    if (!parse_real(tok[15 + k], false, phys[k]))
      return Status::err(TLBM_ERR_FORMAT, "params.lbm: malformed value on line " +
                                              std::to_string(16 + k));
  if (tok.size() > 21 && !parse_token(tok[21], &p->p_ref_idx))
    return Status::err(TLBM_ERR_FORMAT, "params.lbm: malformed pRefIdx");
  if (tok.size() > 22 && !parse_token(tok[22], &p->ss_data_flag))
    return Status::err(TLBM_ERR_FORMAT, "params.lbm: malformed ssDataFlag");
  return Status::ok();
}

Status parse_int_file(const std::string& path, int64_t n, std::vector<int32_t>* out) {
  std::string text;
  Status s = read_text(path, &text);
  if (!s.good()) return s;
  const bool any = n < 0;
  if (any) out->clear();
  else out->assign(static_cast<size_t>(n), 0);
  const char* c = text.data();
  const char* end = c + text.size();
  int64_t k = 0;
  while (true) {
    while (c < end && (*c == ' ' || *c == '\n' || *c == '\t' || *c == '\r')) ++c;
    if (c >= end) break;
    bool neg = false;
    if (*c == '-' || *c == '+') {
      neg = (*c == '-');
      ++c;
    }
    if (c >= end || *c < '0' || *c > '9')
      return Status::err(TLBM_ERR_FORMAT, path + ": non-integer value at entry " +
                                              std::to_string(k));
    int64_t v = 0;
    while (c < end && *c >= '0' && *c <= '9') {
      v = v * 10 + (*c - '0');
      if (v > 2147483647LL) return Status::err(TLBM_ERR_FORMAT, path + ": value out of range");
      ++c;
    }
    if (c < end && !(*c == ' ' || *c == '\n' || *c == '\t' || *c == '\r'))
      return Status::err(TLBM_ERR_FORMAT, path + ": non-integer value at entry " +
                                              std::to_string(k));
    if (any) {
      out->push_back(static_cast<int32_t>(neg ? -v : v));
      ++k;
      continue;
    }
    if (k >= n)
      return Status::err(TLBM_ERR_FORMAT, path + " has more than nx*ny*nz = " +
                                              std::to_string(n) + " values");
    (*out)[k++] = static_cast<int32_t>(neg ? -v : v);
  }
  if (!any && k != n)
    return Status::err(TLBM_ERR_FORMAT, path + " has " + std::to_string(k) +
                                            " values, expected nx*ny*nz = " + std::to_string(n));
  return Status::ok();
}

Status apply_config_file(const std::string& path, tlbm_options* opt) {
  std::ifstream in(path);
  if (!in.is_open()) return Status::ok();  // optional
  std::string key, val;
  while (in >> key >> val) {
    if (key == "precision") {
      if (val == "f64") opt->precision = TLBM_PREC_F64;
      else if (val == "f32") opt->precision = TLBM_PREC_F32;
      else if (val == "bf16") opt->precision = TLBM_PREC_BF16;
      else if (val == "f16") opt->precision = TLBM_PREC_F16;
      else if (val == "bf16m") opt->precision = TLBM_PREC_BF16M;
      else return Status::err(TLBM_ERR_INVALID_ARGUMENT, path + ": unknown precision " + val);
    } else if (key == "arithmetic") {
      if (val == "reference") opt->arithmetic = TLBM_ARITH_REFERENCE;
      else if (val == "fast") opt->arithmetic = TLBM_ARITH_FAST;
      else return Status::err(TLBM_ERR_INVALID_ARGUMENT, path + ": unknown arithmetic " + val);
    } else if (key == "block_x") {
      opt->block_x = std::atoi(val.c_str());
    } else if (key == "block_y") {
      opt->block_y = std::atoi(val.c_str());
    } else if (key == "device") {
      opt->device = std::atoi(val.c_str());
    } else if (key == "rbgk") {
      opt->rbgk = std::atoi(val.c_str()) != 0;
    } else if (key == "mrt") {
      opt->mrt = std::atoi(val.c_str()) != 0;
    } else if (key == "mrt_ghost_rate") {
      opt->mrt_ghost_rate = static_cast<float>(std::atof(val.c_str()));
    } else if (key == "f64_pipe") {
      opt->f64_pipe = std::atoi(val.c_str()) != 0;
    } else {
      return Status::err(TLBM_ERR_INVALID_ARGUMENT, path + ": unknown key " + key);
    }
  }
  return Status::ok();
}

// ----------------------------------------------------------------------------- engine

namespace {

int lattice_q(const char* s) {
  if (!std::strcmp(s, "D3Q15")) return 15;
  if (!std::strcmp(s, "D3Q19")) return 19;
  if (!std::strcmp(s, "D3Q27")) return 27;
  return 0;
}

// MPI_File_write_at with MPI_MODE_CREATE|MPI_MODE_WRONLY: create, keep existing bytes
Status write_at(const std::string& path, const void* buf, size_t bytes, size_t offset) {
  int fd = ::open(path.c_str(), O_WRONLY | O_CREAT, 0644);
  if (fd < 0) return Status::err(TLBM_ERR_IO, "Error opening file to write " + path);
  const char* p = static_cast<const char*>(buf);
  size_t done = 0;
  while (done < bytes) {
    ssize_t w = ::pwrite(fd, p + done, bytes - done, static_cast<off_t>(offset + done));
    if (w < 0) {
      if (errno == EINTR) continue;
      ::close(fd);
      return Status::err(TLBM_ERR_IO, "Error writing " + path);
    }
    done += static_cast<size_t>(w);
  }
  ::close(fd);
  return Status::ok();
}

}  // namespace

Status Engine::check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status::ok();
  return Status::err(TLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TLBM_TRY(expr)                 \
  do {                                 \
    Status _s = (expr);                \
    if (!_s.good()) return _s;         \
  } while (0)
#define TLBM_CUDA(expr) TLBM_TRY(check((expr), #expr))

Engine::~Engine() {
  if (stream_) cudaStreamSynchronize(stream_);
  if (copy_stream_) cudaStreamSynchronize(copy_stream_);
  for (auto& g : graph_)
    if (g) cudaGraphExecDestroy(g);
  cudaFree(d_type_);
  for (auto p : d_f_) cudaFree(p);
  for (auto p : d_macro_) cudaFree(p);
  for (auto p : d_force_) cudaFree(p);
  for (auto p : d_avg_) cudaFree(p);
  for (auto p : d_uyq_) cudaFree(p);
  cudaFree(d_stage_);
  cudaFree(d_order_);
  cudaFree(d_partial_);
  cudaFree(d_mass_);
  cudaFree(d_inlet_d_);
  cudaFree(d_inlet_f_);
  delete static_cast<mlp::Closure*>(h_closure_);
  cudaFree(d_closure_w_);
  cudaFree(d_ss_);
  cudaFree(d_ss_stage_);
  if (h_pinned_) cudaFreeHost(h_pinned_);
  if (outputs_ready_) cudaEventDestroy(outputs_ready_);
  if (copies_done_) cudaEventDestroy(copies_done_);
  if (macros_ready_) cudaEventDestroy(macros_ready_);
  if (copy_stream_) cudaStreamDestroy(copy_stream_);
  if (stream_) cudaStreamDestroy(stream_);
}

void Engine::drop_graphs() {
  for (auto& g : graph_) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

Status Engine::create(const tlbm_problem& prob, const int32_t* nd_type, const int32_t* parts,
                      int size, const std::string& workdir, const tlbm_options& opt,
                      Engine** out) {
  TraceRange trace("tlbm_create");
  *out = nullptr;
  Engine* e = new (std::nothrow) Engine();
  if (!e) return Status::err(TLBM_ERR_NO_MEMORY, "out of host memory");
  e->prob_ = prob;
  e->opt_ = opt;
  e->workdir_ = workdir;
  Status s = e->init(nd_type, parts, size);
  if (!s.good()) {
    delete e;
    return s;
  }
  *out = e;
  return Status::ok();
}

Status Engine::check_host_inputs(const int32_t* nd_type, const int32_t* parts, int size,
                                 uint8_t* types) {
  // node types: the reference's codes only (python/FluidChannel.py:1386-1397); checked and
  // narrowed to bytes in chunks on several host threads, one branch-free pass per chunk (a
  // branch and an early exit per node kept the loop scalar: ~26 ms for 33.5 M nodes); a chunk
  // that holds a bad code is scanned again for its first one
  {
    struct Chunk {
      int64_t bad = -1;
      bool type5 = false;
    };
    std::vector<Chunk> chunks;
    uint8_t* const out = types;
    for_chunks(n_, &chunks, [&](int64_t begin, int64_t end, Chunk* c) {
      // codes 0, 1, 2, 3, 5; a negative code is a large unsigned value
      const auto bad_code = [](uint32_t t) { return (t > 5u) | (t == 4u); };
      unsigned bad = 0, five = 0;
      for (int64_t g = begin; g < end; ++g) {
        const uint32_t t = static_cast<uint32_t>(nd_type[g]);
        out[g] = static_cast<uint8_t>(t);
        bad |= static_cast<unsigned>(bad_code(t));
        five |= static_cast<unsigned>(t == 5u);
      }
      c->type5 = five != 0;
      if (bad) {
        for (int64_t g = begin; g < end; ++g) {
          if (bad_code(static_cast<uint32_t>(nd_type[g]))) {
            c->bad = g;
            break;
          }
        }
      }
    });
    for (const Chunk& c : chunks) {
      if (c.bad >= 0)
        return Status::err(TLBM_ERR_OUT_OF_RANGE, "ndType.lbm: node " + std::to_string(c.bad) +
                                                      " has unknown type " +
                                                      std::to_string(nd_type[c.bad]));
      has_type5_ |= c.type5;
    }
  }

  // partitions: the reference indexes partSizes[p] with p < size (src/TLBM_Partition.cpp:224)
  if (size < 1) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "size must be >= 1");
  int32_t max_part = 0;
  identity_order_ = true;
  if (parts) {
    for (int64_t g = 0; g < n_; ++g) {
      const int32_t p = parts[g];
      if (p < 0 || p >= size)
        return Status::err(TLBM_ERR_OUT_OF_RANGE,
                           "parts.lbm: node " + std::to_string(g) + " is in partition " +
                               std::to_string(p) + " but the job size is " +
                               std::to_string(size));
      max_part = std::max(max_part, p);
      if (g > 0 && p < parts[g - 1]) identity_order_ = false;
    }
  }
  if (parts && !identity_order_) {
    // nodes sorted by (partition, global id): the concatenation of every rank's localNdList
    // written at its writeOffset (src/TLBM_Partition.cpp:244-248, :542-561)
    std::vector<int64_t> count(static_cast<size_t>(max_part) + 2, 0);
    for (int64_t g = 0; g < n_; ++g) count[parts[g] + 1]++;
    for (int p = 0; p <= max_part; ++p) count[p + 1] += count[p];
    order_.assign(static_cast<size_t>(n_), 0);
    for (int64_t g = 0; g < n_; ++g) order_[count[parts[g]]++] = static_cast<int32_t>(g);
  }
  // cut size of partition 0: (node, speed) pairs of rank 0 whose push target lies elsewhere
  cut_size_ = 0;
  if (parts) {
    bool multi = false;
    for (int64_t g = 0; g < n_ && !multi; ++g) multi = parts[g] != parts[0];
    if (multi) {
      const int nx = prob_.nx, ny = prob_.ny, nz = prob_.nz;
      const int64_t nxy = static_cast<int64_t>(nx) * ny;
      auto tables = [&](int q, const int** ex, const int** ey, const int** ez) {
        static const int e15x[] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
        static const int e15y[] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
        static const int e15z[] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
        static int e19x[19], e19y[19], e19z[19], e27x[27], e27y[27], e27z[27];
        for (int i = 0; i < 19; ++i) {
          e19x[i] = Lattice<19>::ex(i); e19y[i] = Lattice<19>::ey(i); e19z[i] = Lattice<19>::ez(i);
        }
        for (int i = 0; i < 27; ++i) {
          e27x[i] = Lattice<27>::ex(i); e27y[i] = Lattice<27>::ey(i); e27z[i] = Lattice<27>::ez(i);
        }
        if (q == 15) { *ex = e15x; *ey = e15y; *ez = e15z; }
        else if (q == 19) { *ex = e19x; *ey = e19y; *ez = e19z; }
        else { *ex = e27x; *ey = e27y; *ez = e27z; }
      };
      const int *ex, *ey, *ez;
      tables(q_, &ex, &ey, &ez);
      for (int64_t g = 0; g < n_; ++g) {
        if (parts[g] != 0) continue;
        const int z = static_cast<int>(g / nxy);
        const int y = static_cast<int>((g - z * nxy) / nx);
        const int x = static_cast<int>(g - z * nxy - static_cast<int64_t>(y) * nx);
        for (int i = 0; i < q_; ++i) {
          const int tx = ((x + ex[i]) % nx + nx) % nx, ty = ((y + ey[i]) % ny + ny) % ny,
                    tz = ((z + ez[i]) % nz + nz) % nz;
          const int64_t tg = tx + static_cast<int64_t>(ty) * nx + tz * nxy;
          if (parts[tg] != 0) cut_size_++;
        }
      }
    }
  }

  return Status::ok();
}

Status Engine::init_device() {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  TLBM_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  launch_.stream = stream_;

  const size_t n = static_cast<size_t>(n_);
  TLBM_CUDA(cudaMalloc(&d_type_, n));
  for (auto& p : d_f_) TLBM_CUDA(cudaMalloc(&p, buffer_bytes(store_, q_, n_)));
  for (auto& p : d_macro_) TLBM_CUDA(cudaMalloc(&p, n * ob_));
  for (auto& p : d_force_) TLBM_CUDA(cudaMalloc(&p, n * ob_));
  if (prob_.time_avg_flag == 1) {
    for (auto& p : d_avg_) {
      TLBM_CUDA(cudaMalloc(&p, n * ob_));
      TLBM_CUDA(cudaMemsetAsync(p, 0, n * ob_, stream_));
    }
  }
  for (auto& p : d_uyq_) {
    TLBM_CUDA(cudaMalloc(&p, 32 * 8));
    TLBM_CUDA(cudaMemsetAsync(p, 0, 32 * 8, stream_));
  }

  pb_.nx = prob_.nx;
  pb_.ny = prob_.ny;
  pb_.nz = prob_.nz;
  pb_.nxy = prob_.nx * prob_.ny;
  pb_.n = n_;
  pb_.nd_type = d_type_;
  pb_.omega = prob_.omega;
  pb_.nu = (1.0 / prob_.omega - 0.5) / 3.0;
  pb_.cs = prob_.cs;
  pb_.u_bc = prob_.u_lbm;
  pb_.rho_bc = prob_.rho_lbm;
  pb_.dynamics = prob_.dynamics;
  // moment-space collision: dynamics 2 with rbgk (ghost rate 1), dynamics 3 with mrt
  pb_.mcoll = 0;
  pb_.ghost_omega = 1.0;
  if (opt_.rbgk && prob_.dynamics == 2) pb_.mcoll = 1;
  if (opt_.mrt && prob_.dynamics == 3) {
    pb_.mcoll = 1;
    pb_.ghost_omega = opt_.mrt_ghost_rate > 0.0f ? opt_.mrt_ghost_rate : 1.2;
  }
  fill_derived(pb_, q_, sb_);
  pb_.fx = fx_ ? 1 : 0;
  if (pb_.fx) fx::fill_consts(pb_.fxk, prob_.omega, prob_.cs, pb_.nu);

  const int nb = mass_blocks(pb_);
  TLBM_CUDA(cudaMalloc(&d_partial_, nb * sizeof(double)));
  TLBM_CUDA(cudaMalloc(&d_mass_, sizeof(double)));

  // f = w*rho in both buffers (initialize_data_arrays, src/TLBM_Partition.cpp:458-465)
  for (auto p : d_f_) {
    TLBM_CUDA(launch_init_uniform(q_, store_, pb_, p, prob_.rho_lbm, launch_));
    ++launches_;
  }
  return Status::ok();
}

Status Engine::init(const int32_t* nd_type, const int32_t* parts, int size) {
  q_ = lattice_q(prob_.lattice);
  if (!q_) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "Invalid Lattice Structure!");
  if (prob_.nx < 1 || prob_.ny < 1 || prob_.nz < 1)
    return Status::err(TLBM_ERR_FORMAT, "params.lbm: lattice dimensions must be positive");
  n_ = static_cast<int64_t>(prob_.nx) * prob_.ny * prob_.nz;
  if (n_ * q_ > (int64_t(1) << 40) || n_ >= (int64_t(1) << 31))
    return Status::err(TLBM_ERR_UNSUPPORTED, "lattice too large for one device (N >= 2^31)");
  if (prob_.nz > 65535 || prob_.ny > 65535 * 64)
    return Status::err(TLBM_ERR_UNSUPPORTED, "nz > 65535 is not supported");
  if (prob_.plot_freq <= 0)
    return Status::err(TLBM_ERR_FORMAT, "params.lbm: plotFreq must be positive");
  switch (opt_.precision) {
    case TLBM_PREC_F64: store_ = kStoreF64; break;
    case TLBM_PREC_F32: store_ = kStoreF32; break;
    case TLBM_PREC_BF16: store_ = kStoreBF16; break;
    case TLBM_PREC_F16: store_ = kStoreF16; break;
    case TLBM_PREC_BF16M: store_ = kStoreBF16M; break;
    default: return Status::err(TLBM_ERR_INVALID_ARGUMENT, "unknown precision option");
  }
  ref_arith_ = (opt_.arithmetic == TLBM_ARITH_REFERENCE);
  if (ref_arith_ && (store_ == kStoreBF16 || store_ == kStoreF16 || store_ == kStoreBF16M))
    return Status::err(TLBM_ERR_INVALID_ARGUMENT,
                       "16-bit storage has no reference arithmetic; use TLBM_ARITH_FAST");
  if ((opt_.rbgk || opt_.mrt) && ref_arith_)
    return Status::err(TLBM_ERR_UNSUPPORTED,
                       "the regularised and moment-space collisions have no reference arithmetic "
                       "(the reference streams without relaxation for dynamics 2 and 3): use "
                       "TLBM_ARITH_FAST");
  if (opt_.mrt && opt_.mrt_ghost_rate >= 2.0f)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "mrt_ghost_rate must lie in (0, 2)");
  if (opt_.closure != TLBM_CLOSURE_PARAMS)
    return Status::err(TLBM_ERR_UNSUPPORTED, "closure option not available");
  // FP64 in fast arithmetic: fluid nodes collide in exact fixed point (physics_fx.cuh), and the
  // populations stay in its Q1.62 format between steps unless a moment-space collision runs
  fx_ = store_ == kStoreF64 && !ref_arith_ && !opt_.f64_pipe &&
        fx_collision_ok(prob_.omega, prob_.cs);
  const bool mcoll = (opt_.rbgk && prob_.dynamics == 2) || (opt_.mrt && prob_.dynamics == 3);
  if (fx_ && !mcoll && fx_storage_ok(prob_.omega, prob_.cs, prob_.rho_lbm)) store_ = kStoreFX;
  sb_ = store_bytes(store_);
  ob_ = (store_ == kStoreF64 || store_ == kStoreFX) ? 8 : 4;

  int bx = opt_.block_x, by = opt_.block_y;
  if (bx <= 0) bx = prob_.nx >= 128 ? 128 : 32;
  if (by <= 0) by = std::max(1, 128 / bx);
  if (bx * by > 128 || bx % 32 != 0)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT,
                       "block_x must be a multiple of 32 and block_x*block_y <= 128");
  launch_.bx = bx;
  launch_.by = by;

  // The host checks of the inputs (node types, partitions, the cut size) run on a second thread
  // while this one sets up the device (stream, buffers, the initial populations, none of which
  // depend on them): 33.5 M nodes take ~3 ms of each.  An input error is reported before any
  // device error, as when the checks ran first.
  const size_t n = static_cast<size_t>(n_);
  std::unique_ptr<uint8_t[]> types(new (std::nothrow) uint8_t[n]);
  if (!types) return Status::err(TLBM_ERR_NO_MEMORY, "out of host memory for the node types");
  Status host = Status::ok();
  auto checks = [&] {  // no exception may leave a thread
    try {
      host = check_host_inputs(nd_type, parts, size, types.get());
    } catch (const std::bad_alloc&) {
      host = Status::err(TLBM_ERR_NO_MEMORY, "out of host memory checking the inputs");
    }
  };
  std::thread checker;
  try {
    checker = std::thread(checks);
  } catch (const std::system_error&) {
    checks();  // no thread to be had: the checks first, as before
  }
  const Status device = init_device();
  if (checker.joinable()) checker.join();
  TLBM_TRY(host);
  TLBM_TRY(device);
  pb_.has_type5 = has_type5_ ? 1 : 0;
  TLBM_CUDA(cudaMemcpy(d_type_, types.get(), n, cudaMemcpyHostToDevice));
  if (!identity_order_) {
    TLBM_CUDA(cudaMalloc(&d_order_, n * sizeof(int32_t)));
    TLBM_CUDA(cudaMemcpy(d_order_, order_.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice));
    TLBM_CUDA(cudaMalloc(&d_stage_, n * ob_));
  }
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  if (prob_.restart_flag) {
    // load_restart_data (src/TLBM_Partition.cpp:481-540): the datasets velocity/{x,y,z} and
    // density/rho of restart.h5, read as NATIVE_FLOAT in global node order; without
    // restart.h5, the same four fields as raw float32 files restart_{ux,uy,uz,rho}.b_dat
    if (workdir_.empty())
      return Status::err(TLBM_ERR_INVALID_ARGUMENT,
                         "restart flag set without a directory: use tlbm_load_restart");
    std::vector<std::vector<float>> r(4);
    const std::string h5file = workdir_ + "/restart.h5";
    if (std::ifstream(h5file).good()) {
      const char* sets[4] = {"velocity/x", "velocity/y", "velocity/z", "density/rho"};
      for (int k = 0; k < 4; ++k) {
        std::vector<uint64_t> dims;
        const std::string e = h5::read_f32(h5file, sets[k], &r[k], &dims);
        if (!e.empty()) return Status::err(TLBM_ERR_FORMAT, "restart data: " + e);
        if (r[k].size() != n)
          return Status::err(TLBM_ERR_FORMAT, "restart.h5: " + std::string(sets[k]) +
                                                  " must hold nx*ny*nz values");
      }
    } else {
      const char* names[4] = {"restart_ux.b_dat", "restart_uy.b_dat", "restart_uz.b_dat",
                              "restart_rho.b_dat"};
      for (int k = 0; k < 4; ++k) {
        std::string bytes;
        Status s = read_text(workdir_ + "/" + names[k], &bytes);
        if (!s.good())
          return Status::err(TLBM_ERR_IO, std::string("restart data: ") + s.msg +
                                              " (and no restart.h5)");
        if (bytes.size() != n * sizeof(float))
          return Status::err(TLBM_ERR_FORMAT,
                             std::string(names[k]) + " must hold nx*ny*nz floats");
        r[k].resize(n);
        std::memcpy(r[k].data(), bytes.data(), bytes.size());
      }
    }
    TLBM_TRY(load_restart(r[0].data(), r[1].data(), r[2].data(), r[3].data()));
  }

  // write_node_ordering (src/TLBM_Partition.cpp:542-561)
  if (!workdir_.empty()) {
    std::vector<int32_t> ord;
    const int32_t* op = order_.data();
    if (identity_order_) {
      ord.resize(n);
      for (size_t g = 0; g < n; ++g) ord[g] = static_cast<int32_t>(g);
      op = ord.data();
    }
    TLBM_TRY(write_at(workdir_ + "/ordering.b_dat", op, n * sizeof(int32_t), 0));
  }
  return load_subspace();
}

// Sub-space output: tLBM_write_params.py writes the subset node list to ssNds.lbm and the flag
// to params.lbm line 23 (python/tLBM_write_params.py:110-117, :166); the reference reads the
// flag (src/Problem.cpp:32) but never uses it.  Here each dump also writes ss_ux{n},
// ss_uy{n}, ss_uz{n} and ss_density{n}.b_dat: the dump's values at the listed nodes, in list
// order, gathered on the device.
Status Engine::load_subspace() {
  if (prob_.ss_data_flag != 1 || workdir_.empty()) return Status::ok();
  TLBM_TRY(parse_int_file(workdir_ + "/ssNds.lbm", -1, &ss_));
  for (size_t k = 0; k < ss_.size(); ++k)
    if (ss_[k] < 0 || ss_[k] >= n_)
      return Status::err(TLBM_ERR_OUT_OF_RANGE, "ssNds.lbm: entry " + std::to_string(k) +
                                                    " is not a node of the lattice");
  if (ss_.empty()) return Status::ok();
  const size_t m = ss_.size();
  TLBM_CUDA(cudaMalloc(&d_ss_, m * sizeof(int32_t)));
  TLBM_CUDA(cudaMemcpy(d_ss_, ss_.data(), m * sizeof(int32_t), cudaMemcpyHostToDevice));
  TLBM_CUDA(cudaMalloc(&d_ss_stage_, m * ob_));
  return Status::ok();
}

Status Engine::write_subspace(const std::string& d) {
  const size_t m = ss_.size();
  std::vector<char> host(m * ob_);
  const char* names[4] = {"ss_ux", "ss_uy", "ss_uz", "ss_density"};
  for (int k = 0; k < 4; ++k) {
    if (m) {
      TLBM_CUDA(launch_gather(d_macro_[k], d_ss_, static_cast<int64_t>(m), ob_, d_ss_stage_,
                              launch_));
      ++launches_;
      TLBM_CUDA(cudaMemcpyAsync(host.data(), d_ss_stage_, m * ob_, cudaMemcpyDeviceToHost,
                                stream_));
      TLBM_CUDA(cudaStreamSynchronize(stream_));
    }
    TLBM_TRY(write_at(workdir_ + "/" + names[k] + d + ".b_dat", host.data(), m * ob_, 0));
  }
  return Status::ok();
}

Status Engine::enqueue_step(int is_even) {
  // take_LBM_time_step: isEven -> fIn = fEven, fOut = fOdd (src/TLBM_Partition.cpp:913-920).
  // Here the pull reads the buffer the reference calls fIn and writes the other one.
  const int src = is_even ? 0 : 1;
  const int dst = 1 - src;
  StepArgs a{};
  a.pb = pb_;
  a.src = d_f_[src];
  a.dst = d_f_[dst];
  a.time_avg = (prob_.time_avg_flag == 1) ? 1 : 0;
  for (int k = 0; k < 4; ++k) a.avg[k] = d_avg_[k];
  const int par = is_even ? 1 : 0;
  a.uyq_cur = d_uyq_[par];
  a.uyq_prev = d_uyq_[1 - par];
  if (ref_arith_) {
    if (has_type5_) {
      TLBM_CUDA(launch_quirk_uy_ref(q_, sb_, pb_, a.src, d_uyq_[par], launch_));
      ++launches_;
    }
    TLBM_CUDA(launch_step_ref(q_, sb_, a, launch_));
  } else {
    a.closure = h_closure_;
    TLBM_CUDA(launch_step_fast(q_, store_, a, launch_));
    if (has_type5_) ++launches_;
  }
  ++launches_;
  last_src_ = src;
  last_dst_ = dst;
  outputs_fresh_ = false;
  ++steps_;
  return Status::ok();
}

Status Engine::step(int is_even) {
  TraceRange trace("tlbm_step");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  return enqueue_step(is_even);
}

Status Engine::build_graph(int parity) {
  // two consecutive steps starting with is_even = parity, captured once
  if (graph_[parity]) return Status::ok();
  cudaGraph_t g = nullptr;
  TLBM_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
  const int64_t l0 = launches_;
  Status s = enqueue_step(parity);
  if (s.good()) s = enqueue_step(1 - parity);
  cudaError_t e = cudaStreamEndCapture(stream_, &g);
  launches_ = l0;
  steps_ -= 2;
  if (!s.good()) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  TLBM_CUDA(e);
  e = cudaGraphInstantiate(&graph_[parity], g, 0);
  cudaGraphDestroy(g);
  TLBM_CUDA(e);
  return Status::ok();
}

Status Engine::run(int first_ts, int nsteps) {
  TraceRange trace("tlbm_run");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (nsteps < 0) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "nsteps < 0");
  int ts = first_ts;
  const int64_t per_step = has_type5_ ? 2 : 1;
  if (nsteps >= 2) {
    const int parity = ts % 2;
    TLBM_TRY(build_graph(parity));
    while (nsteps >= 2) {
      TLBM_CUDA(cudaGraphLaunch(graph_[parity], stream_));
      launches_ += 2 * per_step;
      steps_ += 2;
      ts += 2;
      nsteps -= 2;
    }
    // the last captured step had is_even = 1 - parity, i.e. it pulled from buffer `parity`
    last_src_ = parity;
    last_dst_ = 1 - parity;
    outputs_fresh_ = false;
  }
  if (nsteps == 1) TLBM_TRY(enqueue_step(ts % 2));
  return Status::ok();
}

Status Engine::time_steps(int first_ts, int nsteps, float* ms) {
  TraceRange trace("tlbm_time_steps");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  cudaEvent_t e0, e1;
  TLBM_CUDA(cudaEventCreate(&e0));
  TLBM_CUDA(cudaEventCreate(&e1));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  TLBM_CUDA(cudaEventRecord(e0, stream_));
  Status s = run(first_ts, nsteps);
  if (s.good()) s = check(cudaEventRecord(e1, stream_), "cudaEventRecord");
  if (s.good()) s = check(cudaEventSynchronize(e1), "step loop");
  if (s.good()) s = check(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return s;
}

Status Engine::synchronize() {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  if (copy_stream_) TLBM_CUDA(cudaStreamSynchronize(copy_stream_));
  copies_pending_ = false;
  return Status::ok();
}

Status Engine::compute_outputs(cudaEvent_t macros_done) {
  if (last_src_ < 0)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "no time step has been taken yet");
  if (outputs_fresh_) {
    if (macros_done) TLBM_CUDA(cudaEventRecord(macros_done, stream_));
    return Status::ok();
  }
  // an asynchronous copy may still be reading the output fields
  if (copies_pending_) TLBM_CUDA(cudaStreamWaitEvent(stream_, copies_done_, 0));
  // macroscopic values of the last step, recomputed from its (untouched) pull source
  if (ref_arith_)
    TLBM_CUDA(launch_macros_ref(q_, sb_, pb_, d_f_[last_src_], d_macro_, launch_));
  else
    TLBM_CUDA(launch_macros_fast(q_, store_, pb_, d_f_[last_src_], d_macro_, launch_));
  if (macros_done) TLBM_CUDA(cudaEventRecord(macros_done, stream_));
  if (ref_arith_)
    TLBM_CUDA(launch_force_ref(q_, sb_, pb_, d_f_[last_dst_], d_force_, launch_));
  else
    TLBM_CUDA(launch_force_fast(q_, store_, pb_, d_f_[last_dst_], d_force_, launch_));
  launches_ += 2;
  outputs_fresh_ = true;
  return Status::ok();
}

Status Engine::fetch(const void* dev, void* host, bool wait) {
  const size_t bytes = static_cast<size_t>(n_) * ob_;
  const void* from = dev;
  if (!identity_order_) {
    TLBM_CUDA(launch_gather(dev, d_order_, n_, ob_, d_stage_, launch_));
    ++launches_;
    from = d_stage_;
  }
  TLBM_CUDA(cudaMemcpyAsync(host, from, bytes, cudaMemcpyDeviceToHost, stream_));
  if (wait) TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::write_fields(const std::string* names, const void* const* dev, int k) {
  // The page-locked staging buffer of the dump files: a slot per field, made at the first dump
  // (runs without file dumps never pay the pinning).  Every field is queued into its slot (the
  // gathers and copies are stream-ordered, so the one gather buffer is reused safely), then the
  // k files are written by k host threads at once: on GB300's host a 1.9 GB FP64 dump of
  // 512x256x256 takes ~290 ms written file after file and ~60 ms in parallel.
  if (k < 1 || k > 7) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "1 to 7 fields per dump");
  const size_t bytes = static_cast<size_t>(n_) * ob_;
  if (!h_pinned_) TLBM_CUDA(cudaMallocHost(&h_pinned_, 7 * bytes));
  char* const base = static_cast<char*>(h_pinned_);
  for (int j = 0; j < k; ++j) TLBM_TRY(fetch(dev[j], base + j * bytes, false));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  std::vector<Status> st(static_cast<size_t>(k));
  auto write_one = [&](int j) {  // no exception may leave a thread
    try {
      st[j] = write_at(workdir_ + "/" + names[j], base + j * bytes, bytes, 0);
    } catch (const std::bad_alloc&) {
      st[j] = Status::err(TLBM_ERR_NO_MEMORY, "out of host memory writing a dump file");
    }
  };
  std::vector<std::thread> pool;
  for (int j = 1; j < k; ++j) {
    try {
      pool.emplace_back(write_one, j);
    } catch (const std::system_error&) {
      write_one(j);  // no thread to be had: this one in turn
    }
  }
  write_one(0);
  for (auto& t : pool) t.join();
  for (const Status& s : st)
    if (!s.good()) return s;
  return Status::ok();
}

Status Engine::write_data() {
  TraceRange trace("tlbm_write_data");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (workdir_.empty()) return Status::err(TLBM_ERR_IO, "no output directory");
  TLBM_TRY(compute_outputs());
  const std::string d = std::to_string(dump_num_);
  const std::string names[7] = {"ux" + d + ".b_dat", "uy" + d + ".b_dat", "uz" + d + ".b_dat",
                                "density" + d + ".b_dat", "Fx" + d + ".b_dat",
                                "Fy" + d + ".b_dat", "Fz" + d + ".b_dat"};
  const void* dev[7] = {d_macro_[0], d_macro_[1], d_macro_[2], d_macro_[3],
                        d_force_[0], d_force_[1], d_force_[2]};
  TLBM_TRY(write_fields(names, dev, 7));
  if (prob_.ss_data_flag == 1) TLBM_TRY(write_subspace(d));
  ++dump_num_;
  return Status::ok();
}

Status Engine::write_time_avg_data() {
  TraceRange trace("tlbm_write_time_avg_data");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (prob_.time_avg_flag != 1)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "time averaging is off (params.lbm line 15)");
  if (workdir_.empty()) return Status::err(TLBM_ERR_IO, "no output directory");
  const std::string names[4] = {"uAvg.b_dat", "vAvg.b_dat", "wAvg.b_dat", "rhoAvg.b_dat"};
  const void* dev[4] = {d_avg_[0], d_avg_[1], d_avg_[2], d_avg_[3]};
  TLBM_TRY(write_fields(names, dev, 4));
  return Status::ok();
}

Status Engine::processed(bool time_avg, float* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (prob_.p_ref_idx < 0 || prob_.p_ref_idx >= n_)
    return Status::err(TLBM_ERR_OUT_OF_RANGE, "params.lbm: pRef_idx outside the lattice");
  const void* f[7] = {};
  if (time_avg) {
    if (prob_.time_avg_flag != 1)
      return Status::err(TLBM_ERR_INVALID_ARGUMENT, "time averaging is off (params.lbm line 15)");
    for (int k = 0; k < 4; ++k) f[k] = d_avg_[k];
  } else {
    TLBM_TRY(compute_outputs());
    for (int k = 0; k < 4; ++k) f[k] = d_macro_[k];
    for (int k = 0; k < 3; ++k) f[4 + k] = d_force_[k];
  }
  const size_t planes = time_avg ? kPostAvgFields : kPostFields;
  const size_t bytes = static_cast<size_t>(n_) * 4 * planes;
  float* d = nullptr;
  TLBM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), bytes, stream_));
  const PostFactors k = post_factors(prob_, time_avg);
  cudaError_t e;
  if (ob_ == 4) {
    PostInputs<float> in;
    const float** p[7] = {&in.ux, &in.uy, &in.uz, &in.rho, &in.fx, &in.fy, &in.fz};
    for (int i = 0; i < 7; ++i) *p[i] = static_cast<const float*>(f[i]);
    e = launch_post(in, nullptr, n_, prob_.p_ref_idx, k, d, stream_);
  } else {
    PostInputs<double> in;
    const double** p[7] = {&in.ux, &in.uy, &in.uz, &in.rho, &in.fx, &in.fy, &in.fz};
    for (int i = 0; i < 7; ++i) *p[i] = static_cast<const double*>(f[i]);
    e = launch_post(in, nullptr, n_, prob_.p_ref_idx, k, d, stream_);
  }
  ++launches_;
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::write_processed(bool time_avg) {
  if (workdir_.empty()) return Status::err(TLBM_ERR_IO, "no output directory");
  std::vector<float> host(static_cast<size_t>(n_) * (time_avg ? kPostAvgFields : kPostFields));
  TLBM_TRY(processed(time_avg, host.data()));
  const std::string d = std::to_string(proc_num_);
  std::string err;
  const bool ok = time_avg ? post_write(workdir_, "timeAvg.h5", "timeAvg.xmf", prob_,
                                        host.data(), true, &err)
                           : post_write(workdir_, "out" + d + ".h5", "data" + d + ".xmf", prob_,
                                        host.data(), false, &err);
  if (!ok) return Status::err(TLBM_ERR_IO, err);
  if (!time_avg) ++proc_num_;
  return Status::ok();
}

Status Engine::copy_macros(void* ux, void* uy, void* uz, void* rho) {
  TraceRange trace("tlbm_copy_macros");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  TLBM_TRY(compute_outputs());
  void* o[4] = {ux, uy, uz, rho};
  const size_t bytes = static_cast<size_t>(n_) * ob_;
  for (int k = 0; k < 4; ++k) {
    if (!o[k]) continue;
    TLBM_CUDA(cudaMemcpyAsync(o[k], d_macro_[k], bytes, cudaMemcpyDeviceToHost, stream_));
  }
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::copy_force(void* fx, void* fy, void* fz) {
  TraceRange trace("tlbm_copy_force");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  TLBM_TRY(compute_outputs());
  void* o[3] = {fx, fy, fz};
  const size_t bytes = static_cast<size_t>(n_) * ob_;
  for (int k = 0; k < 3; ++k) {
    if (!o[k]) continue;
    TLBM_CUDA(cudaMemcpyAsync(o[k], d_force_[k], bytes, cudaMemcpyDeviceToHost, stream_));
  }
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::copy_outputs_async(void* const host[7]) {
  TraceRange trace("tlbm_copy_outputs_async");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (!copy_stream_) {  // all four or none
    cudaStream_t cs = nullptr;
    cudaEvent_t ready = nullptr, done = nullptr, macros = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&macros, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      if (macros) cudaEventDestroy(macros);
      if (done) cudaEventDestroy(done);
      if (ready) cudaEventDestroy(ready);
      if (cs) cudaStreamDestroy(cs);
      TLBM_CUDA(e);
    }
    copy_stream_ = cs;
    outputs_ready_ = ready;
    copies_done_ = done;
    macros_ready_ = macros;
  }
  TLBM_TRY(compute_outputs(macros_ready_));
  TLBM_CUDA(cudaEventRecord(outputs_ready_, stream_));
  const size_t bytes = static_cast<size_t>(n_) * ob_;
  const void* dev[7] = {d_macro_[0], d_macro_[1], d_macro_[2], d_macro_[3],
                        d_force_[0], d_force_[1], d_force_[2]};
  // Page-locked destinations are written by a copy kernel on the copy stream: on GB300 its
  // stores reach page-locked host memory at the copy engines' rate (~190 GB/s), and some
  // copy-engine transfers issued from an application process ran at ~16 GB/s.  Other
  // destinations take cudaMemcpyAsync.  ux..rho start as soon as they are computed, while the
  // force kernel runs; Fx..Fz follow it.
  for (int group = 0; group < 2; ++group) {
    TLBM_CUDA(cudaStreamWaitEvent(copy_stream_, group == 0 ? macros_ready_ : outputs_ready_, 0));
    const void* ksrc[4];
    void* kdst[4];
    int nk = 0;
    for (int k = group == 0 ? 0 : 4; k < (group == 0 ? 4 : 7); ++k) {
      if (!host[k]) continue;
      cudaPointerAttributes at{};
      const bool pinned = cudaPointerGetAttributes(&at, host[k]) == cudaSuccess &&
                          at.type == cudaMemoryTypeHost &&
                          reinterpret_cast<uintptr_t>(host[k]) % 16 == 0 && bytes % 16 == 0;
      cudaGetLastError();  // a pageable pointer can leave an error state behind
      if (pinned) {
        ksrc[nk] = dev[k];
        kdst[nk] = at.devicePointer ? at.devicePointer : host[k];
        ++nk;
      } else {
        TLBM_CUDA(cudaMemcpyAsync(host[k], dev[k], bytes, cudaMemcpyDeviceToHost, copy_stream_));
      }
    }
    if (nk > 0) {
      if (sms_ == 0) TLBM_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount,
                                                      opt_.device));
      Launch cl = launch_;
      cl.stream = copy_stream_;
      TLBM_CUDA(launch_copy_words(ksrc, kdst, nk, bytes, 2 * sms_, cl));
      ++launches_;
    }
  }
  TLBM_CUDA(cudaEventRecord(copies_done_, copy_stream_));
  copies_pending_ = true;
  return Status::ok();
}

Status Engine::copy_populations(int which, void* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (last_src_ < 0) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "no time step taken yet");
  const size_t bytes = static_cast<size_t>(n_) * q_ * ob_;
  void* d = nullptr;
  TLBM_CUDA(cudaMallocAsync(&d, bytes, stream_));
  // which = 0: post-stream fOut = pull of the last destination; 1: post-collision values
  cudaError_t e = launch_to_aos(q_, store_, pb_, d_f_[last_dst_], which == 0 ? 1 : 0, d, ob_,
                                launch_);
  ++launches_;
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::copy_adjacency(int32_t* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  const size_t bytes = static_cast<size_t>(n_) * q_ * sizeof(int32_t);
  void* d = nullptr;
  TLBM_CUDA(cudaMallocAsync(&d, bytes, stream_));
  cudaError_t e = launch_adjacency(q_, pb_, static_cast<int32_t*>(d), launch_);
  ++launches_;
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, bytes, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Engine::mass(double* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  // the populations the next step will pull (after a step: its destination)
  const int buf = last_dst_ >= 0 ? last_dst_ : 1;
  TLBM_CUDA(launch_mass(q_, store_, pb_, d_f_[buf], d_partial_, mass_blocks(pb_), d_mass_,
                        launch_));
  launches_ += 2;
  TLBM_CUDA(cudaMemcpyAsync(out, d_mass_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  if (!std::isfinite(*out))
    return Status::err(TLBM_ERR_NUMERIC, "total mass is not finite: the run has diverged");
  return Status::ok();
}

Status Engine::load_restart(const float* ux, const float* uy, const float* uz,
                            const float* rho) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (!ux || !uy || !uz || !rho) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "NULL field");
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  const size_t bytes = static_cast<size_t>(n_) * sizeof(float);
  void* d = nullptr;
  TLBM_CUDA(cudaMalloc(&d, 4 * bytes));
  char* db = static_cast<char*>(d);
  const void* m[4] = {db, db + bytes, db + 2 * bytes, db + 3 * bytes};
  const float* h[4] = {ux, uy, uz, rho};
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    e = cudaMemcpy(const_cast<void*>(m[k]), h[k], bytes, cudaMemcpyHostToDevice);
  // f = feq of every node, placed so that the next pull returns it at its own node
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = launch_init_equilibrium(q_, store_, pb_, d_f_[b], m, 4, launch_);
    ++launches_;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  cudaFree(d);
  TLBM_CUDA(e);
  last_src_ = last_dst_ = -1;
  outputs_fresh_ = false;
  return Status::ok();
}

Status Engine::set_inlet_profile(const double* uz) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (ref_arith_)
    return Status::err(TLBM_ERR_UNSUPPORTED,
                       "an inlet profile changes the reference's physics: fast arithmetic only");
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  drop_graphs();
  if (!uz) {
    pb_.inlet_d = nullptr;
    pb_.inlet_f = nullptr;
    return Status::ok();
  }
  const size_t nxy = static_cast<size_t>(pb_.nxy);
  std::vector<float> uf(nxy);
  for (size_t k = 0; k < nxy; ++k) uf[k] = static_cast<float>(uz[k]);
  if (!d_inlet_d_) TLBM_CUDA(cudaMalloc(&d_inlet_d_, nxy * sizeof(double)));
  if (!d_inlet_f_) TLBM_CUDA(cudaMalloc(&d_inlet_f_, nxy * sizeof(float)));
  TLBM_CUDA(cudaMemcpy(d_inlet_d_, uz, nxy * sizeof(double), cudaMemcpyHostToDevice));
  TLBM_CUDA(cudaMemcpy(d_inlet_f_, uf.data(), nxy * sizeof(float), cudaMemcpyHostToDevice));
  pb_.inlet_d = d_inlet_d_;
  pb_.inlet_f = d_inlet_f_;
  return Status::ok();
}

Status Engine::set_closure(const float* params, const float* scale, const float* shift,
                           float out_scale, float tau_min) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (ref_arith_)
    return Status::err(TLBM_ERR_UNSUPPORTED,
                       "the learned closure has no reference arithmetic: use TLBM_ARITH_FAST");
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  drop_graphs();
  if (!params) {
    delete static_cast<mlp::Closure*>(h_closure_);
    h_closure_ = nullptr;
    return Status::ok();
  }
  if (!scale || !shift || !(tau_min > 0.5f) || !std::isfinite(out_scale))
    return Status::err(TLBM_ERR_INVALID_ARGUMENT,
                       "closure needs 8 scales and shifts, a finite out_scale and tau_min > 1/2");
  // the tensor-core image: weights rounded to BF16 once here, biases FP32 (mlp.cuh)
  mlp::MmaWeights img;
  mlp::build_mma_weights(params, &img);
  if (!d_closure_w_) TLBM_CUDA(cudaMalloc(&d_closure_w_, sizeof(mlp::MmaWeights)));
  TLBM_CUDA(cudaMemcpy(d_closure_w_, &img, sizeof(img), cudaMemcpyHostToDevice));
  mlp::Closure c{};
  c.w = static_cast<const mlp::MmaWeights*>(d_closure_w_);
  for (int k = 0; k < mlp::kIn; ++k) {
    c.scale[k] = scale[k];
    c.shift[k] = shift[k];
    c.offset[k] = -shift[k] * scale[k];
  }
  c.out_scale = out_scale;
  c.tau_min = tau_min;
  if (!h_closure_) h_closure_ = new mlp::Closure();
  *static_cast<mlp::Closure*>(h_closure_) = c;
  return Status::ok();
}

Status Engine::filtered(int f, void* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (f < 1 || prob_.nx % f || prob_.ny % f || prob_.nz % f)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "the filter width must divide nx, ny and nz");
  TLBM_TRY(compute_outputs());
  const size_t nc = static_cast<size_t>(prob_.nx / f) * (prob_.ny / f) * (prob_.nz / f);
  void* d = nullptr;
  TLBM_CUDA(cudaMallocAsync(&d, 10 * nc * ob_, stream_));
  cudaError_t e = launch_box_filter(d_macro_, ob_, prob_.nx, prob_.ny, prob_.nz, f, d, stream_);
  ++launches_;
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, 10 * nc * ob_, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

}  // namespace tlbm
