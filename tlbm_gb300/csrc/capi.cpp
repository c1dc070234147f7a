// capi.cpp -- the extern "C" boundary (include/tlbm.h): status codes, no exceptions across it.
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tlbm.h"
#include "engine.h"

struct tlbm_handle {
  tlbm::Engine* engine = nullptr;
  std::string error;
};

namespace {

thread_local std::string g_create_error;

tlbm_status fail_create(const tlbm::Status& s) {
  g_create_error = s.msg;
  return s.code;
}

tlbm_status wrap(tlbm_handle* h, const tlbm::Status& s) {
  if (!s.good() && h) h->error = s.msg;
  return s.code;
}

bool valid(const tlbm_handle* h) { return h && h->engine; }

tlbm_status create_common(const tlbm_problem& prob, const int32_t* nd, const int32_t* parts,
                          int size, const std::string& workdir, const tlbm_options& opt,
                          tlbm_handle** out) {
  tlbm::Engine* e = nullptr;
  tlbm::Status s = tlbm::Engine::create(prob, nd, parts, size, workdir, opt, &e);
  if (!s.good()) return fail_create(s);
  tlbm_handle* h = new (std::nothrow) tlbm_handle();
  if (!h) {
    delete e;
    return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
  }
  h->engine = e;
  *out = h;
  return TLBM_OK;
}

tlbm_status create_from_dir(const char* workdir, int rank, int size, tlbm_options opt,
                            tlbm_handle** out) {
  try {
    if (!out) return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "out is NULL"));
    *out = nullptr;
    if (!workdir) workdir = ".";
    if (rank != 0)
      return fail_create(tlbm::Status::err(
          TLBM_ERR_INVALID_ARGUMENT, "rank must be 0: one process drives the whole lattice"));
    const std::string dir(workdir);
    std::string text;
    tlbm::Status s = tlbm::read_text(dir + "/params.lbm", &text);
    if (!s.good()) return fail_create(s);
    tlbm_problem prob;
    // `real` values are parsed in the precision that computes with them
    s = tlbm::parse_params(text, opt.precision != TLBM_PREC_F64, &prob);
    if (!s.good()) return fail_create(s);
    if (prob.nx < 1 || prob.ny < 1 || prob.nz < 1)
      return fail_create(tlbm::Status::err(TLBM_ERR_FORMAT, "params.lbm: bad lattice size"));
    const int64_t n = static_cast<int64_t>(prob.nx) * prob.ny * prob.nz;
    if (std::strcmp(prob.lattice, "D3Q15") && std::strcmp(prob.lattice, "D3Q19") &&
        std::strcmp(prob.lattice, "D3Q27"))
      return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "Invalid Lattice Structure!"));
    std::vector<int32_t> parts, nd;
    s = tlbm::parse_int_file(dir + "/parts.lbm", n, &parts);
    if (!s.good()) return fail_create(s);
    s = tlbm::parse_int_file(dir + "/ndType.lbm", n, &nd);
    if (!s.good()) return fail_create(s);
    return create_common(prob, nd.data(), parts.data(), size, dir, opt, out);
  } catch (const std::bad_alloc&) {
    return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
  } catch (const std::exception& ex) {
    return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, ex.what()));
  }
}

}  // namespace

extern "C" {

void tlbm_default_options(tlbm_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof(*opt));
  opt->struct_size = sizeof(tlbm_options);
  opt->precision = TLBM_PREC_F32;
  opt->arithmetic = TLBM_ARITH_REFERENCE;
  opt->closure = TLBM_CLOSURE_PARAMS;
}

tlbm_status tlbm_create(const char* workdir, int rank, int size, tlbm_handle** out) {
  tlbm_options opt;
  tlbm_default_options(&opt);
  tlbm::Status s = tlbm::apply_config_file(std::string(workdir ? workdir : ".") + "/tlbm.cfg", &opt);
  if (!s.good()) return fail_create(s);
  return create_from_dir(workdir, rank, size, opt, out);
}

tlbm_status tlbm_create_ex(const char* workdir, int rank, int size, const tlbm_options* opt,
                           tlbm_handle** out) {
  tlbm_options o;
  tlbm_default_options(&o);
  if (opt) {
    if (opt->struct_size < (int)offsetof(tlbm_options, reserved) ||
        opt->struct_size > (int)sizeof(tlbm_options))
      return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "bad options.struct_size"));
    std::memcpy(&o, opt, static_cast<size_t>(opt->struct_size));
  }
  return create_from_dir(workdir, rank, size, o, out);
}

tlbm_status tlbm_create_from_arrays(const tlbm_problem* prob, const int32_t* nd_type,
                                    const int32_t* parts, const char* workdir,
                                    const tlbm_options* opt, tlbm_handle** out) {
  try {
    if (!out || !prob || !nd_type)
      return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "NULL argument"));
    *out = nullptr;
    tlbm_options o;
    tlbm_default_options(&o);
    if (opt) {
      if (opt->struct_size < (int)offsetof(tlbm_options, reserved) ||
          opt->struct_size > (int)sizeof(tlbm_options))
        return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "bad options.struct_size"));
      std::memcpy(&o, opt, static_cast<size_t>(opt->struct_size));
    }
    int size = 1;
    if (parts) {
      const int64_t n = static_cast<int64_t>(prob->nx) * prob->ny * prob->nz;
      for (int64_t g = 0; g < n; ++g)
        if (parts[g] + 1 > size) size = parts[g] + 1;
    }
    return create_common(*prob, nd_type, parts, size, workdir ? std::string(workdir) : std::string(),
                         o, out);
  } catch (const std::bad_alloc&) {
    return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
  }
}

tlbm_status tlbm_destroy(tlbm_handle* h) {
  if (!h) return TLBM_ERR_INVALID_ARGUMENT;
  delete h->engine;
  delete h;
  return TLBM_OK;
}

#define TLBM_CALL(h, expr)                                                        \
  do {                                                                            \
    if (!valid(h)) return TLBM_ERR_INVALID_ARGUMENT;                              \
    try {                                                                         \
      return wrap(h, (expr));                                                     \
    } catch (const std::bad_alloc&) {                                             \
      return wrap(h, tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory")); \
    }                                                                             \
  } while (0)

tlbm_status tlbm_step(tlbm_handle* h, int is_even) { TLBM_CALL(h, h->engine->step(is_even ? 1 : 0)); }
tlbm_status tlbm_run(tlbm_handle* h, int first_ts, int nsteps) {
  TLBM_CALL(h, h->engine->run(first_ts, nsteps));
}
tlbm_status tlbm_time_steps(tlbm_handle* h, int first_ts, int nsteps, float* ms) {
  if (!ms) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->time_steps(first_ts, nsteps, ms));
}
tlbm_status tlbm_synchronize(tlbm_handle* h) { TLBM_CALL(h, h->engine->synchronize()); }
tlbm_status tlbm_write_data(tlbm_handle* h) { TLBM_CALL(h, h->engine->write_data()); }
tlbm_status tlbm_write_time_avg_data(tlbm_handle* h) {
  TLBM_CALL(h, h->engine->write_time_avg_data());
}

int tlbm_get_num_ts(const tlbm_handle* h) { return valid(h) ? h->engine->problem().num_ts : -1; }
int tlbm_get_ts_rep_freq(const tlbm_handle* h) {
  return valid(h) ? h->engine->problem().ts_rep_freq : -1;
}
int tlbm_get_plot_freq(const tlbm_handle* h) { return valid(h) ? h->engine->problem().plot_freq : -1; }
int tlbm_get_warmup_ts(const tlbm_handle* h) { return valid(h) ? h->engine->problem().warmup_ts : -1; }
int tlbm_get_num_global_nodes(const tlbm_handle* h) {
  if (!valid(h)) return -1;
  const tlbm_problem& p = h->engine->problem();
  return p.nx * p.ny * p.nz;
}
int tlbm_get_time_avg_flag(const tlbm_handle* h) {
  return valid(h) ? h->engine->problem().time_avg_flag : -1;
}
int tlbm_is_restart(const tlbm_handle* h) { return valid(h) ? h->engine->problem().restart_flag : -1; }
int tlbm_get_cut_size(const tlbm_handle* h) { return valid(h) ? h->engine->cut_size() : -1; }

tlbm_status tlbm_get_options(const tlbm_handle* h, tlbm_options* out) {
  if (!valid(h) || !out || out->struct_size < static_cast<int>(sizeof(int)) ||
      out->struct_size > static_cast<int>(sizeof(tlbm_options)))
    return TLBM_ERR_INVALID_ARGUMENT;
  const int n = out->struct_size;
  std::memcpy(out, &h->engine->options(), static_cast<size_t>(n));
  out->struct_size = n;
  return TLBM_OK;
}

const char* tlbm_get_last_error(const tlbm_handle* h) {
  if (!h) return g_create_error.c_str();
  return h->error.c_str();
}

const char* tlbm_status_string(tlbm_status s) {
  switch (s) {
    case TLBM_OK: return "ok";
    case TLBM_ERR_IO: return "i/o error";
    case TLBM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TLBM_ERR_FORMAT: return "malformed input";
    case TLBM_ERR_OUT_OF_RANGE: return "value out of range";
    case TLBM_ERR_CUDA: return "CUDA error";
    case TLBM_ERR_NUMERIC: return "non-finite result";
    case TLBM_ERR_UNSUPPORTED: return "unsupported";
    case TLBM_ERR_TIMEOUT: return "device wait timed out";
    case TLBM_ERR_NO_MEMORY: return "out of memory";
    default: return "unknown status";
  }
}

int tlbm_output_bytes(const tlbm_handle* h) { return valid(h) ? h->engine->output_bytes() : -1; }
int tlbm_num_speeds(const tlbm_handle* h) { return valid(h) ? h->engine->q() : -1; }

tlbm_status tlbm_copy_macros(tlbm_handle* h, void* ux, void* uy, void* uz, void* rho) {
  TLBM_CALL(h, h->engine->copy_macros(ux, uy, uz, rho));
}
tlbm_status tlbm_copy_force(tlbm_handle* h, void* fx, void* fy, void* fz) {
  TLBM_CALL(h, h->engine->copy_force(fx, fy, fz));
}
tlbm_status tlbm_copy_outputs_async(tlbm_handle* h, void* ux, void* uy, void* uz, void* rho,
                                    void* fx, void* fy, void* fz) {
  void* const host[7] = {ux, uy, uz, rho, fx, fy, fz};
  TLBM_CALL(h, h->engine->copy_outputs_async(host));
}
tlbm_status tlbm_host_alloc(size_t bytes, void** out) {
  if (!out) return TLBM_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (bytes == 0) return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "0 bytes"));
  const cudaError_t e = cudaMallocHost(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail_create(tlbm::Status::err(e == cudaErrorMemoryAllocation ? TLBM_ERR_NO_MEMORY
                                                                        : TLBM_ERR_CUDA,
                                         std::string("cudaMallocHost: ") + cudaGetErrorString(e)));
  }
  return TLBM_OK;
}
tlbm_status tlbm_host_free(void* p) {
  if (!p) return TLBM_OK;
  const cudaError_t e = cudaFreeHost(p);
  if (e != cudaSuccess)
    return fail_create(tlbm::Status::err(TLBM_ERR_CUDA,
                                         std::string("cudaFreeHost: ") + cudaGetErrorString(e)));
  return TLBM_OK;
}
tlbm_status tlbm_copy_populations(tlbm_handle* h, int which, void* out) {
  if (!out) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->copy_populations(which, out));
}
tlbm_status tlbm_copy_adjacency(tlbm_handle* h, int32_t* out) {
  if (!out) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->copy_adjacency(out));
}
tlbm_status tlbm_mass(tlbm_handle* h, double* mass) {
  if (!mass) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->mass(mass));
}
int64_t tlbm_kernel_launches(const tlbm_handle* h) { return valid(h) ? h->engine->launches() : -1; }

tlbm_status tlbm_load_restart(tlbm_handle* h, const float* ux, const float* uy, const float* uz,
                              const float* rho) {
  TLBM_CALL(h, h->engine->load_restart(ux, uy, uz, rho));
}

tlbm_status tlbm_set_inlet_profile(tlbm_handle* h, const double* uz) {
  TLBM_CALL(h, h->engine->set_inlet_profile(uz));
}
tlbm_status tlbm_set_closure_mlp(tlbm_handle* h, const float* params, const float* scale,
                                 const float* shift, float out_scale, float tau_min) {
  TLBM_CALL(h, h->engine->set_closure(params, scale, shift, out_scale, tau_min));
}
tlbm_status tlbm_filtered_fields(tlbm_handle* h, int factor, void* out) {
  if (!out) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->filtered(factor, out));
}

tlbm_status tlbm_processed_fields(tlbm_handle* h, int time_avg, float* out) {
  if (!out) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_CALL(h, h->engine->processed(time_avg != 0, out));
}

tlbm_status tlbm_write_processed_data(tlbm_handle* h, int time_avg) {
  TLBM_CALL(h, h->engine->write_processed(time_avg != 0));
}

tlbm_status tlbm_process_output_dir(const char* workdir, int device, int* dumps) {
  int done = 0;
  try {
    tlbm::Status s = tlbm::post_process_dir(workdir ? workdir : ".", device, &done);
    if (dumps) *dumps = done;
    if (!s.good()) return fail_create(s);
    return TLBM_OK;
  } catch (const std::bad_alloc&) {
    if (dumps) *dumps = done;
    return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
  }
}

}  // extern "C"

// ---------------------------------------------------------------------------- ensembles

#include "ensemble.h"

struct tlbm_ensemble {
  tlbm::Ensemble* e = nullptr;
  std::string error;
};

namespace {
tlbm_status wrap_e(tlbm_ensemble* h, const tlbm::Status& s) {
  if (!s.good() && h) h->error = s.msg;
  return s.code;
}
bool valid_e(const tlbm_ensemble* h) { return h && h->e; }
}  // namespace

#define TLBM_ECALL(h, expr)                                                          \
  do {                                                                               \
    if (!valid_e(h)) return TLBM_ERR_INVALID_ARGUMENT;                               \
    try {                                                                            \
      return wrap_e(h, (expr));                                                      \
    } catch (const std::bad_alloc&) {                                                \
      return wrap_e(h, tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory")); \
    }                                                                                \
  } while (0)

extern "C" {

tlbm_status tlbm_ensemble_create(int n, const tlbm_problem* problems,
                                 const int32_t* const* nd_types, const tlbm_options* opt,
                                 tlbm_ensemble** out) {
  try {
    if (!out || !problems || !nd_types || n < 1)
      return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "bad ensemble arguments"));
    *out = nullptr;
    tlbm_options o;
    tlbm_default_options(&o);
    if (opt) {
      if (opt->struct_size < (int)offsetof(tlbm_options, reserved) ||
          opt->struct_size > (int)sizeof(tlbm_options))
        return fail_create(tlbm::Status::err(TLBM_ERR_INVALID_ARGUMENT, "bad options.struct_size"));
      std::memcpy(&o, opt, static_cast<size_t>(opt->struct_size));
    }
    tlbm::Ensemble* e = nullptr;
    tlbm::Status s = tlbm::Ensemble::create(n, problems, nd_types, o, &e);
    if (!s.good()) return fail_create(s);
    tlbm_ensemble* h = new (std::nothrow) tlbm_ensemble();
    if (!h) {
      delete e;
      return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
    }
    h->e = e;
    *out = h;
    return TLBM_OK;
  } catch (const std::bad_alloc&) {
    return fail_create(tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory"));
  }
}

tlbm_status tlbm_ensemble_destroy(tlbm_ensemble* h) {
  if (!h) return TLBM_ERR_INVALID_ARGUMENT;
  delete h->e;
  delete h;
  return TLBM_OK;
}

tlbm_status tlbm_ensemble_set_tiles(tlbm_ensemble* h, int bx, int by, int cpt) {
  TLBM_ECALL(h, h->e->set_tiles(bx, by, cpt));
}
tlbm_status tlbm_ensemble_autotune(tlbm_ensemble* h, int steps, int* bx, int* by, int* cpt) {
  TLBM_ECALL(h, h->e->autotune(steps, bx, by, cpt));
}
tlbm_status tlbm_ensemble_run(tlbm_ensemble* h, int first_ts, int nsteps) {
  TLBM_ECALL(h, h->e->run(first_ts, nsteps));
}
tlbm_status tlbm_ensemble_time_steps(tlbm_ensemble* h, int first_ts, int nsteps, float* ms) {
  if (!ms) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_ECALL(h, h->e->time_steps(first_ts, nsteps, ms));
}
tlbm_status tlbm_ensemble_copy_macros(tlbm_ensemble* h, int channel, void* ux, void* uy, void* uz,
                                      void* rho) {
  TLBM_ECALL(h, h->e->copy_macros(channel, ux, uy, uz, rho));
}
tlbm_status tlbm_ensemble_mass(tlbm_ensemble* h, int channel, double* mass) {
  if (!mass) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_ECALL(h, h->e->mass(channel, mass));
}
int64_t tlbm_ensemble_cells(const tlbm_ensemble* h) { return valid_e(h) ? h->e->cells() : -1; }
int64_t tlbm_ensemble_kernel_launches(const tlbm_ensemble* h) {
  return valid_e(h) ? h->e->launches() : -1;
}
const char* tlbm_ensemble_last_error(const tlbm_ensemble* h) {
  if (!h) return g_create_error.c_str();
  return h->error.c_str();
}

}  // extern "C"
