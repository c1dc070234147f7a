// capi_mlp.cpp -- C ABI of the learned closure's trainer (include/tlbm.h).
#include <new>
#include <string>

#include "../../include/tlbm.h"
#include "mlp.cuh"
#include "mlp_trainer.h"

struct tlbm_mlp {
  tlbm::MlpTrainer* t = nullptr;
  std::string error;
};

namespace {
thread_local std::string g_mlp_create_error;

tlbm_status wrap_m(tlbm_mlp* h, const tlbm::Status& s) {
  if (!s.good() && h) h->error = s.msg;
  return s.code;
}
bool valid_m(const tlbm_mlp* h) { return h && h->t; }
}  // namespace

#define TLBM_MCALL(h, expr)                                                          \
  do {                                                                               \
    if (!valid_m(h)) return TLBM_ERR_INVALID_ARGUMENT;                               \
    try {                                                                            \
      return wrap_m(h, (expr));                                                      \
    } catch (const std::bad_alloc&) {                                                \
      return wrap_m(h, tlbm::Status::err(TLBM_ERR_NO_MEMORY, "out of host memory")); \
    }                                                                                \
  } while (0)

extern "C" {

int tlbm_mlp_num_params(void) { return tlbm::mlp::kParams; }

tlbm_status tlbm_mlp_create(int64_t n, const float* features, const float* targets,
                            uint64_t seed, int device, tlbm_mlp** out) {
  try {
    if (!out) return TLBM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    tlbm::MlpTrainer* t = nullptr;
    tlbm::Status s = tlbm::MlpTrainer::create(n, features, targets, seed, device, &t);
    if (!s.good()) {
      g_mlp_create_error = s.msg;
      return s.code;
    }
    tlbm_mlp* h = new (std::nothrow) tlbm_mlp();
    if (!h) {
      delete t;
      return TLBM_ERR_NO_MEMORY;
    }
    h->t = t;
    *out = h;
    return TLBM_OK;
  } catch (const std::bad_alloc&) {
    g_mlp_create_error = "out of host memory";
    return TLBM_ERR_NO_MEMORY;
  }
}

tlbm_status tlbm_mlp_destroy(tlbm_mlp* h) {
  if (!h) return TLBM_ERR_INVALID_ARGUMENT;
  delete h->t;
  delete h;
  return TLBM_OK;
}

tlbm_status tlbm_mlp_set_params(tlbm_mlp* h, const float* params) {
  if (!params) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_MCALL(h, h->t->set_params(params));
}
tlbm_status tlbm_mlp_get_params(tlbm_mlp* h, float* params) {
  if (!params) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_MCALL(h, h->t->get_params(params));
}
tlbm_status tlbm_mlp_loss_grad(tlbm_mlp* h, int64_t first, int64_t count, float* loss,
                               float* grad) {
  TLBM_MCALL(h, h->t->loss_grad(first, count, loss, grad));
}
tlbm_status tlbm_mlp_train(tlbm_mlp* h, int epochs, int64_t batch, float lr, float* epoch_loss) {
  TLBM_MCALL(h, h->t->train(epochs, batch, lr, epoch_loss));
}
tlbm_status tlbm_mlp_predict(tlbm_mlp* h, int64_t n, const float* features, float* y) {
  if (!features || !y) return TLBM_ERR_INVALID_ARGUMENT;
  TLBM_MCALL(h, h->t->predict(n, features, y));
}
const char* tlbm_mlp_last_error(const tlbm_mlp* h) {
  if (!h) return g_mlp_create_error.c_str();
  return h->error.c_str();
}

}  // extern "C"
