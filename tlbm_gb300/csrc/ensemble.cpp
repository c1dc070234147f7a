// ensemble.cpp -- host side of the batched ensemble: one arena, a tile list, graph-replayed
// persistent launches, and the tile-shape autotuner.
#include "ensemble.h"

#include <algorithm>
#include <cstring>

#include "trace.h"

namespace tlbm {

#define TLBM_TRY(expr)         \
  do {                         \
    Status _s = (expr);        \
    if (!_s.good()) return _s; \
  } while (0)
#define TLBM_CUDA(expr) TLBM_TRY(check((expr), #expr))

Status Ensemble::check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return Status::ok();
  return Status::err(TLBM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

Ensemble::~Ensemble() {
  if (stream_) cudaStreamSynchronize(stream_);
  drop_graphs();
  cudaFree(arena_);
  cudaFree(d_ch_);
  cudaFree(d_tiles_);
  cudaFree(d_partial_);
  cudaFree(d_mass_);
  if (stream_) cudaStreamDestroy(stream_);
}

void Ensemble::drop_graphs() {
  for (auto& g : graph_) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

Status Ensemble::create(int n, const tlbm_problem* probs, const int32_t* const* nd_types,
                        const tlbm_options& opt, Ensemble** out) {
  TraceRange trace("tlbm_ensemble_create");
  *out = nullptr;
  Ensemble* e = new (std::nothrow) Ensemble();
  if (!e) return Status::err(TLBM_ERR_NO_MEMORY, "out of host memory");
  e->opt_ = opt;
  Status s = e->init(n, probs, nd_types);
  if (!s.good()) {
    delete e;
    return s;
  }
  *out = e;
  return Status::ok();
}

Status Ensemble::init(int n, const tlbm_problem* probs, const int32_t* const* nd_types) {
  if (n < 1 || n > 65535) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "1..65535 channels");
  switch (opt_.precision) {
    case TLBM_PREC_F64: store_ = kStoreF64; break;
    case TLBM_PREC_F32: store_ = kStoreF32; break;
    case TLBM_PREC_BF16: store_ = kStoreBF16; break;
    case TLBM_PREC_F16: store_ = kStoreF16; break;
    case TLBM_PREC_BF16M:
      return Status::err(TLBM_ERR_UNSUPPORTED, "ensembles take f64, f32, bf16 or f16 storage");
    default: return Status::err(TLBM_ERR_INVALID_ARGUMENT, "unknown precision option");
  }
  // FP64 channels: populations held as Q1.62 when every channel's collision runs in fixed point
  // with a density inside that format's range, as a single-lattice handle of each would
  if (store_ == kStoreF64 && !opt_.f64_pipe) {
    bool all = true;
    for (int k = 0; k < n; ++k)
      all &= fx_storage_ok(probs[k].omega, probs[k].cs, probs[k].rho_lbm);
    if (all) store_ = kStoreFX;
  }
  sb_ = store_bytes(store_);
  ob_ = (store_ == kStoreF64 || store_ == kStoreFX) ? 8 : 4;
  prob_.assign(probs, probs + n);
  ch_.resize(n);
  size_t total = 0;
  auto align = [](size_t b) { return (b + 255) & ~size_t(255); };
  std::vector<size_t> off_type(n), off_f(n);
  for (int k = 0; k < n; ++k) {
    const tlbm_problem& p = probs[k];
    int q = 0;
    if (!std::strcmp(p.lattice, "D3Q15")) q = 15;
    if (!std::strcmp(p.lattice, "D3Q19")) q = 19;
    if (!q)
      return Status::err(TLBM_ERR_UNSUPPORTED, "channel " + std::to_string(k) +
                                                   ": ensembles take D3Q15 or D3Q19 lattices");
    if (p.nx < 1 || p.ny < 1 || p.nz < 1 || p.nz > 65535)
      return Status::err(TLBM_ERR_INVALID_ARGUMENT, "channel " + std::to_string(k) + ": bad size");
    const int64_t cells = static_cast<int64_t>(p.nx) * p.ny * p.nz;
    if (cells >= (int64_t(1) << 31))
      return Status::err(TLBM_ERR_UNSUPPORTED, "channel too large");
    for (int64_t g = 0; g < cells; ++g) {
      const int32_t t = nd_types[k][g];
      if (!(t == 0 || t == 1 || t == 2 || t == 3))
        return Status::err(TLBM_ERR_OUT_OF_RANGE,
                           "channel " + std::to_string(k) + ": node type " + std::to_string(t) +
                               " (ensembles take types 0-3)");
    }
    EnsembleChannel& c = ch_[k];
    std::memset(&c, 0, sizeof(c));
    c.q = q;
    DevProblem& pb = c.step[0].pb;
    pb.nx = p.nx;
    pb.ny = p.ny;
    pb.nz = p.nz;
    pb.nxy = p.nx * p.ny;
    pb.n = cells;
    pb.omega = p.omega;
    pb.nu = (1.0 / p.omega - 0.5) / 3.0;
    pb.cs = p.cs;
    pb.u_bc = p.u_lbm;
    pb.rho_bc = p.rho_lbm;
    pb.dynamics = p.dynamics;
    pb.has_type5 = 0;
    fill_derived(pb, q, sb_);
    // FP64 channels collide fluid nodes in exact fixed point, as a single-lattice handle does
    pb.fx = ((store_ == kStoreF64 || store_ == kStoreFX) && !opt_.f64_pipe &&
             fx_collision_ok(p.omega, p.cs))
                ? 1
                : 0;
    if (pb.fx) fx::fill_consts(pb.fxk, p.omega, p.cs, pb.nu);
    c.div_nx = make_fast_div(static_cast<uint32_t>(p.nx));
    off_type[k] = total;
    total += align(static_cast<size_t>(cells));
    off_f[k] = total;
    total += 2 * align(static_cast<size_t>(cells) * q * sb_);
    cells_ += cells;
  }
  TLBM_CUDA(cudaSetDevice(opt_.device));
  TLBM_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  TLBM_CUDA(cudaMalloc(&arena_, total));
  char* base = static_cast<char*>(arena_);
  int max_nb = 1;
  for (int k = 0; k < n; ++k) {
    EnsembleChannel& c = ch_[k];
    const size_t cells = static_cast<size_t>(c.pb().n);
    std::vector<uint8_t> types(cells);
    for (size_t g = 0; g < cells; ++g) types[g] = static_cast<uint8_t>(nd_types[k][g]);
    uint8_t* dt = reinterpret_cast<uint8_t*>(base + off_type[k]);
    TLBM_CUDA(cudaMemcpy(dt, types.data(), cells, cudaMemcpyHostToDevice));
    c.step[0].pb.nd_type = dt;
    void* f0 = base + off_f[k];
    void* f1 = base + off_f[k] + align(cells * c.q * sb_);
    c.step[0].src = f0;
    c.step[0].dst = f1;
    c.step[1] = c.step[0];
    c.step[1].src = f1;
    c.step[1].dst = f0;
    max_nb = std::max(max_nb, mass_blocks(c.pb()));
  }
  TLBM_CUDA(cudaMalloc(&d_partial_, max_nb * sizeof(double)));
  TLBM_CUDA(cudaMalloc(&d_mass_, sizeof(double)));
  TLBM_TRY(reset_populations());
  return set_tiles(opt_.block_x > 0 ? opt_.block_x : 128, opt_.block_y > 0 ? opt_.block_y : 1, 1);
}

Status Ensemble::reset_populations() {
  Launch l;
  l.stream = stream_;
  for (size_t k = 0; k < ch_.size(); ++k) {
    for (int b = 0; b < 2; ++b) {
      TLBM_CUDA(launch_init_uniform(ch_[k].q, store_, ch_[k].pb(), ch_[k].f(b),
                                    prob_[k].rho_lbm, l));
      ++launches_;
    }
  }
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  last_src_ = -1;
  return Status::ok();
}

Status Ensemble::set_tiles(int bx, int by, int cpt) {
  if (bx < 32 || bx % 32 != 0 || by < 1 || bx * by > 256 || cpt < 1 || cpt > 8)
    return Status::err(TLBM_ERR_INVALID_ARGUMENT,
                       "tiles: bx a multiple of 32, bx*by <= 256, 1 <= cells_per_thread <= 8");
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  // a tile: bx*by threads x cpt consecutive cells of one z-plane
  const int cells = bx * by * cpt;
  std::vector<EnsembleTile> tiles;
  for (size_t k = 0; k < ch_.size(); ++k) {
    const EnsembleChannel& c = ch_[k];
    const int per_plane = (c.pb().nxy + cells - 1) / cells;
    if (static_cast<int64_t>(tiles.size()) + static_cast<int64_t>(per_plane) * c.pb().nz >
        (int64_t(1) << 30))
      return Status::err(TLBM_ERR_UNSUPPORTED, "too many tiles");
    for (int z = 0; z < c.pb().nz; ++z)
      for (int t = 0; t < per_plane; ++t)
        tiles.push_back({static_cast<int>(k), z, t * cells, 0});
  }
  n_tiles_ = static_cast<int>(tiles.size());
  cudaFree(d_ch_);
  cudaFree(d_tiles_);
  d_ch_ = nullptr;
  d_tiles_ = nullptr;
  TLBM_CUDA(cudaMalloc(&d_ch_, ch_.size() * sizeof(EnsembleChannel)));
  TLBM_CUDA(cudaMemcpy(d_ch_, ch_.data(), ch_.size() * sizeof(EnsembleChannel),
                       cudaMemcpyHostToDevice));
  TLBM_CUDA(cudaMalloc(&d_tiles_, tiles.size() * sizeof(EnsembleTile)));
  TLBM_CUDA(cudaMemcpy(d_tiles_, tiles.data(), tiles.size() * sizeof(EnsembleTile),
                       cudaMemcpyHostToDevice));
  int sms = 0;
  TLBM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opt_.device));
  const int per_sm = ensemble_resident_blocks(store_, bx * by);
  grid_ = std::max(1, std::min(n_tiles_, sms * per_sm));
  bx_ = bx;
  by_ = by;
  cpt_ = cpt;
  drop_graphs();
  return Status::ok();
}

Status Ensemble::enqueue(int is_even) {
  EnsembleArgs a{};
  a.channels = d_ch_;
  a.tiles = d_tiles_;
  a.n_tiles = n_tiles_;
  a.src = is_even ? 0 : 1;
  a.cells_per_thread = cpt_;
  TLBM_CUDA(launch_ensemble_step(store_, a, bx_ * by_, grid_, stream_));
  ++launches_;
  last_src_ = a.src;
  return Status::ok();
}

Status Ensemble::run(int first_ts, int nsteps) {
  TraceRange trace("tlbm_ensemble_run");
  TLBM_CUDA(cudaSetDevice(opt_.device));
  int ts = first_ts;
  if (nsteps >= 2) {
    const int parity = ts % 2;
    if (!graph_[parity]) {
      cudaGraph_t g = nullptr;
      TLBM_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
      const int64_t l0 = launches_;
      Status s = enqueue(parity);
      if (s.good()) s = enqueue(1 - parity);
      cudaError_t e = cudaStreamEndCapture(stream_, &g);
      launches_ = l0;
      if (!s.good()) {
        if (g) cudaGraphDestroy(g);
        return s;
      }
      TLBM_CUDA(e);
      e = cudaGraphInstantiate(&graph_[parity], g, 0);
      cudaGraphDestroy(g);
      TLBM_CUDA(e);
    }
    while (nsteps >= 2) {
      TLBM_CUDA(cudaGraphLaunch(graph_[parity], stream_));
      launches_ += 2;
      ts += 2;
      nsteps -= 2;
    }
    last_src_ = parity;  // the last step had is_even = 1 - parity
  }
  if (nsteps == 1) TLBM_TRY(enqueue(ts % 2));
  return Status::ok();
}

Status Ensemble::time_steps(int first_ts, int nsteps, float* ms) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  cudaEvent_t e0, e1;
  TLBM_CUDA(cudaEventCreate(&e0));
  TLBM_CUDA(cudaEventCreate(&e1));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  TLBM_CUDA(cudaEventRecord(e0, stream_));
  Status s = run(first_ts, nsteps);
  if (s.good()) s = check(cudaEventRecord(e1, stream_), "cudaEventRecord");
  if (s.good()) s = check(cudaEventSynchronize(e1), "ensemble steps");
  if (s.good()) s = check(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return s;
}

// Tile shapes tried by the autotuner: (threads, 1, cells per thread); a tile is threads x cells
// per thread consecutive cells of a z-plane.
static const int kCandidates[][3] = {{64, 1, 1},  {128, 1, 1}, {256, 1, 1}, {64, 1, 2},
                                     {128, 1, 2}, {256, 1, 2}, {128, 1, 4}, {256, 1, 4}};

Status Ensemble::autotune(int steps, int* bx, int* by, int* cpt) {
  TraceRange trace("tlbm_ensemble_autotune");
  if (steps < 2) steps = 2;
  float best = 0.0f;
  int pick = -1;
  for (int c = 0; c < static_cast<int>(sizeof(kCandidates) / sizeof(kCandidates[0])); ++c) {
    TLBM_TRY(set_tiles(kCandidates[c][0], kCandidates[c][1], kCandidates[c][2]));
    TLBM_TRY(run(0, 2));
    float ms = 0.0f;
    TLBM_TRY(time_steps(2, steps, &ms));
    if (pick < 0 || ms < best) {
      best = ms;
      pick = c;
    }
  }
  TLBM_TRY(set_tiles(kCandidates[pick][0], kCandidates[pick][1], kCandidates[pick][2]));
  TLBM_TRY(reset_populations());  // tuning steps are discarded: back to the initial state
  if (bx) *bx = bx_;
  if (by) *by = by_;
  if (cpt) *cpt = cpt_;
  return Status::ok();
}

Status Ensemble::copy_macros(int channel, void* ux, void* uy, void* uz, void* rho) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (channel < 0 || channel >= static_cast<int>(ch_.size()))
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "no such channel");
  if (last_src_ < 0) return Status::err(TLBM_ERR_INVALID_ARGUMENT, "no time step taken yet");
  const EnsembleChannel& c = ch_[channel];
  const size_t bytes = static_cast<size_t>(c.pb().n) * ob_;
  void* d = nullptr;
  TLBM_CUDA(cudaMallocAsync(&d, 4 * bytes, stream_));
  char* db = static_cast<char*>(d);
  void* outs[4] = {db, db + bytes, db + 2 * bytes, db + 3 * bytes};
  Launch l;
  l.stream = stream_;
  cudaError_t e = launch_macros_fast(c.q, store_, c.pb(), c.f(last_src_), outs, l);
  ++launches_;
  void* host[4] = {ux, uy, uz, rho};
  for (int k = 0; k < 4 && e == cudaSuccess; ++k)
    if (host[k]) e = cudaMemcpyAsync(host[k], outs[k], bytes, cudaMemcpyDeviceToHost, stream_);
  cudaFreeAsync(d, stream_);
  TLBM_CUDA(e);
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

Status Ensemble::mass(int channel, double* out) {
  TLBM_CUDA(cudaSetDevice(opt_.device));
  if (channel < 0 || channel >= static_cast<int>(ch_.size()))
    return Status::err(TLBM_ERR_INVALID_ARGUMENT, "no such channel");
  const EnsembleChannel& c = ch_[channel];
  const int buf = last_src_ >= 0 ? 1 - last_src_ : 1;
  Launch l;
  l.stream = stream_;
  TLBM_CUDA(launch_mass(c.q, store_, c.pb(), c.f(buf), d_partial_, mass_blocks(c.pb()), d_mass_, l));
  launches_ += 2;
  TLBM_CUDA(cudaMemcpyAsync(out, d_mass_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
  TLBM_CUDA(cudaStreamSynchronize(stream_));
  return Status::ok();
}

}  // namespace tlbm
