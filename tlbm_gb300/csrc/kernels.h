// kernels.h -- host-side launch interface of the CUDA kernels (no CUDA types beyond the stream).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "grid.cuh"

namespace tlbm {

// storage kinds of the population arrays
enum StoreKind : int {
  kStoreF64 = 0,
  kStoreF32 = 1,
  kStoreBF16 = 2,
  kStoreF16 = 3,
  kStoreBF16M = 4,  // BF16 remainders after a per-cell moment shift (storage.cuh)
  kStoreFX = 5,     // FP64 populations held as 64-bit fixed point, Q1.62 (storage.cuh)
};
inline int store_bytes(int k) {
  return (k == kStoreF64 || k == kStoreFX) ? 8 : (k == kStoreF32 ? 4 : 2);
}
// FP64 populations in fast arithmetic: the fluid collision runs in fixed point when its rate
// constants exist (0 < omega < 2, cs >= 0); the populations are held as Q1.62 (kStoreFX) when,
// in addition, the run's density keeps them well inside its range |f| < 2
inline bool fx_collision_ok(double omega, double cs) {
  return omega > 0.0 && omega < 2.0 && cs >= 0.0;
}
inline bool fx_storage_ok(double omega, double cs, double rho) {
  return fx_collision_ok(omega, cs) && rho >= 0.5 && rho < 2.0;
}
// bytes of one population buffer: Q planes, then (moment-shifted kind) a float4 per cell
inline size_t buffer_bytes(int k, int q, int64_t n) {
  const size_t planes = static_cast<size_t>(n) * q * store_bytes(k);
  if (k != kStoreBF16M) return planes;
  return ((planes + 15) / 16) * 16 + static_cast<size_t>(n) * 16;
}

struct StepArgs {
  DevProblem pb;
  const void* src;   // populations after the previous step's collision (pull source)
  void* dst;         // populations after this step's collision
  void* avg[4];      // time-average sums of ux, uy, uz, rho (null when off)
  int time_avg;
  const void* uyq_cur;   // uy of nodes 0..Q-1 in this step   (type-5 quirk, see ref::set_uz)
  const void* uyq_prev;  // uy of nodes 0..Q-1 in the previous step
  const void* closure;   // learned closure (mlp::Closure in HOST memory; the launch copies it
                         // into the kernel's parameters) or null
};

struct Launch {
  int bx = 32, by = 4;
  cudaStream_t stream = nullptr;
};

// ---- reference arithmetic (bit-identical to the CPU reference); R = double or float
cudaError_t launch_step_ref(int q, int rbytes, const StepArgs& a, const Launch& l);
// macroscopic values of every node, recomputed from the step's pull source: out[4] in R
cudaError_t launch_macros_ref(int q, int rbytes, const DevProblem& pb, const void* src,
                              void* const out[4], const Launch& l);
// uy of nodes 0..min(Q,n)-1 (the type-5 quirk) from the pull source
cudaError_t launch_quirk_uy_ref(int q, int rbytes, const DevProblem& pb, const void* src,
                                void* uy_out, const Launch& l);
// calc_force on the post-stream populations (pull of `dst`): out[3] in R
cudaError_t launch_force_ref(int q, int rbytes, const DevProblem& pb, const void* dst,
                             void* const out[3], const Launch& l);

// ---- fast arithmetic (FMA, reassociated); storage kind k, compute in double (f64) or float
cudaError_t launch_step_fast(int q, int store, const StepArgs& a, const Launch& l);
cudaError_t launch_macros_fast(int q, int store, const DevProblem& pb, const void* src,
                               void* const out[4], const Launch& l);
cudaError_t launch_force_fast(int q, int store, const DevProblem& pb, const void* dst,
                              void* const out[3], const Launch& l);

// ---- storage-generic utilities
// f_i = w_i * rho in both buffers (initialize_data_arrays, src/TLBM_Partition.cpp:448-479);
// for the 16-bit kinds the stored value is f_i - w_i.
cudaError_t launch_init_uniform(int q, int store, const DevProblem& pb, void* f, double rho,
                                const Launch& l);
// f = feq(u, rho) per node, placed so that the first pull reads it back at its own node
// (restart initialisation, src/TLBM_Partition.cpp:527-532)
cudaError_t launch_init_equilibrium(int q, int store, const DevProblem& pb, void* f,
                                    const void* const macro[4], int macro_bytes,
                                    const Launch& l);
// populations in the reference's AoS layout; post_stream=1 gathers c - e_i
cudaError_t launch_to_aos(int q, int store, const DevProblem& pb, const void* f, int post_stream,
                          void* out, int out_bytes, const Launch& l);
cudaError_t launch_adjacency(int q, const DevProblem& pb, int32_t* out, const Launch& l);
// deterministic FP64 sum of all populations: partial sums per block into `partial`
// (nblocks doubles), then one block folds them into *out
int mass_blocks(const DevProblem& pb);
cudaError_t launch_mass(int q, int store, const DevProblem& pb, const void* f, double* partial,
                        int nblocks, double* out, const Launch& l);
// out[k] = in[order[k]] for element size `bytes`
// dst[k][0 .. bytes) = src[k][0 .. bytes) for k < count <= 8, by a kernel (every pointer 16-byte
// aligned, bytes a multiple of 16; dst may be page-locked host memory, written through the
// GPU's loads and stores instead of a copy engine); `blocks` CTAs of 256 threads
cudaError_t launch_copy_words(const void* const* src, void* const* dst, int count, size_t bytes,
                              int blocks, const Launch& l);
cudaError_t launch_gather(const void* in, const int32_t* order, int64_t n, int bytes, void* out,
                          const Launch& l);

}  // namespace tlbm
