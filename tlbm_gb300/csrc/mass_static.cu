// mass_static.cu -- the FP64 mass reduction for callers that cannot allocate device memory.
//
// Who needs it: applications that reserve the whole GPU up front for their own memory pool
// (a cudaMalloc issued by a library inside them fails or fragments that pool), and solver
// loops whose policy forbids any allocation once the run has started (allocation can block
// and its latency is unbounded).  tlbm_mass allocates its partial-sum buffer when a handle is
// created; tlbm_mass_static computes the same quantity -- the FP64 sum of every population --
// from a population array and an output the caller owns, with no allocation at all.
//
// Its scratch is g_mass_scratch below: kMassStaticMaxBlocks doubles (512 KiB), a file-scope
// __device__ array that is part of this library's device image, so every GPU that loads the
// library holds it until the process exits.  In host code the name g_mass_scratch is only a
// stand-in for the symbol, not a device address: each call, with the device current, asks the
// runtime for the array's device address (cudaGetSymbolAddress) when its stream is not being
// captured, and keeps it per device for a call made during a capture.  Make the first call on
// a device before any stream capture.
//
// All calls share the array and it keeps the last call's partial sums.  Every call writes each
// partial it later reads, so nothing has to be cleared between calls; calls that overlap on the
// GPU (two streams, or two host threads) race on the array and must be ordered by the caller.
// The sum is not checked: a diverged run yields NaN or Inf in *mass (tlbm_mass returns
// TLBM_ERR_NUMERIC instead), so the caller tests it with isfinite after synchronizing.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/tlbm.h"
#include "kernels.h"
#include "lattice.cuh"
#include "storage.cuh"

namespace tlbm {
namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerThread = 4;
constexpr int kCellsPerBlock = kThreads * kCellsPerThread;
constexpr int kMassStaticMaxBlocks = 65536;  // 512 KiB of doubles
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_mass_scratch[kMassStaticMaxBlocks];

std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

__device__ double block_sum_static(double v) {
  __shared__ double part[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) part[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = lane < kThreads / 32 ? part[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;
}

// block b sums cells [b*kCellsPerBlock, (b+1)*kCellsPerBlock) in a fixed order
template <class L, int K>
__global__ void __launch_bounds__(kThreads) k_mass_static_partial(
    const typename Store<K>::T* __restrict__ f, int64_t n, double* scratch) {
  using S = Store<K>;
  const size_t nn = static_cast<size_t>(n);
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kCellsPerThread; ++k) {
    const int64_t c = static_cast<int64_t>(blockIdx.x) * kCellsPerBlock + k * kThreads + threadIdx.x;
    if (c >= n) break;
    double cell = 0.0;
#pragma unroll
    for (int i = 0; i < L::Q; ++i) {
      if constexpr (S::kShifted)
        cell += static_cast<double>(weight<L, float>(i)) + static_cast<double>(f[i * nn + c]);
      else
        cell += static_cast<double>(f[i * nn + c]);
    }
    acc += cell;
  }
  const double b = block_sum_static(acc);
  if (threadIdx.x == 0) scratch[blockIdx.x] = b;
}

__global__ void __launch_bounds__(kThreads) k_mass_static_final(const double* scratch, int nb,
                                                                double* out) {
  double acc = 0.0;
  for (int k = threadIdx.x; k < nb; k += kThreads) acc += scratch[k];
  const double b = block_sum_static(acc);
  if (threadIdx.x == 0) *out = b;
}

template <class L, int K>
cudaError_t launch_partial(const void* f, int64_t n, int nb, double* scratch, cudaStream_t s) {
  k_mass_static_partial<L, K><<<nb, kThreads, 0, s>>>(
      static_cast<const typename Store<K>::T*>(f), n, scratch);
  return cudaGetLastError();
}

cudaError_t dispatch_partial(int q, int store, const void* f, int64_t n, int nb, double* scratch,
                             cudaStream_t s) {
#define TLBM_MS_CASE(QQ, KK) \
  if (q == QQ && store == KK) return launch_partial<Lattice<QQ>, KK>(f, n, nb, scratch, s);
  TLBM_MS_CASE(15, kStoreF64) TLBM_MS_CASE(15, kStoreF32) TLBM_MS_CASE(15, kStoreBF16)
  TLBM_MS_CASE(15, kStoreF16) TLBM_MS_CASE(19, kStoreF64) TLBM_MS_CASE(19, kStoreF32)
  TLBM_MS_CASE(19, kStoreBF16) TLBM_MS_CASE(19, kStoreF16) TLBM_MS_CASE(27, kStoreF64)
  TLBM_MS_CASE(27, kStoreF32) TLBM_MS_CASE(27, kStoreBF16) TLBM_MS_CASE(27, kStoreF16)
#undef TLBM_MS_CASE
  return cudaErrorInvalidValue;
}

}  // namespace
}  // namespace tlbm

extern "C" tlbm_status tlbm_mass_static(int q, int precision, int64_t n_cells,
                                        const void* populations, double* mass, void* stream) {
  using namespace tlbm;
  if (q != 15 && q != 19 && q != 27) return TLBM_ERR_INVALID_ARGUMENT;
  if (precision < TLBM_PREC_F64 || precision > TLBM_PREC_F16) return TLBM_ERR_INVALID_ARGUMENT;
  if (!populations || !mass || n_cells < 1) return TLBM_ERR_INVALID_ARGUMENT;
  // one partial sum per kCellsPerBlock cells must fit the static scratch array
  const int64_t nb64 = (n_cells + kCellsPerBlock - 1) / kCellsPerBlock;
  if (nb64 > kMassStaticMaxBlocks) return TLBM_ERR_OUT_OF_RANGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TLBM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Outside stream capture the array's address is looked up on every call, so an address kept
  // from before a cudaDeviceReset (or from another context on this device) is never used; a
  // call on a capturing stream uses the address of the last call outside capture.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return TLBM_ERR_CUDA;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_mass_scratch);
      if (e != cudaSuccess || !p) return TLBM_ERR_CUDA;
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  if (!scratch) return TLBM_ERR_CUDA;
  const int store = precision == TLBM_PREC_F64   ? kStoreF64
                    : precision == TLBM_PREC_F32 ? kStoreF32
                    : precision == TLBM_PREC_BF16 ? kStoreBF16
                                                  : kStoreF16;
  const int nb = static_cast<int>(nb64);
  cudaError_t e = dispatch_partial(q, store, populations, n_cells, nb, scratch, s);
  if (e == cudaSuccess) {
    k_mass_static_final<<<1, kThreads, 0, s>>>(scratch, nb, mass);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return TLBM_ERR_CUDA;
  return TLBM_OK;
}
