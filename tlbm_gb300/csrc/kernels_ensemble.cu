// kernels_ensemble.cu -- one persistent launch steps a batch of independent channels.
//
// Channels differ in size, lattice (D3Q15 or D3Q19), Reynolds number and geometry.  Each
// z-plane of each channel is cut into tiles of (threads x cells_per_thread) consecutive cells
// in x-fastest order, so a tile's loads and stores are contiguous and its threads idle only in
// the last tile of a plane, whatever the channel's width.  The tiles of all channels form one
// list, and a grid of (SM count x resident blocks) CTAs walks it with a fixed stride, so the
// schedule is static and every cell is computed by the same cell_step as the single-lattice
// kernel (identical results).  The host replays the step launches from a CUDA graph; the
// autotuner picks (threads, cells_per_thread).
#include "ensemble.h"
#include "step_fast.cuh"

namespace tlbm {
namespace {

__device__ __forceinline__ int fast_div(int n, FastDiv d) {
  return static_cast<int>((__umulhi(static_cast<uint32_t>(n), d.m) + static_cast<uint32_t>(n)) >>
                          d.l);
}

template <int K>
__global__ void __launch_bounds__(256) k_ensemble_step(EnsembleArgs a) {
  constexpr bool kFx = K == kStoreF64 || K == kStoreFX;  // fluid nodes in fixed point
  for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
    const EnsembleTile tile = a.tiles[t];
    const EnsembleChannel& ch = a.channels[tile.channel];
    const StepArgs& s = ch.step[a.src];
    const int nxy = s.pb.nxy;
    for (int k = 0; k < a.cells_per_thread; ++k) {
      const int r = tile.r0 + k * blockDim.x + threadIdx.x;
      if (r >= nxy) break;
      const int y = fast_div(r, ch.div_nx);
      const int x = r - y * s.pb.nx;
      if (ch.q == 19) {
        if (s.pb.cs > 0)
          cell_step<Lattice<19>, K, fast::kClosureSmag, false, true, kFx>(s, x, y, tile.z);
        else
          cell_step<Lattice<19>, K, fast::kClosureNone, false, true, kFx>(s, x, y, tile.z);
      } else {
        if (s.pb.cs > 0)
          cell_step<Lattice<15>, K, fast::kClosureSmag, false, true, kFx>(s, x, y, tile.z);
        else
          cell_step<Lattice<15>, K, fast::kClosureNone, false, true, kFx>(s, x, y, tile.z);
      }
    }
  }
}

template <int K>
int resident_blocks(int threads) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ensemble_step<K>, threads, 0) !=
      cudaSuccess)
    return 1;
  return b > 0 ? b : 1;
}

}  // namespace

int ensemble_resident_blocks(int store, int threads) {
  switch (store) {
    case kStoreF64: return resident_blocks<kStoreF64>(threads);
    case kStoreFX: return resident_blocks<kStoreFX>(threads);
    case kStoreF32: return resident_blocks<kStoreF32>(threads);
    case kStoreBF16: return resident_blocks<kStoreBF16>(threads);
    case kStoreF16: return resident_blocks<kStoreF16>(threads);
    default: return 1;
  }
}

cudaError_t launch_ensemble_step(int store, const EnsembleArgs& a, int threads, int grid,
                                 cudaStream_t s) {
  const dim3 block(threads, 1, 1);
  switch (store) {
    case kStoreF64: k_ensemble_step<kStoreF64><<<grid, block, 0, s>>>(a); break;
    case kStoreFX: k_ensemble_step<kStoreFX><<<grid, block, 0, s>>>(a); break;
    case kStoreF32: k_ensemble_step<kStoreF32><<<grid, block, 0, s>>>(a); break;
    case kStoreBF16: k_ensemble_step<kStoreBF16><<<grid, block, 0, s>>>(a); break;
    case kStoreF16: k_ensemble_step<kStoreF16><<<grid, block, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tlbm
