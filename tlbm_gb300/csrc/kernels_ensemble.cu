// kernels_ensemble.cu -- one persistent launch steps a batch of independent channels.
//
// Channels differ in size, lattice (D3Q15 or D3Q19), Reynolds number and geometry.  Each is
// cut into tiles of (bx * cells_per_thread) x by cells of one z-plane; the tiles of all
// channels form one list.  A grid of (SM count x resident blocks) CTAs walks that list with a
// fixed stride, so the schedule is static and every cell is computed by the same cell_step as
// the single-lattice kernel (identical results).  The host replays the step launches from a
// CUDA graph; the autotuner picks (bx, by, cells_per_thread).
#include "ensemble.h"
#include "step_fast.cuh"

namespace tlbm {
namespace {

template <int K>
__global__ void __launch_bounds__(256) k_ensemble_step(EnsembleArgs a) {
  for (int t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
    const EnsembleChannel& ch = a.channels[a.tile_channel[t]];
    const StepArgs& s = ch.step[a.src];
    const int local = t - ch.tile_begin;
    const int per_plane = ch.tiles_x * ch.tiles_y;
    const int z = local / per_plane;
    const int r = local - z * per_plane;
    const int tyi = r / ch.tiles_x;
    const int txi = r - tyi * ch.tiles_x;
    const int y = tyi * a.by + threadIdx.y;
    if (y >= s.pb.ny) continue;
    for (int k = 0; k < a.cells_per_thread; ++k) {
      const int x = (txi * a.cells_per_thread + k) * a.bx + threadIdx.x;
      if (x >= s.pb.nx) break;
      if (ch.q == 19) {
        if (s.pb.cs > 0)
          cell_step<Lattice<19>, K, fast::kClosureSmag>(s, x, y, z);
        else
          cell_step<Lattice<19>, K, fast::kClosureNone>(s, x, y, z);
      } else {
        if (s.pb.cs > 0)
          cell_step<Lattice<15>, K, fast::kClosureSmag>(s, x, y, z);
        else
          cell_step<Lattice<15>, K, fast::kClosureNone>(s, x, y, z);
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
    case kStoreF32: return resident_blocks<kStoreF32>(threads);
    case kStoreBF16: return resident_blocks<kStoreBF16>(threads);
    case kStoreF16: return resident_blocks<kStoreF16>(threads);
    default: return 1;
  }
}

cudaError_t launch_ensemble_step(int store, const EnsembleArgs& a, int grid, cudaStream_t s) {
  const dim3 block(a.bx, a.by, 1);
  switch (store) {
    case kStoreF64: k_ensemble_step<kStoreF64><<<grid, block, 0, s>>>(a); break;
    case kStoreF32: k_ensemble_step<kStoreF32><<<grid, block, 0, s>>>(a); break;
    case kStoreBF16: k_ensemble_step<kStoreBF16><<<grid, block, 0, s>>>(a); break;
    case kStoreF16: k_ensemble_step<kStoreF16><<<grid, block, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tlbm
