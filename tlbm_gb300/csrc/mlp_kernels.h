// mlp_kernels.h -- launchers of the learned-closure kernels (kernels_mlp.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace tlbm {

size_t mlp_grad_smem();
// mean loss and gradient over samples index[first .. first+count) (index may be null: identity);
// grad holds kParams gradients then the mean loss; partial: nblocks * (kParams + 1) floats
cudaError_t launch_mlp_grad(const float* wbf, const float* feats, const float* targets,
                            const int64_t* index, int64_t first, int64_t count, float* partial,
                            int nblocks, float* grad, cudaStream_t s);
cudaError_t launch_mlp_adam(float* w, float* wbf, float* m, float* v, const float* grad, float lr,
                            int step, cudaStream_t s);
cudaError_t launch_mlp_round(const float* w, float* wbf, cudaStream_t s);
cudaError_t launch_mlp_predict(const float* wbf, const float* feats, int64_t n, float* y,
                               cudaStream_t s);
// fine macroscopic fields (ux, uy, uz, rho) -> 10 box-filtered coarse fields
cudaError_t launch_box_filter(const void* const macro[4], int bytes, int nx, int ny, int nz,
                              int f, void* out, cudaStream_t s);

}  // namespace tlbm
