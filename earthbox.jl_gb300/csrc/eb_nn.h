// eb_nn.h -- launchers of the tensor-core kernels used by the learned preconditioner.
#pragma once
#include "eb_nn_gemm.cuh"

namespace nn {
// D = A . B^T on the tensor cores (see eb_nn_gemm.cuh); splits > 1 splits K across CTAs
// and writes one FP32 partial per split (epilogue mode 0).
template <class ALoad>
cudaError_t launch_gemm(const ALoad& A, const MatLoader& B, int64_t M, int32_t N, int64_t K, const Epilogue& ep,
                        int32_t splits, cudaStream_t s, int32_t* err);
}  // namespace nn
