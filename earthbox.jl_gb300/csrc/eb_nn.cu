// eb_nn.cu -- tensor-core building blocks of the learned preconditioner: the tcgen05 GEMM
// launcher (eb_nn_gemm.cuh) and host-array entry points that run one GEMM or one
// convolution on temporary device buffers (used by the tests to check the tensor-core
// path against an FP32 product of the same BF16 operands).
#include "eb_internal.h"
#include "eb_nn.h"

#include <vector>

namespace nn {

bool valid_bn(int32_t bn) { return bn >= 16 && bn <= 256 && bn % 16 == 0; }

int32_t pick_bn(int32_t n) {
  if (n <= 256) return (n + 15) / 16 * 16;
  return 128;
}

template <class ALoad>
cudaError_t launch_gemm(const ALoad& A, const MatLoader& B, int64_t M, int32_t N, int64_t K, const Epilogue& ep,
                        int32_t splits, cudaStream_t s, int32_t* err) {
  const int32_t bn = pick_bn(N);
  if (!valid_bn(bn) || M <= 0 || N <= 0 || K <= 0 || splits < 1) return cudaErrorInvalidValue;
  const int64_t nchunks = (K + kChunkK - 1) / kChunkK;
  const int32_t kc_per = (int32_t)((nchunks + splits - 1) / splits);
  const size_t smem = gemm_smem_bytes(bn);
  cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16<ALoad>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((M + kTileM - 1) / kTileM), (unsigned)((N + bn - 1) / bn), (unsigned)splits);
  k_gemm_bf16<ALoad><<<grid, kGemmThreads, smem, s>>>(A, B, M, N, bn, K, kc_per, ep, err);
  return cudaGetLastError();
}
template cudaError_t launch_gemm<MatLoader>(const MatLoader&, const MatLoader&, int64_t, int32_t, int64_t,
                                            const Epilogue&, int32_t, cudaStream_t, int32_t*);
template cudaError_t launch_gemm<ConvLoader>(const ConvLoader&, const MatLoader&, int64_t, int32_t, int64_t,
                                             const Epilogue&, int32_t, cudaStream_t, int32_t*);

namespace {
// device copies of host arrays, freed on scope exit
struct Scratch {
  std::vector<void*> p;
  ~Scratch() { for (void* q : p) cudaFree(q); }
  template <class T>
  T* get(size_t n, const T* host = nullptr) {
    void* d = nullptr;
    if (cudaMalloc(&d, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
    p.push_back(d);
    if (host && cudaMemcpy(d, host, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    if (!host) cudaMemset(d, 0, n * sizeof(T));
    return static_cast<T*>(d);
  }
};
int finish(int32_t* d_err, cudaError_t e) {
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return EB_CUDA_ERROR;
  int32_t h = 0;
  if (cudaMemcpy(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return EB_CUDA_ERROR;
  return h ? EB_CUDA_ERROR : EB_OK;
}
}  // namespace

}  // namespace nn

using namespace nn;

extern "C" int eb_nn_gemm_bf16(int64_t M, int32_t N, int64_t K, const uint16_t* A, const uint16_t* B, float* D,
                               int32_t splits) {
  if (M <= 0 || N <= 0 || K <= 0 || K % 8 != 0 || !A || !B || !D || splits < 1) return EB_BAD_INPUT;
  Scratch s;
  const uint16_t* dA = s.get<uint16_t>((size_t)M * K, A);
  const uint16_t* dB = s.get<uint16_t>((size_t)N * K, B);
  float* dD = s.get<float>((size_t)splits * M * N);
  int32_t* derr = s.get<int32_t>(1);
  if (!dA || !dB || !dD || !derr) return EB_CUDA_ERROR;
  const MatLoader la{dA, K, M, K}, lb{dB, K, N, K};
  const Epilogue ep{dD, nullptr, nullptr, N, 0, 0};
  int rc = finish(derr, launch_gemm(la, lb, M, N, K, ep, splits, 0, derr));
  if (rc) return rc;
  std::vector<float> part((size_t)splits * M * N);
  if (cudaMemcpy(part.data(), dD, part.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return EB_CUDA_ERROR;
  for (size_t k = 0; k < (size_t)M * N; ++k) {
    float t = 0.f;
    for (int32_t q = 0; q < splits; ++q) t += part[(size_t)q * M * N + k];
    D[k] = t;
  }
  return EB_OK;
}

extern "C" int eb_nn_conv2d_bf16(int32_t B, int32_t H, int32_t W, int32_t C, int32_t Cout, int32_t taps,
                                 int32_t flip, const uint16_t* x, const uint16_t* w, const float* bias,
                                 int32_t mode, float* y32, uint16_t* y16) {
  if (B <= 0 || H <= 0 || W <= 0 || C <= 0 || C % 8 || Cout <= 0 || (taps != 1 && taps != 9) || !x || !w ||
      mode < 0 || mode > 2 || (mode == 0 && !y32) || (mode > 0 && !y16))
    return EB_BAD_INPUT;
  const int64_t P = (int64_t)B * H * W, K = (int64_t)taps * C;
  Scratch s;
  const uint16_t* dx = s.get<uint16_t>((size_t)P * C, x);
  const uint16_t* dw = s.get<uint16_t>((size_t)Cout * K, w);
  const float* db = bias ? s.get<float>((size_t)Cout, bias) : nullptr;
  float* d32 = mode == 0 ? s.get<float>((size_t)P * Cout) : nullptr;
  uint16_t* d16 = mode > 0 ? s.get<uint16_t>((size_t)P * Cout) : nullptr;
  int32_t* derr = s.get<int32_t>(1);
  if (!dx || !dw || (bias && !db) || (!d32 && !d16) || !derr) return EB_CUDA_ERROR;
  const ConvLoader la{dx, B, H, W, C, taps, flip};
  const MatLoader lb{dw, K, Cout, K};
  const Epilogue ep{d32, d16, db, Cout, 0, mode};
  int rc = finish(derr, launch_gemm(la, lb, P, Cout, K, ep, 1, 0, derr));
  if (rc) return rc;
  cudaError_t e = mode == 0 ? cudaMemcpy(y32, d32, (size_t)P * Cout * 4, cudaMemcpyDeviceToHost)
                            : cudaMemcpy(y16, d16, (size_t)P * Cout * 2, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? EB_OK : EB_CUDA_ERROR;
}
