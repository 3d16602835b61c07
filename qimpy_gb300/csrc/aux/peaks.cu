// FMA-pipe throughput probe: the FP64 / FP32 CUDA-core roofline denominators
// (the measured-peaks file records only HBM copy and bf16 tensor rates).
#include "../qgb_common.cuh"

namespace qgb {

template <typename T>
__global__ void k_fma_burn(int iters, T seed, T* out) {
  T a0 = seed + T(threadIdx.x), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
  T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
  const T m = T(0.999999), c = T(1e-7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      a0 = a0 * m + c; a1 = a1 * m + c; a2 = a2 * m + c; a3 = a3 * m + c;
      a4 = a4 * m + c; a5 = a5 * m + c; a6 = a6 * m + c; a7 = a7 * m + c;
    }
  }
  const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == T(-12345.678)) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace qgb

extern "C" int qgb_fma_burn(int dtype, int blocks, int threads, int iters, void* out, void* stream) {
  using namespace qgb;
  if (blocks < 1 || threads < 32 || iters < 1 || !out) return fail(QGB_ERR_INVALID, "bad fma_burn arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == QGB_F64)
    k_fma_burn<double><<<blocks, threads, 0, st>>>(iters, 1.0, static_cast<double*>(out));
  else
    k_fma_burn<float><<<blocks, threads, 0, st>>>(iters, 1.0f, static_cast<float*>(out));
  QGB_LAUNCH_CHECK("k_fma_burn");
  return QGB_OK;
}
