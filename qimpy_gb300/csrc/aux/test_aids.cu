// Test aids of the tensor-core path (include/qimpy_gb300_aux.h): the raw
// split-BF16x3 GEMM, checked against an exact product of the same splits, and
// a launch whose pipeline wait runs out, checked for its error word and a
// clean return.  They call internal functions of libqimpy_gb300.so.
#include "../qgb_common.cuh"

namespace qgb {
int tc_gemm_test(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo, int M, int N, int K,
                 int lda, int ldb, float* D, int* err, void* ws, size_t ws_bytes, cudaStream_t st);
int tc_wait_timeout_test(const void* ab, float* ws, int* err, unsigned long long timeout_ns, cudaStream_t st);
}  // namespace qgb

extern "C" int qgb_tc_gemm_bf16x3(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo, int M,
                                  int N, int K, int lda, int ldb, float* D, int* dev_error, void* workspace,
                                  size_t workspace_bytes, void* stream) {
  return qgb::tc_gemm_test(a_hi, a_lo, b_hi, b_lo, M, N, K, lda, ldb, D, dev_error, workspace, workspace_bytes,
                           static_cast<cudaStream_t>(stream));
}

extern "C" int qgb_tc_wait_timeout_test(const void* operands, float* workspace, int* dev_error,
                                        unsigned long long timeout_ns, void* stream) {
  return qgb::tc_wait_timeout_test(operands, workspace, dev_error, timeout_ns, static_cast<cudaStream_t>(stream));
}
