/*
 * qimpy_gb300 auxiliary library (libqimpy_gb300_aux.so): measurement and test
 * aids, kept out of the product ABI of qimpy_gb300.h.  No counterpart in the
 * reference.  Same conventions: device pointers, asynchronous on `stream`,
 * 0 or a QGB_ERR_* status, message from qgb_last_error().
 */
#ifndef QIMPY_GB300_AUX_H
#define QIMPY_GB300_AUX_H

#include "qimpy_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Measurement aid: `blocks` x `threads` threads each run 8 independent FMA
 * chains of 8*iters steps (64*iters FMAs = 128*iters flops per thread).
 * Timed by the caller; gives the FP64/FP32 CUDA-core peak used as a roofline
 * denominator.  `out` (`blocks` reals of the dtype) receives nothing in practice.
 */
int qgb_fma_burn(int dtype, int blocks, int threads, int iters, void* out, void* stream);

/*
 * Test aid: the tensor-core GEMM alone, D (FP32 [M][N], N <= 64) =
 * A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T with bf16 K-major A [M][lda],
 * B [N][ldb] (lda, ldb multiples of 8).  workspace >= ceil(M/128)*128*64*4 B.
 */
int qgb_tc_gemm_bf16x3(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo, int M, int N,
                       int K, int lda, int ldb, float* D, int* dev_error, void* workspace,
                       size_t workspace_bytes, void* stream);

/*
 * Test aid for the bounded pipeline waits: one tensor-core GEMM CTA whose TMA
 * producer issues no copies, so the MMA issuer's first wait gives up after
 * `timeout_ns` and records error 3 in *dev_error; the kernel then frees its
 * tensor memory and returns with no copy or MMA in flight.  operands: 192 x 64
 * bf16 (24 KB, 16-byte aligned); workspace: 128 x 64 floats.
 */
int qgb_tc_wait_timeout_test(const void* operands, float* workspace, int* dev_error,
                             unsigned long long timeout_ns, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QIMPY_GB300_AUX_H */
