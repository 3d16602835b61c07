// Nonlocal pseudopotential terms <beta|psi>, D, |beta> as complex GEMMs.
//
// Replaces Wavefunction.proj = beta ^ C (qimpy/dft/electrons/_wavefunction.py:106-123,
// _wavefunction_dot.py:18-107) and beta @ (D_all @ proj)
// (qimpy/dft/electrons/_hamiltonian.py:22-24, _wavefunction_dot.py:137-191).
// Row-major [k][rows][n_tot] arrays are column-major (n_tot x rows) matrices, so
//   projT (P x nb)   = beta^H C            (ZGEMM C,N over the basis)
//   DpT  (P x nb)    = D_a projT_a per atom block a (strided-batched, block-diagonal D)
//   out  (n_tot x nb) += beta DpT          (ZGEMM N,N)
// These are plain library GEMMs (cuBLAS), batched over k.
#include <cublas_v2.h>

#include <mutex>
#include <unordered_map>

#include "qgb_common.cuh"

namespace qgb {

static const char* cublas_name(cublasStatus_t s) {
  switch (s) {
    case CUBLAS_STATUS_SUCCESS: return "success";
    case CUBLAS_STATUS_NOT_INITIALIZED: return "not initialized";
    case CUBLAS_STATUS_ALLOC_FAILED: return "alloc failed";
    case CUBLAS_STATUS_INVALID_VALUE: return "invalid value";
    case CUBLAS_STATUS_ARCH_MISMATCH: return "arch mismatch";
    case CUBLAS_STATUS_EXECUTION_FAILED: return "execution failed";
    case CUBLAS_STATUS_INTERNAL_ERROR: return "internal error";
    case CUBLAS_STATUS_NOT_SUPPORTED: return "not supported";
    default: return "unknown";
  }
}

#define QGB_CUBLAS(expr)                                                             \
  do {                                                                               \
    cublasStatus_t s_ = (expr);                                                      \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                 \
      return ::qgb::fail(QGB_ERR_CUBLAS, "%s: %s", #expr, cublas_name(s_));          \
  } while (0)

// One cuBLAS handle per (host thread, device), created on the first nonlocal
// call of that thread.  A handle binds one stream at a time: threads sharing a
// handle would race between cublasSetStream and the GEMM launch, putting one
// thread's GEMM on another thread's stream.
static int get_handle(cublasHandle_t* h) {
  static thread_local std::unordered_map<int, cublasHandle_t> handles;
  int dev = 0;
  QGB_CUDA_CHECK(cudaGetDevice(&dev));
  auto it = handles.find(dev);
  if (it == handles.end()) {
    cublasHandle_t nh;
    QGB_CUBLAS(cublasCreate(&nh));
    it = handles.emplace(dev, nh).first;
  }
  *h = it->second;
  return QGB_OK;
}

int project(int dtype, const void* beta, const void* C, void* projT, int nk, int P, int nb,
            int n_tot, cudaStream_t st) {
  if (nk < 0 || P < 0 || nb < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad project sizes");
  if (nk == 0 || P == 0 || nb == 0) return QGB_OK;
  if (!beta || !C || !projT) return fail(QGB_ERR_INVALID, "NULL pointer in project");
  cublasHandle_t h;
  int rc = get_handle(&h);
  if (rc) return rc;
  QGB_CUBLAS(cublasSetStream(h, st));
  const long long sA = (long long)P * n_tot, sB = (long long)nb * n_tot, sC = (long long)nb * P;
  if (dtype == QGB_F64) {
    const cuDoubleComplex one{1, 0}, zero{0, 0};
    QGB_CUBLAS(cublasZgemmStridedBatched(h, CUBLAS_OP_C, CUBLAS_OP_N, P, nb, n_tot, &one,
                                         (const cuDoubleComplex*)beta, n_tot, sA,
                                         (const cuDoubleComplex*)C, n_tot, sB, &zero,
                                         (cuDoubleComplex*)projT, P, sC, nk));
  } else {
    const cuComplex one{1, 0}, zero{0, 0};
    QGB_CUBLAS(cublasCgemmStridedBatched(h, CUBLAS_OP_C, CUBLAS_OP_N, P, nb, n_tot, &one,
                                         (const cuComplex*)beta, n_tot, sA, (const cuComplex*)C,
                                         n_tot, sB, &zero, (cuComplex*)projT, P, sC, nk));
  }
  return QGB_OK;
}

int apply_nonlocal(int dtype, const void* beta, const void* D, int n_atoms, int pa,
                   const void* projT, void* out, int nk, int nb, int n_tot, void* work,
                   cudaStream_t st) {
  const int P = n_atoms * pa;
  if (nk < 0 || n_atoms < 0 || pa < 0 || nb < 0 || n_tot < 1)
    return fail(QGB_ERR_INVALID, "bad apply_nonlocal sizes");
  if (nk == 0 || P == 0 || nb == 0) return QGB_OK;
  if (!beta || !D || !projT || !out || !work) return fail(QGB_ERR_INVALID, "NULL pointer in apply_nonlocal");
  cublasHandle_t h;
  int rc = get_handle(&h);
  if (rc) return rc;
  QGB_CUBLAS(cublasSetStream(h, st));
  const size_t eb = elem_bytes(dtype);
  for (int k = 0; k < nk; ++k) {
    const char* pk = static_cast<const char*>(projT) + (size_t)k * nb * P * eb;
    char* wk = static_cast<char*>(work) + (size_t)k * nb * P * eb;
    if (dtype == QGB_F64) {
      const cuDoubleComplex one{1, 0}, zero{0, 0};
      QGB_CUBLAS(cublasZgemmStridedBatched(h, CUBLAS_OP_T, CUBLAS_OP_N, pa, nb, pa, &one,
                                           (const cuDoubleComplex*)D, pa, (long long)pa * pa,
                                           (const cuDoubleComplex*)pk, P, pa, &zero,
                                           (cuDoubleComplex*)wk, P, pa, n_atoms));
    } else {
      const cuComplex one{1, 0}, zero{0, 0};
      QGB_CUBLAS(cublasCgemmStridedBatched(h, CUBLAS_OP_T, CUBLAS_OP_N, pa, nb, pa, &one,
                                           (const cuComplex*)D, pa, (long long)pa * pa,
                                           (const cuComplex*)pk, P, pa, &zero, (cuComplex*)wk,
                                           P, pa, n_atoms));
    }
  }
  const long long sA = (long long)P * n_tot, sB = (long long)nb * P, sC = (long long)nb * n_tot;
  if (dtype == QGB_F64) {
    const cuDoubleComplex one{1, 0};
    QGB_CUBLAS(cublasZgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, n_tot, nb, P, &one,
                                         (const cuDoubleComplex*)beta, n_tot, sA,
                                         (const cuDoubleComplex*)work, P, sB, &one,
                                         (cuDoubleComplex*)out, n_tot, sC, nk));
  } else {
    const cuComplex one{1, 0};
    QGB_CUBLAS(cublasCgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_N, n_tot, nb, P, &one,
                                         (const cuComplex*)beta, n_tot, sA, (const cuComplex*)work,
                                         P, sB, &one, (cuComplex*)out, n_tot, sC, nk));
  }
  return QGB_OK;
}

}  // namespace qgb
