// FP64 Hermitian eigensolver for the Davidson subspace problems, batched over
// k-points.
//
// Each Davidson iteration diagonalises one small dense Hermitian matrix per
// k-point (qimpy/dft/electrons/_davidson.py:164-168 and the eighg of
// qimpy/math/_linalg.py:143-183).  torch.linalg.eigh on CUDA loops over the
// batch with one syevd per matrix, each with its own host synchronisation.
// This entry point hands the whole batch to cuSOLVER's batched syev in one
// call on the caller's stream, in FP64 on the GPU.
//
// Layout: A is [nk][n][n] row-major Hermitian, which read column-major is
// conj(A).  cuSOLVER therefore returns the eigenvectors of conj(A) in columns:
// on exit A[k][j][c] = conj(v_j[c]) for eigenvector v_j of the input, i.e. the
// row-major array holds V^H.  Eigenvalues are equal for A and conj(A).
#include <cusolverDn.h>

#include <unordered_map>
#include <vector>

#include "qgb_common.cuh"

namespace qgb {

static const char* cusolver_name(cusolverStatus_t s) {
  switch (s) {
    case CUSOLVER_STATUS_SUCCESS: return "success";
    case CUSOLVER_STATUS_NOT_INITIALIZED: return "not initialized";
    case CUSOLVER_STATUS_ALLOC_FAILED: return "alloc failed";
    case CUSOLVER_STATUS_INVALID_VALUE: return "invalid value";
    case CUSOLVER_STATUS_ARCH_MISMATCH: return "arch mismatch";
    case CUSOLVER_STATUS_EXECUTION_FAILED: return "execution failed";
    case CUSOLVER_STATUS_INTERNAL_ERROR: return "internal error";
    case CUSOLVER_STATUS_NOT_SUPPORTED: return "not supported";
    default: return "unknown";
  }
}

#define QGB_CUSOLVER(expr)                                                           \
  do {                                                                               \
    cusolverStatus_t s_ = (expr);                                                    \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                               \
      return ::qgb::fail(QGB_ERR_CUSOLVER, "%s: %s", #expr, cusolver_name(s_));      \
  } while (0)

struct Solver {
  cusolverDnHandle_t h = nullptr;
  cusolverDnParams_t p = nullptr;
};

// One cuSOLVER handle per (host thread, device): the serving loop advances
// requests from several threads, each on its own stream, and a handle's stream
// binding is per handle.  Handles live until the process exits.
static int get_solver(Solver* out) {
  static thread_local std::unordered_map<int, Solver> solvers;
  int dev = 0;
  QGB_CUDA_CHECK(cudaGetDevice(&dev));
  auto it = solvers.find(dev);
  if (it == solvers.end()) {
    Solver s;
    QGB_CUSOLVER(cusolverDnCreate(&s.h));
    QGB_CUSOLVER(cusolverDnCreateParams(&s.p));
    it = solvers.emplace(dev, s).first;
  }
  *out = it->second;
  return QGB_OK;
}

// Few large matrices (the Gamma-only cells' expanded subspaces, n in the
// hundreds) go through the divide-and-conquer syevd one matrix at a time; many
// small ones through the batched syev.
static bool per_matrix(int64_t nk, int64_t n) { return n >= 128 && nk <= 2; }

static int query(const Solver& s, int64_t nk, int64_t n, size_t* dev_bytes, size_t* host_bytes) {
  if (per_matrix(nk, n)) {
    QGB_CUSOLVER(cusolverDnXsyevd_bufferSize(s.h, s.p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                             CUDA_C_64F, nullptr, n, CUDA_R_64F, nullptr, CUDA_C_64F, dev_bytes,
                                             host_bytes));
    return QGB_OK;
  }
  QGB_CUSOLVER(cusolverDnXsyevBatched_bufferSize(s.h, s.p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                                 CUDA_C_64F, nullptr, n, CUDA_R_64F, nullptr, CUDA_C_64F,
                                                 dev_bytes, host_bytes, nk));
  return QGB_OK;
}

}  // namespace qgb

using namespace qgb;

extern "C" {

size_t qgb_subspace_eigh_workspace_bytes(int64_t nk, int64_t n) {
  if (nk < 1 || n < 1) return 0;
  Solver s;
  size_t dev_bytes = 0, host_bytes = 0;
  if (get_solver(&s) != QGB_OK || query(s, nk, n, &dev_bytes, &host_bytes) != QGB_OK) return 0;
  return dev_bytes + 256;
}

int qgb_subspace_eigh(void* A, double* W, int* info, int64_t nk, int64_t n, void* workspace,
                      size_t workspace_bytes, void* stream) {
  if (nk < 0 || n < 0) return fail(QGB_ERR_INVALID, "bad subspace_eigh sizes nk=%lld n=%lld", (long long)nk,
                                   (long long)n);
  if (nk == 0 || n == 0) return QGB_OK;
  if (!A || !W || !info) return fail(QGB_ERR_INVALID, "NULL pointer in subspace_eigh");
  Solver s;
  int rc = get_solver(&s);
  if (rc) return rc;
  size_t dev_bytes = 0, host_bytes = 0;
  rc = query(s, nk, n, &dev_bytes, &host_bytes);
  if (rc) return rc;
  if (dev_bytes > 0 && (!workspace || workspace_bytes < dev_bytes))
    return fail(QGB_ERR_WORKSPACE, "subspace_eigh workspace %zu < %zu", workspace_bytes, dev_bytes);
  // Host workspace is used by the host side of the call only; one per thread.
  static thread_local std::vector<unsigned char> host;
  if (host.size() < host_bytes + 1) host.resize(host_bytes + 1);
  QGB_CUSOLVER(cusolverDnSetStream(s.h, (cudaStream_t)stream));
  if (per_matrix(nk, n)) {
    for (int64_t k = 0; k < nk; ++k)
      QGB_CUSOLVER(cusolverDnXsyevd(s.h, s.p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_64F,
                                    static_cast<double2*>(A) + k * n * n, n, CUDA_R_64F, W + k * n, CUDA_C_64F,
                                    workspace, dev_bytes, host.data(), host_bytes, info + k));
    return QGB_OK;
  }
  QGB_CUSOLVER(cusolverDnXsyevBatched(s.h, s.p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_64F, A,
                                      n, CUDA_R_64F, W, CUDA_C_64F, workspace, dev_bytes, host.data(), host_bytes,
                                      info, nk));
  return QGB_OK;
}

}  // extern "C"
