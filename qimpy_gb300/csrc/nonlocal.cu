// Nonlocal pseudopotential terms <beta|psi>, D, |beta> on the CUDA cores.
//
// Replaces Wavefunction.proj = beta ^ C (qimpy/dft/electrons/_wavefunction.py:106-123,
// _wavefunction_dot.py:18-107) and beta @ (D_all @ proj)
// (qimpy/dft/electrons/_hamiltonian.py:22-24, _wavefunction_dot.py:137-191):
//   projT[k][b][p] = sum_g conj(beta[k][p][g]) C[k][b][g]   (gram, split-K)
//   Dp[k][b]       = D_a projT[k][b]_a per atom block a      (block-diagonal D)
//   out[k][b][g]  += sum_p beta[k][p][g] Dp[k][b][p]         (rotate, accumulate)
// with the band-space product kernels of bandgemm.cu (hand-written, FP64 or
// FP32; the mixed form's tensor-core chain is tc_gemm.cu).
#include "bandgemm.cuh"

namespace qgb {

size_t project_workspace_bytes(int dtype, int nk, int P, int nb, int n_tot) {
  return gram_workspace_bytes(dtype, nk, P, nb, n_tot);
}

int project(int dtype, const void* beta, const void* C, void* projT, int nk, int P, int nb, int n_tot, void* ws,
            size_t ws_bytes, cudaStream_t st) {
  if (nk < 0 || P < 0 || nb < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad project sizes");
  if (nk == 0 || P == 0 || nb == 0) return QGB_OK;
  if (!beta || !C || !projT) return fail(QGB_ERR_INVALID, "NULL pointer in project");
  // i = projector p (rows of beta), j = band b (rows of C); projT[k][b][p]: oi = 1, oj = P.
  return gram(dtype, dtype, beta, static_cast<long long>(P) * n_tot, n_tot, C, static_cast<long long>(nb) * n_tot,
              n_tot, nk, P, nb, n_tot, projT, static_cast<long long>(nb) * P, 1, P, ws, ws_bytes, st);
}

int apply_nonlocal(int dtype, const void* beta, const void* D, int n_atoms, int pa, const void* projT, void* out,
                   int nk, int nb, int n_tot, void* work, cudaStream_t st) {
  const int P = n_atoms * pa;
  if (nk < 0 || n_atoms < 0 || pa < 0 || nb < 0 || n_tot < 1)
    return fail(QGB_ERR_INVALID, "bad apply_nonlocal sizes");
  if (nk == 0 || P == 0 || nb == 0) return QGB_OK;
  if (!beta || !D || !projT || !out || !work) return fail(QGB_ERR_INVALID, "NULL pointer in apply_nonlocal");
  int rc = dapply(dtype, projT, D, n_atoms, pa, nb, nk, work, st);
  if (rc) return rc;
  // out[k][b][g] += sum_p beta[k][p][g] Dp[k][b][p]: i = p, j = b, W(p, b) = Dp[b*P + p].
  return rotate(dtype, beta, static_cast<long long>(P) * n_tot, n_tot, work, static_cast<long long>(nb) * P, 1, P,
                nk, P, nb, n_tot, out, static_cast<long long>(nb) * n_tot, n_tot, true, st);
}

}  // namespace qgb
