// Internal interface of the band-space products (bandgemm.cu) for the other
// translation units of the library.
#pragma once

#include "qgb_common.cuh"

namespace qgb {

// Bytes of split-K partial sums a gram() call of these extents needs (0: none).
size_t gram_workspace_bytes(int dtype, int nk, int M, int N, int K);

// out(i, j) (complex of out_dtype, at out + k*out_batch + i*oi + j*oj) =
// sum_g [w_g] conj(A[k][i][g]) B[k][j][g]; real_out keeps the real part.
int gram(int dtype, int out_dtype, const void* A, long long a_batch, int lda, const void* B, long long b_batch,
         int ldb, int nk, int M, int N, int K, void* out, long long out_batch, int oi, int oj, void* ws,
         size_t ws_bytes, cudaStream_t st, const double* weight = nullptr, bool real_out = false);

// out[k][j][g] (+)= sum_i W(i, j) X[k][i][g], W(i, j) = W[k*w_batch + i*wi + j*wj].
int rotate(int dtype, const void* X, long long x_batch, int ldx, const void* W, long long w_batch, int wi, int wj,
           int nk, int Kin, int Nout, int G, void* out, long long out_batch, int ldo, bool accumulate,
           cudaStream_t st);

// Dp[k][b][a pa + r] = sum_c D[a][r][c] proj[k][b][a pa + c].
int dapply(int dtype, const void* proj, const void* D, int n_atoms, int pa, int nb, int nk, void* Dp,
           cudaStream_t st);

}  // namespace qgb
