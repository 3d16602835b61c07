// Band-space complex products on the CUDA cores: the overlap (Gram) products
// of Wavefunction.dot and the projections <beta|psi>, the band rotations of
// Wavefunction.matmul and the back-projection beta (D proj), and the
// block-diagonal D apply.
//
// Replaces (qimpy/dft/electrons/_wavefunction_dot.py:18-107, 137-191;
// _wavefunction.py:106-123; qimpy/dft/electrons/_hamiltonian.py:22-24):
//   gram    out(i, j) = sum_g conj(A[i][g]) B[j][g]     (long g, small i/j)
//   rotate  out[j][g] (+)= sum_i W(i, j) X[i][g]         (short i, long g)
//   dapply  Dp[b][a pa + r] = sum_c D[a][r][c] proj[b][a pa + c]
// Arrays are batched over k-points with explicit strides.  GB300's FP64 rate
// (about 1 TFLOP/s) bounds the FP64 products, so they are register-tiled DFMA
// loops with shared-memory staging; the FP32 forms use the same tiling.
// Every product is deterministic: split-K partial tiles are summed by a
// second kernel in a fixed order (no atomics), so repeated calls, and calls
// from different host threads, give identical bits.
#include <algorithm>
#include <type_traits>

#include "bandgemm.cuh"

namespace qgb {
namespace bg {

constexpr int kSms = 152;  // GB300 streaming multiprocessors

template <typename T>
__device__ __forceinline__ void cmac_conj(cplx_t<T>& acc, const cplx_t<T>& a, const cplx_t<T>& b) {
  // acc += conj(a) * b
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(-a.y, b.x, acc.y);
}
template <typename T>
__device__ __forceinline__ void cmac(cplx_t<T>& acc, const cplx_t<T>& a, const cplx_t<T>& b) {
  // acc += a * b
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

// ---------------------------------------------------------------------------
// Gram / projection: out(i, j) = sum_g conj(A[i][g]) B[j][g]
// ---------------------------------------------------------------------------
//
// CTA: BI (i) x BJ (j) outputs of one k and one g range (split-K), 256
// threads as TI x TJ (TI TJ = 256), each 4 x 4 outputs: 64 x 64 in general,
// 128 x 32 or 32 x 128 when one side has at most 32 rows (the projections of
// a 32-band block), so that no thread multiplies padding.  g is staged 16 at a
// time: A and B tiles are loaded along g (coalesced rows) and stored
// transposed, [g][i] and [g][j], so each thread reads 4 consecutive i (or j)
// per g.
constexpr int GK = 16;   // g per stage
constexpr int GPAD = 1;  // row padding (elements) of the transposed tiles

struct GramArgs {
  const void* A;
  const void* B;
  long long a_batch, b_batch;  // element strides between k-points
  int lda, ldb;                // element stride between rows i (A) / j (B)
  int M, N, K;                 // i, j, g extents
  int splits, g_per_split;     // split-K (g_per_split a multiple of GK)
  void* partial;               // splits > 1: [split][k][M][N] of cplx_t<T>
  void* out;                   // splits == 1: OutT at out + k*out_batch + i*oi + j*oj
  long long out_batch;
  int oi, oj;
  const double* weight;        // optional per-g weight w_g (shared by all k): sum_g w_g conj(A) B
  int real_out;                // keep only the real part (imaginary part written as 0)
};

template <typename T, typename OutT, int TI>
__global__ void __launch_bounds__(256) k_gram(const GramArgs a) {
  using C2 = cplx_t<T>;
  using O2 = cplx_t<OutT>;
  constexpr int TJ = 256 / TI, BI = 4 * TI, BJ = 4 * TJ;
  __shared__ C2 As[GK][BI + GPAD];
  __shared__ C2 Bs[GK][BJ + GPAD];
  const int tid = threadIdx.x, tx = tid % TJ, ty = tid / TJ;
  const int i0 = blockIdx.x * BI, j0 = blockIdx.y * BJ;
  const int k = blockIdx.z / a.splits, split = blockIdx.z % a.splits;
  const int g_begin = split * a.g_per_split;
  const int g_end = min(a.K, g_begin + a.g_per_split);
  const C2* A = static_cast<const C2*>(a.A) + k * a.a_batch;
  const C2* B = static_cast<const C2*>(a.B) + k * a.b_batch;
  C2 acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = mk<T>(T(0), T(0));
  for (int g0 = g_begin; g0 < g_end; g0 += GK) {
#pragma unroll
    for (int r = 0; r < BI * GK / 256; ++r) {
      const int e = tid + 256 * r, row = e >> 4, gg = e & 15, g = g0 + gg;
      As[gg][row] = (g < g_end && i0 + row < a.M) ? A[static_cast<long long>(i0 + row) * a.lda + g]
                                                  : mk<T>(T(0), T(0));
    }
#pragma unroll
    for (int r = 0; r < BJ * GK / 256; ++r) {
      const int e = tid + 256 * r, row = e >> 4, gg = e & 15, g = g0 + gg;
      const bool g_ok = g < g_end;
      C2 bv = (g_ok && j0 + row < a.N) ? B[static_cast<long long>(j0 + row) * a.ldb + g] : mk<T>(T(0), T(0));
      if (a.weight != nullptr && g_ok) {
        const T w = static_cast<T>(a.weight[g]);
        bv.x *= w;
        bv.y *= w;
      }
      Bs[gg][row] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int gg = 0; gg < GK; ++gg) {
      C2 av[4], bv[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) av[p] = As[gg][ty * 4 + p];
#pragma unroll
      for (int q = 0; q < 4; ++q) bv[q] = Bs[gg][tx * 4 + q];
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cmac_conj<T>(acc[p][q], av[p], bv[q]);
    }
    __syncthreads();
  }
  if (a.splits == 1) {
    O2* out = static_cast<O2*>(a.out) + k * a.out_batch;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int i = i0 + ty * 4 + p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + tx * 4 + q;
        if (i < a.M && j < a.N)
          out[static_cast<long long>(i) * a.oi + static_cast<long long>(j) * a.oj] =
              mk<OutT>(static_cast<OutT>(acc[p][q].x), a.real_out ? OutT(0) : static_cast<OutT>(acc[p][q].y));
      }
    }
  } else {
    const int nk = gridDim.z / a.splits;
    C2* part = static_cast<C2*>(a.partial) + (static_cast<long long>(split) * nk + k) * a.M * a.N;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int i = i0 + ty * 4 + p;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int j = j0 + tx * 4 + q;
        if (i < a.M && j < a.N) part[static_cast<long long>(i) * a.N + j] = acc[p][q];
      }
    }
  }
}

// Sum of the split-K partials in split order (accumulated in OutT's precision
// or better), written with the caller's output strides.
template <typename T, typename OutT>
__global__ void k_gram_reduce(const cplx_t<T>* __restrict__ partial, int splits, int nk, int M, int N,
                              cplx_t<OutT>* __restrict__ out, long long out_batch, int oi, int oj, int real_out) {
  using Acc = typename std::conditional<sizeof(T) >= sizeof(OutT), T, OutT>::type;
  const long long per_k = static_cast<long long>(M) * N;
  const long long total = per_k * nk;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int k = static_cast<int>(e / per_k);
    const long long r = e - k * per_k;
    const int i = static_cast<int>(r / N), j = static_cast<int>(r - static_cast<long long>(i) * N);
    Acc re = 0, im = 0;
    for (int s = 0; s < splits; ++s) {
      const cplx_t<T> v = partial[(static_cast<long long>(s) * nk + k) * per_k + r];
      re += static_cast<Acc>(v.x);
      im += static_cast<Acc>(v.y);
    }
    out[k * out_batch + static_cast<long long>(i) * oi + static_cast<long long>(j) * oj] =
        mk<OutT>(static_cast<OutT>(re), real_out ? OutT(0) : static_cast<OutT>(im));
  }
}

struct GramPlan {
  int shape;  // threads along i: 16 (64 x 64 tiles), 32 (128 x 32) or 8 (32 x 128)
  int ti, tj, splits, g_per_split;
  size_t partial_bytes;
};
static GramPlan gram_plan(int nk, int M, int N, int K, size_t elem) {
  GramPlan p;
  // Skinny tiles for skinny outputs; otherwise the tile shape that pads the
  // output least (M = 256 projectors x N = 160 bands: 128 x 32 tiles cover it
  // exactly, 64 x 64 tiles would compute 20% more), the square 64 x 64 tile
  // on ties, as its loads feed the most multiply-adds.
  auto padded = [M, N](int shape) {
    const long long bi = 4 * shape, bj = 4 * (256 / shape);
    return ((M + bi - 1) / bi) * bi * ((N + bj - 1) / bj) * bj;
  };
  p.shape = (N <= 32 && M > 32) ? 32 : ((M <= 32 && N > 32) ? 8 : 16);
  for (const int shape : {16, 32, 8})
    if (padded(shape) < padded(p.shape)) p.shape = shape;
  const int bi = 4 * p.shape, bj = 4 * (256 / p.shape);
  p.ti = (M + bi - 1) / bi;
  p.tj = (N + bj - 1) / bj;
  const int tiles = p.ti * p.tj * nk;
  const int kchunks = (K + GK - 1) / GK;
  // Enough CTAs for two waves over the SMs, with at least 8 stages of g each.
  int splits = std::max(1, std::min((2 * kSms + tiles - 1) / tiles, (kchunks + 7) / 8));
  const int chunks_per_split = (kchunks + splits - 1) / splits;
  p.g_per_split = chunks_per_split * GK;
  p.splits = (K + p.g_per_split - 1) / p.g_per_split;
  if (p.splits < 1) p.splits = 1;
  p.partial_bytes = p.splits > 1 ? static_cast<size_t>(p.splits) * nk * M * N * elem : 0;
  return p;
}

// ---------------------------------------------------------------------------
// Rotation / back-projection: out[j][g] (+)= sum_i W(i, j) X[i][g]
// ---------------------------------------------------------------------------
//
// CTA: TJ*8 (j) x 128 (g) outputs of one k, 256 threads as 32 (g) x 8 (j);
// each thread TJ j-values x 4 consecutive g.  i is staged 16 at a time: the
// X tile [16][128] along g (coalesced), the W tile [16][TJ*8].
constexpr int RG = 128;
constexpr int RK = 16;

struct RotArgs {
  const void* X;
  const void* W;
  void* out;
  long long x_batch, w_batch, out_batch;  // element strides between k-points
  int ldx, ldo;                           // element stride between rows i (X) / j (out)
  int wi, wj;                             // W(i, j) = W[i*wi + j*wj]
  int Kin, Nout, G;                       // i, j, g extents
  int accumulate;
};

template <typename T, int TJ>
__global__ void __launch_bounds__(256) k_rotate(const RotArgs a) {
  using C2 = cplx_t<T>;
  constexpr int BJ = TJ * 8;
  __shared__ C2 Xs[RK][RG];
  __shared__ C2 Ws[RK][BJ];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int g0 = blockIdx.x * RG, j0 = blockIdx.y * BJ, k = blockIdx.z;
  const C2* X = static_cast<const C2*>(a.X) + k * a.x_batch;
  const C2* W = static_cast<const C2*>(a.W) + k * a.w_batch;
  C2 acc[TJ][4];
#pragma unroll
  for (int p = 0; p < TJ; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = mk<T>(T(0), T(0));
  for (int i0 = 0; i0 < a.Kin; i0 += RK) {
#pragma unroll
    for (int r = 0; r < RK * RG / 256; ++r) {
      const int e = tid + 256 * r, ii = e / RG, gg = e % RG;
      const int i = i0 + ii, g = g0 + gg;
      Xs[ii][gg] = (i < a.Kin && g < a.G) ? X[static_cast<long long>(i) * a.ldx + g] : mk<T>(T(0), T(0));
    }
    for (int e = tid; e < RK * BJ; e += 256) {
      const int ii = e / BJ, jj = e % BJ, i = i0 + ii, j = j0 + jj;
      Ws[ii][jj] = (i < a.Kin && j < a.Nout) ? W[static_cast<long long>(i) * a.wi + static_cast<long long>(j) * a.wj]
                                             : mk<T>(T(0), T(0));
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < RK; ++ii) {
      C2 xv[4], wv[TJ];
#pragma unroll
      for (int q = 0; q < 4; ++q) xv[q] = Xs[ii][tx * 4 + q];
#pragma unroll
      for (int p = 0; p < TJ; ++p) wv[p] = Ws[ii][ty * TJ + p];
#pragma unroll
      for (int p = 0; p < TJ; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cmac<T>(acc[p][q], wv[p], xv[q]);
    }
    __syncthreads();
  }
  C2* out = static_cast<C2*>(a.out) + k * a.out_batch;
#pragma unroll
  for (int p = 0; p < TJ; ++p) {
    const int j = j0 + ty * TJ + p;
    if (j >= a.Nout) continue;
    C2* row = out + static_cast<long long>(j) * a.ldo;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int g = g0 + tx * 4 + q;
      if (g < a.G) {
        C2 v = acc[p][q];
        if (a.accumulate) {
          const C2 o = row[g];
          v.x += o.x;
          v.y += o.y;
        }
        row[g] = v;
      }
    }
  }
}

// Dp[k][b][a*pa + r] = sum_c D[a][r][c] proj[k][b][a*pa + c]  (one thread per output)
template <typename T>
__global__ void k_dapply(const cplx_t<T>* __restrict__ proj, const cplx_t<T>* __restrict__ D, int n_atoms, int pa,
                         int nb, int nk, cplx_t<T>* __restrict__ Dp) {
  const int P = n_atoms * pa;
  const long long total = static_cast<long long>(nk) * nb * P;
  for (long long e = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; e < total;
       e += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long kb = e / P;
    const int p = static_cast<int>(e - kb * P), atom = p / pa, r = p - atom * pa;
    const cplx_t<T>* x = proj + kb * P + atom * pa;
    const cplx_t<T>* d = D + (static_cast<long long>(atom) * pa + r) * pa;
    cplx_t<T> acc = mk<T>(T(0), T(0));
    for (int c = 0; c < pa; ++c) cmac<T>(acc, d[c], x[c]);
    Dp[e] = acc;
  }
}

}  // namespace bg

using namespace bg;

// Workspace (bytes) of a Gram product: the split-K partial tiles.
size_t gram_workspace_bytes(int dtype, int nk, int M, int N, int K) {
  if (nk < 1 || M < 1 || N < 1 || K < 1) return 0;
  return gram_plan(nk, M, N, K, elem_bytes(dtype)).partial_bytes;
}

template <typename T, typename OutT>
static void launch_gram(int shape, dim3 grid, const GramArgs& g, cudaStream_t st) {
  if (shape == 32)
    k_gram<T, OutT, 32><<<grid, 256, 0, st>>>(g);
  else if (shape == 8)
    k_gram<T, OutT, 8><<<grid, 256, 0, st>>>(g);
  else
    k_gram<T, OutT, 16><<<grid, 256, 0, st>>>(g);
}

// out(i, j) of type out_dtype (complex) = sum_g conj(A(i, g)) B(j, g), per k.
int gram(int dtype, int out_dtype, const void* A, long long a_batch, int lda, const void* B, long long b_batch,
         int ldb, int nk, int M, int N, int K, void* out, long long out_batch, int oi, int oj, void* ws,
         size_t ws_bytes, cudaStream_t st, const double* weight, bool real_out) {
  if (nk < 0 || M < 0 || N < 0 || K < 0) return fail(QGB_ERR_INVALID, "negative gram extent");
  if (nk == 0 || M == 0 || N == 0) return QGB_OK;
  if (!A || !B || !out) return fail(QGB_ERR_INVALID, "NULL pointer in gram");
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (out_dtype != QGB_F64 && out_dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown out dtype %d", out_dtype);
  if (dtype == QGB_F64 && out_dtype == QGB_F32) return fail(QGB_ERR_UNSUPPORTED, "FP64 gram to FP32 output");
  if (K == 0) return fail(QGB_ERR_INVALID, "gram over an empty basis");
  const GramPlan p = gram_plan(nk, M, N, K, elem_bytes(dtype));
  if (p.splits > 1 && (!ws || ws_bytes < p.partial_bytes))
    return fail(QGB_ERR_WORKSPACE, "gram workspace %zu B < %zu B", ws_bytes, p.partial_bytes);
  GramArgs g{A, B, a_batch, b_batch, lda, ldb, M, N, K, p.splits, p.g_per_split, ws, out, out_batch, oi, oj,
             weight, real_out ? 1 : 0};
  const dim3 grid(p.ti, p.tj, nk * p.splits);
  if (dtype == QGB_F64) {
    launch_gram<double, double>(p.shape, grid, g, st);
  } else if (out_dtype == QGB_F64) {
    launch_gram<float, double>(p.shape, grid, g, st);
  } else {
    launch_gram<float, float>(p.shape, grid, g, st);
  }
  QGB_LAUNCH_CHECK("k_gram");
  if (p.splits > 1) {
    const long long total = static_cast<long long>(nk) * M * N;
    const unsigned blocks = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 8 * kSms));
    if (dtype == QGB_F64) {
      k_gram_reduce<double, double><<<blocks, 256, 0, st>>>(static_cast<const double2*>(ws), p.splits, nk, M, N,
                                                            static_cast<double2*>(out), out_batch, oi, oj, g.real_out);
    } else if (out_dtype == QGB_F64) {
      k_gram_reduce<float, double><<<blocks, 256, 0, st>>>(static_cast<const float2*>(ws), p.splits, nk, M, N,
                                                           static_cast<double2*>(out), out_batch, oi, oj, g.real_out);
    } else {
      k_gram_reduce<float, float><<<blocks, 256, 0, st>>>(static_cast<const float2*>(ws), p.splits, nk, M, N,
                                                          static_cast<float2*>(out), out_batch, oi, oj, g.real_out);
    }
    QGB_LAUNCH_CHECK("k_gram_reduce");
  }
  return QGB_OK;
}

// out[k][j][g] (+)= sum_i W(i, j) X[k][i][g] with W(i, j) = W[k*w_batch + i*wi + j*wj].
int rotate(int dtype, const void* X, long long x_batch, int ldx, const void* W, long long w_batch, int wi, int wj,
           int nk, int Kin, int Nout, int G, void* out, long long out_batch, int ldo, bool accumulate,
           cudaStream_t st) {
  if (nk < 0 || Kin < 0 || Nout < 0 || G < 0) return fail(QGB_ERR_INVALID, "negative rotate extent");
  if (nk == 0 || Nout == 0 || G == 0) return QGB_OK;
  if (!out || (Kin > 0 && (!X || !W))) return fail(QGB_ERR_INVALID, "NULL pointer in rotate");
  RotArgs r{X, W, out, x_batch, w_batch, out_batch, ldx, ldo, wi, wj, Kin, Nout, G, accumulate ? 1 : 0};
  if (dtype == QGB_F64) {
    constexpr int TJ = 4;
    const dim3 grid((G + RG - 1) / RG, (Nout + TJ * 8 - 1) / (TJ * 8), nk);
    k_rotate<double, TJ><<<grid, 256, 0, st>>>(r);
  } else if (dtype == QGB_F32) {
    constexpr int TJ = 8;
    const dim3 grid((G + RG - 1) / RG, (Nout + TJ * 8 - 1) / (TJ * 8), nk);
    k_rotate<float, TJ><<<grid, 256, 0, st>>>(r);
  } else {
    return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  }
  QGB_LAUNCH_CHECK("k_rotate");
  return QGB_OK;
}

int dapply(int dtype, const void* proj, const void* D, int n_atoms, int pa, int nb, int nk, void* Dp,
           cudaStream_t st) {
  const long long total = static_cast<long long>(nk) * nb * n_atoms * pa;
  if (total == 0) return QGB_OK;
  const unsigned blocks = static_cast<unsigned>(std::min<long long>((total + 255) / 256, 8 * kSms));
  if (dtype == QGB_F64)
    k_dapply<double><<<blocks, 256, 0, st>>>(static_cast<const double2*>(proj), static_cast<const double2*>(D),
                                             n_atoms, pa, nb, nk, static_cast<double2*>(Dp));
  else
    k_dapply<float><<<blocks, 256, 0, st>>>(static_cast<const float2*>(proj), static_cast<const float2*>(D), n_atoms,
                                            pa, nb, nk, static_cast<float2*>(Dp));
  QGB_LAUNCH_CHECK("k_dapply");
  return QGB_OK;
}

}  // namespace qgb
