// In-shared-memory batched 1D FFT passes built from the register codelets.
//
// A length-L transform with L = L1 * L2 is two passes of small DFTs (the
// "four-step" split without the reordering step):
//
//   inverse, natural in -> permuted out (SIGN +1)
//     pass 1: for each n1 < L1: DFT_L2 over x[n1 + L1 n2], times W[n1][k2],
//             stored back at n1 + L1 k2
//     pass 2: for each k2 < L2: DFT_L1 over the block [L1 k2, L1 k2 + L1)
//   forward, permuted in -> natural out (SIGN -1)
//     pass A: for each a < L2: DFT_L1 over the block [L1 a, L1 a + L1),
//             output c times conj(W[c][a])
//     pass B: for each c < L1: DFT_L2 over x[c + L1 a] -> natural index c + L1 d
//
// with W[i][j] = exp(+2 pi i i j / L).  Real-space index r = a + L2 b lives at
// position L1 a + b ("digit-permuted" order); every pass reads and writes the
// same addresses from one thread, so a pass needs no barrier inside it.
//
// All data and twiddles live in the kernel's dynamic shared memory and are
// addressed by element offsets from its base, so every access is a plain
// shared-memory load or store.
#pragma once

#include "codelets.cuh"
#include "qgb_common.cuh"

namespace qgb {

extern __shared__ __align__(16) unsigned char qgb_smem[];

template <typename T> __device__ __forceinline__ cplx_t<T>* smem_c() {
  return reinterpret_cast<cplx_t<T>*>(qgb_smem);
}

// One codelet applied in place to smem[off + j * stride], j < R, with an
// optional twiddle multiply by smem[tw + j * tw_stride] (tw < 0: none) on the
// outputs; the table holds exp(+i...), conjugated when SIGN < 0.
template <typename T, int S, int R>
__device__ __forceinline__ void codelet_inplace(int off, int stride, int tw, int tw_stride, int lim,
                                                int tw_lim) {
  cplx_t<T>* sm = smem_c<T>();
  T re[R], im[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (!QGB_OK_IDX(off + j * stride, lim, 10 + R)) return;
    const cplx_t<T> v = sm[off + j * stride];
    re[j] = v.x;
    im[j] = v.y;
  }
  Codelet<R, S>::run(re, im);
  if (tw >= 0) {
#pragma unroll
    for (int j = 1; j < R; ++j) {
      if (!QGB_OK_IDX(tw + j * tw_stride, tw_lim, 40 + R)) return;
      const cplx_t<T> w = sm[tw + j * tw_stride];
      const T wy = (S > 0) ? w.y : -w.y;
      const T xr = re[j] * w.x - im[j] * wy;
      const T xi = re[j] * wy + im[j] * w.x;
      re[j] = xr;
      im[j] = xi;
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) sm[off + j * stride] = mk<T>(re[j], im[j]);
}

// Geometry of one pass: item `it` in [0, nbatch * nsub) is (batch = it % nbatch,
// sub = it / nbatch); its codelet elements sit at shared offsets
//   base + boff(batch) + sub * sstride + j * estride,
// boff(batch) = (bmap ? bmap[batch] : batch) * bstride, bmap in global memory.
struct Pass {
  const int* bmap;
  int base, nbatch, bstride, nsub, sstride, estride;
  int tw, tw_sub, tw_el;  // tw < 0: no twiddles
  int lim, tw_lim;        // bounds of the data and twiddle regions (debug checks)
};

template <typename T, int S, int R>
__device__ __forceinline__ void run_pass_R(const Pass ps) {
  const int nitems = ps.nbatch * ps.nsub;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / ps.nbatch;
    const int b = it - sub * ps.nbatch;
    const int boff = (ps.bmap != nullptr ? __ldg(ps.bmap + b) : b) * ps.bstride;
    codelet_inplace<T, S, R>(ps.base + boff + sub * ps.sstride, ps.estride,
                             ps.tw >= 0 ? ps.tw + sub * ps.tw_sub : -1, ps.tw_el, ps.lim, ps.tw_lim);
  }
}

template <typename T, int S>
__device__ __forceinline__ void run_pass(int R, const Pass ps) {
  switch (R) {
    case 2: run_pass_R<T, S, 2>(ps); break;
    case 3: run_pass_R<T, S, 3>(ps); break;
    case 4: run_pass_R<T, S, 4>(ps); break;
    case 5: run_pass_R<T, S, 5>(ps); break;
    case 6: run_pass_R<T, S, 6>(ps); break;
    case 7: run_pass_R<T, S, 7>(ps); break;
    case 8: run_pass_R<T, S, 8>(ps); break;
    case 9: run_pass_R<T, S, 9>(ps); break;
    case 10: run_pass_R<T, S, 10>(ps); break;
    case 12: run_pass_R<T, S, 12>(ps); break;
    case 14: run_pass_R<T, S, 14>(ps); break;
    case 15: run_pass_R<T, S, 15>(ps); break;
    case 16: run_pass_R<T, S, 16>(ps); break;
    default: break;  // R == 1: identity
  }
}

// Inverse transform (natural -> permuted) of nbatch pencils starting at shared
// offset `base`, element stride es; twiddles at shared offset W; `lim` bounds
// the data region.  Ends with __syncthreads().
template <typename T>
__device__ __forceinline__ void fft_inverse(int base, const int* bmap, int nbatch, int bstride, int es,
                                            int L1, int L2, int W, int lim) {
  if (L2 > 1) {
    run_pass<T, +1>(L2, Pass{bmap, base, nbatch, bstride, L1, es, L1 * es, W, L2, 1, lim, W + L1 * L2});
    __syncthreads();
  }
  if (L1 > 1) {
    run_pass<T, +1>(L1, Pass{bmap, base, nbatch, bstride, L2, L1 * es, es, -1, 0, 0, lim, 0});
    __syncthreads();
  }
}

// Forward transform (permuted -> natural) of nbatch pencils.  Ends with __syncthreads().
template <typename T>
__device__ __forceinline__ void fft_forward(int base, const int* bmap, int nbatch, int bstride, int es,
                                            int L1, int L2, int W, int lim) {
  if (L1 > 1) {
    run_pass<T, -1>(L1, Pass{bmap, base, nbatch, bstride, L2, L1 * es, es, (L2 > 1) ? W : -1, 1, L2, lim,
                             W + L1 * L2});
    __syncthreads();
  }
  if (L2 > 1) {
    run_pass<T, -1>(L2, Pass{bmap, base, nbatch, bstride, L1, es, L1 * es, -1, 0, 0, lim, 0});
    __syncthreads();
  }
}

}  // namespace qgb
