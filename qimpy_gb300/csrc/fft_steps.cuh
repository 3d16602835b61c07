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
#pragma once

#include "codelets.cuh"
#include "qgb_common.cuh"

namespace qgb {

// One codelet applied in place to p[j * stride], j < R, with an optional
// twiddle multiply tw[j * tw_stride] on the outputs (table holds exp(+i...),
// conjugated when SIGN < 0).
template <typename T, int S, int R>
__device__ __forceinline__ void codelet_inplace(cplx_t<T>* __restrict__ p, int stride,
                                                const cplx_t<T>* __restrict__ tw, int tw_stride) {
  T re[R], im[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const cplx_t<T> v = p[j * stride];
    re[j] = v.x;
    im[j] = v.y;
  }
  Codelet<R, S>::run(re, im);
  if (tw != nullptr) {
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const cplx_t<T> w = tw[j * tw_stride];
      const T wy = (S > 0) ? w.y : -w.y;
      const T xr = re[j] * w.x - im[j] * wy;
      const T xi = re[j] * wy + im[j] * w.x;
      re[j] = xr;
      im[j] = xi;
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) p[j * stride] = mk<T>(re[j], im[j]);
}

// Geometry of one pass: item `it` in [0, nbatch * nsub) is (batch = it % nbatch,
// sub = it / nbatch); its codelet elements sit at
//   base + boff(batch) + sub * sstride + j * estride,
// boff(batch) = (bmap ? bmap[batch] : batch) * bstride.
template <typename T> struct Pass {
  cplx_t<T>* base;
  const int* bmap;
  int nbatch, bstride, nsub, sstride, estride;
  const cplx_t<T>* tw;  // nullptr: no twiddles
  int tw_sub, tw_el;
};

template <typename T, int S, int R>
__device__ __noinline__ void run_pass_R(const Pass<T> ps) {
  const int nitems = ps.nbatch * ps.nsub;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / ps.nbatch;
    const int b = it - sub * ps.nbatch;
    const int boff = (ps.bmap ? ps.bmap[b] : b) * ps.bstride;
    codelet_inplace<T, S, R>(ps.base + boff + sub * ps.sstride, ps.estride,
                             ps.tw ? ps.tw + sub * ps.tw_sub : nullptr, ps.tw_el);
  }
}

template <typename T, int S>
__device__ void run_pass(int R, const Pass<T>& ps) {
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

// Inverse transform (natural -> permuted) of nbatch pencils, element stride es.
// Ends with __syncthreads().
template <typename T>
__device__ void fft_inverse(cplx_t<T>* base, const int* bmap, int nbatch, int bstride, int es,
                            int L1, int L2, const cplx_t<T>* W) {
  if (L2 > 1) {
    run_pass<T, +1>(L2, Pass<T>{base, bmap, nbatch, bstride, L1, es, L1 * es, W, L2, 1});
    __syncthreads();
  }
  if (L1 > 1) {
    run_pass<T, +1>(L1, Pass<T>{base, bmap, nbatch, bstride, L2, L1 * es, es, nullptr, 0, 0});
    __syncthreads();
  }
}

// Forward transform (permuted -> natural) of nbatch pencils.  Ends with __syncthreads().
template <typename T>
__device__ void fft_forward(cplx_t<T>* base, const int* bmap, int nbatch, int bstride, int es,
                            int L1, int L2, const cplx_t<T>* W) {
  if (L1 > 1) {
    run_pass<T, -1>(L1, Pass<T>{base, bmap, nbatch, bstride, L2, L1 * es, es,
                                (L2 > 1) ? W : nullptr, 1, L2});
    __syncthreads();
  }
  if (L2 > 1) {
    run_pass<T, -1>(L2, Pass<T>{base, bmap, nbatch, bstride, L1, es, L1 * es, nullptr, 0, 0});
    __syncthreads();
  }
}

}  // namespace qgb
