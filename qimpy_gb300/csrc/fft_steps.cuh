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

// ---------------------------------------------------------------------------
// Packed FP32: two pencils per thread
// ---------------------------------------------------------------------------
//
// sm_100+ executes two FP32 additions, multiplications or FMAs in one
// instruction on a register pair (__fadd2_rn / __fmul2_rn / __ffma2_rn, each
// lane rounded as its scalar counterpart).  f32x2 holds one value of two
// independent pencils; the generated codelets run on it unchanged, so a thread
// transforms two adjacent pencils (two complex elements next to each other in
// shared memory, one 16-byte access) for about the instructions of one.
struct f32x2 {
  float2 v;
  __device__ __forceinline__ f32x2() {}
  __device__ __forceinline__ explicit f32x2(float2 x) : v(x) {}
  __device__ __forceinline__ explicit f32x2(double c) : v(make_float2(static_cast<float>(c), static_cast<float>(c))) {}
};
__device__ __forceinline__ f32x2 operator+(f32x2 a, f32x2 b) { return f32x2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ f32x2 operator-(f32x2 a, f32x2 b) {
  return f32x2(__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v));
}
__device__ __forceinline__ f32x2 operator-(f32x2 a) { return f32x2(__fmul2_rn(a.v, make_float2(-1.f, -1.f))); }
__device__ __forceinline__ f32x2 operator*(f32x2 a, f32x2 b) { return f32x2(__fmul2_rn(a.v, b.v)); }

// Elements j of the two pencils at smem[off + j*stride] and smem[off + 1 + j*stride]
// (off even, stride even: 16-byte aligned pairs).
template <int R>
__device__ __forceinline__ bool load_x2(int off, int stride, int lim, f32x2* re, f32x2* im) {
  const float2* sm = smem_c<float>();
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (!QGB_OK_IDX(off + j * stride + 1, lim, 60 + R)) return false;
    const float4 q = *reinterpret_cast<const float4*>(sm + off + j * stride);
    re[j] = f32x2(make_float2(q.x, q.z));
    im[j] = f32x2(make_float2(q.y, q.w));
  }
  return true;
}
template <int R>
__device__ __forceinline__ void store_x2(int off, int stride, const f32x2* re, const f32x2* im) {
  float2* sm = smem_c<float>();
#pragma unroll
  for (int j = 0; j < R; ++j)
    *reinterpret_cast<float4*>(sm + off + j * stride) = make_float4(re[j].v.x, im[j].v.x, re[j].v.y, im[j].v.y);
}

// x * conj?(w) for a twiddle w shared by both lanes (SIGN > 0: w, else conj(w)).
template <int S>
__device__ __forceinline__ void twiddle_x2(f32x2& re, f32x2& im, float2 w) {
  const float wy = (S > 0) ? w.y : -w.y;
  const float2 wx2 = make_float2(w.x, w.x), wy2 = make_float2(wy, wy), nwy2 = make_float2(-wy, -wy);
  const float2 xr = __ffma2_rn(im.v, nwy2, __fmul2_rn(re.v, wx2));
  const float2 xi = __ffma2_rn(im.v, wx2, __fmul2_rn(re.v, wy2));
  re = f32x2(xr);
  im = f32x2(xi);
}

template <int S, int R>
__device__ __forceinline__ void codelet_x2(int off, int stride, int tw, int tw_stride, int lim, int tw_lim) {
  f32x2 re[R], im[R];
  if (!load_x2<R>(off, stride, lim, re, im)) return;
  Codelet<R, S>::run(re, im);
  if (tw >= 0) {
    const float2* sm = smem_c<float>();
#pragma unroll
    for (int j = 1; j < R; ++j) {
      if (!QGB_OK_IDX(tw + j * tw_stride, tw_lim, 80 + R)) return;
      twiddle_x2<S>(re[j], im[j], sm[tw + j * tw_stride]);
    }
  }
  store_x2<R>(off, stride, re, im);
}

// A pass over pairs of adjacent pencils: needs bmap == nullptr, bstride == 1,
// nbatch even and even base, sstride and estride (FP32 data only).
template <int S, int R>
__device__ __forceinline__ void run_pass_x2_R(const Pass ps) {
  const int npairs = ps.nbatch >> 1;
  const int nitems = npairs * ps.nsub;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / npairs;
    const int b = 2 * (it - sub * npairs);
    codelet_x2<S, R>(ps.base + b + sub * ps.sstride, ps.estride, ps.tw >= 0 ? ps.tw + sub * ps.tw_sub : -1,
                     ps.tw_el, ps.lim, ps.tw_lim);
  }
}

template <int S>
__device__ __forceinline__ void run_pass_x2(int R, const Pass ps) {
  switch (R) {
    case 2: run_pass_x2_R<S, 2>(ps); break;
    case 3: run_pass_x2_R<S, 3>(ps); break;
    case 4: run_pass_x2_R<S, 4>(ps); break;
    case 5: run_pass_x2_R<S, 5>(ps); break;
    case 6: run_pass_x2_R<S, 6>(ps); break;
    case 7: run_pass_x2_R<S, 7>(ps); break;
    case 8: run_pass_x2_R<S, 8>(ps); break;
    case 9: run_pass_x2_R<S, 9>(ps); break;
    case 10: run_pass_x2_R<S, 10>(ps); break;
    case 12: run_pass_x2_R<S, 12>(ps); break;
    case 14: run_pass_x2_R<S, 14>(ps); break;
    case 15: run_pass_x2_R<S, 15>(ps); break;
    case 16: run_pass_x2_R<S, 16>(ps); break;
    default: break;  // R == 1: identity
  }
}

// A pass with two items per thread in general position (any Pass): thread t
// takes items t and t + H (H = ceil(nitems / 2)), so that each lane's accesses
// stay consecutive across the warp as in run_pass; the two items' elements and
// twiddles are loaded separately (8 bytes each) and transformed together with
// the packed instructions (FP32 data only).
template <int S, int R>
__device__ __forceinline__ void run_pass_pairs_R(const Pass ps) {
  float2* sm = smem_c<float>();
  const int nitems = ps.nbatch * ps.nsub;
  const int H = (nitems + 1) >> 1;
  for (int it0 = threadIdx.x; it0 < H; it0 += blockDim.x) {
    const int it1 = it0 + H;
    const bool dual = it1 < nitems;
    const int sub0 = it0 / ps.nbatch, b0 = it0 - sub0 * ps.nbatch;
    const int sub1 = dual ? it1 / ps.nbatch : sub0, b1 = dual ? it1 - sub1 * ps.nbatch : b0;
    const int off0 = ps.base + (ps.bmap != nullptr ? __ldg(ps.bmap + b0) : b0) * ps.bstride + sub0 * ps.sstride;
    const int off1 = ps.base + (ps.bmap != nullptr ? __ldg(ps.bmap + b1) : b1) * ps.bstride + sub1 * ps.sstride;
    f32x2 re[R], im[R];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      ok = ok && QGB_OK_IDX(off0 + j * ps.estride, ps.lim, 70 + R) && QGB_OK_IDX(off1 + j * ps.estride, ps.lim, 70 + R);
      const float2 v0 = ok ? sm[off0 + j * ps.estride] : make_float2(0.f, 0.f);
      const float2 v1 = ok ? sm[off1 + j * ps.estride] : make_float2(0.f, 0.f);
      re[j] = f32x2(make_float2(v0.x, v1.x));
      im[j] = f32x2(make_float2(v0.y, v1.y));
    }
    if (!ok) continue;
    Codelet<R, S>::run(re, im);
    if (ps.tw >= 0) {
      const int t0 = ps.tw + sub0 * ps.tw_sub, t1 = ps.tw + sub1 * ps.tw_sub;
#pragma unroll
      for (int j = 1; j < R; ++j) {
        if (!QGB_OK_IDX(t0 + j * ps.tw_el, ps.tw_lim, 90 + R) || !QGB_OK_IDX(t1 + j * ps.tw_el, ps.tw_lim, 90 + R))
          continue;
        const float2 w0 = sm[t0 + j * ps.tw_el], w1 = sm[t1 + j * ps.tw_el];
        const float2 wx2 = make_float2(w0.x, w1.x);
        const float2 wy2 = (S > 0) ? make_float2(w0.y, w1.y) : make_float2(-w0.y, -w1.y);
        const float2 nwy2 = make_float2(-wy2.x, -wy2.y);
        const float2 xr = __ffma2_rn(im[j].v, nwy2, __fmul2_rn(re[j].v, wx2));
        const float2 xi = __ffma2_rn(im[j].v, wx2, __fmul2_rn(re[j].v, wy2));
        re[j] = f32x2(xr);
        im[j] = f32x2(xi);
      }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      sm[off0 + j * ps.estride] = make_float2(re[j].v.x, im[j].v.x);
      if (dual) sm[off1 + j * ps.estride] = make_float2(re[j].v.y, im[j].v.y);
    }
  }
}

template <int S>
__device__ __forceinline__ void run_pass_pairs(int R, const Pass ps) {
  switch (R) {
    case 2: run_pass_pairs_R<S, 2>(ps); break;
    case 3: run_pass_pairs_R<S, 3>(ps); break;
    case 4: run_pass_pairs_R<S, 4>(ps); break;
    case 5: run_pass_pairs_R<S, 5>(ps); break;
    case 6: run_pass_pairs_R<S, 6>(ps); break;
    case 7: run_pass_pairs_R<S, 7>(ps); break;
    case 8: run_pass_pairs_R<S, 8>(ps); break;
    case 9: run_pass_pairs_R<S, 9>(ps); break;
    case 10: run_pass_pairs_R<S, 10>(ps); break;
    case 12: run_pass_pairs_R<S, 12>(ps); break;
    case 14: run_pass_pairs_R<S, 14>(ps); break;
    case 15: run_pass_pairs_R<S, 15>(ps); break;
    case 16: run_pass_pairs_R<S, 16>(ps); break;
    default: break;  // R == 1: identity
  }
}

// One pass of the y/z transforms: scalar items (the paired form measured
// slower there: two 8-byte accesses per element pair, separate twiddles per
// lane and twice the registers).
template <typename T, int S>
__device__ __forceinline__ void run_pass_any(int R, const Pass ps) {
  run_pass<T, S>(R, ps);
}

// Inverse transform (natural -> permuted) of nbatch pencils starting at shared
// offset `base`, element stride es; twiddles at shared offset W; `lim` bounds
// the data region.  Ends with __syncthreads().
template <typename T>
__device__ __forceinline__ void fft_inverse(int base, const int* bmap, int nbatch, int bstride, int es,
                                            int L1, int L2, int W, int lim) {
  if (L2 > 1) {
    run_pass_any<T, +1>(L2, Pass{bmap, base, nbatch, bstride, L1, es, L1 * es, W, L2, 1, lim, W + L1 * L2});
    __syncthreads();
  }
  if (L1 > 1) {
    run_pass_any<T, +1>(L1, Pass{bmap, base, nbatch, bstride, L2, L1 * es, es, -1, 0, 0, lim, 0});
    __syncthreads();
  }
}

// Forward transform (permuted -> natural) of nbatch pencils.  Ends with __syncthreads().
template <typename T>
__device__ __forceinline__ void fft_forward(int base, const int* bmap, int nbatch, int bstride, int es,
                                            int L1, int L2, int W, int lim) {
  if (L1 > 1) {
    run_pass_any<T, -1>(L1, Pass{bmap, base, nbatch, bstride, L2, L1 * es, es, (L2 > 1) ? W : -1, 1, L2, lim,
                                 W + L1 * L2});
    __syncthreads();
  }
  if (L2 > 1) {
    run_pass_any<T, -1>(L2, Pass{bmap, base, nbatch, bstride, L1, es, L1 * es, -1, 0, 0, lim, 0});
    __syncthreads();
  }
}

}  // namespace qgb
