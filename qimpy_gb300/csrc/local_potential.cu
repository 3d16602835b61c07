// Local-potential apply V*psi on the G-sphere: scatter -> 3D inverse FFT -> *V(r)
// -> 3D forward FFT -> gather (+ KE*psi), for a block of bands at every k.
//
// Replaces Basis.apply_potential (qimpy/dft/electrons/_basis_ops.py:39-113, with
// _KernelCommon.expand_ifft 152-163 and _ApplyPotentialKernel.__call__ 183-199)
// and fuses Basis.apply_ke (_basis_ops.py:29-36).  FFT conventions follow
// qimpy/grid/_fft.py: inverse unnormalised, forward scaled by 1/N.
//
// The 3D transform is split by the G-sphere's structure.  In-sphere points are
// sorted by linear grid index, so each "slab" (points sharing the first grid
// index i0) is a contiguous range of the basis, and only the n_slabs i0 values
// the sphere touches carry data:
//   k_ifft_yz      one CTA per (k, band, slab): scatter the slab's points into
//                  an N1 x N2 plane in shared memory, inverse z-FFT on the rows
//                  the sphere touches, inverse y-FFT on all columns, store the
//                  plane (real-space y, z in permuted order) to the workspace.
//   k_xpass        one CTA per (k, band, y-row): gather the slabs' rows into
//                  N2 pencils along x, inverse x-FFT, multiply by V(r), forward
//                  x-FFT, keep only the slab rows, store back.
//   k_fft_yz_gather one CTA per (k, band, slab): forward y-FFT on all columns,
//                  forward z-FFT on the touched rows, gather the slab's points,
//                  scale by 1/N and add KE*psi.
// Versus three full-grid passes each way this skips the empty x-planes in the
// y/z passes and the empty z-rows in the z passes.  Where both factors of an
// axis exceed 1, the passes next to global memory read or write it directly:
// the first inverse y pass reads untouched rows as zero (no zero fill), the
// last inverse y pass and the last forward x pass store straight to the
// planes, and the first inverse x pass and the first forward y pass read
// straight from them, so shared memory sees each element in the inner passes
// only.  With QGB_ACCUMULATE the gather adds to `out` (the mixed H.psi writes
// its nonlocal term there first, on another stream).
#include <algorithm>
#include <mutex>

#include "fft_steps.cuh"

namespace qgb {

static constexpr int kThreads = 256;

struct LocalParams {
  int nb_total;  // bands in C / out (stride of the band axis)
  int b0;        // first band of this chunk
  int nb;        // bands in this chunk
  unsigned flags;
};

template <typename T>
__device__ __forceinline__ void load_twiddles(int dst, const cplx_t<T>* src, int count) {
  cplx_t<T>* sm = smem_c<T>();
  for (int i = threadIdx.x; i < count; i += blockDim.x) sm[dst + i] = src[i];
}

// Plane workspace index of (k, band-in-chunk, slab).
__device__ __forceinline__ size_t plane_index(const qgb_sphere& s, int k, int b, int nb, int slab) {
  return (static_cast<size_t>(k) * nb + b) * s.max_slabs + slab;
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One complex element global -> shared without a register round trip (8 B
// for FP32, 16 B for FP64): many copies stay in flight per thread.
template <typename T>
__device__ __forceinline__ void cp_async_elem(cplx_t<T>* smem_dst, const cplx_t<T>* gsrc) {
  if constexpr (sizeof(cplx_t<T>) == 16) {
    cp_async16(smem_dst, gsrc);
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst))),
                 "l"(gsrc)
                 : "memory");
  }
}


// ---------------------------------------------------------------------------
// y passes of the y/z kernels with the plane's boundaries folded in (used when
// both y factors exceed 1).  Rows y of the shared plane sit at offset y * ld,
// columns c < nz; `rowmask[y]` marks the rows the slab's sphere points touch.
// ---------------------------------------------------------------------------

// Inverse pass 1 (radix R = L2) over rows sub + j * L1 with the pass-1
// twiddles; untouched rows are read as zero (they are never zero-filled).
template <typename T, int R>
__device__ __forceinline__ void ypass_inv1_R(const int* rowmask, int nz, int L1, int ld, int W, int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L1;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / nz;
    const int c = it - sub * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int y = sub + j * L1;
      const int off = y * ld + c;
      if (!QGB_OK_IDX(off, lim, 64)) return;
      cplx_t<T> v = mk<T>(T(0), T(0));
      if (rowmask[y]) v = sm[off];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, +1>::run(re, im);
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const cplx_t<T> w = sm[W + sub * R + j];
      const T xr = re[j] * w.x - im[j] * w.y;
      const T xi = re[j] * w.y + im[j] * w.x;
      re[j] = xr;
      im[j] = xi;
    }
#pragma unroll
    for (int j = 0; j < R; ++j) sm[(sub + j * L1) * ld + c] = mk<T>(re[j], im[j]);
  }
}

// Inverse pass 2 (radix R = L1) over rows sub * L1 + j, stored straight to the
// plane in global memory (row stride N2), in the permuted order of the rows.
template <typename T, int R>
__device__ __forceinline__ void ypass_inv2_R(cplx_t<T>* __restrict__ out, int N2, int nz, int L2, int ld, int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L2;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / nz;
    const int c = it - sub * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int off = (sub * R + j) * ld + c;
      if (!QGB_OK_IDX(off, lim, 65)) return;
      const cplx_t<T> v = sm[off];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, +1>::run(re, im);
#pragma unroll
    for (int j = 0; j < R; ++j) out[static_cast<size_t>(sub * R + j) * N2 + c] = mk<T>(re[j], im[j]);
  }
}

// Forward pass A (radix R = L1) over rows a * L1 + j, read straight from the
// plane in global memory, times the conjugated pass-A twiddles.
template <typename T, int R>
__device__ __forceinline__ void ypass_fwdA_R(const cplx_t<T>* __restrict__ in, int N2, int nz, int L2, int ld, int W,
                                             int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L2;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int a = it / nz;
    const int c = it - a * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const cplx_t<T> v = in[static_cast<size_t>(a * R + j) * N2 + c];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, -1>::run(re, im);
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const cplx_t<T> w = sm[W + a + j * L2];
      const T xr = re[j] * w.x + im[j] * w.y;
      const T xi = im[j] * w.x - re[j] * w.y;
      re[j] = xr;
      im[j] = xi;
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int off = (a * R + j) * ld + c;
      if (!QGB_OK_IDX(off, lim, 66)) return;
      sm[off] = mk<T>(re[j], im[j]);
    }
  }
}

// Forward pass B (radix R = L2) over rows sub + j * L1 (natural order out);
// only the rows the slab's sphere points touch are stored.
template <typename T, int R>
__device__ __forceinline__ void ypass_fwdB_R(const int* rowmask, int nz, int L1, int ld, int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L1;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / nz;
    const int c = it - sub * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int off = (sub + j * L1) * ld + c;
      if (!QGB_OK_IDX(off, lim, 67)) return;
      const cplx_t<T> v = sm[off];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, -1>::run(re, im);
#pragma unroll
    for (int j = 0; j < R; ++j)
      if (rowmask[sub + j * L1]) sm[(sub + j * L1) * ld + c] = mk<T>(re[j], im[j]);
  }
}

// kind 0: inverse pass 1; 1: inverse pass 2 (to global); 2: forward pass A
// (from global); 3: forward pass B.  R is the pass's radix.
template <typename T, int KIND>
__device__ __forceinline__ void ypass(int R, const int* rowmask, cplx_t<T>* g, int N2, int nz, int L1, int L2,
                                      int ld, int W, int lim) {
#define QGB_YP(RR)                                                                  \
  case RR:                                                                          \
    if constexpr (KIND == 0) ypass_inv1_R<T, RR>(rowmask, nz, L1, ld, W, lim);      \
    if constexpr (KIND == 1) ypass_inv2_R<T, RR>(g, N2, nz, L2, ld, lim);           \
    if constexpr (KIND == 2) ypass_fwdA_R<T, RR>(g, N2, nz, L2, ld, W, lim);        \
    if constexpr (KIND == 3) ypass_fwdB_R<T, RR>(rowmask, nz, L1, ld, lim);         \
    break;
  switch (R) {
    QGB_YP(2) QGB_YP(3) QGB_YP(4) QGB_YP(5) QGB_YP(6) QGB_YP(7) QGB_YP(8) QGB_YP(9) QGB_YP(10) QGB_YP(12)
    QGB_YP(14) QGB_YP(15) QGB_YP(16)
    default: break;
  }
#undef QGB_YP
}

template <typename T>
__device__ __forceinline__ void body_ifft_yz(const qgb_sphere& s, const LocalParams& lp,
                                             const cplx_t<T>* __restrict__ C, cplx_t<T>* __restrict__ planes,
                                             const int slab, const int b, const int k) {
  using C2 = cplx_t<T>;
  if (slab >= s.n_slabs[k]) return;
  const int N1 = s.N[1], N2 = s.N[2], ld = N2 + 1;
  const int L1y = s.L1[1], L2y = s.L2[1];
  const bool fold = L1y > 1 && L2y > 1;  // y passes with the plane's boundaries folded in
  // Shared layout: plane [N1][ld], W_y [N1], W_z [N2], row mask [N1] int.
  const int lim = N1 * ld, Wy = lim, Wz = Wy + N1;
  C2* sm = smem_c<T>();
  int* rowmask = reinterpret_cast<int*>(sm + Wz + N2);
  const C2* tw = static_cast<const C2*>(s.twiddle);
  load_twiddles<T>(Wy, tw + s.tw_off[1], N1);
  load_twiddles<T>(Wz, tw + s.tw_off[2], N2);
  const C2 zero = mk<T>(T(0), T(0));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int r0 = s.row_start[k * (s.max_slabs + 1) + slab];
  const int nrows = s.row_start[k * (s.max_slabs + 1) + slab + 1] - r0;
  const int* rows = s.rows + r0;
  if (fold) {
    // Only the touched rows are zero-filled: the first y pass reads the others as zero.
    for (int y = threadIdx.x; y < N1; y += blockDim.x) rowmask[y] = 0;
    for (int i = warp; i < nrows; i += nwarps) {
      const int y = rows[i];
      if (!QGB_OK_IDX(y, N1, 68)) continue;
      for (int c = lane; c < N2; c += 32) sm[y * ld + c] = zero;
    }
  } else {
    for (int r = warp; r < N1; r += nwarps)
      for (int c = lane; c < N2; c += 32) sm[r * ld + c] = zero;
  }
  __syncthreads();
  if (fold) {
    for (int i = threadIdx.x; i < nrows; i += blockDim.x) {
      const int y = rows[i];
      if (QGB_OK_IDX(y, N1, 68)) rowmask[y] = 1;
    }
  }

  // Scatter this slab's coefficients (contiguous in the basis) into the plane.
  const int g0 = s.slab_start[k * (s.max_slabs + 1) + slab];
  const int g1 = s.slab_start[k * (s.max_slabs + 1) + slab + 1];
  const C2* Cb = C + (static_cast<size_t>(k) * lp.nb_total + lp.b0 + b) * s.n_tot;
  const int* yz = s.yz + static_cast<size_t>(k) * s.n_tot;
  for (int g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
    if (!QGB_OK_IDX(g, s.n[k], 1)) continue;
    const int v = yz[g];
    const int pos = (v >> 16) * ld + (v & 0xFFFF);
    if (!QGB_OK_IDX(pos, lim, 2) || !QGB_OK_IDX(v & 0xFFFF, N2, 3)) continue;
    cp_async_elem<T>(sm + pos, Cb + g);
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();

  // Inverse z-FFT along the rows this slab touches (row stride ld, element stride 1).
  fft_inverse<T>(0, rows, nrows, ld, 1, s.L1[2], s.L2[2], Wz, lim);
  if (!QGB_OK_IDX(plane_index(s, k, b, lp.nb, slab), (long long)s.nk * lp.nb * s.max_slabs, 4)) return;
  C2* out = planes + plane_index(s, k, b, lp.nb, slab) * (static_cast<size_t>(N1) * N2);
  if (fold) {
    // Inverse y-FFT along all N2 columns; its second pass stores the plane.
    ypass<T, 0>(L2y, rowmask, nullptr, N2, N2, L1y, L2y, ld, Wy, lim);
    __syncthreads();
    ypass<T, 1>(L1y, rowmask, out, N2, N2, L1y, L2y, ld, Wy, lim);
    return;
  }
  // Inverse y-FFT along all N2 columns (column stride 1, element stride ld).
  fft_inverse<T>(0, nullptr, N2, 1, ld, L1y, L2y, Wy, lim);
  for (int r = warp; r < N1; r += nwarps)
    for (int c = lane; c < N2; c += 32) out[r * N2 + c] = sm[r * ld + c];
}

template <typename T>
__device__ __forceinline__ void body_xpass(const qgb_sphere& s, const LocalParams& lp,
                                           cplx_t<T>* __restrict__ planes, const int r1, const int b, const int k) {
  using C2 = cplx_t<T>;
  const int N0 = s.N[0], N1 = s.N[1], N2 = s.N[2], ld = N2 + 1;
  const int L1 = s.L1[0], L2 = s.L2[0];
  const int lim = N0 * ld, Wx = lim;  // shared layout: pencils (x rows of N2 columns), W_x
  C2* sm = smem_c<T>();
  const C2* tw = static_cast<const C2*>(s.twiddle);
  load_twiddles<T>(Wx, tw + s.tw_off[0], N0);
  const C2 zero = mk<T>(T(0), T(0));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  for (int r = warp; r < N0; r += nwarps)
    for (int c = lane; c < N2; c += 32) sm[r * ld + c] = zero;
  __syncthreads();

  const int nslabs = s.n_slabs[k];
  const int* i0 = s.slab_i0 + k * s.max_slabs;
  const size_t plane = static_cast<size_t>(N1) * N2;
  C2* base = planes + plane_index(s, k, b, lp.nb, 0) * plane + static_cast<size_t>(r1) * N2;
  for (int sl = warp; sl < nslabs; sl += nwarps) {
    const int x = i0[sl];
    if (!QGB_OK_IDX(x, N0, 5) ||
        !QGB_OK_IDX(plane_index(s, k, b, lp.nb, sl), (long long)s.nk * lp.nb * s.max_slabs, 6))
      continue;
    const C2* src = base + sl * plane;
    for (int c = lane; c < N2; c += 32) sm[x * ld + c] = src[c];
  }
  __syncthreads();

  // Inverse x pass 1 (natural in).
  if (L2 > 1) {
    run_pass<T, +1>(L2, Pass{nullptr, 0, N2, 1, L1, ld, L1 * ld, Wx, L2, 1, lim, Wx + N0});
    __syncthreads();
  }
  // Inverse pass 2, multiply by V at the permuted real-space position, forward
  // pass A: the same thread owns block [L1 a, L1 a + L1) of a column in all three.
  {
    const T* V = static_cast<const T*>(s.V);
    const int nitems = N2 * L2;
    for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
      const int a = it / N2;
      const int c = it - a * N2;
      const int p = c + a * L1 * ld;
      const T* Vp = V + (static_cast<size_t>(a) * L1 * N1 + r1) * N2 + c;
      if (!QGB_OK_IDX(c + (a * L1 + L1 - 1) * ld, lim, 7) ||
          !QGB_OK_IDX(((long long)(a * L1 + L1 - 1) * N1 + r1) * N2 + c, (long long)N0 * N1 * N2, 8) ||
          !QGB_OK_IDX((L1 - 1) * L2 + a, N0, 9))
        continue;
      // L1 is a codelet size; dispatch once per item.
      switch (L1) {
#define QGB_XMID(R)                                                                        \
  case R: {                                                                                \
    T re[R], im[R];                                                                        \
    _Pragma("unroll") for (int j = 0; j < R; ++j) {                                        \
      const C2 v = sm[p + j * ld];                                                         \
      re[j] = v.x;                                                                         \
      im[j] = v.y;                                                                         \
    }                                                                                      \
    Codelet<R, +1>::run(re, im);                                                           \
    _Pragma("unroll") for (int j = 0; j < R; ++j) {                                        \
      const T vv = Vp[static_cast<size_t>(j) * N1 * N2];                                   \
      re[j] *= vv;                                                                         \
      im[j] *= vv;                                                                         \
    }                                                                                      \
    Codelet<R, -1>::run(re, im);                                                           \
    if (L2 > 1) {                                                                          \
      _Pragma("unroll") for (int j = 1; j < R; ++j) {                                      \
        const C2 w = sm[Wx + j * L2 + a];                                                  \
        const T xr = re[j] * w.x + im[j] * w.y;                                            \
        const T xi = im[j] * w.x - re[j] * w.y;                                            \
        re[j] = xr;                                                                        \
        im[j] = xi;                                                                        \
      }                                                                                    \
    }                                                                                      \
    _Pragma("unroll") for (int j = 0; j < R; ++j) sm[p + j * ld] = mk<T>(re[j], im[j]);    \
  } break;
        QGB_XMID(1)
        QGB_XMID(2)
        QGB_XMID(3)
        QGB_XMID(4)
        QGB_XMID(5)
        QGB_XMID(6)
        QGB_XMID(7)
        QGB_XMID(8)
        QGB_XMID(9)
        QGB_XMID(10)
        QGB_XMID(12)
        QGB_XMID(14)
        QGB_XMID(15)
        QGB_XMID(16)
#undef QGB_XMID
        default: break;
      }
    }
    __syncthreads();
  }
  // Forward pass B (natural out).
  if (L2 > 1) {
    run_pass<T, -1>(L2, Pass{nullptr, 0, N2, 1, L1, ld, L1 * ld, -1, 0, 0, lim, 0});
    __syncthreads();
  }
  for (int sl = warp; sl < nslabs; sl += nwarps) {
    const int x = i0[sl];
    if (!QGB_OK_IDX(x, N0, 5)) continue;
    C2* dst = base + sl * plane;
    for (int c = lane; c < N2; c += 32) dst[c] = sm[x * ld + c];
  }
}

// The x-pass middle step on one item: inverse L1-point DFT, multiply by V,
// forward L1-point DFT, forward-pass twiddles; data at sm[p + j*ld], V at
// Vp[j * vstride] (global or shared), twiddles at sm[Wx + j*L2 + a].
template <typename T, int R, typename VPtr>
__device__ __forceinline__ void xmid_item(cplx_t<T>* sm, int p, int ld, VPtr Vp, size_t vstride, int Wx, int L2,
                                          int a) {
  using C2 = cplx_t<T>;
  T re[R], im[R];
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const C2 v = sm[p + j * ld];
    re[j] = v.x;
    im[j] = v.y;
  }
  Codelet<R, +1>::run(re, im);
#pragma unroll
  for (int j = 0; j < R; ++j) {
    const T vv = Vp[j * vstride];
    re[j] *= vv;
    im[j] *= vv;
  }
  Codelet<R, -1>::run(re, im);
  if (L2 > 1) {
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const C2 w = sm[Wx + j * L2 + a];
      const T xr = re[j] * w.x + im[j] * w.y;
      const T xi = im[j] * w.x - re[j] * w.y;
      re[j] = xr;
      im[j] = xi;
    }
  }
#pragma unroll
  for (int j = 0; j < R; ++j) sm[p + j * ld] = mk<T>(re[j], im[j]);
}

template <typename T, typename VPtr>
__device__ __forceinline__ void xmid_dispatch(int L1, cplx_t<T>* sm, int p, int ld, VPtr Vp, size_t vstride, int Wx,
                                              int L2, int a) {
  switch (L1) {
    case 1: xmid_item<T, 1>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 2: xmid_item<T, 2>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 3: xmid_item<T, 3>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 4: xmid_item<T, 4>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 5: xmid_item<T, 5>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 6: xmid_item<T, 6>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 7: xmid_item<T, 7>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 8: xmid_item<T, 8>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 9: xmid_item<T, 9>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 10: xmid_item<T, 10>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 12: xmid_item<T, 12>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 14: xmid_item<T, 14>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 15: xmid_item<T, 15>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    case 16: xmid_item<T, 16>(sm, p, ld, Vp, vstride, Wx, L2, a); break;
    default: break;
  }
}

// x-pass first inverse pass straight from the slab planes: item (column c,
// sub) is the L2-point DFT over x = sub + j * L1 (natural order), read from the
// plane of slab xs[x] (zero where no slab), times the pass-1 twiddles, stored
// at the same shared rows.  Covers every row, so no zero fill is needed.
template <typename T, int R>
__device__ __forceinline__ void xpass_first_R(const cplx_t<T>* __restrict__ base, size_t plane, const int* xs,
                                              int nz, int L1, int ld, int Wx, int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L1;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / nz;
    const int c = it - sub * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int sl = xs[sub + j * L1];
      cplx_t<T> v = mk<T>(T(0), T(0));
      if (sl >= 0) v = base[static_cast<size_t>(sl) * plane + c];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, +1>::run(re, im);
#pragma unroll
    for (int j = 1; j < R; ++j) {
      const cplx_t<T> w = sm[Wx + sub * R + j];
      const T xr = re[j] * w.x - im[j] * w.y;
      const T xi = re[j] * w.y + im[j] * w.x;
      re[j] = xr;
      im[j] = xi;
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int off = (sub + j * L1) * ld + c;
      if (!QGB_OK_IDX(off, lim, 61)) return;
      sm[off] = mk<T>(re[j], im[j]);
    }
  }
}

// x-pass last forward pass straight to the slab planes: the L2-point DFT over
// the shared rows sub + j * L1 gives natural x = sub + j * L1; only the rows of
// a slab (xs[x] >= 0) are stored.
template <typename T, int R>
__device__ __forceinline__ void xpass_last_R(cplx_t<T>* __restrict__ base, size_t plane, const int* xs, int nz,
                                             int L1, int ld, int lim) {
  cplx_t<T>* sm = smem_c<T>();
  const int nitems = nz * L1;
  for (int it = threadIdx.x; it < nitems; it += blockDim.x) {
    const int sub = it / nz;
    const int c = it - sub * nz;
    T re[R], im[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int off = (sub + j * L1) * ld + c;
      if (!QGB_OK_IDX(off, lim, 62)) return;
      const cplx_t<T> v = sm[off];
      re[j] = v.x;
      im[j] = v.y;
    }
    Codelet<R, -1>::run(re, im);
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int sl = xs[sub + j * L1];
      if (sl >= 0) base[static_cast<size_t>(sl) * plane + c] = mk<T>(re[j], im[j]);
    }
  }
}

template <typename T, bool FIRST>
__device__ __forceinline__ void xpass_outer(int R, cplx_t<T>* base, size_t plane, const int* xs, int nz, int L1,
                                            int ld, int Wx, int lim) {
#define QGB_XO(RR)                                                   \
  case RR:                                                           \
    if constexpr (FIRST)                                             \
      xpass_first_R<T, RR>(base, plane, xs, nz, L1, ld, Wx, lim);    \
    else                                                             \
      xpass_last_R<T, RR>(base, plane, xs, nz, L1, ld, lim);         \
    break;
  switch (R) {
    QGB_XO(2) QGB_XO(3) QGB_XO(4) QGB_XO(5) QGB_XO(6) QGB_XO(7) QGB_XO(8) QGB_XO(9) QGB_XO(10) QGB_XO(12)
    QGB_XO(14) QGB_XO(15) QGB_XO(16)
    default: break;
  }
#undef QGB_XO
}

// x-pass (FP32, N2 % 4 == 0, L2 > 1) with its outer passes on the slab planes:
// the first inverse pass reads the slab rows from global memory (L2) and the
// last forward pass stores the slab rows back, so shared memory sees each
// element in three passes only (no zero fill, staging or write-back).  The
// middle step reads V(r) from global memory (it stays in L2 across the bands).
// Shared layout: pencils [N0][ld = nz + 2] complex, W_x [N0] complex, x -> slab
// table [N0] int.  75 KB for si64 (96^3), so 3 CTAs fit an SM.
template <typename T>
__device__ __forceinline__ void body_xpass_async(const qgb_sphere& s, const LocalParams& lp,
                                                 cplx_t<T>* __restrict__ planes, const int r1, const int b,
                                                 const int k, const int z0, const int nz) {
  using C2 = cplx_t<T>;
  const int N0 = s.N[0], N1 = s.N[1], N2 = s.N[2], ld = nz + 2;
  const int L1 = s.L1[0], L2 = s.L2[0];
  const int lim = N0 * ld, Wx = lim;
  C2* sm = smem_c<T>();
  int* xs = reinterpret_cast<int*>(sm + Wx + N0);
  const C2* tw = static_cast<const C2*>(s.twiddle);
  load_twiddles<T>(Wx, tw + s.tw_off[0], N0);
  for (int x = threadIdx.x; x < N0; x += blockDim.x) xs[x] = -1;
  __syncthreads();
  const int nslabs = s.n_slabs[k];
  const int* i0 = s.slab_i0 + k * s.max_slabs;
  for (int sl = threadIdx.x; sl < nslabs; sl += blockDim.x) {
    const int x = i0[sl];
    if (QGB_OK_IDX(x, N0, 63)) xs[x] = sl;
  }
  __syncthreads();
  const size_t plane = static_cast<size_t>(N1) * N2;
  C2* base = planes + plane_index(s, k, b, lp.nb, 0) * plane + static_cast<size_t>(r1) * N2 + z0;
  xpass_outer<T, true>(L2, base, plane, xs, nz, L1, ld, Wx, lim);
  __syncthreads();
  // V[p0][r1][z0 + c] with p0 = a * L1 + j: j-stride N1 * N2.
  const T* V = static_cast<const T*>(s.V) + static_cast<size_t>(r1) * N2 + z0;
  for (int it = threadIdx.x; it < nz * L2; it += blockDim.x) {
    const int a = it / nz;
    const int c = it - a * nz;
    xmid_dispatch<T>(L1, sm, c + a * L1 * ld, ld, V + static_cast<size_t>(a) * L1 * N1 * N2 + c,
                     static_cast<size_t>(N1) * N2, Wx, L2, a);
  }
  __syncthreads();
  xpass_outer<T, false>(L2, base, plane, xs, nz, L1, ld, Wx, lim);
}

template <typename T>
__device__ __forceinline__ void body_fft_yz_gather(const qgb_sphere& s, const LocalParams& lp, const cplx_t<T>* C,
                                                   cplx_t<T>* out, const cplx_t<T>* __restrict__ planes,
                                                   const int slab, const int b, const int k) {
  using C2 = cplx_t<T>;
  const int nslabs = s.n_slabs[k];
  C2* Ob = out + (static_cast<size_t>(k) * lp.nb_total + lp.b0 + b) * s.n_tot;
  const bool accumulate = (lp.flags & QGB_ACCUMULATE) != 0;
  if (slab == 0 && !accumulate) {  // zero the padding entries of this band
    const int nk_in = s.n[k];
    for (int g = nk_in + threadIdx.x; g < s.n_tot; g += blockDim.x) Ob[g] = mk<T>(T(0), T(0));
  }
  if (slab >= nslabs) return;
  const int N0 = s.N[0], N1 = s.N[1], N2 = s.N[2], ld = N2 + 1;
  const int lim = N1 * ld, Wy = lim, Wz = Wy + N1;
  C2* sm = smem_c<T>();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  if (!QGB_OK_IDX(plane_index(s, k, b, lp.nb, slab), (long long)s.nk * lp.nb * s.max_slabs, 4)) return;
  const C2* in = planes + plane_index(s, k, b, lp.nb, slab) * (static_cast<size_t>(N1) * N2);
  const int L1y = s.L1[1], L2y = s.L2[1];
  const int r0 = s.row_start[k * (s.max_slabs + 1) + slab];
  const int nrows = s.row_start[k * (s.max_slabs + 1) + slab + 1] - r0;
  const C2* tw = static_cast<const C2*>(s.twiddle);
  if (L1y > 1 && L2y > 1) {
    // The first forward y pass reads the plane from global memory; the second
    // stores only the rows the z-FFT and the gather use.
    int* rowmask = reinterpret_cast<int*>(sm + Wz + N2);
    for (int y = threadIdx.x; y < N1; y += blockDim.x) rowmask[y] = 0;
    load_twiddles<T>(Wy, tw + s.tw_off[1], N1);
    load_twiddles<T>(Wz, tw + s.tw_off[2], N2);
    __syncthreads();
    for (int i = threadIdx.x; i < nrows; i += blockDim.x) {
      const int y = s.rows[r0 + i];
      if (QGB_OK_IDX(y, N1, 68)) rowmask[y] = 1;
    }
    ypass<T, 2>(L1y, rowmask, const_cast<C2*>(in), N2, N2, L1y, L2y, ld, Wy, lim);
    __syncthreads();
    ypass<T, 3>(L2y, rowmask, nullptr, N2, N2, L1y, L2y, ld, Wy, lim);
    __syncthreads();
  } else {
    // Stage the plane asynchronously (padded rows are 8-byte aligned only, so one
    // element per copy), then the twiddles while the copies are in flight.
    for (int r = warp; r < N1; r += nwarps)
      for (int c = lane; c < N2; c += 32) cp_async_elem<T>(sm + r * ld + c, in + r * N2 + c);
    cp_async_commit();
    load_twiddles<T>(Wy, tw + s.tw_off[1], N1);
    load_twiddles<T>(Wz, tw + s.tw_off[2], N2);
    cp_async_wait<0>();
    __syncthreads();
    fft_forward<T>(0, nullptr, N2, 1, ld, L1y, L2y, Wy, lim);
  }
  fft_forward<T>(0, s.rows + r0, nrows, ld, 1, s.L1[2], s.L2[2], Wz, lim);

  const int g0 = s.slab_start[k * (s.max_slabs + 1) + slab];
  const int g1 = s.slab_start[k * (s.max_slabs + 1) + slab + 1];
  const C2* Cb = C + (static_cast<size_t>(k) * lp.nb_total + lp.b0 + b) * s.n_tot;
  const int* yz = s.yz + static_cast<size_t>(k) * s.n_tot;
  const T invN = T(1) / (T(N0) * T(N1) * T(N2));
  const bool add_ke = (lp.flags & QGB_ADD_KE) != 0;
  const T* ke = static_cast<const T*>(s.ke) + static_cast<size_t>(k) * s.n_tot;
  for (int g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
    if (!QGB_OK_IDX(g, s.n[k], 1)) continue;
    const int v = yz[g];
    const int pos = (v >> 16) * ld + (v & 0xFFFF);
    if (!QGB_OK_IDX(pos, lim, 2)) continue;
    const C2 f = sm[pos];
    T xr = f.x * invN, xi = f.y * invN;
    if (add_ke) {
      const C2 c = Cb[g];
      const T e = ke[g];
      xr = e * c.x + xr;
      xi = e * c.y + xi;
    }
    if (accumulate) {
      const C2 o = Ob[g];
      xr += o.x;
      xi += o.y;
    }
    Ob[g] = mk<T>(xr, xi);
  }
}


// ---------------------------------------------------------------------------
// Kernels: one sphere (grid = work units of that sphere) ...
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(kThreads) k_ifft_yz(const qgb_sphere s, LocalParams lp,
                                                      const cplx_t<T>* __restrict__ C,
                                                      cplx_t<T>* __restrict__ planes) {
  body_ifft_yz<T>(s, lp, C, planes, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_xpass(const qgb_sphere s, LocalParams lp,
                                                    cplx_t<T>* __restrict__ planes) {
  body_xpass<T>(s, lp, planes, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 3) k_xpass_async(const qgb_sphere s, LocalParams lp,
                                                          cplx_t<T>* __restrict__ planes) {
  body_xpass_async<T>(s, lp, planes, blockIdx.x, blockIdx.y, blockIdx.z, 0, s.N[2]);
}

// C and out may alias (in-place apply): no __restrict__ on them.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_fft_yz_gather(const qgb_sphere s, LocalParams lp,
                                                            const cplx_t<T>* C, cplx_t<T>* out,
                                                            const cplx_t<T>* __restrict__ planes) {
  body_fft_yz_gather<T>(s, lp, C, out, planes, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ... and a batch of independent spheres (cells / k-point sets / band blocks
// with their own grids and bases) in one launch per phase.  Work unit u of the
// concatenated unit ranges starts[i] <= u < starts[i + 1] belongs to item
// i = unit_item[u]; units are (k, band, slab) for the y/z phases and (k, band,
// y-row) for the x phase, in that order (slab / row fastest).  Each CTA runs
// `upc` consecutive units, so it stages an item and its sphere descriptor in
// shared memory once for a run of units of that item rather than once per
// unit (the three dependent loads behind it cost about as much as the FFT work
// of one unit on the smallest grids).

struct BatchCtx {
  qgb_batch_item it;
  qgb_sphere s;
};

// Stage item i's context when it differs from the one staged (uniform across
// the CTA); returns the unit's index within its item.
__device__ __forceinline__ long long batch_unit(BatchCtx& ctx, int& staged, const qgb_batch_item* __restrict__ items,
                                                const int* __restrict__ unit_item,
                                                const long long* __restrict__ starts, long long u) {
  const int i = __ldg(unit_item + u);
  if (i != staged) {
    if (threadIdx.x == 0) {
      ctx.it = items[i];
      ctx.s = *ctx.it.sphere;
    }
    staged = i;
    __syncthreads();
  }
  return u - __ldg(starts + i);
}

#define QGB_BATCH_UNITS_BEGIN                                                       \
  __shared__ BatchCtx ctx;                                                          \
  int staged = -1;                                                                  \
  const long long u_begin = static_cast<long long>(blockIdx.x) * upc;               \
  const long long u_end = u_begin + upc < n_units ? u_begin + upc : n_units;        \
  for (long long u = u_begin; u < u_end; ++u) {                                     \
    const long long local = batch_unit(ctx, staged, items, unit_item, starts, u);   \
    const qgb_sphere& s = ctx.s;                                                    \
    const LocalParams lp{ctx.it.nb, 0, ctx.it.nb, ctx.it.flags};
#define QGB_BATCH_UNITS_END                                                         \
    __syncthreads(); /* shared memory and ctx are reused by the next unit */        \
  }

template <typename T>
__global__ void __launch_bounds__(kThreads) k_ifft_yz_batched(const qgb_batch_item* __restrict__ items,
                                                              const int* __restrict__ unit_item,
                                                              const long long* __restrict__ starts,
                                                              long long n_units, int upc) {
  QGB_BATCH_UNITS_BEGIN
  const int slab = static_cast<int>(local % s.max_slabs);
  const long long rest = local / s.max_slabs;
  body_ifft_yz<T>(s, lp, static_cast<const cplx_t<T>*>(ctx.it.C), static_cast<cplx_t<T>*>(ctx.it.planes), slab,
                  static_cast<int>(rest % ctx.it.nb), static_cast<int>(rest / ctx.it.nb));
  QGB_BATCH_UNITS_END
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_xpass_batched(const qgb_batch_item* __restrict__ items,
                                                            const int* __restrict__ unit_item,
                                                            const long long* __restrict__ starts,
                                                            long long n_units, int upc) {
  QGB_BATCH_UNITS_BEGIN
  const int r1 = static_cast<int>(local % s.N[1]);
  const long long rest = local / s.N[1];
  const int b = static_cast<int>(rest % ctx.it.nb), k = static_cast<int>(rest / ctx.it.nb);
  if (sizeof(T) == 4 && s.N[2] % 4 == 0 && s.L2[0] > 1)
    body_xpass_async<T>(s, lp, static_cast<cplx_t<T>*>(ctx.it.planes), r1, b, k, 0, s.N[2]);
  else
    body_xpass<T>(s, lp, static_cast<cplx_t<T>*>(ctx.it.planes), r1, b, k);
  QGB_BATCH_UNITS_END
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_fft_yz_gather_batched(const qgb_batch_item* __restrict__ items,
                                                                    const int* __restrict__ unit_item,
                                                                    const long long* __restrict__ starts,
                                                                    long long n_units, int upc) {
  QGB_BATCH_UNITS_BEGIN
  const int slab = static_cast<int>(local % s.max_slabs);
  const long long rest = local / s.max_slabs;
  body_fft_yz_gather<T>(s, lp, static_cast<const cplx_t<T>*>(ctx.it.C), static_cast<cplx_t<T>*>(ctx.it.out),
                        static_cast<const cplx_t<T>*>(ctx.it.planes), slab, static_cast<int>(rest % ctx.it.nb),
                        static_cast<int>(rest / ctx.it.nb));
  QGB_BATCH_UNITS_END
}

template <typename T>
__global__ void k_apply_ke(const qgb_sphere s, int nb, const cplx_t<T>* __restrict__ C,
                           cplx_t<T>* __restrict__ out) {
  const size_t total = static_cast<size_t>(s.nk) * nb * s.n_tot;
  const T* ke = static_cast<const T*>(s.ke);
  for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<size_t>(gridDim.x) * blockDim.x) {
    const size_t g = i % s.n_tot;
    const size_t k = i / (static_cast<size_t>(nb) * s.n_tot);
    const T e = ke[k * s.n_tot + g];
    const cplx_t<T> c = C[i];
    out[i] = mk<T>(e * c.x, e * c.y);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

#ifdef QGB_DEBUG_CHECKS
// Debug builds: copy out and clear the first recorded range violation
// (site, index, limit, packed block index); site 0 = none.
int debug_violation(unsigned long long* out4) {
  QGB_CUDA_CHECK(cudaDeviceSynchronize());
  QGB_CUDA_CHECK(cudaMemcpyFromSymbol(out4, g_qgb_violation, 4 * sizeof(unsigned long long)));
  const unsigned long long zero[4] = {0, 0, 0, 0};
  QGB_CUDA_CHECK(cudaMemcpyToSymbol(g_qgb_violation, zero, sizeof(zero)));
  return QGB_OK;
}
#endif

static bool codelet_size(int R) {
  switch (R) {
    case 1: case 2: case 3: case 4: case 5: case 6: case 7: case 8: case 9: case 10:
    case 12: case 14: case 15: case 16:
      return true;
    default:
      return false;
  }
}

size_t plane_smem_bytes(const qgb_sphere& s, int dtype) {
  const size_t e = elem_bytes(dtype);
  const size_t yz = (static_cast<size_t>(s.N[1]) * (s.N[2] + 1) + s.N[1] + s.N[2]) * e + s.N[1] * sizeof(int);
  const size_t x = (static_cast<size_t>(s.N[0]) * (s.N[2] + 1) + s.N[0]) * e;
  return std::max(yz, x);
}

// The asynchronous x-pass: FP32 with 16-byte aligned rows of V and of the planes.
static bool xpass_async_ok(const qgb_sphere& s, int dtype) { return dtype == QGB_F32 && s.N[2] % 4 == 0 && s.L2[0] > 1; }

static size_t xpass_async_smem_bytes(const qgb_sphere& s) {
  const size_t cplx = static_cast<size_t>(s.N[0]) * (s.N[2] + 2) + s.N[0];
  return cplx * 8 + static_cast<size_t>(s.N[0]) * 4;
}

int validate_sphere(const qgb_sphere* s, int dtype, bool need_potential = true) {
  if (s == nullptr) return fail(QGB_ERR_INVALID, "sphere descriptor is NULL");
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (s->nk < 1 || s->n_tot < 1 || s->max_slabs < 1)
    return fail(QGB_ERR_INVALID, "empty sphere (nk=%d n_tot=%d max_slabs=%d)", s->nk, s->n_tot,
                s->max_slabs);
  for (int a = 0; a < 3; ++a) {
    if (s->N[a] < 1 || s->N[a] > 65535)
      return fail(QGB_ERR_INVALID, "grid dimension %d = %d out of range", a, s->N[a]);
    if (!codelet_size(s->L1[a]) || !codelet_size(s->L2[a]) || s->L1[a] * s->L2[a] != s->N[a])
      return fail(QGB_ERR_INVALID, "axis %d: N=%d is not L1*L2 with L1=%d, L2=%d codelet sizes",
                  a, s->N[a], s->L1[a], s->L2[a]);
  }
  if (s->max_slabs > s->N[0]) return fail(QGB_ERR_INVALID, "max_slabs %d > N0", s->max_slabs);
  if (!s->n || !s->n_slabs || !s->slab_start || !s->slab_i0 || !s->yz || !s->row_start ||
      !s->rows || !s->twiddle || !s->ke)
    return fail(QGB_ERR_INVALID, "sphere descriptor has a NULL table");
  if (need_potential && !s->V) return fail(QGB_ERR_INVALID, "sphere descriptor has no potential V");
  if (plane_smem_bytes(*s, dtype) > 227 * 1024 || (xpass_async_ok(*s, dtype) && xpass_async_smem_bytes(*s) > 227 * 1024))
    return fail(QGB_ERR_UNSUPPORTED, "grid %dx%dx%d needs %zu B of shared memory per plane (max 227 KB)",
                s->N[0], s->N[1], s->N[2], plane_smem_bytes(*s, dtype));
  return QGB_OK;
}

size_t plane_bytes_per_band(const qgb_sphere& s, int dtype) {
  return static_cast<size_t>(s.nk) * s.max_slabs * s.N[1] * s.N[2] * elem_bytes(dtype);
}

// Kernels' shared-memory limits are raised lazily (raise_smem_limit: per
// kernel and device, to the largest size asked for so far).
static int launch_xpass_async(const qgb_sphere& s, const LocalParams& lp, float2* planes, cudaStream_t st) {
  const size_t smx = xpass_async_smem_bytes(s);
  if (int rc = raise_smem_limit(k_xpass_async<float>, smx)) return rc;
  const dim3 g2(s.N[1], lp.nb, s.nk);
  k_xpass_async<float><<<g2, kThreads, smx, st>>>(s, lp, planes);
  QGB_LAUNCH_CHECK("k_xpass_async");
  return QGB_OK;
}

template <typename T>
static int launch_chunk(const qgb_sphere& s, const LocalParams& lp, const void* C, void* out,
                        void* planes, cudaStream_t st, size_t smem, cudaEvent_t gather_after) {
  using C2 = cplx_t<T>;
  const dim3 g1(s.max_slabs, lp.nb, s.nk);
  k_ifft_yz<T><<<g1, kThreads, smem, st>>>(s, lp, static_cast<const C2*>(C), static_cast<C2*>(planes));
  QGB_LAUNCH_CHECK("k_ifft_yz");
  if (sizeof(T) == 4 && xpass_async_ok(s, QGB_F32)) {
    const int rc = launch_xpass_async(s, lp, static_cast<float2*>(planes), st);
    if (rc) return rc;
  } else {
    const dim3 g2(s.N[1], lp.nb, s.nk);
    k_xpass<T><<<g2, kThreads, smem, st>>>(s, lp, static_cast<C2*>(planes));
    QGB_LAUNCH_CHECK("k_xpass");
  }
  if (gather_after) QGB_CUDA_CHECK(cudaStreamWaitEvent(st, gather_after, 0));
  k_fft_yz_gather<T><<<g1, kThreads, smem, st>>>(s, lp, static_cast<const C2*>(C),
                                                static_cast<C2*>(out), static_cast<const C2*>(planes));
  QGB_LAUNCH_CHECK("k_fft_yz_gather");
  return QGB_OK;
}

template <typename T>
static int set_smem_limits(size_t smem) {
  int rc;
  if ((rc = raise_smem_limit(k_ifft_yz<T>, smem))) return rc;
  if ((rc = raise_smem_limit(k_xpass<T>, smem))) return rc;
  return raise_smem_limit(k_fft_yz_gather<T>, smem);
}

// gather_after (optional): an event the gather kernels wait for, so that a
// term written into `out` on another stream (QGB_ACCUMULATE) can be produced
// while the inverse and x passes run.
int apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb,
                    unsigned flags, void* ws, size_t ws_bytes, cudaStream_t st, cudaEvent_t gather_after = nullptr) {
  int rc = validate_sphere(s, dtype);
  if (rc) return rc;
  if (nb < 0) return fail(QGB_ERR_INVALID, "nb = %d < 0", nb);
  if (nb == 0) return QGB_OK;
  // C == out is allowed: every chunk reads its bands of C (k_ifft_yz, and the
  // KE term in k_fft_yz_gather before the same thread stores) before writing them.
  if (!C || !out) return fail(QGB_ERR_INVALID, "NULL wavefunction pointer");
  const size_t per_band = plane_bytes_per_band(*s, dtype);
  if (!ws || ws_bytes < per_band)
    return fail(QGB_ERR_WORKSPACE, "workspace %zu B < %zu B needed for one band", ws_bytes, per_band);
  const int chunk = static_cast<int>(std::min<size_t>(nb, std::min<size_t>(ws_bytes / per_band, 65535)));
  const size_t smem = plane_smem_bytes(*s, dtype);
  rc = (dtype == QGB_F64) ? set_smem_limits<double>(smem) : set_smem_limits<float>(smem);
  if (rc) return rc;
  for (int b0 = 0; b0 < nb; b0 += chunk) {
    LocalParams lp{nb, b0, std::min(chunk, nb - b0), flags};
    rc = (dtype == QGB_F64) ? launch_chunk<double>(*s, lp, C, out, ws, st, smem, gather_after)
                            : launch_chunk<float>(*s, lp, C, out, ws, st, smem, gather_after);
    if (rc) return rc;
  }
  return QGB_OK;
}

size_t sphere_smem_bytes(const qgb_sphere& s, int dtype) {
  size_t smem = plane_smem_bytes(s, dtype);
  if (xpass_async_ok(s, dtype)) smem = std::max(smem, xpass_async_smem_bytes(s));
  return smem;
}

// The y/z kernels get the y/z-phase shared memory and the x kernel its own
// (the largest sphere of the batch sets each): giving all three the largest
// size would cost the kernels of the smaller phase CTAs per SM.
template <typename T>
static int launch_batched(const qgb_batch_item* items, const int* slab_item, const long long* slab_starts,
                          const int* row_item, const long long* row_starts, long long n_slab, long long n_row,
                          size_t smem_yz, size_t smem_x, cudaStream_t st) {
  int rc;
  if ((rc = raise_smem_limit(k_ifft_yz_batched<T>, smem_yz))) return rc;
  if ((rc = raise_smem_limit(k_fft_yz_gather_batched<T>, smem_yz))) return rc;
  if ((rc = raise_smem_limit(k_xpass_batched<T>, smem_x))) return rc;
  // Units per CTA: up to 8 while the grid keeps at least 32 CTAs per SM.
  auto upc_for = [](long long n) { return static_cast<int>(std::max(1LL, std::min(8LL, n / (152LL * 32)))); };
  auto ctas = [](long long n, int upc) { return static_cast<unsigned>((n + upc - 1) / upc); };
  const int us = upc_for(n_slab), ur = upc_for(n_row);
  k_ifft_yz_batched<T><<<ctas(n_slab, us), kThreads, smem_yz, st>>>(items, slab_item, slab_starts, n_slab, us);
  QGB_LAUNCH_CHECK("k_ifft_yz_batched");
  k_xpass_batched<T><<<ctas(n_row, ur), kThreads, smem_x, st>>>(items, row_item, row_starts, n_row, ur);
  QGB_LAUNCH_CHECK("k_xpass_batched");
  k_fft_yz_gather_batched<T><<<ctas(n_slab, us), kThreads, smem_yz, st>>>(items, slab_item, slab_starts, n_slab,
                                                                          us);
  QGB_LAUNCH_CHECK("k_fft_yz_gather_batched");
  return QGB_OK;
}

int apply_potential_batched(const qgb_batch_item* items, int n_items, const int* slab_item,
                            const long long* slab_starts, const int* row_item, const long long* row_starts,
                            long long n_slab, long long n_row, int dtype, size_t smem_yz, size_t smem_x,
                            cudaStream_t st) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (n_items < 0 || n_slab < 0 || n_row < 0) return fail(QGB_ERR_INVALID, "negative batch sizes");
  if (n_items == 0 || n_slab == 0) return QGB_OK;
  if (!items || !slab_starts || !row_starts || !slab_item || !row_item) return fail(QGB_ERR_INVALID, "NULL batch table");
  if (n_slab > 0x7FFFFFFFLL || n_row > 0x7FFFFFFFLL) return fail(QGB_ERR_UNSUPPORTED, "batch too large for one grid");
  if (smem_yz > 227 * 1024 || smem_x > 227 * 1024)
    return fail(QGB_ERR_UNSUPPORTED, "batched shared memory %zu / %zu B > 227 KB", smem_yz, smem_x);
  if (smem_x < smem_yz) return fail(QGB_ERR_INVALID, "smem_x %zu < smem_yz %zu", smem_x, smem_yz);
  return dtype == QGB_F64 ? launch_batched<double>(items, slab_item, slab_starts, row_item, row_starts, n_slab, n_row,
                                                   smem_yz, smem_x, st)
                          : launch_batched<float>(items, slab_item, slab_starts, row_item, row_starts, n_slab, n_row,
                                                  smem_yz, smem_x, st);
}

int apply_ke(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, cudaStream_t st) {
  if (s == nullptr) return fail(QGB_ERR_INVALID, "sphere descriptor is NULL");
  if (nb < 0 || !C || !out || !s->ke) return fail(QGB_ERR_INVALID, "bad apply_ke arguments");
  if (nb == 0) return QGB_OK;
  const size_t total = static_cast<size_t>(s->nk) * nb * s->n_tot;
  const int blocks = static_cast<int>(std::min<size_t>((total + 255) / 256, 152 * 16));
  if (dtype == QGB_F64)
    k_apply_ke<double><<<blocks, 256, 0, st>>>(*s, nb, static_cast<const double2*>(C), static_cast<double2*>(out));
  else
    k_apply_ke<float><<<blocks, 256, 0, st>>>(*s, nb, static_cast<const float2*>(C), static_cast<float2*>(out));
  QGB_LAUNCH_CHECK("k_apply_ke");
  return QGB_OK;
}


// ---------------------------------------------------------------------------
// Density: rho(r) = sum_kb prefac[k][b] |psi_kb(r)|^2, psi = IFFT(scatter(C))
// (replaces Basis.collect_density, qimpy/dft/electrons/_basis_ops.py:207-296,
// single spin without spinors, with accum_norm_ of qimpy/math/_linalg.py:31-58).
// k_ifft_yz leaves each band's slab planes (y, z inverse-transformed); then
// k_density_x, one CTA per (k, y-row, z-range, group of bands): for each band
// of its group it stages the slab rows of its y-row, runs the inverse x-FFT and
// adds prefac |psi|^2 into per-thread register accumulators, and at the end
// adds them into rho (natural real-space order) with one atomicAdd per grid
// point.  rho is FP64 for both precisions.
// ---------------------------------------------------------------------------

template <typename T> struct DensityRegs { static constexpr int value = sizeof(T) == 4 ? 64 : 32; };

__device__ __forceinline__ int digit_perm(int p, int L1, int L2) { return p / L1 + L2 * (p - (p / L1) * L1); }

template <typename T>
__global__ void __launch_bounds__(kThreads) k_density_x(const qgb_sphere s, LocalParams lp,
                                                        const cplx_t<T>* __restrict__ planes,
                                                        const double* __restrict__ prefac, double* __restrict__ rho,
                                                        int zs, int bpc) {
  using C2 = cplx_t<T>;
  constexpr int R = DensityRegs<T>::value;
  const int N0 = s.N[0], N1 = s.N[1], N2 = s.N[2];
  const int r1 = blockIdx.x / zs, zp = blockIdx.x - r1 * zs;
  const int nz_max = (N2 + zs - 1) / zs, z0 = zp * nz_max;
  const int nz = min(nz_max, N2 - z0);
  const int k = blockIdx.z;
  if (nz <= 0) return;
  const int ld = nz + 1, lim = N0 * ld, Wx = lim;
  C2* sm = smem_c<T>();
  const C2* tw = static_cast<const C2*>(s.twiddle);
  load_twiddles<T>(Wx, tw + s.tw_off[0], N0);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int nslabs = s.n_slabs[k];
  const int* i0 = s.slab_i0 + k * s.max_slabs;
  const size_t plane = static_cast<size_t>(N1) * N2;
  const int total = N0 * nz;  // <= R * kThreads (host-checked)
  const int step_px = kThreads / nz, step_c = kThreads - step_px * nz;
  T acc[R];
#pragma unroll
  for (int j = 0; j < R; ++j) acc[j] = T(0);
  const int b_begin = blockIdx.y * bpc, b_end = min(lp.nb, b_begin + bpc);
  for (int b = b_begin; b < b_end; ++b) {
    for (int r = warp; r < N0; r += nwarps)
      for (int c = lane; c < nz; c += 32) sm[r * ld + c] = mk<T>(T(0), T(0));
    __syncthreads();
    if (!QGB_OK_IDX(plane_index(s, k, b, lp.nb, 0), (long long)s.nk * lp.nb * s.max_slabs, 20)) return;
    const C2* base = planes + plane_index(s, k, b, lp.nb, 0) * plane + static_cast<size_t>(r1) * N2 + z0;
    for (int sl = warp; sl < nslabs; sl += nwarps) {
      const int x = i0[sl];
      for (int c = lane; c < nz; c += 32) sm[x * ld + c] = base[sl * plane + c];
    }
    __syncthreads();
    fft_inverse<T>(0, nullptr, nz, 1, ld, s.L1[0], s.L2[0], Wx, lim);  // ends with __syncthreads
    const T w = static_cast<T>(prefac[static_cast<size_t>(k) * lp.nb_total + lp.b0 + b]);
    int px = threadIdx.x / nz, c = threadIdx.x - (threadIdx.x / nz) * nz;
#pragma unroll
    for (int j = 0; j < R; ++j) {
      if (j * kThreads + static_cast<int>(threadIdx.x) < total) {
        const C2 v = sm[px * ld + c];
        acc[j] += w * (v.x * v.x + v.y * v.y);
      }
      px += step_px;
      c += step_c;
      if (c >= nz) {
        c -= nz;
        ++px;
      }
    }
    __syncthreads();  // the tile is refilled for the next band
  }
  // Natural real-space order: every axis of the stored data is digit-permuted.
  const int y = digit_perm(r1, s.L1[1], s.L2[1]);
  int px = threadIdx.x / nz, c = threadIdx.x - (threadIdx.x / nz) * nz;
#pragma unroll
  for (int j = 0; j < R; ++j) {
    if (j * kThreads + static_cast<int>(threadIdx.x) < total) {
      const int x = digit_perm(px, s.L1[0], s.L2[0]);
      const int z = digit_perm(z0 + c, s.L1[2], s.L2[2]);
      atomicAdd(rho + (static_cast<size_t>(x) * N1 + y) * N2 + z, static_cast<double>(acc[j]));
    }
    px += step_px;
    c += step_c;
    if (c >= nz) {
      c -= nz;
      ++px;
    }
  }
}

static int density_zsplit(const qgb_sphere& s, int dtype) {
  const long long cap = static_cast<long long>(dtype == QGB_F64 ? DensityRegs<double>::value
                                                                : DensityRegs<float>::value) * kThreads;
  int zs = 1;
  while (static_cast<long long>(s.N[0]) * ((s.N[2] + zs - 1) / zs) > cap) ++zs;
  return zs;
}

template <typename T>
static int launch_density_chunk(const qgb_sphere& s, const LocalParams& lp, const void* C, void* planes,
                                const double* prefac, double* rho, size_t smem_yz, cudaStream_t st) {
  using C2 = cplx_t<T>;
  const dim3 g1(s.max_slabs, lp.nb, s.nk);
  k_ifft_yz<T><<<g1, kThreads, smem_yz, st>>>(s, lp, static_cast<const C2*>(C), static_cast<C2*>(planes));
  QGB_LAUNCH_CHECK("k_ifft_yz");
  const int zs = density_zsplit(s, sizeof(T) == 8 ? QGB_F64 : QGB_F32);
  const int nz = (s.N[2] + zs - 1) / zs;
  const size_t smem = (static_cast<size_t>(s.N[0]) * (nz + 1) + s.N[0]) * sizeof(C2);
  if (int rc = raise_smem_limit(k_density_x<T>, smem)) return rc;
  // Groups of bands per CTA: enough CTAs to cover the SMs a few times over.
  const long long base = static_cast<long long>(s.N[1]) * zs * s.nk;
  const int groups = static_cast<int>(std::min<long long>(lp.nb, std::max<long long>(1, (4LL * 152 + base - 1) / base)));
  const int bpc = (lp.nb + groups - 1) / groups;
  const dim3 g2(s.N[1] * zs, (lp.nb + bpc - 1) / bpc, s.nk);
  k_density_x<T><<<g2, kThreads, smem, st>>>(s, lp, static_cast<const C2*>(planes), prefac, rho, zs, bpc);
  QGB_LAUNCH_CHECK("k_density_x");
  return QGB_OK;
}

int collect_density(const qgb_sphere* s, int dtype, const void* C, int nb, const double* prefac, double* rho,
                    unsigned flags, void* ws, size_t ws_bytes, cudaStream_t st) {
  int rc = validate_sphere(s, dtype, false);  // the density needs no potential
  if (rc) return rc;
  if (nb < 0) return fail(QGB_ERR_INVALID, "nb = %d < 0", nb);
  if (!rho) return fail(QGB_ERR_INVALID, "NULL density pointer");
  const size_t N = static_cast<size_t>(s->N[0]) * s->N[1] * s->N[2];
  if (!(flags & QGB_ACCUMULATE)) QGB_CUDA_CHECK(cudaMemsetAsync(rho, 0, N * sizeof(double), st));
  if (nb == 0) return QGB_OK;
  if (!C || !prefac) return fail(QGB_ERR_INVALID, "NULL wavefunction or prefactor pointer");
  const size_t per_band = plane_bytes_per_band(*s, dtype);
  if (!ws || ws_bytes < per_band)
    return fail(QGB_ERR_WORKSPACE, "workspace %zu B < %zu B needed for one band", ws_bytes, per_band);
  const int chunk = static_cast<int>(std::min<size_t>(nb, std::min<size_t>(ws_bytes / per_band, 65535)));
  const size_t smem = plane_smem_bytes(*s, dtype);
  rc = (dtype == QGB_F64) ? set_smem_limits<double>(smem) : set_smem_limits<float>(smem);
  if (rc) return rc;
  for (int b0 = 0; b0 < nb; b0 += chunk) {
    LocalParams lp{nb, b0, std::min(chunk, nb - b0), 0u};
    rc = (dtype == QGB_F64) ? launch_density_chunk<double>(*s, lp, C, ws, prefac, rho, smem, st)
                            : launch_density_chunk<float>(*s, lp, C, ws, prefac, rho, smem, st);
    if (rc) return rc;
  }
  return QGB_OK;
}

}  // namespace qgb
