// Shared types and error plumbing of the qimpy_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/qimpy_gb300.h"

namespace qgb {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };
template <typename T> using cplx_t = typename Cplx<T>::type;

template <typename T> __device__ __forceinline__ cplx_t<T> mk(T x, T y) {
  cplx_t<T> r;
  r.x = x;
  r.y = y;
  return r;
}

// Debug builds (-DQGB_DEBUG_CHECKS) range-check every shared and global access of
// the local-potential kernels: a violation records (site, index, limit) in a device
// word and the access is skipped, so a bad index is reported instead of faulting.
#ifdef QGB_DEBUG_CHECKS
static __device__ unsigned long long g_qgb_violation[4];
__device__ __forceinline__ bool qgb_in_range(long long idx, long long lim, int site) {
  if (idx >= 0 && idx < lim) return true;
  if (atomicCAS(&g_qgb_violation[0], 0ull, (unsigned long long)site) == 0ull) {
    g_qgb_violation[1] = (unsigned long long)idx;
    g_qgb_violation[2] = (unsigned long long)lim;
    g_qgb_violation[3] = ((unsigned long long)blockIdx.x << 32) | (blockIdx.y << 16) | blockIdx.z;
  }
  return false;
}
#define QGB_OK_IDX(idx, lim, site) ::qgb::qgb_in_range((long long)(idx), (long long)(lim), (site))
#else
#define QGB_OK_IDX(idx, lim, site) true
#endif

// Error state of the calling host thread.
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);

#define QGB_CUDA_CHECK(expr)                                                        \
  do {                                                                              \
    cudaError_t e_ = (expr);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return ::qgb::fail(QGB_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,              \
                         cudaGetErrorString(e_), __FILE__, __LINE__);               \
  } while (0)

#define QGB_LAUNCH_CHECK(what)                                                      \
  do {                                                                              \
    cudaError_t e_ = cudaGetLastError();                                            \
    if (e_ != cudaSuccess)                                                          \
      return ::qgb::fail(QGB_ERR_CUDA, "launch of %s failed: %s", what,             \
                         cudaGetErrorString(e_));                                   \
  } while (0)

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`.  The attribute belongs to the device's context, so the size
// raised so far is kept per (kernel, device); the check and the raise are one
// step under a lock, so host threads launching for different sizes cannot
// lower a limit another thread is about to launch with.
int raise_smem_limit(const void* kernel, size_t bytes);
template <typename K>
inline int raise_smem_limit(K* kernel, size_t bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(kernel), bytes);
}

inline size_t elem_bytes(int dtype) { return dtype == QGB_F64 ? 16 : 8; }
inline size_t real_bytes(int dtype) { return dtype == QGB_F64 ? 8 : 4; }

}  // namespace qgb
