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

inline size_t elem_bytes(int dtype) { return dtype == QGB_F64 ? 16 : 8; }
inline size_t real_bytes(int dtype) { return dtype == QGB_F64 ? 8 : 4; }

}  // namespace qgb
