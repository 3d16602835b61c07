// Band-wise passes of the Davidson iteration, each one read of the bands
// (one CTA per (k, band) row, FP64 sums in a fixed tree order):
//
//   band_norm_ke  ||c_b|| and sum_g |c_bg|^2 KE_g
//                 (Wavefunction.band_norm / band_ke, qimpy/dft/electrons/_wavefunction.py:226-247)
//   residual      R = HC - eps C, optionally preconditioned R / (x + e^-x) with
//                 x = KE / KEref_b, stored and/or reduced to ||R||
//                 (qimpy/dft/electrons/_davidson.py:92-99 and 177-180)
//   normalize     null bands (norm below a cut) re-randomised with the seeded
//                 xorshift generator, then C_b / ||C_b|| with the padding zeroed
//                 (_davidson.py:101-115 and 181-183; Wavefunction.randomize_selected,
//                 _wavefunction_init.py:127-188; constrain, _wavefunction.py:264-275)
//
// The null-band test runs on the device, so an iteration needs no host
// synchronisation to decide whether to randomise.
#include "qgb_common.cuh"

namespace qgb {
namespace dvo {

constexpr int kThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kThreads / 32; ++w) s += red[w];
  return s;  // valid in thread 0
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_band_stats(const cplx_t<T>* __restrict__ C, int nb_all, int b0, int nb, int n_tot,
                 const double* __restrict__ ke, const double* __restrict__ weight, double* __restrict__ norm,
                 double* __restrict__ bke) {
  __shared__ double red[2][kThreads / 32];
  const int row = blockIdx.x, k = row / nb, b = row - k * nb;
  const cplx_t<T>* c = C + (static_cast<long long>(k) * nb_all + b0 + b) * n_tot;
  const double* kek = ke ? ke + static_cast<long long>(k) * n_tot : nullptr;
  double s0 = 0.0, s1 = 0.0;
  for (int g = threadIdx.x; g < n_tot; g += kThreads) {
    const cplx_t<T> v = c[g];
    double a = static_cast<double>(v.x) * v.x + static_cast<double>(v.y) * v.y;
    if (weight) a *= weight[g];
    s0 += a;
    if (kek) s1 += a * kek[g];
  }
  s0 = block_sum(s0, red[0]);
  s1 = block_sum(s1, red[1]);
  if (threadIdx.x == 0) {
    if (norm) norm[row] = sqrt(s0);
    if (bke) bke[row] = s1;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_residual(const cplx_t<T>* __restrict__ HC, const cplx_t<T>* __restrict__ C, int nb_all, int b0, int nb,
               int n_tot, const double* __restrict__ eig, int eig_ld, const double* __restrict__ ke,
               const double* __restrict__ KEref, const double* __restrict__ weight, cplx_t<T>* __restrict__ out,
               double* __restrict__ norm) {
  __shared__ double red[kThreads / 32];
  const int row = blockIdx.x, k = row / nb, b = row - k * nb;
  const long long off = (static_cast<long long>(k) * nb_all + b0 + b) * n_tot;
  const cplx_t<T>* h = HC + off;
  const cplx_t<T>* c = C + off;
  cplx_t<T>* o = out ? out + static_cast<long long>(row) * n_tot : nullptr;
  const T e = static_cast<T>(eig[static_cast<long long>(k) * eig_ld + b0 + b]);
  const bool pre = KEref != nullptr;
  const T inv_ref = pre ? static_cast<T>(1.0 / KEref[row]) : T(0);
  const double* kek = pre ? ke + static_cast<long long>(k) * n_tot : nullptr;
  double s = 0.0;
  for (int g = threadIdx.x; g < n_tot; g += kThreads) {
    const cplx_t<T> hv = h[g], cv = c[g];
    T rx = hv.x - e * cv.x, ry = hv.y - e * cv.y;
    if (pre) {
      T x = static_cast<T>(kek[g]) * inv_ref;
      x += exp(-x);  // stays ~1 where KE ~ 0
      rx /= x;
      ry /= x;
    }
    if (o) o[g] = mk<T>(rx, ry);
    const double a = static_cast<double>(rx) * rx + static_cast<double>(ry) * ry;
    s += weight ? a * weight[g] : a;
  }
  if (norm) {
    s = block_sum(s, red);
    if (threadIdx.x == 0) norm[row] = sqrt(s);
  }
}

// One draw of the reference's generator: xorshift (13, 7, 17) on a signed
// 64-bit state (left shifts wrap, the right shift is arithmetic), mapped to a
// uniform in (0, 1) as 2^-64 x + 1/2.
__device__ __forceinline__ double xorshift_uniform(long long& x) {
  x ^= static_cast<long long>(static_cast<unsigned long long>(x) << 13);
  x ^= x >> 7;
  x ^= static_cast<long long>(static_cast<unsigned long long>(x) << 17);
  return ldexp(static_cast<double>(x), -64) + 0.5;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_normalize(cplx_t<T>* __restrict__ X, int nb, int n_tot, const int* __restrict__ n, double* __restrict__ norm,
                double cut, long long seed, long long n_max, const double* __restrict__ ke) {
  const int row = blockIdx.x, k = row / nb, b = row - k * nb;
  cplx_t<T>* x = X + static_cast<long long>(row) * n_tot;
  const double nv = norm[row];
  const bool low = nv < cut;
  const int nk_g = n[k];
  const T scale = low ? T(1) : static_cast<T>(1.0 / nv);
  const double* kek = ke + static_cast<long long>(k) * n_tot;
  for (int g = threadIdx.x; g < n_tot; g += kThreads) {
    cplx_t<T> v = mk<T>(T(0), T(0));
    if (g < nk_g) {
      if (low) {
        long long st = (1 + seed) + g + n_max * (b + static_cast<long long>(nb) * k);
        xorshift_uniform(st);  // warm-up pair: one complex deviate discarded
        xorshift_uniform(st);
        const double u0 = xorshift_uniform(st), u1 = xorshift_uniform(st);
        const double amp = sqrt(-2.0 * log(u0));
        double sn, cs;
        sincospi(2.0 * u1, &sn, &cs);
        const double t = (4.0 / 3.0) * kek[g], t2 = t * t;
        const double damp = 1.0 / (1.0 + t2 * t2 * t2);
        v = mk<T>(static_cast<T>(amp * cs * damp), static_cast<T>(amp * sn * damp));
      } else {
        const cplx_t<T> c = x[g];
        v = mk<T>(c.x * scale, c.y * scale);
      }
    }
    x[g] = v;
  }
  __syncthreads();
  if (low && threadIdx.x == 0) norm[row] = 1.0;  // the reference's estimate for a randomised band
}

}  // namespace dvo

using namespace dvo;

static int rows_ok(int nk, int nb, int n_tot) {
  if (nk < 0 || nb < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad band extents (nk %d, nb %d, n_tot %d)", nk, nb, n_tot);
  if (static_cast<long long>(nk) * nb > 0x7fffffffLL) return fail(QGB_ERR_INVALID, "too many bands");
  return QGB_OK;
}

}  // namespace qgb

using namespace qgb;

extern "C" int qgb_band_norm_ke(int dtype, const void* C, int nb_all, int b0, int nb, int nk, int n_tot,
                                const double* ke, const double* weight, double* norm, double* band_ke, void* stream) {
  if (int rc = rows_ok(nk, nb, n_tot)) return rc;
  if (b0 < 0 || b0 + nb > nb_all) return fail(QGB_ERR_INVALID, "bands [%d, %d) outside %d", b0, b0 + nb, nb_all);
  if (nk * nb == 0) return QGB_OK;
  if (!C || (band_ke && !ke)) return fail(QGB_ERR_INVALID, "NULL pointer in band_norm_ke");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == QGB_F64)
    k_band_stats<double><<<nk * nb, kThreads, 0, st>>>(static_cast<const double2*>(C), nb_all, b0, nb, n_tot, ke,
                                                       weight, norm, band_ke);
  else if (dtype == QGB_F32)
    k_band_stats<float><<<nk * nb, kThreads, 0, st>>>(static_cast<const float2*>(C), nb_all, b0, nb, n_tot, ke,
                                                      weight, norm, band_ke);
  else
    return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  QGB_LAUNCH_CHECK("k_band_stats");
  return QGB_OK;
}

extern "C" int qgb_residual(int dtype, const void* HC, const void* C, int nb_all, int b0, int nb, int nk, int n_tot,
                            const double* eig, int eig_ld, const double* ke, const double* KEref, const double* weight,
                            void* out, double* norm, void* stream) {
  if (int rc = rows_ok(nk, nb, n_tot)) return rc;
  if (b0 < 0 || b0 + nb > nb_all || b0 + nb > eig_ld)
    return fail(QGB_ERR_INVALID, "bands [%d, %d) outside %d (eig_ld %d)", b0, b0 + nb, nb_all, eig_ld);
  if (nk * nb == 0) return QGB_OK;
  if (!HC || !C || !eig || (KEref && !ke)) return fail(QGB_ERR_INVALID, "NULL pointer in residual");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == QGB_F64)
    k_residual<double><<<nk * nb, kThreads, 0, st>>>(static_cast<const double2*>(HC), static_cast<const double2*>(C),
                                                     nb_all, b0, nb, n_tot, eig, eig_ld, ke, KEref, weight,
                                                     static_cast<double2*>(out), norm);
  else if (dtype == QGB_F32)
    k_residual<float><<<nk * nb, kThreads, 0, st>>>(static_cast<const float2*>(HC), static_cast<const float2*>(C),
                                                    nb_all, b0, nb, n_tot, eig, eig_ld, ke, KEref, weight,
                                                    static_cast<float2*>(out), norm);
  else
    return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  QGB_LAUNCH_CHECK("k_residual");
  return QGB_OK;
}

extern "C" int qgb_normalize_bands(int dtype, void* X, int nb, int nk, int n_tot, const int32_t* n, double* norm,
                                   double norm_cut, long long seed, long long n_max, const double* ke, void* stream) {
  if (int rc = rows_ok(nk, nb, n_tot)) return rc;
  if (nk * nb == 0) return QGB_OK;
  if (!X || !n || !norm || !ke) return fail(QGB_ERR_INVALID, "NULL pointer in normalize_bands");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == QGB_F64)
    k_normalize<double><<<nk * nb, kThreads, 0, st>>>(static_cast<double2*>(X), nb, n_tot, n, norm, norm_cut, seed,
                                                      n_max, ke);
  else if (dtype == QGB_F32)
    k_normalize<float><<<nk * nb, kThreads, 0, st>>>(static_cast<float2*>(X), nb, n_tot, n, norm, norm_cut, seed,
                                                     n_max, ke);
  else
    return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  QGB_LAUNCH_CHECK("k_normalize");
  return QGB_OK;
}
