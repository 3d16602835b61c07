// Projectors beta[k][p][g] generated on the device.
//
// Replaces Ions.get_projectors (qimpy/dft/ions/_ions_projectors.py:14-72):
//   beta[k][a pa + j][g] = i^l S_lm(q) R_s(|q|) exp(-2 pi i (iG + k) . tau_a) / sqrt(Omega),
//   q = (iG + k) Gbasis^T,
// for every atom a (fractional position tau_a) and every projector j of the
// atom template (shells s of angular momentum l, all 2l + 1 real solid
// harmonics S_lm(q) = |q|^l Y_lm, m = -l..l, l = 1 ordered (y, z, x) as in
// qimpy/math/spherical_harmonics.py:80-83; i^l is the reference's reciprocal
// phase, get_harmonics_tilde, spherical_harmonics.py:111-137).  The radial
// part R_s is either
//   * a Gaussian shell: (-1)^l (2 pi)^{3/2} sigma^{2l+3} exp(-sigma^2 |q|^2 / 2),
//     so that beta is the Fourier transform of r^l Y_lm exp(-r^2 / (2 sigma^2)); or
//   * a quintic blip spline on a uniform |q| grid of spacing dq, evaluated like
//     the reference's Interpolator (qimpy/math/quintic_spline.py:57-130):
//     R(x) = sum_{j<6} c[i + j] sum_{p<6} t^p B[p][j], i = floor(x/dq),
//     t = x/dq - i, with B the quintic B-spline's polynomial pieces.
// Padding entries (g >= n[k]) are zero.  One thread per (k, g): the template
// values of all shells are formed once, then every atom's phase multiplies
// them and each store is coalesced along g.
#include <algorithm>

#include "qgb_common.cuh"

namespace qgb {
namespace pj {

constexpr int kThreads = 128;
constexpr int kMaxShells = 8;
constexpr int kMaxPAtom = 40;  // kMaxShells shells of l <= 2

struct Params {
  int nk, n_tot, n_atoms, n_shells, p_atom;
  double Gb[9];  // row-major: q_i = sum_j Gb[3 i + j] (iG_j + k_j)
  double inv_sqrt_vol;
  int l[kMaxShells], kind[kMaxShells], n_coeff[kMaxShells];
  double sigma[kMaxShells], dq[kMaxShells];
  const double* coeff[kMaxShells];
};

// Quintic B-spline pieces: weight of coefficient c[i + j] at fractional
// position t is sum_p t^p kBlip[p][j] / 66.
__constant__ double kBlip[6][6] = {
    {+1.0, 26.0, 66.0, 26.0, 1.0, 0.0},   {-5.0, -50.0, 0.0, 50.0, 5.0, 0.0},
    {+10.0, 20.0, -60.0, 20.0, 10.0, 0.0}, {-10.0, 20.0, 0.0, -20.0, 10.0, 0.0},
    {+5.0, -20.0, 30.0, -20.0, 5.0, 0.0},  {-1.0, 5.0, -10.0, 10.0, -5.0, 1.0}};

__device__ double blip_eval(const double* __restrict__ c, int n_coeff, double dq, double x) {
  const double u = x / dq;
  const int i = static_cast<int>(floor(u));
  const double t = u - i;
  double tp[6];
  tp[0] = 1.0;
#pragma unroll
  for (int p = 1; p < 6; ++p) tp[p] = tp[p - 1] * t;
  double y = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int idx = i + j;
    if (idx < 0 || idx >= n_coeff) continue;  // outside the table: no contribution
    double f = 0.0;
#pragma unroll
    for (int p = 0; p < 6; ++p) f += tp[p] * kBlip[p][j];
    y += c[idx] * (f * (1.0 / 66.0));
  }
  return y;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_projectors(const Params P, const int* __restrict__ n,
                                                         const int* __restrict__ iG, const double* __restrict__ kpt,
                                                         const double* __restrict__ pos, cplx_t<T>* __restrict__ beta) {
  const int k = blockIdx.y;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= P.n_tot) return;
  const long long P_tot = static_cast<long long>(P.n_atoms) * P.p_atom;
  cplx_t<T>* out = beta + static_cast<long long>(k) * P_tot * P.n_tot + g;
  if (g >= n[k]) {
    for (long long p = 0; p < P_tot; ++p) out[p * P.n_tot] = mk<T>(T(0), T(0));
    return;
  }
  const int* ig = iG + (static_cast<long long>(k) * P.n_tot + g) * 3;
  const double f0 = ig[0] + kpt[3 * k], f1 = ig[1] + kpt[3 * k + 1], f2 = ig[2] + kpt[3 * k + 2];
  const double x = P.Gb[0] * f0 + P.Gb[1] * f1 + P.Gb[2] * f2;
  const double y = P.Gb[3] * f0 + P.Gb[4] * f1 + P.Gb[5] * f2;
  const double z = P.Gb[6] * f0 + P.Gb[7] * f1 + P.Gb[8] * f2;
  const double q2 = x * x + y * y + z * z;
  // Template values i^l S_lm(q) R_s(|q|), as (re, im).
  double tre[kMaxPAtom], tim[kMaxPAtom];
  int j = 0;
  for (int s = 0; s < P.n_shells; ++s) {
    const int l = P.l[s];
    double R;
    if (P.kind[s] == QGB_RADIAL_GAUSSIAN) {
      const double sg = P.sigma[s];
      double pw = sg * sg * sg;
      for (int e = 0; e < l; ++e) pw *= sg * sg;
      R = 15.749609945722419 * pw * exp(-0.5 * sg * sg * q2);  // (2 pi)^{3/2} sigma^{2l+3}
      if (l & 1) R = -R;
    } else {
      R = blip_eval(P.coeff[s], P.n_coeff[s], P.dq[s], sqrt(q2));
    }
    double S[5];
    int nm;
    if (l == 0) {
      S[0] = 0.28209479177387814;  // 1 / (2 sqrt(pi))
      nm = 1;
    } else if (l == 1) {
      const double c1 = 0.4886025119029199;  // sqrt(3 / (4 pi))
      S[0] = c1 * y;
      S[1] = c1 * z;
      S[2] = c1 * x;
      nm = 3;
    } else {
      const double a = 1.0925484305920792, b = 0.31539156525252005, c = 0.5462742152960396;
      S[0] = a * x * y;
      S[1] = a * y * z;
      S[2] = b * (3.0 * z * z - q2);
      S[3] = a * x * z;
      S[4] = c * (x * x - y * y);
      nm = 5;
    }
    // i^l: 1, i, -1, -i
    for (int m = 0; m < nm; ++m, ++j) {
      const double v = S[m] * R;
      switch (l & 3) {
        case 0: tre[j] = v; tim[j] = 0.0; break;
        case 1: tre[j] = 0.0; tim[j] = v; break;
        case 2: tre[j] = -v; tim[j] = 0.0; break;
        default: tre[j] = 0.0; tim[j] = -v; break;
      }
    }
  }
  for (int a = 0; a < P.n_atoms; ++a) {
    const double t = f0 * pos[3 * a] + f1 * pos[3 * a + 1] + f2 * pos[3 * a + 2];
    double sn, cs;
    sincospi(-2.0 * t, &sn, &cs);
    cs *= P.inv_sqrt_vol;
    sn *= P.inv_sqrt_vol;
    cplx_t<T>* o = out + static_cast<long long>(a) * P.p_atom * P.n_tot;
    for (int jj = 0; jj < P.p_atom; ++jj)
      o[static_cast<long long>(jj) * P.n_tot] =
          mk<T>(static_cast<T>(tre[jj] * cs - tim[jj] * sn), static_cast<T>(tre[jj] * sn + tim[jj] * cs));
  }
}

}  // namespace pj
}  // namespace qgb

using namespace qgb;

extern "C" int qgb_make_projectors(int dtype, int nk, int n_tot, const int32_t* n, const int32_t* iG,
                                   const double* k, const double* Gbasis, int n_atoms, const double* positions,
                                   int n_shells, const qgb_projector_shell* shells, double volume, void* beta,
                                   void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (nk < 0 || n_tot < 0 || n_atoms < 0 || n_shells < 0) return fail(QGB_ERR_INVALID, "negative sizes");
  if (n_shells > pj::kMaxShells) return fail(QGB_ERR_UNSUPPORTED, "%d shells > %d", n_shells, pj::kMaxShells);
  if (!(volume > 0.0)) return fail(QGB_ERR_INVALID, "cell volume %g <= 0", volume);
  if (!Gbasis || (n_shells && !shells)) return fail(QGB_ERR_INVALID, "NULL Gbasis or shells");
  pj::Params P{};
  P.nk = nk;
  P.n_tot = n_tot;
  P.n_atoms = n_atoms;
  P.n_shells = n_shells;
  for (int i = 0; i < 9; ++i) P.Gb[i] = Gbasis[i];
  P.inv_sqrt_vol = 1.0 / sqrt(volume);
  int p_atom = 0;
  for (int s = 0; s < n_shells; ++s) {
    const qgb_projector_shell& sh = shells[s];
    if (sh.l < 0 || sh.l > 2) return fail(QGB_ERR_UNSUPPORTED, "shell %d: l = %d (0..2 supported)", s, sh.l);
    if (sh.kind == QGB_RADIAL_GAUSSIAN) {
      if (!(sh.sigma > 0.0)) return fail(QGB_ERR_INVALID, "shell %d: sigma %g <= 0", s, sh.sigma);
    } else if (sh.kind == QGB_RADIAL_BLIP) {
      if (!sh.coeff || sh.n_coeff < 6 || !(sh.dq > 0.0))
        return fail(QGB_ERR_INVALID, "shell %d: blip table needs coeff, n_coeff >= 6 and dq > 0", s);
    } else {
      return fail(QGB_ERR_INVALID, "shell %d: unknown radial kind %d", s, sh.kind);
    }
    P.l[s] = sh.l;
    P.kind[s] = sh.kind;
    P.sigma[s] = sh.sigma;
    P.coeff[s] = sh.coeff;
    P.n_coeff[s] = sh.n_coeff;
    P.dq[s] = sh.dq;
    p_atom += 2 * sh.l + 1;
  }
  P.p_atom = p_atom;
  if (nk == 0 || n_tot == 0 || n_atoms == 0 || p_atom == 0) return QGB_OK;
  if (nk > 65535) return fail(QGB_ERR_UNSUPPORTED, "nk %d > 65535", nk);
  if (!n || !iG || !k || !positions || !beta) return fail(QGB_ERR_INVALID, "NULL device pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 grid((n_tot + pj::kThreads - 1) / pj::kThreads, nk);
  if (dtype == QGB_F64)
    pj::k_projectors<double><<<grid, pj::kThreads, 0, st>>>(P, n, iG, k, positions, static_cast<double2*>(beta));
  else
    pj::k_projectors<float><<<grid, pj::kThreads, 0, st>>>(P, n, iG, k, positions, static_cast<float2*>(beta));
  QGB_LAUNCH_CHECK("k_projectors");
  return QGB_OK;
}
