// Real (Gamma-point) wavefunctions on the half-sphere basis.
//
// The reference stores a real wavefunction by its coefficients on the half
// mesh Gz >= 0 (qimpy/dft/electrons/_basis_real.py:10-106; H-mesh basis at
// _basis.py:168) and transforms it with c2r / r2c FFTs (_basis_ops.py:119-163,
// qimpy/grid/_fft.py).  Here two real bands travel in one complex transform of
// the full Gamma sphere: with c(-G) = conj(c(G)),
//     z(G) = c_a(G) + i c_b(G)  <->  z(r) = psi_a(r) + i psi_b(r), both real,
// so V z(r) = V psi_a + i V psi_b and its transform W(G) gives back
//     (V psi_a)(G) = (W(G) + conj(W(-G))) / 2,
//     (V psi_b)(G) = (W(G) - conj(W(-G))) / (2i).
// The local potential of nb real bands therefore costs the complex kernels'
// work for ceil(nb / 2) bands:
//   k_pack_real     half-basis pairs of bands -> full-sphere complex rows
//   (apply_potential on the full sphere, local_potential.cu)
//   k_unpack_real   full-sphere rows -> half-basis bands (+ KE C)
// The unpacked Gz = 0 plane is Hermitian by construction, as the reference's
// symmetrisation (BasisReal.symmetrize, _basis_real.py:68-106) makes it;
// k_symmetrize_real applies that symmetrisation to other half-basis bands.
// Overlaps and projections use the weights 1 (Gz = 0) / 2 (elsewhere) and
// keep the real part (_wavefunction_dot.py:55-88).
#include <algorithm>

#include "bandgemm.cuh"

namespace qgb {

int validate_sphere(const qgb_sphere* s, int dtype, bool need_potential = true);
size_t plane_bytes_per_band(const qgb_sphere& s, int dtype);
int apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, unsigned flags,
                    void* ws, size_t ws_bytes, cudaStream_t st,
                    cudaEvent_t gather_after = nullptr);

namespace rb {

constexpr int kThreads = 256;
constexpr unsigned kConj = 0x80000000u;

// Half-basis coefficient of one full-sphere entry e = pack[j]: c[h0] (Gz > 0),
// conj(c[h0]) (Gz < 0, bit 31 of e.x), or on the Gz = 0 plane the Hermitian
// part (c[h0] + conj(c[h1])) / 2 with h1 = e.y the half index of -G -- what
// the reference's c2r transform sees of a plane that is not Hermitian.
template <typename T>
__device__ __forceinline__ cplx_t<T> half_coeff(const cplx_t<T>* __restrict__ c, int2 e) {
  const unsigned e0 = static_cast<unsigned>(e.x);
  cplx_t<T> a = c[e0 & ~kConj];
  if (e0 & kConj) a.y = -a.y;
  if (e.y >= 0) {
    const cplx_t<T> p = c[e.y];
    a = mk<T>(T(0.5) * (a.x + p.x), T(0.5) * (a.y - p.y));
  }
  return a;
}

template <typename T>
__global__ void k_pack_real(const cplx_t<T>* __restrict__ C, int nb, int n_tot_half, const int2* __restrict__ pack,
                            int n_full, int n_tot_full, cplx_t<T>* __restrict__ Z) {
  const int q = blockIdx.y;
  const int b0 = 2 * q, b1 = 2 * q + 1;
  const cplx_t<T>* ca = C + static_cast<long long>(b0) * n_tot_half;
  const cplx_t<T>* cb = C + static_cast<long long>(b1) * n_tot_half;
  cplx_t<T>* z = Z + static_cast<long long>(q) * n_tot_full;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n_tot_full; j += gridDim.x * blockDim.x) {
    cplx_t<T> v = mk<T>(T(0), T(0));
    if (j < n_full) {
      const int2 e = __ldg(pack + j);
      const cplx_t<T> a = half_coeff<T>(ca, e);
      const cplx_t<T> b = b1 < nb ? half_coeff<T>(cb, e) : mk<T>(T(0), T(0));
      v = mk<T>(a.x - b.y, a.y + b.x);  // a + i b
    }
    z[j] = v;
  }
}

template <typename T>
__global__ void k_unpack_real(const cplx_t<T>* __restrict__ W, int n_tot_full, const int* __restrict__ unpack,
                              int n_half, const cplx_t<T>* __restrict__ C, const T* __restrict__ ke, int nb,
                              int n_tot_half, unsigned flags, cplx_t<T>* __restrict__ out) {
  const int b = blockIdx.y;
  const cplx_t<T>* w = W + static_cast<long long>(b / 2) * n_tot_full;
  const cplx_t<T>* c = C + static_cast<long long>(b) * n_tot_half;
  cplx_t<T>* o = out + static_cast<long long>(b) * n_tot_half;
  const bool odd = b & 1;
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < n_tot_half; h += gridDim.x * blockDim.x) {
    T x = T(0), y = T(0);
    if (h < n_half) {
      const cplx_t<T> wp = w[__ldg(unpack + 2 * h)], wm = w[__ldg(unpack + 2 * h + 1)];
      if (!odd) {  // (W(G) + conj(W(-G))) / 2
        x = T(0.5) * (wp.x + wm.x);
        y = T(0.5) * (wp.y - wm.y);
      } else {  // (W(G) - conj(W(-G))) / (2i)
        x = T(0.5) * (wp.y + wm.y);
        y = T(-0.5) * (wp.x - wm.x);
      }
      if (flags & QGB_ADD_KE) {
        const cplx_t<T> cv = c[h];
        const T e = ke[h];
        x += e * cv.x;
        y += e * cv.y;
      }
    }
    if (flags & QGB_ACCUMULATE) {
      const cplx_t<T> ov = o[h];
      x += ov.x;
      y += ov.y;
    }
    o[h] = mk<T>(x, y);
  }
}

// c(G) <- (c(G) + conj(c(-G))) / 2 on the Gz = 0 plane, pairs (h, partner):
// the lower index of a pair writes both entries; a self-partner (G = 0) keeps
// its real part.
template <typename T>
__global__ void k_symmetrize_real(cplx_t<T>* __restrict__ X, int n_tot_half, const int* __restrict__ plane,
                                  int n_plane) {
  cplx_t<T>* x = X + static_cast<long long>(blockIdx.y) * n_tot_half;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_plane; i += gridDim.x * blockDim.x) {
    const int h = __ldg(plane + 2 * i), p = __ldg(plane + 2 * i + 1);
    if (h == p) {
      x[h].y = T(0);
    } else if (h < p) {
      const cplx_t<T> a = x[h], c = x[p];
      const cplx_t<T> m = mk<T>(T(0.5) * (a.x + c.x), T(0.5) * (a.y - c.y));
      x[h] = m;
      x[p] = mk<T>(m.x, -m.y);
    }
  }
}

static inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

int check_map(const qgb_real_map* m, const qgb_sphere* full) {
  if (!m || !full) return fail(QGB_ERR_INVALID, "NULL real-basis map or sphere");
  if (m->n_half < 1 || m->n_tot_half < m->n_half || m->n_full < m->n_half || m->n_plane < 0 ||
      m->n_plane > m->n_half)
    return fail(QGB_ERR_INVALID, "bad real-basis map sizes");
  if (full->nk != 1 || full->n_tot != m->n_tot_full || m->n_tot_full < m->n_full)
    return fail(QGB_ERR_INVALID, "full sphere (nk %d, n_tot %d) does not match the map (n_tot_full %d)",
                full->nk, full->n_tot, m->n_tot_full);
  if (!m->pack || !m->unpack || (m->n_plane && !m->plane) || !m->ke || !m->weight)
    return fail(QGB_ERR_INVALID, "NULL table in the real-basis map");
  return QGB_OK;
}

// Workspace: packed rows Z, their transform W, D proj, Gram partials, slab planes.
struct RealLayout {
  size_t z, w, dp, part, planes, total;
};
static RealLayout real_layout(const qgb_sphere& full, const qgb_real_map& m, int nb, int P, int dtype) {
  RealLayout L;
  const int nz = (nb + 1) / 2;
  const size_t eb = elem_bytes(dtype);
  L.z = align256(static_cast<size_t>(nz) * m.n_tot_full * eb);
  L.w = L.z;
  L.dp = P > 0 ? align256(static_cast<size_t>(nb) * P * eb) : 0;
  L.part = P > 0 ? align256(gram_workspace_bytes(dtype, 1, P, nb, m.n_tot_half)) : 0;
  L.planes = plane_bytes_per_band(full, dtype) * static_cast<size_t>(std::max(nz, 1));
  L.total = L.z + L.w + L.dp + L.part + L.planes;
  return L;
}

}  // namespace rb

using namespace rb;

int check_real_map(const qgb_real_map* m, const qgb_sphere* full) { return check_map(m, full); }

static int real_pack(int dtype, const qgb_real_map* m, const void* C, int nb, void* Z, cudaStream_t st) {
  const int nz = (nb + 1) / 2;
  if (nz == 0) return QGB_OK;
  const dim3 grid(static_cast<unsigned>(std::min(64, (m->n_tot_full + kThreads - 1) / kThreads)), nz);
  const int2* pack = reinterpret_cast<const int2*>(m->pack);
  if (dtype == QGB_F64)
    k_pack_real<double><<<grid, kThreads, 0, st>>>(static_cast<const double2*>(C), nb, m->n_tot_half, pack,
                                                   m->n_full, m->n_tot_full, static_cast<double2*>(Z));
  else
    k_pack_real<float><<<grid, kThreads, 0, st>>>(static_cast<const float2*>(C), nb, m->n_tot_half, pack,
                                                  m->n_full, m->n_tot_full, static_cast<float2*>(Z));
  QGB_LAUNCH_CHECK("k_pack_real");
  return QGB_OK;
}

static int real_unpack(int dtype, const qgb_real_map* m, const void* W, const void* C, int nb, void* out,
                       unsigned flags, cudaStream_t st) {
  if (nb == 0) return QGB_OK;
  const dim3 grid(static_cast<unsigned>(std::min(64, (m->n_tot_half + kThreads - 1) / kThreads)), nb);
  if (dtype == QGB_F64)
    k_unpack_real<double><<<grid, kThreads, 0, st>>>(static_cast<const double2*>(W), m->n_tot_full, m->unpack,
                                                     m->n_half, static_cast<const double2*>(C),
                                                     static_cast<const double*>(m->ke), nb, m->n_tot_half, flags,
                                                     static_cast<double2*>(out));
  else
    k_unpack_real<float><<<grid, kThreads, 0, st>>>(static_cast<const float2*>(W), m->n_tot_full, m->unpack,
                                                    m->n_half, static_cast<const float2*>(C),
                                                    static_cast<const float*>(m->ke), nb, m->n_tot_half, flags,
                                                    static_cast<float2*>(out));
  QGB_LAUNCH_CHECK("k_unpack_real");
  return QGB_OK;
}

// The local part alone (pack, full-sphere potential with the KE term, unpack):
// workspace Z, W and the slab planes.
size_t real_local_bytes(const qgb_sphere& full, const qgb_real_map& m, int nb, int dtype) {
  const RealLayout L = real_layout(full, m, nb, 0, dtype);
  return L.z + L.w + L.planes;
}

// HC = KE C + V C in the real mode.  With `unpack_after` (an event on another
// stream that writes a term into HC), the unpack waits for it and adds to HC.
int real_local(const qgb_sphere* full, const qgb_real_map* m, int dtype, const void* C, void* HC, int nb, void* ws,
               size_t ws_bytes, cudaStream_t st, cudaEvent_t unpack_after) {
  const RealLayout L = real_layout(*full, *m, nb, 0, dtype);
  if (ws_bytes < L.z + L.w + L.planes) return fail(QGB_ERR_WORKSPACE, "real local workspace too small");
  char* w = static_cast<char*>(ws);
  int rc;
  if ((rc = real_pack(dtype, m, C, nb, w, st))) return rc;
  if ((rc = apply_potential(full, dtype, w, w + L.z, (nb + 1) / 2, 0u, w + L.z + L.w, L.planes, st))) return rc;
  if (unpack_after) QGB_CUDA_CHECK(cudaStreamWaitEvent(st, unpack_after, 0));
  return real_unpack(dtype, m, w + L.z, C, nb, HC, QGB_ADD_KE | (unpack_after ? QGB_ACCUMULATE : 0u), st);
}

}  // namespace qgb

using namespace qgb;

extern "C" size_t qgb_hamiltonian_real_workspace_bytes(const qgb_sphere* full, const qgb_real_map* m, int nb, int P,
                                                       int dtype) {
  if (!full || !m || nb < 0 || P < 0 || (dtype != QGB_F64 && dtype != QGB_F32)) return 0;
  return real_layout(*full, *m, nb, P, dtype).total;
}

extern "C" int qgb_hamiltonian_real(const qgb_sphere* full, const qgb_real_map* m, int dtype, const void* C, void* HC,
                                    int nb, const void* beta, const void* D, int n_atoms, int pa, void* projT,
                                    void* workspace, size_t workspace_bytes, void* stream) {
  int rc = validate_sphere(full, dtype);
  if (rc) return rc;
  if ((rc = check_map(m, full))) return rc;
  if (nb < 0 || n_atoms < 0 || pa < 0) return fail(QGB_ERR_INVALID, "negative sizes");
  if (nb == 0) return QGB_OK;
  if (!C || !HC) return fail(QGB_ERR_INVALID, "NULL wavefunction pointer");
  if (C == HC) return fail(QGB_ERR_INVALID, "C and HC must not alias");
  const int P = n_atoms * pa;
  if (P > 0 && (!beta || !D || !projT)) return fail(QGB_ERR_INVALID, "NULL projector argument with P > 0");
  const RealLayout L = real_layout(*full, *m, nb, P, dtype);
  if (!workspace || workspace_bytes < L.total)
    return fail(QGB_ERR_WORKSPACE, "workspace %zu B < %zu B", workspace_bytes, L.total);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  void* Z = ws;
  void* W = ws + L.z;
  void* Dp = ws + L.z + L.w;
  void* part = ws + L.z + L.w + L.dp;
  void* planes = ws + L.z + L.w + L.dp + L.part;
  const int nz = (nb + 1) / 2;
  if ((rc = real_pack(dtype, m, C, nb, Z, st))) return rc;
  if ((rc = apply_potential(full, dtype, Z, W, nz, 0u, planes, L.planes, st))) return rc;
  if ((rc = real_unpack(dtype, m, W, C, nb, HC, QGB_ADD_KE, st))) return rc;
  if (P == 0) return QGB_OK;
  // <beta|C> = Re sum_G w_G conj(beta) C (the implicit -G partners), stored
  // band-major projT[b][p]; then HC += beta (D proj).
  const int n = m->n_tot_half;
  if ((rc = gram(dtype, dtype, beta, static_cast<long long>(P) * n, n, C, static_cast<long long>(nb) * n, n, 1, P,
                 nb, n, projT, static_cast<long long>(nb) * P, 1, P, part, L.part, st, m->weight, true)))
    return rc;
  if ((rc = dapply(dtype, projT, D, n_atoms, pa, nb, 1, Dp, st))) return rc;
  return rotate(dtype, beta, static_cast<long long>(P) * n, n, Dp, static_cast<long long>(nb) * P, 1, P, 1, P, nb, n,
                HC, static_cast<long long>(nb) * n, n, true, st);
}

extern "C" int qgb_symmetrize_real(int dtype, const qgb_real_map* m, void* X, int nb, void* stream) {
  if (!m || nb < 0 || m->n_plane < 0 || m->n_tot_half < m->n_half || (m->n_plane && !m->plane))
    return fail(QGB_ERR_INVALID, "bad symmetrize_real arguments");
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (nb == 0 || m->n_plane == 0) return QGB_OK;
  if (!X) return fail(QGB_ERR_INVALID, "NULL wavefunction pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const dim3 grid(static_cast<unsigned>(std::min(16, (m->n_plane + kThreads - 1) / kThreads)), nb);
  if (dtype == QGB_F64)
    k_symmetrize_real<double><<<grid, kThreads, 0, st>>>(static_cast<double2*>(X), m->n_tot_half, m->plane,
                                                         m->n_plane);
  else
    k_symmetrize_real<float><<<grid, kThreads, 0, st>>>(static_cast<float2*>(X), m->n_tot_half, m->plane,
                                                        m->n_plane);
  QGB_LAUNCH_CHECK("k_symmetrize_real");
  return QGB_OK;
}
