// extern "C" entry points of libqimpy_gb300 (declared in include/qimpy_gb300.h).
#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>

#include "bandgemm.cuh"

namespace qgb {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int raise_smem_limit(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> raised;
  int dev = 0;
  QGB_CUDA_CHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = raised[{kernel, dev}];
  if (bytes <= have) return QGB_OK;
  QGB_CUDA_CHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
  have = bytes;
  return QGB_OK;
}

int validate_sphere(const qgb_sphere* s, int dtype, bool need_potential = true);
size_t plane_bytes_per_band(const qgb_sphere& s, int dtype);
int apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, unsigned flags,
                    void* ws, size_t ws_bytes, cudaStream_t st,
                    cudaEvent_t gather_after = nullptr);
int apply_ke(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, cudaStream_t st);
size_t project_workspace_bytes(int dtype, int nk, int P, int nb, int n_tot);
int project(int dtype, const void* beta, const void* C, void* projT, int nk, int P, int nb, int n_tot, void* ws,
            size_t ws_bytes, cudaStream_t st);
int apply_nonlocal(int dtype, const void* beta, const void* D, int n_atoms, int pa, const void* projT,
                   void* out, int nk, int nb, int n_tot, void* work, cudaStream_t st);
#ifdef QGB_DEBUG_CHECKS
int debug_violation(unsigned long long* out4);
#endif
size_t sphere_smem_bytes(const qgb_sphere& s, int dtype);
int collect_density(const qgb_sphere* s, int dtype, const void* C, int nb, const double* prefac, double* rho,
                    unsigned flags, void* ws, size_t ws_bytes, cudaStream_t st);
size_t plane_smem_bytes(const qgb_sphere& s, int dtype);
int apply_potential_batched(const qgb_batch_item* items, int n_items, const int* slab_item,
                            const long long* slab_starts, const int* row_item, const long long* row_starts,
                            long long n_slab, long long n_row, int dtype, size_t smem_yz, size_t smem_x,
                            cudaStream_t st);
size_t beta_split_bytes(int nk, int P, int n_tot);
int beta_split(const void* beta, int nk, int P, int n_tot, void* out, size_t out_bytes, cudaStream_t st);
size_t nonlocal_tc_workspace_bytes(int nk, int P, int nb, int n_tot);
int nonlocal_tc(const void* split, const void* D, int n_atoms, int pa, const void* C, void* HC, void* projT,
                int nk, int nb, int n_tot, void* ws, size_t ws_bytes, int* err, cudaStream_t st);
int nonlocal_tc_phase(const void* split, const void* D, int n_atoms, int pa, const void* C, void* HC, void* projT,
                      int nk, int nb, int n_tot, void* ws, size_t ws_bytes, int* err, int phases, cudaStream_t st,
                      const double* weight = nullptr);
int check_real_map(const qgb_real_map* m, const qgb_sphere* full);
size_t gram_tc_workspace_bytes(int nk, int nx, int ny, int n);
size_t rotate_tc_workspace_bytes(int nk, int n_in, int n_out, int n);
int rotate_tc(const void* C, int n_in, int nk, int n, const void* M, int n_out, void* out, bool accumulate,
              void* ws, size_t ws_bytes, int* err, cudaStream_t st);
int gram_tc(const void* X, int nx, const void* Y, int ny, int nk, int n, double2* out, long long out_batch, int oi,
            int oj, void* ws, size_t ws_bytes, int* err, cudaStream_t st);
size_t real_local_bytes(const qgb_sphere& full, const qgb_real_map& m, int nb, int dtype);
int real_local(const qgb_sphere* full, const qgb_real_map* m, int dtype, const void* C, void* HC, int nb, void* ws,
               size_t ws_bytes, cudaStream_t st,
               cudaEvent_t unpack_after = nullptr);

// A side stream and a fork/join event pair per (host thread, device): the mixed
// Hamiltonian runs the C-only part of its nonlocal term there, beside the local
// potential on the caller's stream (the FFT kernels are issue-bound on the CUDA
// cores, the projector GEMMs bound by HBM and the tensor cores).  Fork and join
// are events, so the sequence stays capturable in a CUDA graph.
struct SideStream {
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
static int side_stream(SideStream* out) {
  static thread_local std::unordered_map<int, SideStream> streams;
  int dev = 0;
  QGB_CUDA_CHECK(cudaGetDevice(&dev));
  auto it = streams.find(dev);
  if (it == streams.end()) {
    SideStream s;
    QGB_CUDA_CHECK(cudaStreamCreateWithFlags(&s.side, cudaStreamNonBlocking));
    QGB_CUDA_CHECK(cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming));
    QGB_CUDA_CHECK(cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming));
    it = streams.emplace(dev, s).first;
  }
  *out = it->second;
  return QGB_OK;
}

}  // namespace qgb

using namespace qgb;

extern "C" {

int qgb_abi_version(void) { return QGB_ABI_VERSION; }

const char* qgb_last_error(void) { return g_last_error.c_str(); }

size_t qgb_potential_workspace_bytes(const qgb_sphere* s, int nb, int dtype) {
  if (!s || nb < 0) return 0;
  return plane_bytes_per_band(*s, dtype) * static_cast<size_t>(nb);
}

static inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Workspace of qgb_hamiltonian: [D proj (nk nb P complex) | <beta|psi> split-K
// partials | slab planes], each part 256-byte aligned.
static size_t ham_nonlocal_bytes(const qgb_sphere& s, int nb, int P, int dtype) {
  if (P == 0 || nb == 0) return 0;
  return align256(static_cast<size_t>(s.nk) * nb * P * elem_bytes(dtype)) +
         align256(project_workspace_bytes(dtype, s.nk, P, nb, s.n_tot));
}

size_t qgb_hamiltonian_workspace_bytes(const qgb_sphere* s, int nb, int P, int dtype) {
  if (!s || nb < 0 || P < 0) return 0;
  return ham_nonlocal_bytes(*s, nb, P, dtype) + plane_bytes_per_band(*s, dtype) * static_cast<size_t>(nb);
}

int qgb_permute_real_space(const qgb_sphere* s, int32_t* perm) {
  if (!s || !perm) return fail(QGB_ERR_INVALID, "NULL argument");
  int off = 0;
  for (int a = 0; a < 3; ++a) {
    const int L1 = s->L1[a], L2 = s->L2[a];
    if (L1 < 1 || L2 < 1 || L1 * L2 != s->N[a]) return fail(QGB_ERR_INVALID, "bad factorisation on axis %d", a);
    for (int p = 0; p < s->N[a]; ++p) perm[off + p] = p / L1 + L2 * (p % L1);
    off += s->N[a];
  }
  return QGB_OK;
}

int qgb_apply_ke(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, void* stream) {
  return apply_ke(s, dtype, C, out, nb, static_cast<cudaStream_t>(stream));
}

int qgb_apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, unsigned flags,
                        void* workspace, size_t workspace_bytes, void* stream) {
  return apply_potential(s, dtype, C, out, nb, flags, workspace, workspace_bytes,
                         static_cast<cudaStream_t>(stream));
}

size_t qgb_project_workspace_bytes(int dtype, int nk, int P, int nb, int n_tot) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return 0;
  return project_workspace_bytes(dtype, nk, P, nb, n_tot);
}

int qgb_project(int dtype, const void* beta, const void* C, void* projT, int nk, int P, int nb, int n_tot,
                void* workspace, size_t workspace_bytes, void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  return project(dtype, beta, C, projT, nk, P, nb, n_tot, workspace, workspace_bytes,
                 static_cast<cudaStream_t>(stream));
}

size_t qgb_dot_workspace_bytes(int dtype, int nk, int nx, int ny, int n_tot) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return 0;
  return gram_workspace_bytes(dtype, nk, nx, ny, n_tot);
}

int qgb_dot(int dtype, const void* X, int nx, const void* Y, int ny, int nk, int n_tot, void* out, void* workspace,
            size_t workspace_bytes, void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (nk < 0 || nx < 0 || ny < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad dot sizes");
  return gram(dtype, QGB_F64, X, static_cast<long long>(nx) * n_tot, n_tot, Y, static_cast<long long>(ny) * n_tot,
              n_tot, nk, nx, ny, n_tot, out, static_cast<long long>(nx) * ny, ny, 1, workspace, workspace_bytes,
              static_cast<cudaStream_t>(stream));
}

size_t qgb_matmul_tc_workspace_bytes(int nk, int n_in, int n_out, int n_tot) {
  return rotate_tc_workspace_bytes(nk, n_in, n_out, n_tot);
}

int qgb_matmul_tc(const void* C, int n_in, int nk, int n_tot, const void* M, int n_out, void* out, unsigned flags,
                  void* workspace, size_t workspace_bytes, int* dev_error, void* stream) {
  if (flags & ~QGB_ACCUMULATE) return fail(QGB_ERR_INVALID, "unknown matmul flags 0x%x", flags);
  return rotate_tc(C, n_in, nk, n_tot, M, n_out, out, (flags & QGB_ACCUMULATE) != 0, workspace, workspace_bytes,
                   dev_error, static_cast<cudaStream_t>(stream));
}

size_t qgb_dot_tc_workspace_bytes(int nk, int nx, int ny, int n_tot) {
  return gram_tc_workspace_bytes(nk, nx, ny, n_tot);
}

int qgb_dot_tc(const void* X, int nx, const void* Y, int ny, int nk, int n_tot, void* out, void* workspace,
               size_t workspace_bytes, int* dev_error, void* stream) {
  return gram_tc(X, nx, Y, ny, nk, n_tot, static_cast<double2*>(out), static_cast<long long>(nx) * ny, ny, 1,
                 workspace, workspace_bytes, dev_error, static_cast<cudaStream_t>(stream));
}

int qgb_dot_real(int dtype, const void* X, int nx, const void* Y, int ny, int n_tot, const double* weight, void* out,
                 void* workspace, size_t workspace_bytes, void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (nx < 0 || ny < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad dot sizes");
  if (!weight) return fail(QGB_ERR_INVALID, "NULL weight");
  return gram(dtype, QGB_F64, X, static_cast<long long>(nx) * n_tot, n_tot, Y, static_cast<long long>(ny) * n_tot,
              n_tot, 1, nx, ny, n_tot, out, static_cast<long long>(nx) * ny, ny, 1, workspace, workspace_bytes,
              static_cast<cudaStream_t>(stream), weight, true);
}

int qgb_matmul(int dtype, const void* C, int n_in, int nk, int n_tot, const void* M, int n_out, void* out,
               unsigned flags, void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (nk < 0 || n_in < 0 || n_out < 0 || n_tot < 1) return fail(QGB_ERR_INVALID, "bad matmul sizes");
  if (flags & ~QGB_ACCUMULATE) return fail(QGB_ERR_INVALID, "unknown matmul flags 0x%x", flags);
  if (n_in > 0 && C != nullptr && C == out) return fail(QGB_ERR_INVALID, "C and out must not alias");
  // out[k][j][g] = sum_i M[k][i][j] C[k][i][g]: W(i, j) = M[i*n_out + j].
  return rotate(dtype, C, static_cast<long long>(n_in) * n_tot, n_tot, M, static_cast<long long>(n_in) * n_out,
                n_out, 1, nk, n_in, n_out, n_tot, out, static_cast<long long>(n_out) * n_tot, n_tot,
                (flags & QGB_ACCUMULATE) != 0, static_cast<cudaStream_t>(stream));
}

int qgb_apply_nonlocal(int dtype, const void* beta, const void* D, int n_atoms, int pa, const void* projT,
                       void* out, int nk, int nb, int n_tot, void* work, void* stream) {
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  return apply_nonlocal(dtype, beta, D, n_atoms, pa, projT, out, nk, nb, n_tot, work,
                        static_cast<cudaStream_t>(stream));
}

int qgb_hamiltonian(const qgb_sphere* s, int dtype, const void* C, void* HC, int nb, const void* beta,
                    const void* D, int n_atoms, int pa, void* projT, void* workspace,
                    size_t workspace_bytes, void* stream) {
  int rc = validate_sphere(s, dtype);
  if (rc) return rc;
  if (C == HC) return fail(QGB_ERR_INVALID, "C and HC must not alias");
  if (n_atoms < 0 || pa < 0 || nb < 0) return fail(QGB_ERR_INVALID, "bad nonlocal sizes");
  const int P = n_atoms * pa;
  const size_t nl = ham_nonlocal_bytes(*s, nb, P, dtype);
  if (workspace_bytes < nl) return fail(QGB_ERR_WORKSPACE, "workspace too small for nonlocal term");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  rc = apply_potential(s, dtype, C, HC, nb, QGB_ADD_KE, ws + nl, workspace_bytes - nl, st);
  if (rc) return rc;
  if (P > 0 && nb > 0) {
    if (!projT) return fail(QGB_ERR_INVALID, "projT is NULL with P > 0");
    const size_t dp = align256(static_cast<size_t>(s->nk) * nb * P * elem_bytes(dtype));
    rc = project(dtype, beta, C, projT, s->nk, P, nb, s->n_tot, ws + dp, nl - dp, st);
    if (rc) return rc;
    rc = apply_nonlocal(dtype, beta, D, n_atoms, pa, projT, HC, s->nk, nb, s->n_tot, ws, st);
    if (rc) return rc;
  }
  return QGB_OK;
}

#ifdef QGB_DEBUG_CHECKS
int qgb_debug_violation(unsigned long long* out4) { return qgb::debug_violation(out4); }
#endif

size_t qgb_sphere_smem_bytes(const qgb_sphere* s, int dtype) { return s ? sphere_smem_bytes(*s, dtype) : 0; }

int qgb_collect_density(const qgb_sphere* s, int dtype, const void* C, int nb, const double* prefac, double* rho,
                        unsigned flags, void* workspace, size_t workspace_bytes, void* stream) {
  return collect_density(s, dtype, C, nb, prefac, rho, flags, workspace, workspace_bytes,
                         static_cast<cudaStream_t>(stream));
}
size_t qgb_sphere_smem_bytes_yz(const qgb_sphere* s, int dtype) { return s ? plane_smem_bytes(*s, dtype) : 0; }

int qgb_apply_potential_batched(const qgb_batch_item* items, int n_items, const int* slab_item,
                                const long long* slab_starts, const int* row_item, const long long* row_starts,
                                long long n_slab_units, long long n_row_units, int dtype, size_t smem_yz,
                                size_t smem_x, void* stream) {
  return apply_potential_batched(items, n_items, slab_item, slab_starts, row_item, row_starts, n_slab_units,
                                 n_row_units, dtype, smem_yz, smem_x, static_cast<cudaStream_t>(stream));
}

size_t qgb_beta_split_bytes(int nk, int P, int n_tot) { return beta_split_bytes(nk, P, n_tot); }

int qgb_beta_split(const void* beta, int nk, int P, int n_tot, void* out, size_t out_bytes, void* stream) {
  return beta_split(beta, nk, P, n_tot, out, out_bytes, static_cast<cudaStream_t>(stream));
}

size_t qgb_nonlocal_tc_workspace_bytes(int nk, int P, int nb, int n_tot) {
  return nonlocal_tc_workspace_bytes(nk, P, nb, n_tot);
}

int qgb_apply_nonlocal_tc(const void* beta_split, const void* D, int n_atoms, int pa, const void* C, void* HC,
                          void* projT, int nk, int nb, int n_tot, void* workspace, size_t workspace_bytes,
                          int* dev_error, void* stream) {
  return nonlocal_tc(beta_split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, workspace, workspace_bytes,
                     dev_error, static_cast<cudaStream_t>(stream));
}

int qgb_apply_nonlocal_tc_phase(const void* beta_split, const void* D, int n_atoms, int pa, const void* C,
                                void* HC, void* projT, int nk, int nb, int n_tot, void* workspace,
                                size_t workspace_bytes, int* dev_error, int phases, void* stream) {
  if (phases < 1 || phases > 7 || phases == 4 || phases == 5)
    return fail(QGB_ERR_INVALID, "phases = %d (1, 2 or 3, plus 4 with 2)", phases);
  return nonlocal_tc_phase(beta_split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, workspace, workspace_bytes,
                           dev_error, phases, static_cast<cudaStream_t>(stream));
}

size_t qgb_hamiltonian_mixed_workspace_bytes(const qgb_sphere* s, int nb, int P) {
  if (!s || nb < 0 || P < 0) return 0;
  const size_t nl = (nonlocal_tc_workspace_bytes(s->nk, P, nb, s->n_tot) + 255) / 256 * 256;
  return nl + plane_bytes_per_band(*s, QGB_F32) * static_cast<size_t>(nb);
}

int qgb_hamiltonian_mixed(const qgb_sphere* s, const void* C, void* HC, int nb, const void* beta_split,
                          const void* D, int n_atoms, int pa, void* projT, void* workspace, size_t workspace_bytes,
                          int* dev_error, void* stream) {
  int rc = validate_sphere(s, QGB_F32);
  if (rc) return rc;
  if (C == HC) return fail(QGB_ERR_INVALID, "C and HC must not alias");
  const int P = n_atoms * pa;
  const size_t nl = P > 0 ? (nonlocal_tc_workspace_bytes(s->nk, P, nb, s->n_tot) + 255) / 256 * 256 : 0;
  if (workspace_bytes < nl) return fail(QGB_ERR_WORKSPACE, "workspace too small for the nonlocal term");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  if (P == 0 || nb == 0) return apply_potential(s, QGB_F32, C, HC, nb, QGB_ADD_KE, ws + nl, workspace_bytes - nl, st);
  SideStream f;
  if ((rc = side_stream(&f))) return rc;
  // Fork: the whole nonlocal term on the side stream (split, <beta|psi>,
  // reduce, D, and the back-projection storing HC = beta (D projT)) while the
  // inverse and x passes of the local potential run; their gather kernels wait
  // for it and accumulate KE C + V C into HC.  The nonlocal chain is thus off
  // the critical path.  The join is waited for on every path, so that a
  // capture stays well-formed even when a launch was refused.
  QGB_CUDA_CHECK(cudaEventRecord(f.fork, st));
  QGB_CUDA_CHECK(cudaStreamWaitEvent(f.side, f.fork, 0));
  const int rc_front = nonlocal_tc_phase(beta_split, D, n_atoms, pa, C, HC, projT, s->nk, nb, s->n_tot, ws, nl,
                                         dev_error, 1 | 2 | 4, f.side);
  QGB_CUDA_CHECK(cudaEventRecord(f.join, f.side));
  rc = apply_potential(s, QGB_F32, C, HC, nb, QGB_ADD_KE | QGB_ACCUMULATE, ws + nl, workspace_bytes - nl, st,
                       f.join);
  QGB_CUDA_CHECK(cudaStreamWaitEvent(st, f.join, 0));
  if (rc_front) return rc_front;
  return rc;
}

size_t qgb_hamiltonian_real_mixed_workspace_bytes(const qgb_sphere* full, const qgb_real_map* map, int nb, int P) {
  if (!full || !map || nb < 0 || P < 0) return 0;
  const size_t nl = P > 0 ? (nonlocal_tc_workspace_bytes(1, P, nb, map->n_tot_half) + 255) / 256 * 256 : 0;
  return nl + real_local_bytes(*full, *map, nb, QGB_F32);
}

int qgb_hamiltonian_real_mixed(const qgb_sphere* full, const qgb_real_map* map, const void* C, void* HC, int nb,
                               const void* beta_split, const void* D, int n_atoms, int pa, void* projT,
                               void* workspace, size_t workspace_bytes, int* dev_error, void* stream) {
  int rc = validate_sphere(full, QGB_F32);
  if (rc) return rc;
  if ((rc = check_real_map(map, full))) return rc;
  if (nb < 0 || n_atoms < 0 || pa < 0) return fail(QGB_ERR_INVALID, "negative sizes");
  if (nb == 0) return QGB_OK;
  if (!C || !HC) return fail(QGB_ERR_INVALID, "NULL wavefunction pointer");
  if (C == HC) return fail(QGB_ERR_INVALID, "C and HC must not alias");
  const int P = n_atoms * pa;
  const size_t nl = P > 0 ? (nonlocal_tc_workspace_bytes(1, P, nb, map->n_tot_half) + 255) / 256 * 256 : 0;
  if (!workspace || workspace_bytes < nl + real_local_bytes(*full, *map, nb, QGB_F32))
    return fail(QGB_ERR_WORKSPACE, "workspace %zu B < %zu B", workspace_bytes,
                nl + real_local_bytes(*full, *map, nb, QGB_F32));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* ws = static_cast<char*>(workspace);
  if (P == 0) return real_local(full, map, QGB_F32, C, HC, nb, ws, workspace_bytes, st);
  SideStream f;
  if ((rc = side_stream(&f))) return rc;
  // As qgb_hamiltonian_mixed: the whole nonlocal term (weighted real
  // projection, D, back-projection stored into HC) on the side stream beside
  // the local potential, whose unpack waits for it and adds KE C + V C.
  QGB_CUDA_CHECK(cudaEventRecord(f.fork, st));
  QGB_CUDA_CHECK(cudaStreamWaitEvent(f.side, f.fork, 0));
  const int rc_front = nonlocal_tc_phase(beta_split, D, n_atoms, pa, C, HC, projT, 1, nb, map->n_tot_half, ws, nl,
                                         dev_error, 1 | 2 | 4, f.side, map->weight);
  QGB_CUDA_CHECK(cudaEventRecord(f.join, f.side));
  rc = real_local(full, map, QGB_F32, C, HC, nb, ws + nl, workspace_bytes - nl, st, f.join);
  QGB_CUDA_CHECK(cudaStreamWaitEvent(st, f.join, 0));
  if (rc_front) return rc_front;
  return rc;
}

}  // extern "C"
