// Local-potential apply for callers that cannot allocate device memory.
//
// Some host programs cannot hand this library a workspace: their GPU memory is
// owned by an outer framework (a Fortran or C electronic-structure code that
// reserves the device up front and forbids allocations from plugins), or they
// run in a context where cudaMalloc is not allowed (inside a stream capture, or
// a latency-critical serving loop with a fixed memory budget).  For them,
// qgb_apply_potential_static runs the same kernels as qgb_apply_potential with
// its slab-plane scratch in a fixed file-scope device array instead of a
// caller-provided buffer.  Nothing here allocates.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "qgb_common.cuh"

namespace qgb {

int validate_sphere(const qgb_sphere* s, int dtype, bool need_potential = true);
size_t plane_bytes_per_band(const qgb_sphere& s, int dtype);
int apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, unsigned flags,
                    void* ws, size_t ws_bytes, cudaStream_t st,
                    cudaEvent_t gather_after = nullptr);

// 32 MiB per GPU that loads this library, held until the process exits.
static constexpr size_t kStaticScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mu;
static void* g_scratch_addr[kMaxDevices];
static unsigned long long g_scratch_ctx[kMaxDevices];  // context id the address belongs to

// Unique id of the calling thread's current context (0 if the driver cannot
// tell).  A device reset (cudaDeviceReset, or the primary context released)
// reloads this module at a new address under a new context id.
static unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, so the address is looked up once per device (and
// again after a device reset gave the device a new context) with that device
// current, and cached.
static int static_scratch(void** addr) {
  int dev = 0;
  QGB_CUDA_CHECK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(QGB_ERR_UNSUPPORTED, "device ordinal %d >= %d", dev, kMaxDevices);
  // A thread that has not used the runtime yet may have no current context
  // (id 0): that is no sign of a reset, so it keeps the cached address.
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (g_scratch_addr[dev] == nullptr || (ctx != 0 && g_scratch_ctx[dev] != ctx)) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || p == nullptr)
      return fail(QGB_ERR_CUDA, "cudaGetSymbolAddress(static scratch) on device %d failed: %s", dev,
                  cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev] = current_context_id();  // the lookup made the device's context current
  }
  *addr = g_scratch_addr[dev];
  return QGB_OK;
}

}  // namespace qgb

extern "C" size_t qgb_static_scratch_bytes(void) { return qgb::kStaticScratchBytes; }

extern "C" int qgb_apply_potential_static(const qgb_sphere* s, int dtype, const void* C, void* out, int nb,
                                          unsigned flags, void* stream) {
  using namespace qgb;
  if (s == nullptr) return fail(QGB_ERR_INVALID, "sphere descriptor is NULL");
  if (dtype != QGB_F64 && dtype != QGB_F32) return fail(QGB_ERR_INVALID, "unknown dtype %d", dtype);
  if (s->nk < 1 || s->max_slabs < 1 || s->N[1] < 1 || s->N[2] < 1)
    return fail(QGB_ERR_INVALID, "empty sphere descriptor");
  const size_t per_band = plane_bytes_per_band(*s, dtype);
  if (per_band > kStaticScratchBytes)
    return fail(QGB_ERR_WORKSPACE,
                "one band needs %zu bytes of scratch (nk=%d x %d slabs x %dx%d planes), more than the "
                "fixed %zu-byte scratch of qgb_apply_potential_static; use qgb_apply_potential with a "
                "caller-provided workspace",
                per_band, s->nk, s->max_slabs, s->N[1], s->N[2], kStaticScratchBytes);
  int rc = validate_sphere(s, dtype);
  if (rc) return rc;
  void* scratch = nullptr;
  rc = static_scratch(&scratch);
  if (rc) return rc;
  return apply_potential(s, dtype, C, out, nb, flags, scratch, kStaticScratchBytes,
                         static_cast<cudaStream_t>(stream));
}
