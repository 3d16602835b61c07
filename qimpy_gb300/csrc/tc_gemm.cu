// Tensor-core (tcgen05) split-BF16x3 GEMM and the mixed-precision nonlocal term.
//
// D[m][n] = sum_k A[m][k] B[n][k] (both operands K-major, "TN") is computed as
//   A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T,   x_hi = bf16(x), x_lo = bf16(x - x_hi),
// with FP32 accumulation in tensor memory: about 16 significant bits per
// product, the split-BF16x3 scheme.  The three products run as one K loop
// over three segments, so a CTA accumulates them into one TMEM tile.
//
// Per CTA (128 threads, one 128 x BN output tile, one K range):
//   thread 0 (warp 0)  - TMA producer: 128B-swizzled A and B boxes into an
//                        S-stage shared-memory ring, mbarrier complete_tx;
//   thread 32 (warp 1) - MMA issuer: tcgen05.mma.cta_group::1.kind::f16 with
//                        bf16 inputs and an FP32 accumulator in TMEM, four K=16
//                        steps per 64-wide stage, tcgen05.commit frees the stage;
//   all 4 warps        - epilogue: tcgen05.ld of their 32 TMEM lanes.
// Every mbarrier wait is bounded by a %globaltimer deadline; on timeout the
// kernel records an error code, drains its own TMA copies (bounded), frees its
// TMEM and returns.
//
// Complex products map onto this real GEMM by stacking real and imaginary
// parts as rows (see the nonlocal section below).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "qgb_common.cuh"

namespace qgb {
namespace tc {

constexpr int BM = 128;            // MMA M (rows of A per CTA)
constexpr int BK = 64;             // bf16 elements per stage along K (one 128 B swizzle atom)
constexpr int kThreads = 128;
constexpr unsigned long long kTimeoutNs = 2000000000ull;  // 2 s per pipeline wait
constexpr unsigned long long kDrainNs = 2000000000ull;    // 2 s per drain wait

enum Epi { EPI_PARTIAL = 0, EPI_ADD_HC = 1 };

struct GemmArgs {
  int M, N, K;             // logical sizes (rows of A, rows of B, reduction)
  int kb_per_split;        // 64-wide K blocks per split
  int splits;
  float* partial;          // EPI_PARTIAL: [batch][split][m_tiles*BM][n_tiles*BN]
  int part_ld;             // n_tiles * BN
  long long part_rows;     // m_tiles * BM
  float2* hc;              // EPI_ADD_HC: complex64 [batch][nb][hc_ld], += D
  long long hc_batch_stride;
  int hc_ld, nb;
  int hc_store;            // EPI_ADD_HC: 1 = store D instead of adding it
  int* err;                // device error word (0 = ok)
  unsigned long long timeout_ns;  // limit of each pipeline wait (kTimeoutNs)
  int skip_loads;          // test aid: the producer issues no copies, so the MMA wait runs out
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase with the given parity; false on timeout (error
// `code` recorded) or when another thread already flagged an error.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          unsigned long long limit_ns) {
  const unsigned long long t0 = now_ns();
  for (unsigned it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*reinterpret_cast<volatile int*>(err) != 0) return false;
      if (now_ns() - t0 > limit_ns) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}
// Drain wait: for work this CTA has already issued (TMA copies into its
// shared memory, MMAs into its TMEM), which must land before the CTA frees
// TMEM or exits.  It ignores the error word (an error elsewhere does not
// cancel issued work) and gives up only after its own limit.
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity, int* err, int code) {
  const unsigned long long t0 = now_ns();
  for (unsigned it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255u) == 255u && now_ns() - t0 > kDrainNs) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
// 32 TMEM lanes (one per thread of the warp) x 32 consecutive 32-bit columns.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 B in 8-row (1024 B) swizzle atoms.  Fields: start address >> 4 (bits
// 0-13), leading byte offset >> 4 (16-29, unused for this layout), stride
// byte offset >> 4 (32-45, 1024 B between 8-row groups), descriptor version 1
// (46-47), layout type 2 = SWIZZLE_128B (61-63).
__device__ __forceinline__ uint64_t desc_kmajor_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;
  d |= static_cast<uint64_t>(1024 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(2) << 61;
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// bf16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

template <int BN, int STAGES>
struct Smem {
  static constexpr int A_BYTES = BM * BK * 2;   // 16 KB
  static constexpr int B_BYTES = BN * BK * 2;   // BN x 128 B
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int BAR_OFF = STAGES * STAGE_BYTES;
  static constexpr int TOTAL = BAR_OFF + (2 * STAGES + 1) * 8 + 16 + 1024;  // + alignment slack
};

template <int BN, int STAGES, int EPI>
__global__ void __launch_bounds__(kThreads)
    k_tc_gemm(const __grid_constant__ CUtensorMap mA_hi, const __grid_constant__ CUtensorMap mA_lo,
              const __grid_constant__ CUtensorMap mB_hi, const __grid_constant__ CUtensorMap mB_lo,
              const GemmArgs args) {
  using L = Smem<BN, STAGES>;
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  // 1024-byte alignment for the 128B-swizzled tiles.
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::BAR_OFF);
  uint64_t* empty = full + STAGES;
  uint64_t* tmem_full = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tmem_full + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_tile = blockIdx.x, n_tile = blockIdx.y;
  const int batch = blockIdx.z / args.splits, split = blockIdx.z % args.splits;
  const int nkb_total = (args.K + BK - 1) / BK;
  const int kb0 = split * args.kb_per_split;
  const int kb1 = min(nkb_total, kb0 + args.kb_per_split);
  const int nkb = max(0, kb1 - kb0);
  const int niter = 3 * nkb;  // segments: (hi, hi), (hi, lo), (lo, hi)

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tmem_full, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0 && niter > 0 && !args.skip_loads) {
    // ---------------- TMA producer ----------------
    int issued = 0;
    for (int it = 0; it < niter; ++it) {
      const int s = it % STAGES, use = it / STAGES;
      if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1, args.err, 1, args.timeout_ns)) break;
      const int seg = it / nkb, kb = kb0 + it % nkb;
      unsigned char* a_dst = smem + s * L::STAGE_BYTES;
      unsigned char* b_dst = a_dst + L::A_BYTES;
      mbar_arrive_expect_tx(&full[s], L::STAGE_BYTES);
      tma_load_3d(a_dst, seg == 2 ? &mA_lo : &mA_hi, &full[s], kb * BK, m_tile * BM, batch);
      tma_load_3d(b_dst, seg == 1 ? &mB_lo : &mB_hi, &full[s], kb * BK, n_tile * BN, batch);
      ++issued;
    }
    // Drain: every load issued lands before exit.  Loads before the last
    // STAGES were waited for through the empty barriers (their MMAs consumed
    // them); the last min(STAGES, issued) are waited for here, even after an
    // error.
    for (int it = max(0, issued - STAGES); it < issued; ++it)
      mbar_drain(&full[it % STAGES], (it / STAGES) & 1, args.err, 2);
  } else if (threadIdx.x == 32 && niter > 0) {
    // ---------------- MMA issuer ----------------
    constexpr uint32_t idesc = idesc_bf16_f32(BM, BN);
    for (int it = 0; it < niter; ++it) {
      const int s = it % STAGES, use = it / STAGES;
      if (!mbar_wait(&full[s], use & 1, args.err, 3, args.timeout_ns)) break;
      tc_fence_after();
      const uint32_t a_addr = smem_u32(smem + s * L::STAGE_BYTES);
      const uint32_t b_addr = a_addr + L::A_BYTES;
      const uint64_t adesc = desc_kmajor_sw128(a_addr), bdesc = desc_kmajor_sw128(b_addr);
#pragma unroll
      for (int k = 0; k < BK / 16; ++k)  // K = 16 per MMA: advance 32 B = 2 descriptor units
        umma_bf16(tmem, adesc + 2 * k, bdesc + 2 * k, idesc, (it > 0 || k > 0) ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    umma_commit(tmem_full);  // fires once every MMA issued above has completed
  }
  __syncwarp();

  // ---------------- Epilogue: all four warps ----------------
  // tmem_full is committed after every MMA the issuer launched (also when it
  // stopped early), so this wait drains the tensor cores before TMEM is read
  // or freed, error or not.
  bool ok = niter > 0;
  if (ok) ok = mbar_drain(tmem_full, 0, args.err, 4);
  tc_fence_after();
  // tcgen05.ld is warp-collective: decide per warp.
  ok = __all_sync(0xffffffffu, ok && *reinterpret_cast<volatile int*>(args.err) == 0);
  if (ok) {
    const int row = m_tile * BM + warp * 32 + lane;
    const uint32_t trow = tmem + (static_cast<uint32_t>(warp * 32) << 16);
    if (EPI == EPI_PARTIAL) {
      float* out = args.partial + ((static_cast<long long>(batch) * args.splits + split) * args.part_rows + row) *
                                      args.part_ld + n_tile * BN;
#pragma unroll 1
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(trow + c0, v);
#pragma unroll
        for (int i = 0; i < 32; i += 4)
          *reinterpret_cast<float4*>(out + c0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      }
    } else {
      // Columns [0, BN/2) hold real parts and [BN/2, BN) imaginary parts of
      // bands n_tile*BN/2 + j; rows are basis entries g.
      constexpr int HB = BN / 2;
      const bool row_ok = row < args.M;
      float2* hc = args.hc + batch * args.hc_batch_stride + row;
#pragma unroll 1
      for (int c0 = 0; c0 < HB; c0 += 32) {
        float vr[32], vi[32];
        // All 32 loads of HC first, then the stores: interleaved read-modify-
        // writes through one pointer could alias, which would serialise 32
        // memory round trips per thread.
        float2 o[32];
        if (args.hc_store) {
#pragma unroll
          for (int i = 0; i < 32; ++i) o[i] = make_float2(0.f, 0.f);
        } else if (row_ok) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int b = n_tile * HB + c0 + i;
            o[i] = b < args.nb ? hc[static_cast<long long>(b) * args.hc_ld] : make_float2(0.f, 0.f);
          }
        }
        tmem_ld32(trow + c0, vr);
        tmem_ld32(trow + HB + c0, vi);
        if (row_ok) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int b = n_tile * HB + c0 + i;
            if (b < args.nb) hc[static_cast<long long>(b) * args.hc_ld] = make_float2(o[i].x + vr[i], o[i].y + vi[i]);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, BN);
  }
}

// ---------------------------------------------------------------------------
// Host: tensor maps and launches
// ---------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 3D bf16 tensor [batch][rows][ld] (K innermost, `k_extent` valid), box
// 64 x box_rows x 1 with 128-byte swizzle; out-of-range elements read as zero.
static int make_map(CUtensorMap* m, const void* base, long long k_extent, long long rows, long long batch,
                    long long ld, long long batch_stride, int box_rows) {
  auto enc = encode_fn();
  if (!enc) return fail(QGB_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable from the driver");
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (ld * 2) % 16 || (batch_stride * 2) % 16)
    return fail(QGB_ERR_INVALID, "tensor-map operand not 16-byte aligned (ld=%lld)", ld);
  cuuint64_t dims[3] = {static_cast<cuuint64_t>(k_extent), static_cast<cuuint64_t>(rows),
                        static_cast<cuuint64_t>(batch)};
  cuuint64_t strides[2] = {static_cast<cuuint64_t>(ld * 2), static_cast<cuuint64_t>(batch_stride * 2)};
  cuuint32_t box[3] = {static_cast<cuuint32_t>(BK), static_cast<cuuint32_t>(box_rows), 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(QGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", static_cast<int>(r));
  return QGB_OK;
}

// Operand description for one side: hi/lo bf16 arrays [batch][rows][ld].
struct Operand {
  const void* hi;
  const void* lo;
  long long rows, ld, batch_stride;
};

template <int BN, int STAGES, int EPI>
static int launch(const Operand& A, const Operand& B, int K, int batch, const GemmArgs& args_in,
                  cudaStream_t st) {
  using L = Smem<BN, STAGES>;
  GemmArgs base_args = args_in;
  if (base_args.timeout_ns == 0) base_args.timeout_ns = kTimeoutNs;
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  int rc;
  if ((rc = make_map(&ma_hi, A.hi, K, A.rows, batch, A.ld, A.batch_stride, BM))) return rc;
  if ((rc = make_map(&ma_lo, A.lo, K, A.rows, batch, A.ld, A.batch_stride, BM))) return rc;
  if ((rc = make_map(&mb_hi, B.hi, K, B.rows, batch, B.ld, B.batch_stride, BN))) return rc;
  if ((rc = make_map(&mb_lo, B.lo, K, B.rows, batch, B.ld, B.batch_stride, BN))) return rc;
  if ((rc = raise_smem_limit(k_tc_gemm<BN, STAGES, EPI>, L::TOTAL))) return rc;
  const int m_tiles = static_cast<int>((A.rows + BM - 1) / BM);
  const int n_tiles = static_cast<int>((B.rows + BN - 1) / BN);
  dim3 grid(m_tiles, n_tiles, batch * base_args.splits);
  k_tc_gemm<BN, STAGES, EPI><<<grid, kThreads, L::TOTAL, st>>>(ma_hi, ma_lo, mb_hi, mb_lo, base_args);
  QGB_LAUNCH_CHECK("k_tc_gemm");
  return QGB_OK;
}

// ---------------------------------------------------------------------------
// Split kernels (FP32 -> bf16 hi/lo)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

// Wavefunction rows for the B operand: complex64 C[k][nb][n_tot] -> rows
// r = t*BN + part*HB + j (band t*HB + j, part 0 = real, 1 = imaginary) of
// [k][rows][ld] bf16 hi/lo; bands >= nb give zero rows.  With `weight`
// (real wavefunctions: 1 on the Gz = 0 plane, 2 elsewhere; powers of two, so
// the split stays exact) every coefficient is scaled by w_g.
__global__ void k_split_bands(const float2* __restrict__ C, int nb, int n_tot, int HB, int rows, int ld,
                              const double* __restrict__ weight, __nv_bfloat16* __restrict__ hi,
                              __nv_bfloat16* __restrict__ lo) {
  const int r = blockIdx.y, k = blockIdx.z;
  const int t = r / (2 * HB), rem = r - t * 2 * HB, part = rem / HB, b = t * HB + rem % HB;
  const float2* src = C + (static_cast<long long>(k) * nb + b) * n_tot;
  const long long o = (static_cast<long long>(k) * rows + r) * ld;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ld; g += gridDim.x * blockDim.x) {
    float v = 0.f;
    if (b < nb && g < n_tot) {
      const float2 c = src[g];
      v = part ? c.y : c.x;
      if (weight) v *= static_cast<float>(weight[g]);
    }
    __nv_bfloat16 h, l;
    split_bf16(v, h, l);
    hi[o + g] = h;
    lo[o + g] = l;
  }
}

// Projector operands, once per basis: complex64 beta[k][P][n_tot] ->
//   A  [k][2P][ldA]  rows (Re beta_p; Im beta_p), K = basis  (for <beta|psi>)
//   AT [k][n_tot][ldT] row g = (Re beta_p(g), p < P; Im beta_p(g)), K = 2P
//                                                     (for beta (D proj); skipped when t_hi is NULL)
__global__ void k_split_beta(const float2* __restrict__ beta, int P, int n_tot, int ldA, int ldT,
                             __nv_bfloat16* __restrict__ a_hi, __nv_bfloat16* __restrict__ a_lo,
                             __nv_bfloat16* __restrict__ t_hi, __nv_bfloat16* __restrict__ t_lo) {
  const int p = blockIdx.y, k = blockIdx.z;
  const float2* src = beta + (static_cast<long long>(k) * P + p) * n_tot;
  const long long oa_r = (static_cast<long long>(k) * 2 * P + p) * ldA;
  const long long oa_i = (static_cast<long long>(k) * 2 * P + P + p) * ldA;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ldA; g += gridDim.x * blockDim.x) {
    const float2 c = (g < n_tot) ? src[g] : make_float2(0.f, 0.f);
    __nv_bfloat16 h, l;
    split_bf16(c.x, h, l);
    a_hi[oa_r + g] = h;
    a_lo[oa_r + g] = l;
    if (t_hi != nullptr && g < n_tot) {
      const long long ot = (static_cast<long long>(k) * n_tot + g) * ldT;
      t_hi[ot + p] = h;
      t_lo[ot + p] = l;
    }
    split_bf16(c.y, h, l);
    a_hi[oa_i + g] = h;
    a_lo[oa_i + g] = l;
    if (t_hi != nullptr && g < n_tot) {
      const long long ot = (static_cast<long long>(k) * n_tot + g) * ldT;
      t_hi[ot + P + p] = h;
      t_lo[ot + P + p] = l;
    }
  }
}

// Reduce split-K partials of <beta|psi> into projT[k][b][p] (complex64):
// D rows m < P are Re beta_m, rows P + m are Im beta_m; columns follow the
// band-row order of k_split_bands.
//   Re <b_p|psi_b> = D[p][re b] + D[P+p][im b],  Im = D[p][im b] - D[P+p][re b]
// Threads run along the band columns of a partial row (coalesced reads).
// Block (32, 8): threadIdx.x runs along bands, threadIdx.y strides the splits;
// the 8 partial sums of each band are combined in shared memory.
__global__ void k_reduce_proj(const float* __restrict__ partial, int splits, long long part_rows, int part_ld,
                              int P, int nb, int HB, int real_out, float2* __restrict__ projT) {
  __shared__ float2 acc[8][32];
  const int k = blockIdx.z, p = blockIdx.y;
  const int b = blockIdx.x * 32 + threadIdx.x;
  float re = 0.f, im = 0.f;
  if (b < nb) {
    const int t = b / HB, j = b - t * HB;
    const int c_re = t * 2 * HB + j, c_im = c_re + HB;
    for (int s = threadIdx.y; s < splits; s += 8) {
      const float* D = partial + (static_cast<long long>(k) * splits + s) * part_rows * part_ld;
      const float* r0 = D + static_cast<long long>(p) * part_ld;
      const float* r1 = D + static_cast<long long>(P + p) * part_ld;
      re += r0[c_re] + r1[c_im];
      im += r0[c_im] - r1[c_re];
    }
  }
  acc[threadIdx.y][threadIdx.x] = make_float2(re, im);
  __syncthreads();
  if (threadIdx.y == 0 && b < nb) {
    float2 sum = acc[0][threadIdx.x];
#pragma unroll
    for (int y = 1; y < 8; ++y) {
      sum.x += acc[y][threadIdx.x].x;
      sum.y += acc[y][threadIdx.x].y;
    }
    if (real_out) sum.y = 0.f;  // real wavefunctions: the implicit -G partners cancel it
    projT[(static_cast<long long>(k) * nb + b) * P + p] = sum;
  }
}

// Reduce split-K partials of a Gram product into out (complex128):
// out[k*out_batch + i*oi + j*oj] = <X_i|Y_j>, partial rows i < nx Re X_i,
// nx + i Im X_i; columns follow the band-row order of k_split_bands.  Splits
// are summed in FP64, in split order.
__global__ void k_reduce_gram(const float* __restrict__ partial, int splits, long long part_rows, int part_ld,
                              int nx, int ny, int HB, double2* __restrict__ out, long long out_batch, int oi,
                              int oj) {
  const int k = blockIdx.z, i = blockIdx.y;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ny; j += gridDim.x * blockDim.x) {
    const int t = j / HB, jj = j - t * HB;
    const int c_re = t * 2 * HB + jj, c_im = c_re + HB;
    double re = 0.0, im = 0.0;
    for (int s = 0; s < splits; ++s) {
      const float* D = partial + (static_cast<long long>(k) * splits + s) * part_rows * part_ld;
      const float* r0 = D + static_cast<long long>(i) * part_ld;
      const float* r1 = D + static_cast<long long>(nx + i) * part_ld;
      re += static_cast<double>(r0[c_re]) + static_cast<double>(r1[c_im]);
      im += static_cast<double>(r0[c_im]) - static_cast<double>(r1[c_re]);
    }
    out[k * out_batch + static_cast<long long>(i) * oi + static_cast<long long>(j) * oj] = make_double2(re, im);
  }
}

// Dp[b][p] = sum_q D_atom[a][p'][q'] projT[b][a*pa + q'] (block-diagonal D),
// written as the back-projection B operand: rows r = t*BN + part*HB + j for
// band t*HB + j, K = 2P: real-output row (Re Dp, -Im Dp), imaginary-output
// row (Im Dp, Re Dp).
__global__ void k_dapply_split(const float2* __restrict__ projT, const float2* __restrict__ D, int n_atoms,
                               int pa, int nb, int HB, int rows, int ld, __nv_bfloat16* __restrict__ hi,
                               __nv_bfloat16* __restrict__ lo) {
  const int P = n_atoms * pa;
  const int r = blockIdx.y, k = blockIdx.z;
  const int t = r / (2 * HB), rem = r - t * 2 * HB, part = rem / HB, b = t * HB + rem % HB;
  const long long o = (static_cast<long long>(k) * rows + r) * ld;
  for (int p = threadIdx.x; p < ld; p += blockDim.x) {
    float re = 0.f, im = 0.f;
    if (b < nb && p < P) {
      const int a = p / pa, pp = p - a * pa;
      const float2* Drow = D + (static_cast<long long>(a) * pa + pp) * pa;
      const float2* x = projT + (static_cast<long long>(k) * nb + b) * P + a * pa;
      for (int q = 0; q < pa; ++q) {
        const float2 d = Drow[q], v = x[q];
        re += d.x * v.x - d.y * v.y;
        im += d.x * v.y + d.y * v.x;
      }
    }
    __nv_bfloat16 h, l;
    if (p < P) {
      split_bf16(part ? im : re, h, l);
      hi[o + p] = h;
      lo[o + p] = l;
      split_bf16(part ? re : -im, h, l);
      hi[o + P + p] = h;
      lo[o + P + p] = l;
    } else if (p >= 2 * P) {
      hi[o + p] = __float2bfloat16_rn(0.f);
      lo[o + p] = __float2bfloat16_rn(0.f);
    }
  }
}

// Band rotation operands.  C complex64 [k][n_in][n] -> A [k][n][ldA]: row g =
// (Re C_i(g), i < n_in; Im C_i(g)), K = 2 n_in, through a 32 x 32 shared tile
// (coalesced reads along g, coalesced writes along i).
__global__ void k_split_transpose(const float2* __restrict__ C, int n_in, int n, int ldA,
                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  __shared__ float2 tile[32][33];
  const int k = blockIdx.z;
  const int g0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + r, g = g0 + tx;
    tile[r][tx] = (i < n_in && g < n) ? C[(static_cast<long long>(k) * n_in + i) * n + g] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int g = g0 + r, i = i0 + tx;
    if (g >= n || i >= n_in) continue;
    const float2 v = tile[tx][r];
    const long long o = (static_cast<long long>(k) * n + g) * ldA;
    __nv_bfloat16 h, l;
    split_bf16(v.x, h, l);
    hi[o + i] = h;
    lo[o + i] = l;
    split_bf16(v.y, h, l);
    hi[o + n_in + i] = h;
    lo[o + n_in + i] = l;
  }
}

// Rotation matrix rows for the B operand: M complex64 [k][n_in][n_out] ->
// rows r = t*BN + part*HB + jj (output band j = t*HB + jj) of [k][rows][ld],
// K = 2 n_in: real-output rows (Re M_ij, -Im M_ij), imaginary-output rows
// (Im M_ij, Re M_ij); bands >= n_out and the K padding are zero.
__global__ void k_split_matrix(const float2* __restrict__ M, int n_in, int n_out, int HB, int rows, int ld,
                               __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  const int r = blockIdx.y, k = blockIdx.z;
  const int t = r / (2 * HB), rem = r - t * 2 * HB, part = rem / HB, j = t * HB + rem % HB;
  const long long o = (static_cast<long long>(k) * rows + r) * ld;
  for (int p = threadIdx.x; p < ld; p += blockDim.x) {
    float v = 0.f;
    if (j < n_out && p < 2 * n_in) {
      const int i = p < n_in ? p : p - n_in;
      const float2 m = M[(static_cast<long long>(k) * n_in + i) * n_out + j];
      v = p < n_in ? (part ? m.y : m.x) : (part ? m.x : -m.y);
    }
    __nv_bfloat16 h, l;
    split_bf16(v, h, l);
    hi[o + p] = h;
    lo[o + p] = l;
  }
}

static inline long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

}  // namespace tc

using namespace tc;

// Layout of the per-basis projector split (qgb_beta_split).
struct BetaSplitLayout {
  long long ldA, ldT, a_elems, t_elems;
};
static BetaSplitLayout beta_layout(int nk, int P, int n_tot) {
  BetaSplitLayout L;
  L.ldA = round_up(n_tot, 64);
  L.ldT = round_up(2LL * P, 64);
  L.a_elems = static_cast<long long>(nk) * 2 * P * L.ldA;
  L.t_elems = static_cast<long long>(nk) * n_tot * L.ldT;
  return L;
}
size_t beta_split_bytes(int nk, int P, int n_tot) {
  const BetaSplitLayout L = beta_layout(nk, P, n_tot);
  return static_cast<size_t>(2 * (L.a_elems + L.t_elems)) * 2 + 1024;
}

int beta_split(const void* beta, int nk, int P, int n_tot, void* out, size_t out_bytes, cudaStream_t st) {
  if (nk < 1 || P < 1 || n_tot < 1 || !beta || !out) return fail(QGB_ERR_INVALID, "bad beta_split arguments");
  if (out_bytes < beta_split_bytes(nk, P, n_tot)) return fail(QGB_ERR_WORKSPACE, "beta split buffer too small");
  const BetaSplitLayout L = beta_layout(nk, P, n_tot);
  auto* base = reinterpret_cast<__nv_bfloat16*>(round_up(reinterpret_cast<uintptr_t>(out), 256));
  __nv_bfloat16 *a_hi = base, *a_lo = a_hi + L.a_elems, *t_hi = a_lo + L.a_elems, *t_lo = t_hi + L.t_elems;
  QGB_CUDA_CHECK(cudaMemsetAsync(t_hi, 0, 2 * L.t_elems * 2, st));  // K padding of AT must read as zero
  dim3 grid(static_cast<unsigned>(std::min<long long>(64, (L.ldA + 255) / 256)), P, nk);
  k_split_beta<<<grid, 256, 0, st>>>(static_cast<const float2*>(beta), P, n_tot, static_cast<int>(L.ldA),
                                     static_cast<int>(L.ldT), a_hi, a_lo, t_hi, t_lo);
  QGB_LAUNCH_CHECK("k_split_beta");
  return QGB_OK;
}

// Pipeline depth per tile width: BN = 64 and 128 keep two CTAs per SM
// (96 KB of stages), BN = 256 runs one CTA per SM with 4 stages (192 KB).
template <int BN> constexpr int kStages = (BN == 64) ? 4 : (BN == 128 ? 3 : 4);

// Band-block tile width for the nonlocal GEMMs.
static int pick_bn(int nb) { return nb <= 32 ? 64 : (nb <= 64 ? 128 : 256); }

struct NlWorkspace {
  long long ldB, rowsB, ldB2, partial_floats, psi_elems, b2_elems;
  int splits, kb_per_split, HB, BN;
};
static NlWorkspace nl_layout(int nk, int P, int nb, int n_tot) {
  NlWorkspace W;
  W.BN = pick_bn(nb);
  W.HB = W.BN / 2;
  const long long n_tiles = (nb + W.HB - 1) / W.HB;
  W.rowsB = n_tiles * W.BN;
  W.ldB = round_up(n_tot, 64);
  W.ldB2 = round_up(2LL * P, 64);
  const int nkb = static_cast<int>((n_tot + BK - 1) / BK);
  const int m_tiles = static_cast<int>((2LL * P + BM - 1) / BM);
  const int tiles = m_tiles * static_cast<int>(n_tiles) * nk;
  int splits = std::max(1, std::min(nkb, (2 * 152 + tiles - 1) / tiles));
  W.kb_per_split = (nkb + splits - 1) / splits;
  W.splits = (nkb + W.kb_per_split - 1) / W.kb_per_split;
  W.partial_floats = static_cast<long long>(nk) * W.splits * m_tiles * BM * (n_tiles * W.BN);
  W.psi_elems = static_cast<long long>(nk) * W.rowsB * W.ldB;
  W.b2_elems = static_cast<long long>(nk) * W.rowsB * W.ldB2;
  return W;
}
size_t nonlocal_tc_workspace_bytes(int nk, int P, int nb, int n_tot) {
  const NlWorkspace W = nl_layout(nk, P, nb, n_tot);
  return static_cast<size_t>(W.partial_floats * 4 + 2 * W.psi_elems * 2 + 2 * W.b2_elems * 2) + 4 * 256 + 64;
}

// phases: 1 = steps 1-3 (everything that depends only on C), 2 = step 4 (the
// accumulation into HC), 3 = both; with 4 added, step 4 stores beta (D proj)
// into HC instead of adding it.  Phase 1 may run beside the local potential.
template <int BN>
static int nonlocal_tc_impl(const void* split, const void* D, int n_atoms, int pa, const void* C, void* HC,
                            void* projT, int nk, int nb, int n_tot, const NlWorkspace& W, unsigned char* ws,
                            int* err, int phases, const double* weight, cudaStream_t st) {
  const int P = n_atoms * pa;
  const BetaSplitLayout BL = beta_layout(nk, P, n_tot);
  auto* sbase = reinterpret_cast<const __nv_bfloat16*>(round_up(reinterpret_cast<uintptr_t>(split), 256));
  const __nv_bfloat16 *a_hi = sbase, *a_lo = a_hi + BL.a_elems, *t_hi = a_lo + BL.a_elems,
                      *t_lo = t_hi + BL.t_elems;
  unsigned char* p = reinterpret_cast<unsigned char*>(round_up(reinterpret_cast<uintptr_t>(ws), 256));
  float* partial = reinterpret_cast<float*>(p);
  p += round_up(W.partial_floats * 4, 256);
  auto* b_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* b_lo = b_hi + W.psi_elems;
  p += round_up(2 * W.psi_elems * 2, 256);
  auto* b2_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* b2_lo = b2_hi + W.b2_elems;

  if (phases & 1) {
  // 1. Wavefunctions -> bf16 hi/lo band rows.
  {
    dim3 grid(static_cast<unsigned>(std::min<long long>(32, (W.ldB + 255) / 256)), static_cast<unsigned>(W.rowsB), nk);
    k_split_bands<<<grid, 256, 0, st>>>(static_cast<const float2*>(C), nb, n_tot, W.HB, static_cast<int>(W.rowsB),
                                        static_cast<int>(W.ldB), weight, b_hi, b_lo);
    QGB_LAUNCH_CHECK("k_split_bands");
  }
  // 2. <beta|psi> partials: M = 2P, N = rowsB, K = basis, split-K.
  GemmArgs g1{};
  g1.M = 2 * P;
  g1.N = static_cast<int>(W.rowsB);
  g1.K = n_tot;
  g1.kb_per_split = W.kb_per_split;
  g1.splits = W.splits;
  g1.partial = partial;
  g1.part_ld = static_cast<int>(W.rowsB);
  g1.part_rows = (2LL * P + BM - 1) / BM * BM;
  g1.err = err;
  const int rc = launch<BN, kStages<BN>, EPI_PARTIAL>(
      Operand{a_hi, a_lo, 2LL * P, BL.ldA, 2LL * P * BL.ldA}, Operand{b_hi, b_lo, W.rowsB, W.ldB, W.rowsB * W.ldB},
      n_tot, nk, g1, st);
  if (rc) return rc;
  // 3. Reduce -> projT; apply D; build the back-projection operand.
  {
    dim3 grid((nb + 31) / 32, P, nk);
    k_reduce_proj<<<grid, dim3(32, 8), 0, st>>>(partial, W.splits, g1.part_rows, g1.part_ld, P, nb, W.HB,
                                                weight != nullptr, static_cast<float2*>(projT));
    QGB_LAUNCH_CHECK("k_reduce_proj");
    dim3 grid2(1, static_cast<unsigned>(W.rowsB), nk);
    k_dapply_split<<<grid2, 256, 0, st>>>(static_cast<const float2*>(projT), static_cast<const float2*>(D),
                                          n_atoms, pa, nb, W.HB, static_cast<int>(W.rowsB),
                                          static_cast<int>(W.ldB2), b2_hi, b2_lo);
    QGB_LAUNCH_CHECK("k_dapply_split");
  }
  }
  if (!(phases & 2)) return QGB_OK;
  // 4. HC += beta (D proj): M = basis, N = rowsB, K = 2P.
  GemmArgs g2{};
  g2.M = n_tot;
  g2.N = static_cast<int>(W.rowsB);
  g2.K = 2 * P;
  g2.kb_per_split = static_cast<int>((2LL * P + BK - 1) / BK);
  g2.splits = 1;
  g2.hc = static_cast<float2*>(HC);
  g2.hc_batch_stride = static_cast<long long>(nb) * n_tot;
  g2.hc_ld = n_tot;
  g2.nb = nb;
  g2.hc_store = (phases & 4) ? 1 : 0;
  g2.err = err;
  return launch<BN, kStages<BN>, EPI_ADD_HC>(
      Operand{t_hi, t_lo, n_tot, BL.ldT, static_cast<long long>(n_tot) * BL.ldT},
      Operand{b2_hi, b2_lo, W.rowsB, W.ldB2, W.rowsB * W.ldB2}, 2 * P, nk, g2, st);
}

int nonlocal_tc_phase(const void* split, const void* D, int n_atoms, int pa, const void* C, void* HC, void* projT,
                      int nk, int nb, int n_tot, void* ws, size_t ws_bytes, int* err, int phases, cudaStream_t st,
                      const double* weight) {
  const int P = n_atoms * pa;
  if (nk < 1 || nb < 0 || n_tot < 1 || P < 0) return fail(QGB_ERR_INVALID, "bad nonlocal_tc sizes");
  if (nb == 0 || P == 0) return QGB_OK;
  if (!split || !D || !C || !HC || !projT || !ws || !err) return fail(QGB_ERR_INVALID, "NULL pointer in nonlocal_tc");
  if (ws_bytes < nonlocal_tc_workspace_bytes(nk, P, nb, n_tot))
    return fail(QGB_ERR_WORKSPACE, "nonlocal_tc workspace too small");
  const NlWorkspace W = nl_layout(nk, P, nb, n_tot);
  unsigned char* w = static_cast<unsigned char*>(ws);
  switch (W.BN) {
    case 64:
      return nonlocal_tc_impl<64>(split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, W, w, err, phases, weight,
                                  st);
    case 128:
      return nonlocal_tc_impl<128>(split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, W, w, err, phases, weight,
                                   st);
    default:
      return nonlocal_tc_impl<256>(split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, W, w, err, phases, weight,
                                   st);
  }
}

// ---------------------------------------------------------------------------
// Subspace Gram on the tensor cores (mixed form)
// ---------------------------------------------------------------------------
//
// out[k][i][j] = sum_g conj(X[k][i][g]) Y[k][j][g] for complex64 X, Y: X split
// as the A operand (rows Re X_i, Im X_i, K = basis), Y as band rows (B), the
// split-K split-BF16x3 GEMM into FP32 partials, and the complex combination
// summed over the splits in FP64.
struct GramTcLayout {
  long long ldA, a_elems, partial_floats, psi_elems, ldB, rowsB;
  int splits, kb_per_split, HB, BN;
};
static GramTcLayout gram_tc_layout(int nk, int nx, int ny, int n) {
  GramTcLayout G;
  const NlWorkspace W = nl_layout(nk, nx, ny, n);  // the projection's layout with P -> nx
  G.ldA = round_up(n, 64);
  G.a_elems = static_cast<long long>(nk) * 2 * nx * G.ldA;
  G.partial_floats = W.partial_floats;
  G.psi_elems = W.psi_elems;
  G.ldB = W.ldB;
  G.rowsB = W.rowsB;
  G.splits = W.splits;
  G.kb_per_split = W.kb_per_split;
  G.HB = W.HB;
  G.BN = W.BN;
  return G;
}
size_t gram_tc_workspace_bytes(int nk, int nx, int ny, int n) {
  if (nk < 1 || nx < 1 || ny < 1 || n < 1) return 0;
  const GramTcLayout G = gram_tc_layout(nk, nx, ny, n);
  return static_cast<size_t>(round_up(G.partial_floats * 4, 256) + round_up(2 * G.a_elems * 2, 256) +
                             round_up(2 * G.psi_elems * 2, 256)) + 1024;
}

template <int BN>
static int gram_tc_impl(const GramTcLayout& G, const void* X, int nx, const void* Y, int ny, int nk, int n,
                        double2* out, long long out_batch, int oi, int oj, unsigned char* ws, int* err,
                        cudaStream_t st) {
  unsigned char* p = reinterpret_cast<unsigned char*>(round_up(reinterpret_cast<uintptr_t>(ws), 256));
  float* partial = reinterpret_cast<float*>(p);
  p += round_up(G.partial_floats * 4, 256);
  auto* a_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* a_lo = a_hi + G.a_elems;
  p += round_up(2 * G.a_elems * 2, 256);
  auto* b_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* b_lo = b_hi + G.psi_elems;
  {
    dim3 grid(static_cast<unsigned>(std::min<long long>(64, (G.ldA + 255) / 256)), nx, nk);
    k_split_beta<<<grid, 256, 0, st>>>(static_cast<const float2*>(X), nx, n, static_cast<int>(G.ldA), 0, a_hi,
                                       a_lo, nullptr, nullptr);
    QGB_LAUNCH_CHECK("k_split_beta");
    dim3 grid2(static_cast<unsigned>(std::min<long long>(32, (G.ldB + 255) / 256)), static_cast<unsigned>(G.rowsB),
               nk);
    k_split_bands<<<grid2, 256, 0, st>>>(static_cast<const float2*>(Y), ny, n, G.HB, static_cast<int>(G.rowsB),
                                         static_cast<int>(G.ldB), nullptr, b_hi, b_lo);
    QGB_LAUNCH_CHECK("k_split_bands");
  }
  GemmArgs g{};
  g.M = 2 * nx;
  g.N = static_cast<int>(G.rowsB);
  g.K = n;
  g.kb_per_split = G.kb_per_split;
  g.splits = G.splits;
  g.partial = partial;
  g.part_ld = static_cast<int>(G.rowsB);
  g.part_rows = (2LL * nx + BM - 1) / BM * BM;
  g.err = err;
  const int rc = launch<BN, kStages<BN>, EPI_PARTIAL>(
      Operand{a_hi, a_lo, 2LL * nx, G.ldA, 2LL * nx * G.ldA}, Operand{b_hi, b_lo, G.rowsB, G.ldB, G.rowsB * G.ldB},
      n, nk, g, st);
  if (rc) return rc;
  dim3 grid3(static_cast<unsigned>((ny + 127) / 128), nx, nk);
  k_reduce_gram<<<grid3, 128, 0, st>>>(partial, G.splits, g.part_rows, g.part_ld, nx, ny, G.HB, out, out_batch, oi,
                                       oj);
  QGB_LAUNCH_CHECK("k_reduce_gram");
  return QGB_OK;
}

int gram_tc(const void* X, int nx, const void* Y, int ny, int nk, int n, double2* out, long long out_batch, int oi,
            int oj, void* ws, size_t ws_bytes, int* err, cudaStream_t st) {
  if (nk < 0 || nx < 0 || ny < 0 || n < 1) return fail(QGB_ERR_INVALID, "bad gram_tc sizes");
  if (nk == 0 || nx == 0 || ny == 0) return QGB_OK;
  if (nk > 65535 || nx > 65535) return fail(QGB_ERR_UNSUPPORTED, "gram_tc: nk or nx above 65535");
  if (!X || !Y || !out || !ws || !err) return fail(QGB_ERR_INVALID, "NULL pointer in gram_tc");
  if (ws_bytes < gram_tc_workspace_bytes(nk, nx, ny, n)) return fail(QGB_ERR_WORKSPACE, "gram_tc workspace too small");
  const GramTcLayout G = gram_tc_layout(nk, nx, ny, n);
  unsigned char* w = static_cast<unsigned char*>(ws);
  switch (G.BN) {
    case 64: return gram_tc_impl<64>(G, X, nx, Y, ny, nk, n, out, out_batch, oi, oj, w, err, st);
    case 128: return gram_tc_impl<128>(G, X, nx, Y, ny, nk, n, out, out_batch, oi, oj, w, err, st);
    default: return gram_tc_impl<256>(G, X, nx, Y, ny, nk, n, out, out_batch, oi, oj, w, err, st);
  }
}

// ---------------------------------------------------------------------------
// Band rotation on the tensor cores (mixed form)
// ---------------------------------------------------------------------------
//
// out[k][j][g] (+)= sum_i M[k][i][j] C[k][i][g] for complex64 C, M, out: C
// transposed and split as the A operand (rows g, K = 2 n_in), M as rotation
// rows (B), one split-BF16x3 GEMM accumulating into out in its epilogue.
struct RotTcLayout {
  long long ldA, a_elems, ldB, rowsB, b_elems;
  int HB, BN;
};
static RotTcLayout rot_tc_layout(int nk, int n_in, int n_out, int n) {
  RotTcLayout R;
  R.BN = pick_bn(n_out);
  R.HB = R.BN / 2;
  R.rowsB = (n_out + R.HB - 1) / R.HB * static_cast<long long>(R.BN);
  R.ldA = round_up(2LL * n_in, 64);
  R.ldB = R.ldA;
  R.a_elems = static_cast<long long>(nk) * n * R.ldA;
  R.b_elems = static_cast<long long>(nk) * R.rowsB * R.ldB;
  return R;
}
size_t rotate_tc_workspace_bytes(int nk, int n_in, int n_out, int n) {
  if (nk < 1 || n_in < 1 || n_out < 1 || n < 1) return 0;
  const RotTcLayout R = rot_tc_layout(nk, n_in, n_out, n);
  return static_cast<size_t>(round_up(2 * R.a_elems * 2, 256) + round_up(2 * R.b_elems * 2, 256)) + 1024;
}

template <int BN>
static int rotate_tc_impl(const RotTcLayout& R, const void* C, int n_in, int nk, int n, const void* M, int n_out,
                          void* out, bool accumulate, unsigned char* ws, int* err, cudaStream_t st) {
  unsigned char* p = reinterpret_cast<unsigned char*>(round_up(reinterpret_cast<uintptr_t>(ws), 256));
  auto* a_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* a_lo = a_hi + R.a_elems;
  p += round_up(2 * R.a_elems * 2, 256);
  auto* b_hi = reinterpret_cast<__nv_bfloat16*>(p);
  auto* b_lo = b_hi + R.b_elems;
  // The K padding [2 n_in, ldA) of A is outside the tensor map's K extent and
  // reads as zero; the transpose writes only the valid columns.
  {
    dim3 grid(static_cast<unsigned>((n + 31) / 32), static_cast<unsigned>((n_in + 31) / 32), nk);
    k_split_transpose<<<grid, dim3(32, 8), 0, st>>>(static_cast<const float2*>(C), n_in, n, static_cast<int>(R.ldA),
                                                  a_hi, a_lo);
    QGB_LAUNCH_CHECK("k_split_transpose");
    dim3 grid2(1, static_cast<unsigned>(R.rowsB), nk);
    k_split_matrix<<<grid2, 256, 0, st>>>(static_cast<const float2*>(M), n_in, n_out, R.HB,
                                          static_cast<int>(R.rowsB), static_cast<int>(R.ldB), b_hi, b_lo);
    QGB_LAUNCH_CHECK("k_split_matrix");
  }
  if (!accumulate)
    QGB_CUDA_CHECK(cudaMemsetAsync(out, 0, static_cast<size_t>(nk) * n_out * n * sizeof(float2), st));
  GemmArgs g{};
  g.M = n;
  g.N = static_cast<int>(R.rowsB);
  g.K = 2 * n_in;
  g.kb_per_split = static_cast<int>((2LL * n_in + BK - 1) / BK);
  g.splits = 1;
  g.hc = static_cast<float2*>(out);
  g.hc_batch_stride = static_cast<long long>(n_out) * n;
  g.hc_ld = n;
  g.nb = n_out;
  g.err = err;
  return launch<BN, kStages<BN>, EPI_ADD_HC>(Operand{a_hi, a_lo, n, R.ldA, static_cast<long long>(n) * R.ldA},
                                             Operand{b_hi, b_lo, R.rowsB, R.ldB, R.rowsB * R.ldB}, 2 * n_in, nk, g,
                                             st);
}

int rotate_tc(const void* C, int n_in, int nk, int n, const void* M, int n_out, void* out, bool accumulate,
              void* ws, size_t ws_bytes, int* err, cudaStream_t st) {
  if (nk < 0 || n_in < 0 || n_out < 0 || n < 1) return fail(QGB_ERR_INVALID, "bad rotate_tc sizes");
  if (nk == 0 || n_out == 0) return QGB_OK;
  if (n_in == 0) {
    if (!accumulate) QGB_CUDA_CHECK(cudaMemsetAsync(out, 0, static_cast<size_t>(nk) * n_out * n * 8, st));
    return QGB_OK;
  }
  if (nk > 65535) return fail(QGB_ERR_UNSUPPORTED, "rotate_tc: nk above 65535");
  if (!C || !M || !out || !ws || !err) return fail(QGB_ERR_INVALID, "NULL pointer in rotate_tc");
  if (C == out) return fail(QGB_ERR_INVALID, "C and out must not alias");
  if (ws_bytes < rotate_tc_workspace_bytes(nk, n_in, n_out, n))
    return fail(QGB_ERR_WORKSPACE, "rotate_tc workspace too small");
  const RotTcLayout R = rot_tc_layout(nk, n_in, n_out, n);
  unsigned char* w = static_cast<unsigned char*>(ws);
  switch (R.BN) {
    case 64: return rotate_tc_impl<64>(R, C, n_in, nk, n, M, n_out, out, accumulate, w, err, st);
    case 128: return rotate_tc_impl<128>(R, C, n_in, nk, n, M, n_out, out, accumulate, w, err, st);
    default: return rotate_tc_impl<256>(R, C, n_in, nk, n, M, n_out, out, accumulate, w, err, st);
  }
}

int nonlocal_tc(const void* split, const void* D, int n_atoms, int pa, const void* C, void* HC, void* projT,
                int nk, int nb, int n_tot, void* ws, size_t ws_bytes, int* err, cudaStream_t st) {
  return nonlocal_tc_phase(split, D, n_atoms, pa, C, HC, projT, nk, nb, n_tot, ws, ws_bytes, err, 3, st, nullptr);
}

// Test aid for the bounded waits: one CTA of the GEMM whose producer issues
// no copies, so the MMA issuer's first wait runs out after `timeout_ns` and
// records error 3; no copy or MMA is in flight when it returns.  Operands
// are valid (M = 128, N = 64, K = 64 bf16 rows of `ab`, 128 + 64 rows of 64
// elements), `ws` >= 128 * 64 floats.
int tc_wait_timeout_test(const void* ab, float* ws, int* err, unsigned long long timeout_ns, cudaStream_t st) {
  if (!ab || !ws || !err || timeout_ns == 0) return fail(QGB_ERR_INVALID, "tc_wait_timeout_test arguments");
  const auto* a = static_cast<const __nv_bfloat16*>(ab);
  const auto* b = a + 128 * 64;
  GemmArgs g{};
  g.M = 128;
  g.N = 64;
  g.K = 64;
  g.kb_per_split = 1;
  g.splits = 1;
  g.partial = ws;
  g.part_ld = 64;
  g.part_rows = 128;
  g.err = err;
  g.timeout_ns = timeout_ns;
  g.skip_loads = 1;
  return launch<64, 4, EPI_PARTIAL>(Operand{a, a, 128, 64, 128 * 64}, Operand{b, b, 64, 64, 64 * 64}, 64, 1, g,
                                    st);
}

// Plain TN GEMM for tests: D (FP32 [M][N]) = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T.
int tc_gemm_test(const void* a_hi, const void* a_lo, const void* b_hi, const void* b_lo, int M, int N, int K,
                 int lda, int ldb, float* D, int* err, void* ws, size_t ws_bytes, cudaStream_t st) {
  if (M < 1 || N < 1 || K < 1 || N > 64 || lda % 8 || ldb % 8)
    return fail(QGB_ERR_INVALID, "tc_gemm_test: need N <= 64 and lda, ldb multiples of 8");
  const long long m_rows = (M + BM - 1) / BM * BM;
  if (ws_bytes < static_cast<size_t>(m_rows * 64 * 4)) return fail(QGB_ERR_WORKSPACE, "tc_gemm_test workspace");
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.kb_per_split = (K + BK - 1) / BK;
  g.splits = 1;
  g.partial = static_cast<float*>(ws);
  g.part_ld = 64;
  g.part_rows = m_rows;
  g.err = err;
  int rc = launch<64, 6, EPI_PARTIAL>(Operand{a_hi, a_lo, M, lda, static_cast<long long>(M) * lda},
                                     Operand{b_hi, b_lo, N, ldb, static_cast<long long>(N) * ldb}, K, 1, g, st);
  if (rc) return rc;
  QGB_CUDA_CHECK(cudaMemcpy2DAsync(D, N * sizeof(float), ws, 64 * sizeof(float), N * sizeof(float), M,
                                   cudaMemcpyDeviceToDevice, st));
  return QGB_OK;
}

}  // namespace qgb
