// BF16 GEMM on the 5th-generation tensor cores (tcgen05 + TMA) for the
// threshold MLP's K-major products (sm_103a):
//   C[M, N] = A[M, K] B[K, N],  A row-major [M][K], B stored as B^T [N][K]
// with M % 128 == 0, N % 256 == 0, K % 64 == 0, K <= 256 (the MLP's 256x256
// hidden layers, forward and the backward dH = dZ W^T).
//
// One CTA computes a 128 x 256 tile:
//   * thread 0 initialises one mbarrier per 64-wide K chunk and issues the TMA
//     loads of the chunk's A (128 x 64) and B (256 x 64) boxes with 128-byte
//     swizzle (all chunks of K <= 256 fit in shared memory: 192 KB);
//   * warp 0 allocates 256 TMEM columns (the FP32 accumulator, one lane per
//     row) and frees them at the end;
//   * thread 0 issues tcgen05.mma (kind::f16, M = 128, N = 256, K = 16) four
//     times per chunk as the chunk lands, then tcgen05.commit to an mbarrier;
//   * all four warps read their 32 accumulator lanes with tcgen05.ld and apply
//     the same fused epilogues as the mma.sync kernel in mlp.cu.
// Every mbarrier wait is bounded.  A load wait that gives up sets an error
// word that the host reads; the CTA then drains the copies still in flight
// and the MMAs already issued (with the full bound) before it frees its TMEM.
// Only if that drain also gives up does the CTA exit with work outstanding:
// it then keeps its TMEM and sets a second bit, and the host reports the
// context as unusable.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "common.cuh"

namespace dgb {

__device__ __forceinline__ float gelu_tc(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad_tc(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
         z * 0.3989422804014327f * expf(-0.5f * z * z);
}

namespace tc {

constexpr int BM = 128, BN = 256, BK = 64, MAX_KC = 4;
constexpr uint32_t A_CHUNK = BM * BK * 2;  // 16 KB
constexpr uint32_t B_CHUNK = BN * BK * 2;  // 32 KB
constexpr uint32_t TILE_BYTES = MAX_KC * (A_CHUNK + B_CHUNK);  // 192 KB
constexpr uint32_t SMEM_BYTES = TILE_BYTES + 1024;             // + 1024-byte alignment slack
constexpr uint32_t WAIT_LIMIT = 1u << 22;                      // polls before giving up
constexpr int kErrTimeout = 1;  // a load wait gave up; the CTA drained and skipped its tile
constexpr int kErrSuspect = 2;  // the drain gave up too: copies or MMAs may still be running

// error word of the last launch on this device (nonzero: a bounded wait gave up)
__device__ int g_tc_err;

// polls a CTA spends on each TMA load wait before it gives up (the drain waits
// always use WAIT_LIMIT); lowered only by dgb_mlp_gemm_set_wait_limit
std::atomic<uint32_t> g_load_wait_limit{WAIT_LIMIT};

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B
// BF16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// true once the phase with the given parity has completed; false after
// `limit` polls
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          uint32_t limit = WAIT_LIMIT) {
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with 128-byte swizzle: start address >> 4 (bits 0-13), leading byte offset
// 16 B (unused for swizzled K-major, bits 16-29), stride byte offset 1024 B
// between 8-row groups (bits 32-45), version 1 (bit 46), layout SWIZZLE_128B
// (bits 61-63 = 2).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ void __launch_bounds__(128, 1)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   int M, int N, int K, const float* __restrict__ bias, int epi,
                   const float* __restrict__ aux, float* __restrict__ out32,
                   __nv_bfloat16* __restrict__ out16, int* __restrict__ err,
                   uint32_t load_wait_limit) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t bar_full[MAX_KC];
  __shared__ __align__(8) uint64_t bar_mma;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  __shared__ int stuck;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const uint32_t sA = base, sB = base + MAX_KC * A_CHUNK;
  const int nk = K / BK;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;

  if (threadIdx.x == 0) {
    failed = 0;
    stuck = 0;
    for (int c = 0; c < nk; ++c) mbar_init(smem_u32(&bar_full[c]), 1);
    mbar_init(smem_u32(&bar_mma), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"((uint32_t)BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (threadIdx.x == 0) {
    for (int c = 0; c < nk; ++c) {
      const uint32_t bar = smem_u32(&bar_full[c]);
      mbar_expect_tx(bar, A_CHUNK + B_CHUNK);
      tma_load_2d(sA + c * A_CHUNK, &tmA, c * BK, m0, bar);
      tma_load_2d(sB + c * B_CHUNK, &tmB, c * BK, n0, bar);
    }
    int landed = 0;
    for (int c = 0; c < nk; ++c) {
      if (!mbar_wait(smem_u32(&bar_full[c]), 0, load_wait_limit)) break;
      landed = c + 1;
      tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint64_t a = sw128_desc(sA + c * A_CHUNK + kk * 32);
        const uint64_t b = sw128_desc(sB + c * B_CHUNK + kk * 32);
        umma_bf16(tmem, a, b, (c | kk) != 0);
      }
    }
    if (landed < nk) {
      failed = 1;
      atomicOr(err, kErrTimeout);
      // let the copies still in flight land before the CTA's memory is reused
      for (int c = landed; c < nk; ++c)
        if (!mbar_wait(smem_u32(&bar_full[c]), 0)) {
          stuck = 1;
          atomicOr(err, kErrSuspect);
        }
    }
    umma_commit(smem_u32(&bar_mma));  // arrives once every MMA issued above is done
  }
  __syncthreads();
  // the epilogue's tcgen05.ld is warp-collective: decide per warp
  bool done = __all_sync(0xffffffffu, mbar_wait(smem_u32(&bar_mma), 0));
  if (!done) {
    if (lane == 0) atomicOr(err, kErrTimeout);
    // the MMAs issued so far must finish before their TMEM is freed
    done = __all_sync(0xffffffffu, mbar_wait(smem_u32(&bar_mma), 0));
    if (!done && lane == 0) {
      stuck = 1;
      atomicOr(err, kErrSuspect);
    }
  }
  tc_fence_after();
  if (done && !failed) {
    const int m = m0 + warp * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int col = 0; col < BN; col += 16) {
      float v[16];
      tmem_ld16(lane_base + col, v);
      const int n = n0 + col;
      const int64_t o = (int64_t)m * N + n;  // multiple of 16: 16-byte vector accesses
      if (epi == 1 || epi == 2) {
        const float4* b4 = reinterpret_cast<const float4*>(bias + n);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 b = b4[q];
          v[4 * q] += b.x;
          v[4 * q + 1] += b.y;
          v[4 * q + 2] += b.z;
          v[4 * q + 3] += b.w;
        }
      }
      float w[16];  // the value written to out16
      if (epi == 2) {
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = gelu_tc(v[i]);
      } else if (epi == 3) {
        const float4* a4 = reinterpret_cast<const float4*>(aux + o);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float4 a = a4[q];
          v[4 * q] *= gelu_grad_tc(a.x);
          v[4 * q + 1] *= gelu_grad_tc(a.y);
          v[4 * q + 2] *= gelu_grad_tc(a.z);
          v[4 * q + 3] *= gelu_grad_tc(a.w);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = v[i];
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) w[i] = v[i];
      }
      if (out32) {
        float4* d4 = reinterpret_cast<float4*>(out32 + o);
#pragma unroll
        for (int q = 0; q < 4; ++q)
          d4[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      }
      if (out16) {
        uint4 pk[2];
        uint32_t* pw = reinterpret_cast<uint32_t*>(pk);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const __nv_bfloat162 h2 = __floats2bfloat162_rn(w[2 * i], w[2 * i + 1]);
          pw[i] = *reinterpret_cast<const uint32_t*>(&h2);
        }
        uint4* d16 = reinterpret_cast<uint4*>(out16 + o);
        d16[0] = pk[0];
        d16[1] = pk[1];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0 && !stuck) {  // a CTA with MMAs outstanding keeps its TMEM
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)BN)
                 : "memory");
  }
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// 2-D K-major bf16 operand: rows x K elements, row stride ld elements, box of
// 64 (K) x box_rows with 128-byte swizzle.
static int make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t K, int64_t ld,
                    uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return DGB_ECUDA;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r =
      fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box,
         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return DGB_ECUDA;
  }
  return DGB_OK;
}

}  // namespace tc

// Whether dgb_mlp_gemm runs a product on the tcgen05 kernel.
bool mlp_gemm_tc_aligned(const void* bias, const void* aux, const void* out32, const void* out16) {
  auto al = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  return al(bias) && al(aux) && al(out32) && al(out16);
}

bool mlp_gemm_tc_eligible(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam,
                          int64_t sak, const void* B, int64_t sbk, int64_t sbn) {
  return M > 0 && M % tc::BM == 0 && N > 0 && N % tc::BN == 0 && K > 0 && K % tc::BK == 0 &&
         K <= tc::BK * tc::MAX_KC && sak == 1 && sbk == 1 && sam >= K && sbn >= K &&
         sam % 8 == 0 && sbn % 8 == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
         (reinterpret_cast<uintptr_t>(B) & 15) == 0;
}

int mlp_gemm_tc(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, const void* B,
                int64_t sbn, const float* bias, int32_t epi, const float* aux, float* out32,
                void* out16, cudaStream_t st) {
  CUtensorMap mA, mB;
  int rc = tc::make_map(&mA, A, M, K, sam, tc::BM);
  if (rc) return rc;
  rc = tc::make_map(&mB, B, N, K, sbn, tc::BN);
  if (rc) return rc;
  int* err = nullptr;
  DGB_CUDA_CHECK(cudaGetSymbolAddress(reinterpret_cast<void**>(&err), tc::g_tc_err));
  DGB_CUDA_CHECK(cudaMemsetAsync(err, 0, sizeof(int), st));
  DGB_CUDA_CHECK(cudaFuncSetAttribute(tc::gemm_tc_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)tc::SMEM_BYTES));
  dim3 grid(M / tc::BM, N / tc::BN);
  tc::gemm_tc_kernel<<<grid, 128, tc::SMEM_BYTES, st>>>(
      mA, mB, M, N, K, bias, epi, aux, out32, reinterpret_cast<__nv_bfloat16*>(out16), err,
      tc::g_load_wait_limit.load());
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

}  // namespace dgb

extern "C" int dgb_mlp_gemm_status(void* stream) {
  dgb::clear_error();
  DGB_CUDA_CHECK(cudaStreamSynchronize(dgb::as_stream(stream)));
  int h = 0;
  DGB_CUDA_CHECK(cudaMemcpyFromSymbol(&h, dgb::tc::g_tc_err, sizeof(int)));
  if (h & dgb::tc::kErrSuspect) {
    dgb::set_error("a tcgen05 GEMM wait gave up and its drain did not finish (error bits %d): "
                   "copies or MMAs may still be outstanding, treat this CUDA context as unusable",
                   h);
    return DGB_ETIMEOUT;
  }
  if (h) {
    dgb::set_error("a tcgen05 GEMM load wait gave up (error bits %d); the affected tiles were "
                   "not written, the context is still usable", h);
    return DGB_ETIMEOUT;
  }
  return DGB_OK;
}

extern "C" int dgb_mlp_gemm_set_wait_limit(int64_t polls) {
  dgb::clear_error();
  const uint32_t v = polls < 0 ? dgb::tc::WAIT_LIMIT
                               : (uint32_t)(polls > (int64_t)dgb::tc::WAIT_LIMIT
                                                ? dgb::tc::WAIT_LIMIT : polls);
  dgb::tc::g_load_wait_limit.store(v);
  return DGB_OK;
}

extern "C" int dgb_mlp_gemm_path(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam,
                                 int64_t sak, const void* B, int64_t sbk, int64_t sbn) {
  return dgb::mlp_gemm_tc_eligible(M, N, K, A, sam, sak, B, sbk, sbn) ? 1 : 0;
}
