// Batched tridiagonal solves (Thomas / PCR drop-ins) for sm_103a.
//
// Replaces thomas_solve_cuda_t (triton/t_kernel_thomas.py:13-232) and
// pcr_solve_cuda_t (triton/pcr_kernel_thomas.py:15-226): B independent
// systems with a (B,K-1), b (B,K), c (B,K-1), d (B,K) -> x (B,K).
//
// One group of P lanes owns one system, CH rows per lane, held in registers
// for the whole solve (see chunk_solve.cuh).  Bands with 16-byte aligned
// bases run the bulk-staged kernel (tridiag_bulk.cu: the copy engine fills
// shared-memory stages); others run tridiag_kernel below, which loads each
// lane's rows directly; both do the same arithmetic.  Systems longer than
// 1024 rows run a serial Thomas per thread.  The reference kernels instead
// run one program per system with a scalar loop over K (Thomas) or stage
// every PCR stage through global memory.
#include <atomic>

#include "chunk_solve.cuh"

namespace dgb {

// Bulk-staged solve (tridiag_bulk.cu): DGB_OK when launched, a negative error
// code, or 1 when it does not apply (unaligned bands, stages too large).
int tridiag_bulk(int P, int ch, int64_t B, int64_t K, const float* a, const float* b,
                 const float* c, const float* d, float* x, cudaStream_t st);
int tridiag_bulk(int P, int ch, int64_t B, int64_t K, const double* a, const double* b,
                 const double* c, const double* d, double* x, cudaStream_t st);

template <typename T, int CH, int P>
__global__ void __launch_bounds__(128) tridiag_kernel(int64_t B, int64_t K,
                                                      const T* __restrict__ a,
                                                      const T* __restrict__ b,
                                                      const T* __restrict__ c,
                                                      const T* d, T* x) {
  constexpr int G = 32 / P;  // systems per warp
  const int lane = threadIdx.x & 31;
  const int r = lane % P;
  const int g = lane / P;
  const int64_t warps_total = (int64_t)gridDim.x * (blockDim.x / 32);
  const int64_t warp_id = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int64_t Km1 = K - 1;
  for (int64_t base = warp_id * G; base < B; base += warps_total * G) {
    const int64_t sys = base + g;
    const bool live = sys < B;
    T ra[CH], rb[CH], rc[CH], rd[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int64_t i = (int64_t)r * CH + j;
      const bool in = live && i < K;
      ra[j] = (in && i >= 1) ? a[sys * Km1 + i - 1] : T(0);
      rc[j] = (in && i < Km1) ? c[sys * Km1 + i] : T(0);
      rb[j] = in ? b[sys * K + i] : T(1);
      rd[j] = in ? d[sys * K + i] : T(0);
    }
    chunk_solve<T, CH, P, kFastRcp<T>>(ra, rb, rc, rd, r);
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int64_t i = (int64_t)r * CH + j;
      if (live && i < K) x[sys * K + i] = rd[j];
    }
  }
}

// Instantiated chunk sizes; a system of K rows uses the smallest CH >= K/P.
// Odd only: lane r's rows start r*CH words apart, so an odd CH puts the 32
// lanes of a shared-memory read on 32 different banks (an even CH would
// serialise them gcd(CH, 32)-fold in the bulk-staged kernel).
static const int kChunks[] = {1, 3, 5, 7, 9, 11, 13, 15, 17, 21, 25, 33};
// Longest system on the chunked kernels; longer ones run the serial Thomas.
constexpr int64_t kMaxChunkedK = 1024;

// Blocks for a grid-stride launch: every resident slot filled once (one wave;
// an oversubscribed grid would leave a partial last wave idle-tailed).
// The occupancy query runs once per kernel (no dynamic shared memory, so the
// answer does not depend on the device's size or the call).
template <typename K_>
static int64_t resident_blocks(K_ kern, int threads, int64_t needed, std::atomic<int>& cached) {
  int per_sm = cached.load(std::memory_order_relaxed);
  if (per_sm < 1) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0) !=
            cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    cached.store(per_sm, std::memory_order_relaxed);
  }
  const int64_t cap = (int64_t)device_sm_count() * per_sm;
  return needed < cap ? needed : cap;
}

template <typename T, int P>
static int launch_p(int ch, int64_t B, int64_t K, const T* a, const T* b, const T* c,
                    const T* d, T* x, cudaStream_t st) {
  const int64_t groups = (B + (32 / P) - 1) / (32 / P);
  const int64_t blocks_needed = (groups + 3) / 4;
#define DGB_CASE(CHV)                                                                        \
  case CHV: {                                                                                \
    auto kern = tridiag_kernel<T, CHV, P>;                                                   \
    static std::atomic<int> per_sm{0};                                                       \
    const int blocks = (int)resident_blocks(kern, 128, blocks_needed, per_sm);              \
    kern<<<blocks, 128, 0, st>>>(B, K, a, b, c, d, x);                                       \
  } break;
  switch (ch) {
    DGB_CASE(1) DGB_CASE(3) DGB_CASE(5) DGB_CASE(7) DGB_CASE(9) DGB_CASE(11)
    DGB_CASE(13) DGB_CASE(15) DGB_CASE(17) DGB_CASE(21) DGB_CASE(25) DGB_CASE(33)
    default:
      set_error("internal: no tridiagonal chunk instantiation for %d", ch);
      return DGB_EINVAL;
  }
#undef DGB_CASE
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

// Systems longer than the register-resident chunks hold (K > 1024): one
// thread per system runs the reference's serial Thomas recurrence
// (tridiag/pcr.py:125-183, the loop of t_kernel_thomas.py) with c' in a
// stream-ordered workspace and d' in x, each operation rounded on its own
// (no FMA contraction), so the result equals the sequential CPU Thomas bit
// for bit.  d may alias x.
__device__ __forceinline__ float tri_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double tri_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float tri_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double tri_div(double a, double b) { return __ddiv_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(128)
    thomas_serial_kernel(int64_t B, int64_t K, const T* __restrict__ a, const T* __restrict__ b,
                         const T* __restrict__ c, const T* d, T* x, T* __restrict__ cp) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const T* as = a + s * (K - 1);
  const T* bs = b + s * K;
  const T* cs = c + s * (K - 1);
  const T* ds = d + s * K;
  T* xs = x + s * K;
  T* cps = cp + s * K;
  T denom = bs[0];
  T cprev = tri_div(cs[0], denom);
  T dprev = tri_div(ds[0], denom);
  cps[0] = cprev;
  xs[0] = dprev;
  for (int64_t i = 1; i < K; ++i) {
    const T ai = as[i - 1];
    denom = tri_sub(bs[i], mul_rn(ai, cprev));
    if (i < K - 1) {
      cprev = tri_div(cs[i], denom);
      cps[i] = cprev;
    }
    dprev = tri_div(tri_sub(ds[i], mul_rn(ai, dprev)), denom);
    xs[i] = dprev;
  }
  T xnext = dprev;
  for (int64_t i = K - 2; i >= 0; --i) {
    xnext = tri_sub(xs[i], mul_rn(cps[i], xnext));
    xs[i] = xnext;
  }
}

template <typename T>
static int thomas_serial(int64_t B, int64_t K, const T* a, const T* b, const T* c, const T* d,
                         T* x, cudaStream_t st) {
  T* cp = nullptr;
  DGB_CUDA_CHECK(cudaMallocAsync((void**)&cp, (size_t)B * K * sizeof(T), st));
  thomas_serial_kernel<T><<<(unsigned)((B + 127) / 128), 128, 0, st>>>(B, K, a, b, c, d, x, cp);
  DGB_LAUNCH_CHECK();
  DGB_CUDA_CHECK(cudaFreeAsync(cp, st));
  return DGB_OK;
}

// Lanes per system: wide enough that each lane holds at most 8 rows, and
// always a power of two dividing 32.
static int default_lanes(int64_t K, int method) {
  if (method == DGB_PCR) return 32;
  int P = 4;
  while (P < 32 && (K + P - 1) / P > 8) P <<= 1;
  return P;
}

static int chunk_for(int64_t K, int P) {
  int64_t need = (K + P - 1) / P;
  for (int ch : kChunks)
    if (ch >= need) return ch;
  return -1;
}

template <typename T>
static int solve_t(int method, int64_t B, int64_t K, const T* a, const T* b, const T* c,
                   const T* d, T* x, cudaStream_t st, int lanes) {
  if (K > kMaxChunkedK) return thomas_serial<T>(B, K, a, b, c, d, x, st);
  int P = lanes > 0 ? lanes : default_lanes(K, method);
  int ch = chunk_for(K, P);
  if (ch < 0 && P < 32) {
    P = 32;
    ch = chunk_for(K, P);
  }
  if (ch < 0) return thomas_serial<T>(B, K, a, b, c, d, x, st);
  // bulk-staged kernel when the bands are 16-byte aligned and its stages fit
  const int bulk_rc = tridiag_bulk(P, ch, B, K, a, b, c, d, x, st);
  if (bulk_rc <= 0) return bulk_rc;
  switch (P) {
    case 4: return launch_p<T, 4>(ch, B, K, a, b, c, d, x, st);
    case 8: return launch_p<T, 8>(ch, B, K, a, b, c, d, x, st);
    case 16: return launch_p<T, 16>(ch, B, K, a, b, c, d, x, st);
    case 32: return launch_p<T, 32>(ch, B, K, a, b, c, d, x, st);
    default:
      set_error("lanes per system must be 4, 8, 16 or 32 (got %d)", P);
      return DGB_EINVAL;
  }
}

int tridiag_dispatch(int dtype, int method, int64_t B, int64_t K, const void* a,
                     const void* b, const void* c, const void* d, void* x, void* stream,
                     int lanes) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(method == DGB_THOMAS || method == DGB_PCR, "method must be DGB_THOMAS or DGB_PCR");
  DGB_REQUIRE(B >= 0 && K >= 1, "tridiagonal systems must have K >= 1 (got B=%lld K=%lld)",
              (long long)B, (long long)K);
  if (B == 0) return DGB_OK;
  DGB_REQUIRE(b && d && x, "b, d and x must be non-null");
  DGB_REQUIRE(K == 1 || (a && c), "a and c must be non-null when K > 1");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32)
    return solve_t<float>(method, B, K, (const float*)a, (const float*)b, (const float*)c,
                          (const float*)d, (float*)x, st, lanes);
  return solve_t<double>(method, B, K, (const double*)a, (const double*)b, (const double*)c,
                         (const double*)d, (double*)x, st, lanes);
}

}  // namespace dgb

extern "C" int dgb_tridiag_solve(int dtype, int method, int64_t B, int64_t K, const void* a,
                                 const void* b, const void* c, const void* d, void* x,
                                 void* stream) {
  return dgb::tridiag_dispatch(dtype, method, B, K, a, b, c, d, x, stream, 0);
}

extern "C" int dgb_tridiag_solve_lanes(int dtype, int64_t B, int64_t K, const void* a,
                                       const void* b, const void* c, const void* d, void* x,
                                       int32_t lanes, void* stream) {
  return dgb::tridiag_dispatch(dtype, DGB_THOMAS, B, K, a, b, c, d, x, stream, lanes);
}

// The transpose of tridiag(a, b, c) is tridiag(c, b, a).
extern "C" int dgb_tridiag_solve_transpose(int dtype, int64_t B, int64_t K, const void* a,
                                           const void* b, const void* c, const void* g,
                                           void* y, void* stream) {
  return dgb::tridiag_dispatch(dtype, DGB_THOMAS, B, K, c, b, a, g, y, stream, 0);
}
