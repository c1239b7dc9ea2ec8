// Batched tridiagonal solves (Thomas / PCR drop-ins) for sm_103a.
//
// Replaces thomas_solve_cuda_t (triton/t_kernel_thomas.py:13-232) and
// pcr_solve_cuda_t (triton/pcr_kernel_thomas.py:15-226): B independent
// systems with a (B,K-1), b (B,K), c (B,K-1), d (B,K) -> x (B,K).
//
// One group of P lanes owns one system, CH rows per lane, held in registers
// for the whole solve (see chunk_solve.cuh).  The reference kernels instead
// run one program per system with a scalar loop over K (Thomas) or stage
// every PCR stage through global memory.
#include "chunk_solve.cuh"

namespace dgb {

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
    chunk_solve<T, CH, P>(ra, rb, rc, rd, r);
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const int64_t i = (int64_t)r * CH + j;
      if (live && i < K) x[sys * K + i] = rd[j];
    }
  }
}

// Instantiated chunk sizes; a system of K rows uses the smallest CH >= K/P.
static const int kChunks[] = {1, 2, 3, 4, 5, 6, 7, 8, 10, 12, 13, 16, 24, 32};

template <typename T, int P>
static int launch_p(int ch, int64_t B, int64_t K, const T* a, const T* b, const T* c,
                    const T* d, T* x, cudaStream_t st) {
  const int64_t groups = (B + (32 / P) - 1) / (32 / P);
  const int64_t blocks_needed = (groups + 3) / 4;
  const int64_t max_blocks = (int64_t)device_sm_count() * 16;
  const int blocks = (int)(blocks_needed < max_blocks ? blocks_needed : max_blocks);
#define DGB_CASE(CHV)                                                            \
  case CHV:                                                                      \
    tridiag_kernel<T, CHV, P><<<blocks, 128, 0, st>>>(B, K, a, b, c, d, x);      \
    break;
  switch (ch) {
    DGB_CASE(1) DGB_CASE(2) DGB_CASE(3) DGB_CASE(4) DGB_CASE(5) DGB_CASE(6)
    DGB_CASE(7) DGB_CASE(8) DGB_CASE(10) DGB_CASE(12) DGB_CASE(13) DGB_CASE(16)
    DGB_CASE(24) DGB_CASE(32)
    default:
      set_error("internal: no tridiagonal chunk instantiation for %d", ch);
      return DGB_EINVAL;
  }
#undef DGB_CASE
  DGB_LAUNCH_CHECK();
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
  int P = lanes > 0 ? lanes : default_lanes(K, method);
  int ch = chunk_for(K, P);
  if (ch < 0 && P < 32) {
    P = 32;
    ch = chunk_for(K, P);
  }
  if (ch < 0) {
    set_error("tridiagonal size K=%lld exceeds the supported maximum of 1024", (long long)K);
    return DGB_ERANGE;
  }
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
