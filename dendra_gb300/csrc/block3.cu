// Batched block-tridiagonal solve with 3x3 main blocks and diagonal
// off-diagonal blocks (sm_103a): the multi-layer extracellular cable systems
// (one intracellular and two extracellular unknowns per compartment) that the
// reference's _bwd_euler_bt integrator (integrators/implicit.py:669-1136)
// hands to thomas_solve_cuda_bt (triton/bt_kernel.py:195-262).
//
// Row k of system b:  diag(lower[k-1]) x[k-1] + main[k] x[k] + diag(upper[k]) x[k+1] = rhs[k]
//   lower, upper: (B, K-1, 3);  main: (B, K, 3, 3) row-major;  rhs, x: (B, K, 3).
//
// Block Thomas, one thread per system (the K block rows of one system are a
// strict recurrence):
//   forward   P_0 = main_0,  P_k = main_k - diag(lower_{k-1}) P_{k-1}^{-1} diag(upper_{k-1})
//             r_k = rhs_k - diag(lower_{k-1}) P_{k-1}^{-1} r_{k-1}
//   backward  x_{K-1} = P_{K-1}^{-1} r_{K-1},  x_k = P_k^{-1} (r_k - diag(upper_k) x_{k+1})
// with the 3x3 inverse by cofactors over the determinant.  The inverses and
// r_k go to a scratch area laid out [k][12][B] (system index fastest), so the
// scratch traffic of a warp is coalesced; the inputs are read once, in order.
// transpose = 1 solves A^T y = g instead (main blocks transposed, lower and
// upper exchanged): the adjoint solve of the reference's backward.
#include "common.cuh"

namespace dgb {

template <typename T>
struct Mat3 {
  T a[9];
};

// inverse by cofactors / determinant
template <typename T>
__device__ __forceinline__ Mat3<T> inv3(const Mat3<T>& m) {
  const T* a = m.a;
  const T c0 = a[4] * a[8] - a[5] * a[7];
  const T c3 = a[5] * a[6] - a[3] * a[8];
  const T c6 = a[3] * a[7] - a[4] * a[6];
  const T det = a[0] * c0 + a[1] * c3 + a[2] * c6;
  const T r = T(1) / det;
  Mat3<T> v;
  v.a[0] = c0 * r;
  v.a[1] = (a[2] * a[7] - a[1] * a[8]) * r;
  v.a[2] = (a[1] * a[5] - a[2] * a[4]) * r;
  v.a[3] = c3 * r;
  v.a[4] = (a[0] * a[8] - a[2] * a[6]) * r;
  v.a[5] = (a[2] * a[3] - a[0] * a[5]) * r;
  v.a[6] = c6 * r;
  v.a[7] = (a[1] * a[6] - a[0] * a[7]) * r;
  v.a[8] = (a[0] * a[4] - a[1] * a[3]) * r;
  return v;
}

template <typename T, bool TR>
__device__ __forceinline__ Mat3<T> load_main(const T* __restrict__ p) {
  Mat3<T> m;
#pragma unroll
  for (int i = 0; i < 9; ++i) m.a[i] = __ldg(p + (TR ? (i % 3) * 3 + i / 3 : i));
  return m;
}

template <typename T, bool TR>
__global__ void __launch_bounds__(128) block3_kernel(int64_t B, int64_t K,
                                                     const T* __restrict__ lower,
                                                     const T* __restrict__ mainb,
                                                     const T* __restrict__ upper,
                                                     const T* __restrict__ rhs, T* __restrict__ x,
                                                     T* __restrict__ work) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  // A^T: the sub-diagonal of row k is upper[k-1], the super-diagonal lower[k]
  const T* lo = (TR ? upper : lower) + b * (K - 1) * 3;
  const T* up = (TR ? lower : upper) + b * (K - 1) * 3;
  const T* mb = mainb + b * K * 9;
  const T* rb = rhs + b * K * 3;
  T* xb = x + b * K * 3;
  // scratch [k][12][B]: the 9 entries of P_k^{-1}, then r_k
  auto W = [&](int64_t k, int q) -> T& { return work[(k * 12 + q) * B + b]; };

  Mat3<T> pinv = inv3(load_main<T, TR>(mb));
  T r0 = __ldg(rb), r1 = __ldg(rb + 1), r2 = __ldg(rb + 2);
#pragma unroll
  for (int q = 0; q < 9; ++q) W(0, q) = pinv.a[q];
  W(0, 9) = r0;
  W(0, 10) = r1;
  W(0, 11) = r2;
  for (int64_t k = 1; k < K; ++k) {
    const T u0 = __ldg(up + (k - 1) * 3), u1 = __ldg(up + (k - 1) * 3 + 1),
            u2 = __ldg(up + (k - 1) * 3 + 2);
    const T l0 = __ldg(lo + (k - 1) * 3), l1 = __ldg(lo + (k - 1) * 3 + 1),
            l2 = __ldg(lo + (k - 1) * 3 + 2);
    Mat3<T> m = load_main<T, TR>(mb + k * 9);
    // P_k = main_k - diag(l) P^{-1} diag(u)
    const T lr[3] = {l0, l1, l2}, uc[3] = {u0, u1, u2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) m.a[i * 3 + j] = m.a[i * 3 + j] - lr[i] * (pinv.a[i * 3 + j] * uc[j]);
    // r_k = rhs_k - diag(l) P^{-1} r_{k-1}
    const T w0 = pinv.a[0] * r0 + pinv.a[1] * r1 + pinv.a[2] * r2;
    const T w1 = pinv.a[3] * r0 + pinv.a[4] * r1 + pinv.a[5] * r2;
    const T w2 = pinv.a[6] * r0 + pinv.a[7] * r1 + pinv.a[8] * r2;
    r0 = __ldg(rb + k * 3) - l0 * w0;
    r1 = __ldg(rb + k * 3 + 1) - l1 * w1;
    r2 = __ldg(rb + k * 3 + 2) - l2 * w2;
    pinv = inv3(m);
#pragma unroll
    for (int q = 0; q < 9; ++q) W(k, q) = pinv.a[q];
    W(k, 9) = r0;
    W(k, 10) = r1;
    W(k, 11) = r2;
  }
  // backward substitution
  T x0 = pinv.a[0] * r0 + pinv.a[1] * r1 + pinv.a[2] * r2;
  T x1 = pinv.a[3] * r0 + pinv.a[4] * r1 + pinv.a[5] * r2;
  T x2 = pinv.a[6] * r0 + pinv.a[7] * r1 + pinv.a[8] * r2;
  xb[(K - 1) * 3] = x0;
  xb[(K - 1) * 3 + 1] = x1;
  xb[(K - 1) * 3 + 2] = x2;
  for (int64_t k = K - 2; k >= 0; --k) {
    const T d0 = W(k, 9) - __ldg(up + k * 3) * x0;
    const T d1 = W(k, 10) - __ldg(up + k * 3 + 1) * x1;
    const T d2 = W(k, 11) - __ldg(up + k * 3 + 2) * x2;
    T p[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) p[q] = W(k, q);
    x0 = p[0] * d0 + p[1] * d1 + p[2] * d2;
    x1 = p[3] * d0 + p[4] * d1 + p[5] * d2;
    x2 = p[6] * d0 + p[7] * d1 + p[8] * d2;
    xb[k * 3] = x0;
    xb[k * 3 + 1] = x1;
    xb[k * 3 + 2] = x2;
  }
}

template <typename T>
static int block3_t(int64_t B, int64_t K, const void* lower, const void* mainb, const void* upper,
                    const void* rhs, void* x, void* work, int transpose, cudaStream_t st) {
  const int threads = 128;
  const int64_t blocks = (B + threads - 1) / threads;
  if (transpose) {
    block3_kernel<T, true><<<(unsigned)blocks, threads, 0, st>>>(
        B, K, (const T*)lower, (const T*)mainb, (const T*)upper, (const T*)rhs, (T*)x, (T*)work);
  } else {
    block3_kernel<T, false><<<(unsigned)blocks, threads, 0, st>>>(
        B, K, (const T*)lower, (const T*)mainb, (const T*)upper, (const T*)rhs, (T*)x, (T*)work);
  }
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" size_t dgb_block3_work_size(int dtype, int64_t B, int64_t K) {
  const size_t el = dtype == DGB_F64 ? 8 : 4;
  return (B > 0 && K > 0) ? (size_t)B * (size_t)K * 12 * el : 0;
}

extern "C" int dgb_block3_solve(int dtype, int64_t B, int64_t K, const void* lower,
                                const void* main_blocks, const void* upper, const void* rhs,
                                void* x, void* work, int32_t transpose, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(B >= 1 && K >= 1, "B and K must both be >= 1");
  DGB_REQUIRE(main_blocks && rhs && x && work, "main, rhs, x and work must be non-null");
  DGB_REQUIRE(K == 1 || (lower && upper), "lower and upper must be non-null when K > 1");
  DGB_REQUIRE(transpose == 0 || transpose == 1, "transpose must be 0 or 1");
  DGB_REQUIRE(x != rhs, "x must not alias rhs");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32) return block3_t<float>(B, K, lower, main_blocks, upper, rhs, x, work,
                                               transpose, st);
  return block3_t<double>(B, K, lower, main_blocks, upper, rhs, x, work, transpose, st);
}
