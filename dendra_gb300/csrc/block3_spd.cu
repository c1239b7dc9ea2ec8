// SPD block-Thomas solves of 3x3 block-tridiagonal systems on sm_103a: the
// method="spd" solver of the multi-layer extracellular integrator
// (integrators/implicit.py:669-1136), drop-in for solve_bt_spd_cuda
// (triton/bt_spd_kernel.py:583-755).
//
// Row k: diag(lower[k-1]) x[k-1] + main[k] x[k] + diag(upper[k]) x[k+1] = rhs[k].
// One thread per system, sequential over the rows like the reference:
//   S_0 = main_0;  S_k = main_k - diag(lower_{k-1}) S_{k-1}^-1 diag(upper_{k-1})
//   d_k = rhs_k - lower_{k-1} o S_{k-1}^-1 d_{k-1}
// every S_k factored as L_k L_k^T after symmetrising its off-diagonal pairs
// (midpoints that neither overflow nor lose subnormals); a block that is not
// positive definite gets a diagonal shift tau (its Gershgorin deficit plus a
// margin max(eps_abs, eps_rel trace)), then 10 margins more, and the row is
// reported (info = 1) if that still fails.  Back substitution
//   x_{K-1} = S^-1 d_{K-1},  x_k = S_k^-1 (d_k - upper_k o x_{k+1}).
// The factors are kept (chol) for the backward's solve with the same system.
#include <float.h>

#include "common.cuh"

namespace dgb {

template <typename T>
struct SpdLimits;
template <>
struct SpdLimits<float> {
  static constexpr float half_max = FLT_MAX / 2, twice_tiny = 2 * FLT_MIN;
  static constexpr float eps_rel = 1e-6f, eps_abs = 1e-18f;
};
template <>
struct SpdLimits<double> {
  static constexpr double half_max = DBL_MAX / 2, twice_tiny = 2 * DBL_MIN;
  static constexpr double eps_rel = 1e-12, eps_abs = 1e-30;
};

// (a + b) / 2 without overflow of large finite values or loss of subnormals.
template <typename T>
__device__ __forceinline__ T sym_mid(T a, T b) {
  const T hm = SpdLimits<T>::half_max, tt = SpdLimits<T>::twice_tiny;
  if (fabs(a) <= hm && fabs(b) <= hm) return T(0.5) * (a + b);
  if (fabs(a) < tt) return a + T(0.5) * b;
  if (fabs(b) < tt) return T(0.5) * a + b;
  return T(0.5) * a + T(0.5) * b;
}

// Lower Cholesky factor of a symmetric 3x3 (row-major, lower triangle used);
// false when a pivot is not positive (the factor is then not used).
template <typename T>
__device__ __forceinline__ bool chol3(const T* a, T* L) {
  const bool c0 = a[0] > T(0);
  const T l00 = sqrt(c0 ? a[0] : T(1));
  const T l10 = a[1] / l00, l20 = a[2] / l00;
  const T s11 = a[4] - l10 * l10;
  const bool c1 = s11 > T(0);
  const T l11 = sqrt(c1 ? s11 : T(1));
  const T l21 = (a[5] - l10 * l20) / l11;
  const T s22 = a[8] - l20 * l20 - l21 * l21;
  const bool c2 = s22 > T(0);
  const T l22 = sqrt(c2 ? s22 : T(1));
  L[0] = l00;
  L[1] = T(0);
  L[2] = T(0);
  L[3] = l10;
  L[4] = l11;
  L[5] = T(0);
  L[6] = l20;
  L[7] = l21;
  L[8] = l22;
  return c0 && c1 && c2;
}

template <typename T>
__device__ __forceinline__ bool chol3_bumped(T* a, T* L) {
  const T m01 = sym_mid(a[1], a[3]), m02 = sym_mid(a[2], a[6]), m12 = sym_mid(a[5], a[7]);
  a[1] = a[3] = m01;
  a[2] = a[6] = m02;
  a[5] = a[7] = m12;
  if (chol3(a, L)) return true;
  const T tr = fabs(a[0]) + fabs(a[4]) + fabs(a[8]);
  const T g0 = a[0] - (fabs(a[1]) + fabs(a[2]));
  const T g1 = a[4] - (fabs(a[3]) + fabs(a[5]));
  const T g2 = a[8] - (fabs(a[6]) + fabs(a[7]));
  const T gmin = fmin(g0, fmin(g1, g2));
  const T margin = fmax(SpdLimits<T>::eps_abs, SpdLimits<T>::eps_rel * tr);
  const T tau = gmin > T(0) ? margin : -gmin + margin;
  T b[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) b[q] = a[q];
  b[0] = a[0] + tau;
  b[4] = a[4] + tau;
  b[8] = a[8] + tau;
  if (chol3(b, L)) return true;
  const T tau2 = T(10) * margin;
  b[0] = b[0] + tau2;
  b[4] = b[4] + tau2;
  b[8] = b[8] + tau2;
  return chol3(b, L);
}

// (L L^T)^-1 b
template <typename T>
__device__ __forceinline__ void chol_solve3(const T* L, const T* b, T* x) {
  const T y0 = b[0] / L[0];
  const T y1 = (b[1] - L[3] * y0) / L[4];
  const T y2 = (b[2] - L[6] * y0 - L[7] * y1) / L[8];
  x[2] = y2 / L[8];
  x[1] = (y1 - L[7] * x[2]) / L[4];
  x[0] = (y0 - L[3] * x[1] - L[6] * x[2]) / L[0];
}

template <typename T>
__global__ void __launch_bounds__(128)
    block3_spd_kernel(int64_t B, int64_t K, const T* __restrict__ lower,
                      const T* __restrict__ mainb, const T* __restrict__ upper,
                      const T* __restrict__ rhs, T* __restrict__ x, T* __restrict__ chol,
                      int32_t* __restrict__ info) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const T* lo = lower + s * (K - 1) * 3;
  const T* up = upper + s * (K - 1) * 3;
  const T* M = mainb + s * K * 9;
  const T* d = rhs + s * K * 3;
  T* X = x + s * K * 3;  // modified right-hand sides, then the solution
  T* C = chol + s * K * 9;
  int32_t* I = info + s * K;
  T a[9], L[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) a[q] = M[q];
  I[0] = chol3_bumped(a, L) ? 0 : 1;
#pragma unroll
  for (int q = 0; q < 9; ++q) C[q] = L[q];
  T dk[3] = {d[0], d[1], d[2]};
  X[0] = dk[0];
  X[1] = dk[1];
  X[2] = dk[2];
  for (int64_t k = 1; k < K; ++k) {
    const T u0 = up[(k - 1) * 3], u1 = up[(k - 1) * 3 + 1], u2 = up[(k - 1) * 3 + 2];
    const T l0 = lo[(k - 1) * 3], l1 = lo[(k - 1) * 3 + 1], l2 = lo[(k - 1) * 3 + 2];
    T c0[3], c1[3], c2[3];
    const T e0[3] = {u0, T(0), T(0)}, e1[3] = {T(0), u1, T(0)}, e2[3] = {T(0), T(0), u2};
    chol_solve3(L, e0, c0);
    chol_solve3(L, e1, c1);
    chol_solve3(L, e2, c2);
    const T* Mk = M + k * 9;
    a[0] = Mk[0] - l0 * c0[0];
    a[1] = Mk[1] - l0 * c1[0];
    a[2] = Mk[2] - l0 * c2[0];
    a[3] = Mk[3] - l1 * c0[1];
    a[4] = Mk[4] - l1 * c1[1];
    a[5] = Mk[5] - l1 * c2[1];
    a[6] = Mk[6] - l2 * c0[2];
    a[7] = Mk[7] - l2 * c1[2];
    a[8] = Mk[8] - l2 * c2[2];
    T t[3];
    chol_solve3(L, dk, t);
    dk[0] = d[k * 3] - l0 * t[0];
    dk[1] = d[k * 3 + 1] - l1 * t[1];
    dk[2] = d[k * 3 + 2] - l2 * t[2];
    X[k * 3] = dk[0];
    X[k * 3 + 1] = dk[1];
    X[k * 3 + 2] = dk[2];
    I[k] = chol3_bumped(a, L) ? 0 : 1;
#pragma unroll
    for (int q = 0; q < 9; ++q) C[k * 9 + q] = L[q];
  }
  T xn[3];
  chol_solve3(L, dk, xn);
  X[(K - 1) * 3] = xn[0];
  X[(K - 1) * 3 + 1] = xn[1];
  X[(K - 1) * 3 + 2] = xn[2];
  for (int64_t k = K - 2; k >= 0; --k) {
    const T r[3] = {X[k * 3] - up[k * 3] * xn[0], X[k * 3 + 1] - up[k * 3 + 1] * xn[1],
                    X[k * 3 + 2] - up[k * 3 + 2] * xn[2]};
    chol_solve3(C + k * 9, r, xn);
    X[k * 3] = xn[0];
    X[k * 3 + 1] = xn[1];
    X[k * 3 + 2] = xn[2];
  }
}

// The same system solved with cached factors (the backward's solve).
template <typename T>
__global__ void __launch_bounds__(128)
    block3_spd_chol_kernel(int64_t B, int64_t K, const T* __restrict__ lower,
                           const T* __restrict__ upper, const T* __restrict__ chol,
                           const T* __restrict__ rhs, T* __restrict__ x) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const T* lo = lower + s * (K - 1) * 3;
  const T* up = upper + s * (K - 1) * 3;
  const T* C = chol + s * K * 9;
  const T* d = rhs + s * K * 3;
  T* X = x + s * K * 3;
  T dk[3] = {d[0], d[1], d[2]};
  X[0] = dk[0];
  X[1] = dk[1];
  X[2] = dk[2];
  for (int64_t k = 1; k < K; ++k) {
    T t[3];
    chol_solve3(C + (k - 1) * 9, dk, t);
    dk[0] = d[k * 3] - lo[(k - 1) * 3] * t[0];
    dk[1] = d[k * 3 + 1] - lo[(k - 1) * 3 + 1] * t[1];
    dk[2] = d[k * 3 + 2] - lo[(k - 1) * 3 + 2] * t[2];
    X[k * 3] = dk[0];
    X[k * 3 + 1] = dk[1];
    X[k * 3 + 2] = dk[2];
  }
  T xn[3];
  chol_solve3(C + (K - 1) * 9, dk, xn);
  X[(K - 1) * 3] = xn[0];
  X[(K - 1) * 3 + 1] = xn[1];
  X[(K - 1) * 3 + 2] = xn[2];
  for (int64_t k = K - 2; k >= 0; --k) {
    const T r[3] = {X[k * 3] - up[k * 3] * xn[0], X[k * 3 + 1] - up[k * 3 + 1] * xn[1],
                    X[k * 3 + 2] - up[k * 3 + 2] * xn[2]};
    chol_solve3(C + k * 9, r, xn);
    X[k * 3] = xn[0];
    X[k * 3 + 1] = xn[1];
    X[k * 3 + 2] = xn[2];
  }
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_block3_spd_solve(int dtype, int64_t B, int64_t K, const void* lower,
                                    const void* main_blocks, const void* upper, const void* rhs,
                                    void* x, void* chol, int32_t* info, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(B >= 0 && K >= 1, "K must be >= 1");
  if (B == 0) return DGB_OK;
  DGB_REQUIRE(main_blocks && rhs && x && chol && info && (K == 1 || (lower && upper)),
              "pointers must be non-null");
  DGB_REQUIRE(x != rhs, "x must not alias rhs");
  const unsigned blocks = (unsigned)((B + 127) / 128);
  if (dtype == DGB_F32)
    block3_spd_kernel<float><<<blocks, 128, 0, as_stream(stream)>>>(
        B, K, (const float*)lower, (const float*)main_blocks, (const float*)upper,
        (const float*)rhs, (float*)x, (float*)chol, info);
  else
    block3_spd_kernel<double><<<blocks, 128, 0, as_stream(stream)>>>(
        B, K, (const double*)lower, (const double*)main_blocks, (const double*)upper,
        (const double*)rhs, (double*)x, (double*)chol, info);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_block3_spd_solve_chol(int dtype, int64_t B, int64_t K, const void* lower,
                                         const void* upper, const void* chol, const void* rhs,
                                         void* x, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(B >= 0 && K >= 1, "K must be >= 1");
  if (B == 0) return DGB_OK;
  DGB_REQUIRE(chol && rhs && x && (K == 1 || (lower && upper)), "pointers must be non-null");
  DGB_REQUIRE(x != rhs, "x must not alias rhs");
  const unsigned blocks = (unsigned)((B + 127) / 128);
  if (dtype == DGB_F32)
    block3_spd_chol_kernel<float><<<blocks, 128, 0, as_stream(stream)>>>(
        B, K, (const float*)lower, (const float*)upper, (const float*)chol, (const float*)rhs,
        (float*)x);
  else
    block3_spd_chol_kernel<double><<<blocks, 128, 0, as_stream(stream)>>>(
        B, K, (const double*)lower, (const double*)upper, (const double*)chol,
        (const double*)rhs, (double*)x);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}
