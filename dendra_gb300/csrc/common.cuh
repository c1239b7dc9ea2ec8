// Shared device/host helpers for the dendra_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "../../include/dendra_gb300.h"

namespace dgb {

// ---------------------------------------------------------------------------
// Host-side error reporting (thread-local last error message).
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
void clear_error();

#define DGB_REQUIRE(cond, ...)        \
  do {                                \
    if (!(cond)) {                    \
      ::dgb::set_error(__VA_ARGS__);  \
      return DGB_EINVAL;              \
    }                                 \
  } while (0)

#define DGB_CUDA_CHECK(expr)                                                   \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess) {                                                   \
      ::dgb::set_error("%s failed: %s", #expr, cudaGetErrorString(_e));        \
      return DGB_ECUDA;                                                        \
    }                                                                          \
  } while (0)

#define DGB_LAUNCH_CHECK()                                                     \
  do {                                                                         \
    cudaError_t _e = cudaGetLastError();                                       \
    if (_e != cudaSuccess) {                                                   \
      ::dgb::set_error("kernel launch failed: %s (%s:%d)",                     \
                       cudaGetErrorString(_e), __FILE__, __LINE__);            \
      return DGB_ECUDA;                                                        \
    }                                                                          \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int device_sm_count();

// Reciprocal used by the tridiagonal and tree solves.  Exact mode: the correctly rounded 1/x.
// Fast mode (float only): the hardware approximation rcp.approx.f32 refined by
// one Newton-Raphson step, r' = r + r (1 - x r), which brings it to within
// about one ulp of 1/x for normal x with three instructions and no branch.
// The reference's Triton solves divide with the approximate float division
// (div.full.f32), so the fast mode stays inside its parity tolerances.
template <typename T, bool FAST>
__device__ __forceinline__ T solve_rcp(T x) {
  if constexpr (FAST && sizeof(T) == 4) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return fmaf(r, fmaf(-x, r, 1.0f), r);
  } else {
    return T(1) / x;
  }
}

// float64 reciprocal of the cable solves' pivots: rcp.approx.ftz.f64 refined
// by two Newton-Raphson steps r' = r + r (1 - x r), each of which doubles the
// number of correct bits, so the result is within about one ulp of 1/x for
// normal x, with five instructions and no branch (the correctly rounded
// division adds a rounding correction and a special-case path).
__device__ __forceinline__ double rcp_nr64(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// The tridiagonal drop-ins and the network's tree solve take float systems in
// fast mode, double systems exactly.
template <typename T>
constexpr bool kFastRcp = sizeof(T) == 4;

// ---------------------------------------------------------------------------
// dtype-specific HH arithmetic.  Branch thresholds and polynomial degrees
// follow the reference per dtype:
//   vtrap/exprelr  dendra/models/mechanisms/ops.py:13-125
//   phi1           dendra/models/mechanisms/_cnexp.py:46-93
//   rates          dendra/models/mod/HH.py:24-40
//   cnexp step     dendra/models/mechanisms/_cnexp.py:96-132
// ---------------------------------------------------------------------------
template <typename T>
struct Math;

template <>
struct Math<float> {
  static __device__ __forceinline__ float ex(float x) { return expf(x); }
  static __device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
  static constexpr float kVtrapLocal = 1.0f;
  static __device__ __forceinline__ float even_series(float q) {
    float q2 = q * q;
    float value = q2 * (float)(-691.0 / 1307674368000.0) + (float)(1.0 / 47900160.0);
    value = value * q2 - (float)(1.0 / 1209600.0);
    value = value * q2 + (float)(1.0 / 30240.0);
    value = value * q2 - (float)(1.0 / 720.0);
    value = value * q2 + (float)(1.0 / 12.0);
    return value;
  }
  static __device__ __forceinline__ float phi1(float z) {
    float value = z * (float)(1.0 / 3628800.0) + (float)(1.0 / 362880.0);
    value = value * z + (float)(1.0 / 40320.0);
    value = value * z + (float)(1.0 / 5040.0);
    value = value * z + (float)(1.0 / 720.0);
    value = value * z + (float)(1.0 / 120.0);
    value = value * z + (float)(1.0 / 24.0);
    value = value * z + (float)(1.0 / 6.0);
    value = value * z + 0.5f;
    value = value * z + 1.0f;
    return value;
  }
};

template <>
struct Math<double> {
  static __device__ __forceinline__ double ex(double x) { return exp(x); }
  static __device__ __forceinline__ double fabs_(double x) { return fabs(x); }
  static constexpr double kVtrapLocal = 0.5;
  static __device__ __forceinline__ double even_series(double q) {
    double q2 = q * q;
    double value = q2 * (43867.0 / 5109094217170944000.0) - 3617.0 / 10670622842880000.0;
    value = value * q2 + 1.0 / 74724249600.0;
    value = value * q2 - 691.0 / 1307674368000.0;
    value = value * q2 + 1.0 / 47900160.0;
    value = value * q2 - 1.0 / 1209600.0;
    value = value * q2 + 1.0 / 30240.0;
    value = value * q2 - 1.0 / 720.0;
    value = value * q2 + 1.0 / 12.0;
    return value;
  }
  static __device__ __forceinline__ double phi1(double z) {
    double value = z * (1.0 / 355687428096000.0) + 1.0 / 20922789888000.0;
    value = value * z + 1.0 / 1307674368000.0;
    value = value * z + 1.0 / 87178291200.0;
    value = value * z + 1.0 / 6227020800.0;
    value = value * z + 1.0 / 479001600.0;
    value = value * z + 1.0 / 39916800.0;
    value = value * z + 1.0 / 3628800.0;
    value = value * z + 1.0 / 362880.0;
    value = value * z + 1.0 / 40320.0;
    value = value * z + 1.0 / 5040.0;
    value = value * z + 1.0 / 720.0;
    value = value * z + 1.0 / 120.0;
    value = value * z + 1.0 / 24.0;
    value = value * z + 1.0 / 6.0;
    value = value * z + 0.5;
    value = value * z + 1.0;
    return value;
  }
};

// x / c for a constant integer c whose odd part exceeds 1 (10, 18, 20, 80 in
// the HH rates).  float32: the division.  float64: q = RN(x rc) with rc =
// RN(1/c) (folded at compile time), corrected once by the remainder, RN(q +
// rc RN(x - q c)) with both steps fused multiply-adds (Markstein's
// correction).  The result is the correctly rounded x / c, bit for bit the
// division's (up to the sign of a zero quotient), for finite x away from
// overflow and underflow: x / c is never a rounding midpoint (a midpoint has
// 54 significant bits and an odd last one, so c times it needs more than 53)
// and lies at least ulp/(2c) from one, while q + rc (x - q c) is within about
// 2^-51 ulp of x / c.  Three instructions instead of a division's sequence.
template <typename T>
__device__ __forceinline__ T div_c(T x, T c) {
  if constexpr (sizeof(T) == 8) {
    const T rc = T(1) / c;
    const T q = x * rc;
    return fma(fma(-q, c, x), rc, q);
  } else {
    return x / c;
  }
}

// x / (exp(x/y) - 1) with the local Bernoulli branch (y: a constant that
// div_c accepts).
template <typename T>
__device__ __forceinline__ T vtrap(T x, T y) {
  T q = div_c<T>(x, y);
  if (Math<T>::fabs_(q) <= Math<T>::kVtrapLocal) {
    T even = Math<T>::even_series(q);
    return (y - x / T(2)) + x * (q * even);
  }
  return x / (Math<T>::ex(q) - T(1));
}

// Exact affine step of x' = a - b x over dt.
template <typename T>
__device__ __forceinline__ T cnexp_step(T x, T a, T b, T dt) {
  T rate = a - b * x;
  T coef = -b;
  T z = coef * dt;
  if (Math<T>::fabs_(z) <= T(0.5)) {
    return x + dt * rate * Math<T>::phi1(z);
  }
  T eq = -a / coef;
  return eq + (x - eq) * Math<T>::ex(z);
}

// Rate constants am1 = 0.1, ah1 = 0.07, an1 = 0.01: the reference keeps its
// mechanism GLOBALs as float32 values even in float64 models, so these are the
// float32-rounded values in both precisions (am2 = 4, ah2 = 1, an2 = 0.125 are
// exact either way).
// Advance m, h, n by one cnexp step using the rates at voltage v.
template <typename T>
__device__ __forceinline__ void hh_gates(T v, T q10, T dt, T& m, T& h, T& n) {
  T alpha_m = T(0.1f) * vtrap<T>(-(v + T(40)), T(10));
  T beta_m = T(4.0) * Math<T>::ex(div_c<T>(-(v + T(65)), T(18)));
  T alpha_h = T(0.07f) * Math<T>::ex(div_c<T>(-(v + T(65)), T(20)));
  T beta_h = T(1.0) / (Math<T>::ex(div_c<T>(-(v + T(35)), T(10))) + T(1));
  T alpha_n = T(0.01f) * vtrap<T>(-(v + T(55)), T(10));
  T beta_n = T(0.125) * Math<T>::ex(div_c<T>(-(v + T(65)), T(80)));
  m = cnexp_step<T>(m, q10 * alpha_m, q10 * (alpha_m + beta_m), dt);
  h = cnexp_step<T>(h, q10 * alpha_h, q10 * (alpha_h + beta_h), dt);
  n = cnexp_step<T>(n, q10 * alpha_n, q10 * (alpha_n + beta_n), dt);
}

// ---------------------------------------------------------------------------
// float32 fast-math variant of the gate advance (opt-in, DGB_CABLE_FAST_MATH).
// Same formulas and branch rules as hh_gates, evaluated with fewer
// instructions:
//   * constant divisors become multiplications by the rounded reciprocal;
//   * the remaining divisions use the approximate reciprocal (__fdividef);
//   * three exponentials instead of six, by exact identities:
//       exp(-(v+35)/10) = exp(-(v+40)/10) * e^{0.5}
//       exp(-(v+55)/10) = exp(-(v+40)/10) * e^{-1.5}
//       exp(-(v+65)/20) = (exp(-(v+65)/80))^4
// Each substitution changes a result by a few float32 ulps; the tests hold
// the resulting voltages to the same 1e-3 mV float64 bound as the exact path.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float vtrap_fast(float x, float q, float e) {
  // x / (exp(q) - 1) with q = x / 10 and e = exp(q) supplied by the caller
  if (fabsf(q) <= 1.0f) {
    const float even = Math<float>::even_series(q);
    return (10.0f - x * 0.5f) + x * (q * even);
  }
  return __fdividef(x, e - 1.0f);
}

__device__ __forceinline__ float cnexp_fast(float x, float a, float b, float dt) {
  const float rate = a - b * x;
  const float z = -b * dt;
  if (fabsf(z) <= 0.5f) return x + dt * rate * Math<float>::phi1(z);
  const float eq = __fdividef(a, b);
  return eq + (x - eq) * expf(z);
}

__device__ __forceinline__ void hh_gates_fast(float v, float q10, float dt, float& m, float& h,
                                              float& n) {
  const float xm = -(v + 40.0f), xn = -(v + 55.0f);
  const float qm = xm * 0.1f, qn = xn * 0.1f;
  const float e10 = expf(qm);               // exp(-(v+40)/10)
  const float e_n = e10 * 0.22313016014843f;  // exp(-(v+55)/10) = e10 * e^{-1.5}
  const float e_h = e10 * 1.6487212707001282f; // exp(-(v+35)/10) = e10 * e^{0.5}
  const float u = -(v + 65.0f);
  const float e18 = expf(u * (1.0f / 18.0f));
  const float e80 = expf(u * (1.0f / 80.0f));
  const float e80_2 = e80 * e80;
  const float e20 = e80_2 * e80_2;
  const float alpha_m = 0.1f * vtrap_fast(xm, qm, e10);
  const float beta_m = 4.0f * e18;
  const float alpha_h = 0.07f * e20;
  const float beta_h = __fdividef(1.0f, e_h + 1.0f);
  const float alpha_n = 0.01f * vtrap_fast(xn, qn, e_n);
  const float beta_n = 0.125f * e80;
  m = cnexp_fast(m, q10 * alpha_m, q10 * (alpha_m + beta_m), dt);
  h = cnexp_fast(h, q10 * alpha_h, q10 * (alpha_h + beta_h), dt);
  n = cnexp_fast(n, q10 * alpha_n, q10 * (alpha_n + beta_n), dt);
}

// ---------------------------------------------------------------------------
// float32 fast-math gate advance for code in which all 32 lanes of a warp
// call it together (the persistent cable kernel's row loop).  Same formulas
// as hh_gates_fast with four changes, each tested to the same float64 bound:
//   * exponentials by ex2.approx, with the rates' constant factors folded into
//     the exponent, and reciprocals by rcp.approx;
//   * the cnexp step written as x + k (alpha - s x) phi1(z), k = q10 dt,
//     s = alpha + beta (fewer products per gate);
//   * vtrap evaluates both forms and selects per lane; the branch of the
//     cnexp step is chosen per warp by vote (a side no lane needs is not
//     evaluated, and lanes on different sides both evaluate and select);
//   * when every lane's |z| = |b dt| <= 1/16, phi1 is its Taylor polynomial
//     of degree 4 (truncation below 1.3e-9 relative, under float32
//     rounding) instead of degree 9.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float phi1_deg4(float z) {
  float value = z * (1.0f / 120.0f) + (1.0f / 24.0f);
  value = value * z + (1.0f / 6.0f);
  value = value * z + 0.5f;
  value = value * z + 1.0f;
  return value;
}

// 2^x and 1/x by the hardware approximations (ex2.approx, rcp.approx).
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void hh_gates_fast_warp(float v, float q10, float dt, float& m,
                                                   float& h, float& n) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr float L2E = 1.4426950408889634f;  // log2 e
  const float xm = -(v + 40.0f), xn = -(v + 55.0f);
  const float u = -(v + 65.0f);
  // exp(-(v+40)/10); exp(-(v+55)/10) = e10 e^{-1.5} and exp(-(v+35)/10) =
  // e10 e^{0.5} enter only through e - 1 and e + 1 (one FMA each)
  const float e10 = ex2_approx(xm * (0.1f * L2E));
  // the rates' constant factors ride in the exponent: beta_m = 4 exp(u/18),
  // beta_n = exp(u/80) / 8, alpha_h = 0.07 exp(u/20)
  const float beta_m = ex2_approx(fmaf(u, L2E / 18.0f, 2.0f));
  const float beta_n = ex2_approx(fmaf(u, L2E / 80.0f, -3.0f));
  const float alpha_h = ex2_approx(fmaf(u, L2E / 20.0f, -3.8365012677171206f));  // log2 0.07
  const float beta_h = rcp_approx(fmaf(e10, 1.6487212707001282f, 1.0f));
  // vtrap(x, 10) = x / (exp(x/10) - 1), local series for |x/10| <= 1
  const bool sm = fabsf(xm) <= 10.0f, sn = fabsf(xn) <= 10.0f;
  float vm = xm * rcp_approx(e10 - 1.0f);
  float vn = xn * rcp_approx(fmaf(e10, 0.22313016014843f, -1.0f));
  {
    // both series always: near rest some lane nearly always needs one, and
    // a warp vote with its branch measured costlier than the ten FMAs
    const float qm = xm * 0.1f, qn = xn * 0.1f;
    const float tm = (10.0f - xm * 0.5f) + xm * (qm * Math<float>::even_series(qm));
    const float tn = (10.0f - xn * 0.5f) + xn * (qn * Math<float>::even_series(qn));
    vm = sm ? tm : vm;
    vn = sn ? tn : vn;
  }
  const float alpha_m = 0.1f * vm, alpha_n = 0.01f * vn;
  // cnexp with a = q10 alpha, b = q10 (alpha + beta): z = -b dt, the step
  // x + dt (a - b x) phi1(z) = x + k (alpha - s x) phi1(z) with k = q10 dt,
  // s = alpha + beta (k is loop-invariant in the caller's row loop)
  const float k = q10 * dt;
  const float s_m = alpha_m + beta_m, s_h = alpha_h + beta_h, s_n = alpha_n + beta_n;
  const float zm = -k * s_m, zh = -k * s_h, zn = -k * s_n;
  const float zmax = fmaxf(fabsf(zm), fmaxf(fabsf(zh), fabsf(zn)));
  const float rm = k * fmaf(-s_m, m, alpha_m), rh = k * fmaf(-s_h, h, alpha_h),
              rn = k * fmaf(-s_n, n, alpha_n);
  if (__all_sync(FULL, zmax <= 0.0625f)) {
    m = fmaf(rm, phi1_deg4(zm), m);
    h = fmaf(rh, phi1_deg4(zh), h);
    n = fmaf(rn, phi1_deg4(zn), n);
    return;
  }
  float mt = fmaf(rm, Math<float>::phi1(zm), m);
  float ht = fmaf(rh, Math<float>::phi1(zh), h);
  float nt = fmaf(rn, Math<float>::phi1(zn), n);
  if (__any_sync(FULL, zmax > 0.5f)) {
    // exact relaxation: x_inf + (x - x_inf) e^z, x_inf = a / b = alpha / s
    if (fabsf(zm) > 0.5f) {
      const float eq = alpha_m * rcp_approx(s_m);
      mt = eq + (m - eq) * ex2_approx(zm * L2E);
    }
    if (fabsf(zh) > 0.5f) {
      const float eq = alpha_h * rcp_approx(s_h);
      ht = eq + (h - eq) * ex2_approx(zh * L2E);
    }
    if (fabsf(zn) > 0.5f) {
      const float eq = alpha_n * rcp_approx(s_n);
      nt = eq + (n - eq) * ex2_approx(zn * L2E);
    }
  }
  m = mt;
  h = ht;
  n = nt;
}

// Rounded product that the compiler may not fuse into an FMA.  Used where the
// reference rounds a product before a cancelling add: the extracellular
// voltages field*I (large, then differenced between neighbours), the axial
// coupling g_r (v_r - v) - g_l (v - v_l), the membrane source J - G v and J's
// reversal terms.  A fused product there rounds differently from the
// reference, and spike upstrokes amplify the difference.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// HH affine membrane terms (HH.py:109-116): G = gl + gna + gk, J = gl el + gna ena + gk ek.
template <typename T>
__device__ __forceinline__ void hh_affine(T m, T h, T n, T gnabar, T gkbar, T gl, T el,
                                          T ena, T ek, T& G, T& J) {
  T m3 = m * m * m;
  T n2 = n * n;
  T gna = gnabar * m3 * h;
  T gk = gkbar * (n2 * n2);
  G = gl + gna + gk;
  J = mul_rn(gl, el) + mul_rn(gna, ena) + mul_rn(gk, ek);
}

// hh_affine with the leak's reversal product mul_rn(gl, el) supplied (the same
// value, computed once per cable where gl and el are uniform).
template <typename T>
__device__ __forceinline__ void hh_affine_glel(T m, T h, T n, T gnabar, T gkbar, T gl, T glel,
                                               T ena, T ek, T& G, T& J) {
  T m3 = m * m * m;
  T n2 = n * n;
  T gna = gnabar * m3 * h;
  T gk = gkbar * (n2 * n2);
  G = gl + gna + gk;
  J = glel + mul_rn(gna, ena) + mul_rn(gk, ek);
}

// Rectangular pulse amp on [delay, delay + pw).
template <typename T>
__device__ __forceinline__ T rect_pulse(T t, T amp, T delay, T pw) {
  T stop = delay + pw;
  return (t >= delay && t < stop) ? amp : T(0);
}

}  // namespace dgb
