// Derivatives of the HH gate advance, for the adjoint of the cable update.
//
// Every derivative follows the branch the forward evaluation took: the local
// Bernoulli series of vtrap (|q| <= 1 float32, <= 0.5 float64) or its
// exponential form, and the Taylor phi1 branch of cnexp (|z| <= 0.5) or its
// exact exponential relaxation (mechanisms/ops.py:13-125,
// mechanisms/_cnexp.py:46-132).
#pragma once

#include "common.cuh"

namespace dgb {

// Coefficients c_k of the even series P(u) = sum_k c_k u^k, u = q^2
// (vtrap x/(e^q - 1) = y - x/2 + x q P(q^2) locally).
template <typename T>
struct EvenSeries;
template <>
struct EvenSeries<float> {
  static constexpr int D = 5;
  static __device__ __forceinline__ double c(int k) {
    const double cs[6] = {1.0 / 12.0,        -1.0 / 720.0,     1.0 / 30240.0,
                          -1.0 / 1209600.0,  1.0 / 47900160.0, -691.0 / 1307674368000.0};
    return cs[k];
  }
};
template <>
struct EvenSeries<double> {
  static constexpr int D = 8;
  static __device__ __forceinline__ double c(int k) {
    const double cs[9] = {1.0 / 12.0,
                          -1.0 / 720.0,
                          1.0 / 30240.0,
                          -1.0 / 1209600.0,
                          1.0 / 47900160.0,
                          -691.0 / 1307674368000.0,
                          1.0 / 74724249600.0,
                          -3617.0 / 10670622842880000.0,
                          43867.0 / 5109094217170944000.0};
    return cs[k];
  }
};

// dP/du
template <typename T>
__device__ __forceinline__ T even_series_du(T u) {
  constexpr int D = EvenSeries<T>::D;
  T v = T(D * EvenSeries<T>::c(D));
#pragma unroll
  for (int k = D - 1; k >= 1; --k) v = v * u + T(k * EvenSeries<T>::c(k));
  return v;
}

// d/dx of vtrap(x, y) on the branch the forward took.
template <typename T>
__device__ __forceinline__ T vtrap_dx(T x, T y) {
  const T q = x / y;
  if (Math<T>::fabs_(q) <= Math<T>::kVtrapLocal) {
    const T u = q * q;
    const T P = Math<T>::even_series(q);
    const T dP = even_series_du<T>(u);
    return T(-0.5) + T(2) * q * P + T(2) * q * u * dP;
  }
  const T e = Math<T>::ex(q);
  const T em1 = e - T(1);
  return (em1 - x * e / y) / (em1 * em1);
}

// phi1 polynomial degree (terms z^k / (k+1)!, k = 0..N) and its derivative.
template <typename T>
struct Phi1Deg;
template <>
struct Phi1Deg<float> {
  static constexpr int N = 9;
};
template <>
struct Phi1Deg<double> {
  static constexpr int N = 16;
};

template <typename T>
__device__ __forceinline__ T phi1_dz(T z) {
  constexpr int N = Phi1Deg<T>::N;
  // d/dz sum_{k=0}^{N} z^k/(k+1)! = sum_{k=1}^{N} k z^(k-1)/(k+1)!
  double fact = 1.0;  // (N+1)!
  for (int i = 2; i <= N + 1; ++i) fact *= i;
  T v = T(N / fact);
#pragma unroll
  for (int k = N - 1; k >= 1; --k) {
    fact /= (k + 2);  // now (k+1)!
    v = v * z + T(k / fact);
  }
  return v;
}

// x' = cnexp(x, a, b, dt) and its partials dx'/dx, dx'/da, dx'/db.
template <typename T>
__device__ __forceinline__ T cnexp_partials(T x, T a, T b, T dt, T& dx, T& da, T& db) {
  const T rate = a - b * x;
  const T coef = -b;
  const T z = coef * dt;
  if (Math<T>::fabs_(z) <= T(0.5)) {
    const T ph = Math<T>::phi1(z);
    const T dph = phi1_dz<T>(z);
    dx = T(1) - dt * b * ph;
    da = dt * ph;
    db = dt * (-x) * ph + dt * rate * dph * (-dt);
    return x + dt * rate * ph;
  }
  const T E = Math<T>::ex(z);
  const T eq = -a / coef;
  dx = E;
  da = (T(1) - E) / b;
  db = -(a / (b * b)) * (T(1) - E) - (x - eq) * E * dt;
  return eq + (x - eq) * E;
}

// Gate advance with partials: new gates and, per gate, d(new)/d(old) and
// d(new)/dv.  Same arithmetic as hh_gates for the new values.
template <typename T>
__device__ __forceinline__ void hh_gates_partials(T v, T q10, T dt, T& m, T& h, T& n, T& dm_m,
                                                  T& dm_v, T& dh_h, T& dh_v, T& dn_n, T& dn_v) {
  const T xm = -(v + T(40)), xn = -(v + T(55));
  const T alpha_m = T(0.1f) * vtrap<T>(xm, T(10));
  const T beta_m = T(4.0) * Math<T>::ex(-(v + T(65)) / T(18));
  const T alpha_h = T(0.07f) * Math<T>::ex(-(v + T(65)) / T(20));
  const T eh = Math<T>::ex(-(v + T(35)) / T(10));
  const T beta_h = T(1.0) / (eh + T(1));
  const T alpha_n = T(0.01f) * vtrap<T>(xn, T(10));
  const T beta_n = T(0.125) * Math<T>::ex(-(v + T(65)) / T(80));
  // d/dv of the rates
  const T dam = -T(0.1f) * vtrap_dx<T>(xm, T(10));
  const T dbm = -beta_m / T(18);
  const T dah = -alpha_h / T(20);
  const T dbh = eh / (T(10) * (eh + T(1)) * (eh + T(1)));
  const T dan = -T(0.01f) * vtrap_dx<T>(xn, T(10));
  const T dbn = -beta_n / T(80);
  T pa, pb;
  m = cnexp_partials<T>(m, q10 * alpha_m, q10 * (alpha_m + beta_m), dt, dm_m, pa, pb);
  dm_v = pa * q10 * dam + pb * q10 * (dam + dbm);
  h = cnexp_partials<T>(h, q10 * alpha_h, q10 * (alpha_h + beta_h), dt, dh_h, pa, pb);
  dh_v = pa * q10 * dah + pb * q10 * (dah + dbh);
  n = cnexp_partials<T>(n, q10 * alpha_n, q10 * (alpha_n + beta_n), dt, dn_n, pa, pb);
  dn_v = pa * q10 * dan + pb * q10 * (dan + dbn);
}

// ---------------------------------------------------------------------------
// float32 fast-math variant (DGB_CABLE_FAST_MATH): the same gates and partials
// with the forward fast path's shared exponentials (hh_gates_fast), fast
// exponentials and approximate reciprocals, and a branch-free vtrap (both
// branches evaluated, the forward's branch selected).  Derivatives change by
// a few float32 ulps, far inside the float32 gradient tolerance.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float vtrap_fast_d(float x, float q, float e, float& dvx) {
  const float u = q * q;
  const float P = Math<float>::even_series(q);
  const float dP = even_series_du<float>(u);
  const float ser = (10.0f - x * 0.5f) + x * (q * P);
  const float dser = -0.5f + 2.0f * q * P + 2.0f * q * u * dP;
  const float rinv = __fdividef(1.0f, e - 1.0f);
  const float ex = x * rinv;
  const float dex = rinv * (1.0f - q * e * rinv);
  const bool local = fabsf(q) <= 1.0f;
  dvx = local ? dser : dex;
  return local ? ser : ex;
}

__device__ __forceinline__ float cnexp_partials_fast(float x, float a, float b, float dt,
                                                     float& dx, float& da, float& db) {
  const float rate = a - b * x;
  const float z = -b * dt;
  if (fabsf(z) <= 0.5f) {
    const float ph = Math<float>::phi1(z);
    const float dph = phi1_dz<float>(z);
    dx = 1.0f - dt * b * ph;
    da = dt * ph;
    db = -dt * x * ph - dt * dt * rate * dph;
    return x + dt * rate * ph;
  }
  const float E = __expf(z);
  const float binv = __fdividef(1.0f, b);
  const float eq = a * binv;
  const float omE = 1.0f - E;
  dx = E;
  da = omE * binv;
  db = -eq * binv * omE - (x - eq) * E * dt;
  return eq + (x - eq) * E;
}

__device__ __forceinline__ void hh_gates_partials_fast(float v, float q10, float dt, float& m,
                                                       float& h, float& n, float& dm_m,
                                                       float& dm_v, float& dh_h, float& dh_v,
                                                       float& dn_n, float& dn_v) {
  const float xm = -(v + 40.0f), xn = -(v + 55.0f);
  const float qm = xm * 0.1f, qn = xn * 0.1f;
  const float e10 = __expf(qm);                   // exp(-(v+40)/10)
  const float e_n = e10 * 0.22313016014843f;      // exp(-(v+55)/10)
  const float e_h = e10 * 1.6487212707001282f;    // exp(-(v+35)/10)
  const float u = -(v + 65.0f);
  const float e18 = __expf(u * (1.0f / 18.0f));
  const float e80 = __expf(u * (1.0f / 80.0f));
  const float e80_2 = e80 * e80;
  const float e20 = e80_2 * e80_2;
  float dvm, dvn;
  const float alpha_m = 0.1f * vtrap_fast_d(xm, qm, e10, dvm);
  const float beta_m = 4.0f * e18;
  const float alpha_h = 0.07f * e20;
  const float rh = __fdividef(1.0f, e_h + 1.0f);
  const float beta_h = rh;
  const float alpha_n = 0.01f * vtrap_fast_d(xn, qn, e_n, dvn);
  const float beta_n = 0.125f * e80;
  const float dam = -0.1f * dvm;
  const float dbm = -beta_m * (1.0f / 18.0f);
  const float dah = -alpha_h * (1.0f / 20.0f);
  const float dbh = e_h * rh * rh * 0.1f;
  const float dan = -0.01f * dvn;
  const float dbn = -beta_n * (1.0f / 80.0f);
  float pa, pb;
  m = cnexp_partials_fast(m, q10 * alpha_m, q10 * (alpha_m + beta_m), dt, dm_m, pa, pb);
  dm_v = pa * q10 * dam + pb * q10 * (dam + dbm);
  h = cnexp_partials_fast(h, q10 * alpha_h, q10 * (alpha_h + beta_h), dt, dh_h, pa, pb);
  dh_v = pa * q10 * dah + pb * q10 * (dah + dbh);
  n = cnexp_partials_fast(n, q10 * alpha_n, q10 * (alpha_n + beta_n), dt, dn_n, pa, pb);
  dn_v = pa * q10 * dan + pb * q10 * (dan + dbn);
}

}  // namespace dgb
