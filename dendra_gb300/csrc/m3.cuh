// 3x3 blocks for the block solvers (block3.cu, dhs_block3.cu): row-major
// storage, cofactor inverse, products.
#pragma once

namespace dgb {

template <typename T>
struct M3 {
  T a[9];
};

template <typename T>
__device__ __forceinline__ M3<T> inv3(const M3<T>& m) {
  const T* a = m.a;
  const T c0 = a[4] * a[8] - a[5] * a[7];
  const T c3 = a[5] * a[6] - a[3] * a[8];
  const T c6 = a[3] * a[7] - a[4] * a[6];
  const T det = a[0] * c0 + a[1] * c3 + a[2] * c6;
  const T r = T(1) / det;
  M3<T> v;
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

template <typename T>
__device__ __forceinline__ M3<T> mm(const M3<T>& x, const M3<T>& y) {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      z.a[i * 3 + j] = x.a[i * 3] * y.a[j] + x.a[i * 3 + 1] * y.a[3 + j] + x.a[i * 3 + 2] * y.a[6 + j];
  return z;
}

template <typename T>
__device__ __forceinline__ void mv(const M3<T>& x, const T* v, T* out) {
#pragma unroll
  for (int i = 0; i < 3; ++i) out[i] = x.a[i * 3] * v[0] + x.a[i * 3 + 1] * v[1] + x.a[i * 3 + 2] * v[2];
}

}  // namespace dgb
