// Batched block-tridiagonal solve with 3x3 main blocks and diagonal
// off-diagonal blocks (sm_103a): the multi-layer extracellular cable systems
// (one intracellular and two extracellular unknowns per compartment) that the
// reference's _bwd_euler_bt integrator (integrators/implicit.py:669-1136)
// hands to thomas_solve_cuda_bt (triton/bt_kernel.py:195-262).
//
// Row k of system b:  diag(lower[k-1]) x[k-1] + main[k] x[k] + diag(upper[k]) x[k+1] = rhs[k]
//   lower, upper: (B, K-1, 3);  main: (B, K, 3, 3) row-major;  rhs, x: (B, K, 3).
//
// One warp per system, the block form of the chunked solve of chunk_solve.cuh:
//   1. lane r owns block rows r*ch .. r*ch+ch-1 (identity rows past K) and
//      eliminates them in sequence, leaving x_j = dp_j - ap_j x_first - cp_j x_{j+1}
//      for its rows j >= 1 (ap, cp full 3x3);
//   2. a backward sweep rewrites them as x_j = d2_j - a2_j x_first - c2_j x_next,
//      x_next being the first unknown of the next lane;
//   3. each lane's first row becomes one reduced block row coupling the first
//      unknowns of its neighbours; 5 stages of block PCR across the 32 lanes
//      (warp shuffles) decouple them;
//   4. back substitution.
// Each warp reads its system once, in order (read-only path); the per-row
// factors stay in shared memory planes [q][j][lane] (bank-conflict free).
// transpose = 1 solves A^T y = g instead (main blocks transposed, lower and
// upper exchanged): the adjoint solve of the reference's backward.
#include "chunk_solve.cuh"
#include "common.cuh"
#include "m3.cuh"

namespace dgb {

// diag(d) * x (row scaling) and x * diag(d) (column scaling)
template <typename T>
__device__ __forceinline__ M3<T> dl(const T* d, const M3<T>& x) {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 9; ++i) z.a[i] = d[i / 3] * x.a[i];
  return z;
}
template <typename T>
__device__ __forceinline__ M3<T> dr(const M3<T>& x, const T* d) {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 9; ++i) z.a[i] = x.a[i] * d[i % 3];
  return z;
}

template <typename T>
__device__ __forceinline__ M3<T> shfl_up_m(const M3<T>& x, int s) {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 9; ++i) z.a[i] = shfl_up<T>(x.a[i], s, 32);
  return z;
}
template <typename T>
__device__ __forceinline__ M3<T> shfl_down_m(const M3<T>& x, int s) {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 9; ++i) z.a[i] = shfl_down<T>(x.a[i], s, 32);
  return z;
}

template <typename T>
__device__ __forceinline__ M3<T> zero3() {
  M3<T> z;
#pragma unroll
  for (int i = 0; i < 9; ++i) z.a[i] = T(0);
  return z;
}

// per-row planes: ap (0..8), cp (9..17), dp (18..20)
constexpr int kBlockPlanes = 21;

template <typename T, bool TR>
__device__ void block_system(int64_t b, int K, const T* __restrict__ lower,
                             const T* __restrict__ mainb, const T* __restrict__ upper,
                             const T* __restrict__ rhs, T* __restrict__ x, T* sm, int ch) {
  const int r = threadIdx.x & 31;
  const int last = ch - 1;
  auto S = [&](int q, int j) -> T& { return sm[(q * ch + j) * 32 + r]; };
  // A^T: the sub-diagonal of row i is upper[i-1], the super-diagonal lower[i]
  const T* sub = (TR ? upper : lower) + b * (int64_t)(K - 1) * 3;
  const T* sup = (TR ? lower : upper) + b * (int64_t)(K - 1) * 3;
  const T* mb = mainb + b * (int64_t)K * 9;
  const T* rb = rhs + b * (int64_t)K * 3;
  auto load_row = [&](int i, T* a, M3<T>& m, T* c, T* d) {
    const bool in = i < K;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      a[q] = (in && i > 0) ? __ldg(sub + (i - 1) * 3 + q) : T(0);
      c[q] = (i < K - 1) ? __ldg(sup + i * 3 + q) : T(0);
      d[q] = in ? __ldg(rb + i * 3 + q) : T(0);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q)
      m.a[q] = in ? __ldg(mb + i * 9 + (TR ? (q % 3) * 3 + q / 3 : q)) : (q % 4 == 0 ? T(1) : T(0));
  };

  // ---- 1. local elimination
  T As[3], Cs[3], Ds[3];
  M3<T> Ms;
  load_row(r * ch, As, Ms, Cs, Ds);
  M3<T> ap = zero3<T>(), cp = zero3<T>();
  T dp[3] = {T(0), T(0), T(0)};
  for (int j = 1; j < ch; ++j) {
    T a[3], c[3], d[3];
    M3<T> m;
    load_row(r * ch + j, a, m, c, d);
    if (j == 1) {
      const M3<T> R = inv3(m);
      ap = dr(R, a);
      cp = dr(R, c);
      mv(R, d, dp);
    } else {
      const M3<T> acp = dl(a, cp);
      M3<T> piv;
#pragma unroll
      for (int q = 0; q < 9; ++q) piv.a[q] = m.a[q] - acp.a[q];
      const M3<T> R = inv3(piv);
      const M3<T> Rap = mm(R, dl(a, ap));
#pragma unroll
      for (int q = 0; q < 9; ++q) ap.a[q] = -Rap.a[q];
      cp = dr(R, c);
      T e[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) e[q] = d[q] - a[q] * dp[q];
      mv(R, e, dp);
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      S(q, j) = ap.a[q];
      S(9 + q, j) = cp.a[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) S(18 + q, j) = dp[q];
  }
  // row ch-1 in the form x = De - Ae x_first - Ce x_next
  const M3<T> Ae = ap, Ce = cp;
  const T De[3] = {dp[0], dp[1], dp[2]};

  // ---- 2. backward sweep: rows ch-2 .. 1 in terms of x_first and x_next
  M3<T> a2 = Ae, c2 = Ce;
  T d2[3] = {De[0], De[1], De[2]};
  for (int j = ch - 2; j >= 1; --j) {
    M3<T> apj, cpj;
    T dpj[3];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      apj.a[q] = S(q, j);
      cpj.a[q] = S(9 + q, j);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) dpj[q] = S(18 + q, j);
    T cd[3];
    mv(cpj, d2, cd);
    const M3<T> ca = mm(cpj, a2), cc = mm(cpj, c2);
#pragma unroll
    for (int q = 0; q < 3; ++q) d2[q] = dpj[q] - cd[q];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      a2.a[q] = apj.a[q] - ca.a[q];
      c2.a[q] = -cc.a[q];
      S(q, j) = a2.a[q];
      S(9 + q, j) = c2.a[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) S(18 + q, j) = d2[q];
  }

  // ---- 3. reduced row of this lane, block PCR across the warp
  M3<T> al, be, ga;
  T de[3];
  if (ch == 1) {
    al = zero3<T>();
    ga = zero3<T>();
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      al.a[q * 4] = As[q];
      ga.a[q * 4] = Cs[q];
      de[q] = Ds[q];
    }
    be = Ms;
  } else {
    M3<T> Ae_l = shfl_up_m(Ae, 1), Ce_l = shfl_up_m(Ce, 1);
    T De_l[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) De_l[q] = shfl_up<T>(De[q], 1, 32);
    if (r == 0) {
      Ae_l = zero3<T>();
      Ce_l = zero3<T>();
      De_l[0] = De_l[1] = De_l[2] = T(0);
    }
    const M3<T> t1 = dl(As, Ae_l), t2 = dl(Cs, a2), t3 = dl(As, Ce_l), t4 = dl(Cs, c2);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      al.a[q] = -t1.a[q];
      be.a[q] = Ms.a[q] - t2.a[q] - t3.a[q];
      ga.a[q] = -t4.a[q];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) de[q] = Ds[q] - Cs[q] * d2[q] - As[q] * De_l[q];
  }
#pragma unroll 1
  for (int sh = 1; sh < 32; sh <<= 1) {
    const M3<T> al_l = shfl_up_m(al, sh), be_l = shfl_up_m(be, sh), ga_l = shfl_up_m(ga, sh);
    const M3<T> al_r = shfl_down_m(al, sh), be_r = shfl_down_m(be, sh), ga_r = shfl_down_m(ga, sh);
    T de_l[3], de_r[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      de_l[q] = shfl_up<T>(de[q], sh, 32);
      de_r[q] = shfl_down<T>(de[q], sh, 32);
    }
    const bool hl = r >= sh, hr = r + sh < 32;
    M3<T> nal = zero3<T>(), nga = zero3<T>();
    if (hl) {
      const M3<T> k1 = mm(al, inv3(be_l));
      const M3<T> t = mm(k1, al_l), u = mm(k1, ga_l);
      T w[3];
      mv(k1, de_l, w);
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        nal.a[q] = -t.a[q];
        be.a[q] -= u.a[q];
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) de[q] -= w[q];
    }
    if (hr) {
      const M3<T> k2 = mm(ga, inv3(be_r));
      const M3<T> t = mm(k2, ga_r), u = mm(k2, al_r);
      T w[3];
      mv(k2, de_r, w);
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        nga.a[q] = -t.a[q];
        be.a[q] -= u.a[q];
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) de[q] -= w[q];
    }
    al = nal;
    ga = nga;
  }
  T x0[3];
  mv(inv3(be), de, x0);
  T xe[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    xe[q] = shfl_down<T>(x0[q], 1, 32);
    if (r == 31) xe[q] = T(0);
  }

  // ---- 4. back substitution
  T* xb = x + b * (int64_t)K * 3;
  if (r * ch < K) {
#pragma unroll
    for (int q = 0; q < 3; ++q) xb[r * ch * 3 + q] = x0[q];
  }
  for (int j = 1; j < ch; ++j) {
    const int i = r * ch + j;
    M3<T> aj, cj;
    T dj[3];
    if (j == last) {
      aj = Ae;
      cj = Ce;
      dj[0] = De[0];
      dj[1] = De[1];
      dj[2] = De[2];
    } else {
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        aj.a[q] = S(q, j);
        cj.a[q] = S(9 + q, j);
      }
#pragma unroll
      for (int q = 0; q < 3; ++q) dj[q] = S(18 + q, j);
    }
    T u[3], w[3];
    mv(aj, x0, u);
    mv(cj, xe, w);
    if (i < K) {
#pragma unroll
      for (int q = 0; q < 3; ++q) xb[i * 3 + q] = dj[q] - u[q] - w[q];
    }
  }
}

template <typename T, bool TR>
__global__ void __launch_bounds__(128) block3_kernel(int64_t B, int K, int ch,
                                                     const T* __restrict__ lower,
                                                     const T* __restrict__ mainb,
                                                     const T* __restrict__ upper,
                                                     const T* __restrict__ rhs,
                                                     T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  T* sm = reinterpret_cast<T*>(smem_raw) + (size_t)warp * kBlockPlanes * ch * 32;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; b < B; b += warps)
    block_system<T, TR>(b, K, lower, mainb, upper, rhs, x, sm, ch);
}

// Systems whose chunk planes exceed shared memory: one thread per system runs
// the serial block Thomas recurrence (the algorithm of the reference's
// thomas_bt3_kernel, triton/bt_kernel.py:38-170) with the 3x3 factors
// C'_k = M_k^-1 diag(upper_k) in a stream-ordered workspace and d'_k in x:
//   M_k = main_k - diag(lower_{k-1}) C'_{k-1}
//   d'_k = M_k^-1 (rhs_k - diag(lower_{k-1}) d'_{k-1}),  x_k = d'_k - C'_k x_{k+1}.
template <typename T, bool TR>
__global__ void __launch_bounds__(128)
    block3_serial_kernel(int64_t B, int K, const T* __restrict__ lower,
                         const T* __restrict__ mainb, const T* __restrict__ upper,
                         const T* __restrict__ rhs, T* __restrict__ x, T* __restrict__ cp) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  // the transposed system: main blocks transposed, lower and upper exchanged
  const T* lo = (TR ? upper : lower) + s * (int64_t)(K - 1) * 3;
  const T* up = (TR ? lower : upper) + s * (int64_t)(K - 1) * 3;
  const T* mb = mainb + s * (int64_t)K * 9;
  const T* rs = rhs + s * (int64_t)K * 3;
  T* xs = x + s * (int64_t)K * 3;
  T* cps = cp + s * (int64_t)K * 9;
  M3<T> cprev;
  T dprev[3] = {T(0), T(0), T(0)};
  for (int k = 0; k < K; ++k) {
    M3<T> m;
#pragma unroll
    for (int q = 0; q < 9; ++q) m.a[q] = TR ? mb[k * 9 + (q % 3) * 3 + q / 3] : mb[k * 9 + q];
    T r[3] = {rs[k * 3], rs[k * 3 + 1], rs[k * 3 + 2]};
    if (k > 0) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const T l = lo[(k - 1) * 3 + i];
#pragma unroll
        for (int j = 0; j < 3; ++j) m.a[i * 3 + j] -= l * cprev.a[i * 3 + j];
        r[i] -= l * dprev[i];
      }
    }
    const M3<T> mi = inv3(m);
    mv(mi, r, dprev);
    xs[k * 3] = dprev[0];
    xs[k * 3 + 1] = dprev[1];
    xs[k * 3 + 2] = dprev[2];
    if (k + 1 < K) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) cprev.a[i * 3 + j] = mi.a[i * 3 + j] * up[k * 3 + j];
#pragma unroll
      for (int q = 0; q < 9; ++q) cps[k * 9 + q] = cprev.a[q];
    }
  }
  T xn[3] = {dprev[0], dprev[1], dprev[2]};
  for (int k = K - 2; k >= 0; --k) {
    M3<T> c;
#pragma unroll
    for (int q = 0; q < 9; ++q) c.a[q] = cps[k * 9 + q];
    T cx[3];
    mv(c, xn, cx);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      xn[i] = xs[k * 3 + i] - cx[i];
      xs[k * 3 + i] = xn[i];
    }
  }
}

template <typename T>
static int block3_serial(int64_t B, int K, const void* lower, const void* mainb,
                         const void* upper, const void* rhs, void* x, int transpose,
                         cudaStream_t st) {
  T* cp = nullptr;
  DGB_CUDA_CHECK(cudaMallocAsync((void**)&cp, (size_t)B * K * 9 * sizeof(T), st));
  const unsigned blocks = (unsigned)((B + 127) / 128);
  if (transpose)
    block3_serial_kernel<T, true><<<blocks, 128, 0, st>>>(
        B, K, (const T*)lower, (const T*)mainb, (const T*)upper, (const T*)rhs, (T*)x, cp);
  else
    block3_serial_kernel<T, false><<<blocks, 128, 0, st>>>(
        B, K, (const T*)lower, (const T*)mainb, (const T*)upper, (const T*)rhs, (T*)x, cp);
  DGB_LAUNCH_CHECK();
  DGB_CUDA_CHECK(cudaFreeAsync(cp, st));
  return DGB_OK;
}

template <typename T>
static int block3_t(int64_t B, int K, const void* lower, const void* mainb, const void* upper,
                    const void* rhs, void* x, int transpose, cudaStream_t st) {
  const int ch = (K + 31) / 32;
  const size_t per_warp = (size_t)kBlockPlanes * ch * 32 * sizeof(T);
  int wpb = 4;
  while (wpb > 1 && wpb * per_warp > 227 * 1024) wpb >>= 1;
  if (K > 1024 || wpb * per_warp > 227 * 1024)  // the chunked kernel holds <= 32 rows per lane
    return block3_serial<T>(B, K, lower, mainb, upper, rhs, x, transpose, st);
  const size_t smem = wpb * per_warp;
  auto kern = transpose ? block3_kernel<T, true> : block3_kernel<T, false>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wpb * 32, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t blocks = (int64_t)device_sm_count() * per_sm;
  const int64_t need = (B + wpb - 1) / wpb;
  if (blocks > need) blocks = need;
  kern<<<(unsigned)blocks, wpb * 32, smem, st>>>(B, K, ch, (const T*)lower, (const T*)mainb,
                                                 (const T*)upper, (const T*)rhs, (T*)x);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" size_t dgb_block3_work_size(int dtype, int64_t B, int64_t K) {
  (void)dtype;
  (void)B;
  (void)K;
  return 0;  // the factors stay in shared memory
}

extern "C" int dgb_block3_solve(int dtype, int64_t B, int64_t K, const void* lower,
                                const void* main_blocks, const void* upper, const void* rhs,
                                void* x, void* work, int32_t transpose, void* stream) {
  clear_error();
  (void)work;
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(B >= 1 && K >= 1, "B and K must both be >= 1");
  DGB_REQUIRE(K <= (1 << 26), "K must be <= 2^26, got %lld", (long long)K);
  DGB_REQUIRE(main_blocks && rhs && x, "main, rhs and x must be non-null");
  DGB_REQUIRE(K == 1 || (lower && upper), "lower and upper must be non-null when K > 1");
  DGB_REQUIRE(transpose == 0 || transpose == 1, "transpose must be 0 or 1");
  DGB_REQUIRE(x != rhs, "x must not alias rhs");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32)
    return block3_t<float>(B, (int)K, lower, main_blocks, upper, rhs, x, transpose, st);
  return block3_t<double>(B, (int)K, lower, main_blocks, upper, rhs, x, transpose, st);
}
