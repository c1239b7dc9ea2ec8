// NetStim renewal generators on sm_103a: the per-step transition of
// networks/_netstim_renewal.py (netstim_initial_state :70-91,
// netstim_renewal :94-159) for many generators over many steps in one launch.
//
// One thread owns one generator for the whole run.  Every step it draws one
// unit exponential (as the reference draws a full-shape sample every step,
// _netstim_renewal.py:27-32), or takes it from a caller-supplied table, and
// applies the transition with the reference's arithmetic:
//   due    = t >= next
//   fires  = due && count < number
//   next  += ((interval (1 - noise) + (interval noise) E) * fires) * fires
//   count += fires
// (the gate of the straight-through estimator equals the hard spike in value).
// The clock is t = t0 + k * dt in the state dtype, as the network's exact
// clock (networks/net.py:1942-1947).
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), counter (step low, generator,
// stream, step high), key = the 64-bit seed: runs split at any step continue
// identically.  The uniform is (24 or 53 random bits + 1/2) 2^-24 or 2^-53
// (float32 or float64 state) and the draw is E = -ln(U), rounded to the state
// dtype, with ln evaluated in double precision by the atanh series
//   ln(m 2^e) = e ln 2 + 2 (s + s^3/3 + s^5/5 + ...),  s = (m - 1)/(m + 1),
// m in [sqrt(1/2), sqrt(2)), using only rounded IEEE operations, so the CPU
// oracle reproduces every draw bit for bit.
#include "common.cuh"

namespace dgb {

struct Philox4 {
  uint32_t v[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 uint32_t c3, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
    const uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += W0;
    k1 += W1;
  }
  return Philox4{{c0, c1, c2, c3}};
}

// ln(x) for x in (0, 1], double precision, rounded IEEE operations only.
__device__ __forceinline__ double series_log(double x) {
  int e = 0;
  double m = frexp(x, &e);  // x = m 2^e, m in [1/2, 1): exact
  if (m < 0.70710678118654752440) {
    m = __dmul_rn(m, 2.0);  // exact
    e -= 1;
  }
  const double s = __ddiv_rn(__dsub_rn(m, 1.0), __dadd_rn(m, 1.0));
  const double s2 = __dmul_rn(s, s);
  // 2 (s + s^3/3 + ... + s^23/23): Horner in s^2
  double p = 1.0 / 23.0;
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 21.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 19.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 17.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 15.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 13.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 11.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 9.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 7.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 5.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0 / 3.0);
  p = __dadd_rn(__dmul_rn(p, s2), 1.0);
  const double lm = __dmul_rn(__dmul_rn(2.0, s), p);
  return __dadd_rn(__dmul_rn((double)e, 0.69314718055994530942), lm);
}

// Unit exponential of (step, generator, stream) in dtype T.
template <typename T>
__device__ __forceinline__ T unit_exponential(uint64_t seed, uint64_t step, uint32_t gen,
                                              uint32_t stream) {
  const Philox4 r = philox4x32_10((uint32_t)step, gen, stream, (uint32_t)(step >> 32),
                                  (uint32_t)seed, (uint32_t)(seed >> 32));
  double u;
  if (sizeof(T) == 4) {
    u = ((double)(r.v[0] >> 8) + 0.5) * 5.9604644775390625e-08;  // 2^-24
  } else {
    const uint64_t b = ((uint64_t)r.v[0] << 21) ^ (uint64_t)(r.v[1] >> 11);  // 53 bits
    u = ((double)(b & ((1ull << 53) - 1)) + 0.5) * 1.1102230246251565e-16;  // 2^-53
  }
  return (T)(-series_log(u));
}

__device__ __forceinline__ float add_t(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_t(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_t(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_t(double a, double b) { return __dsub_rn(a, b); }

// Initial clocks (netstim_initial_state): start + (noise interval) E when any
// generator has noise, else start; counts 0.
template <typename T>
__global__ void netstim_init_kernel(int64_t n, const T* __restrict__ interval,
                                    const T* __restrict__ noise, const T* __restrict__ start,
                                    int any_noise, uint64_t seed, const T* __restrict__ draws,
                                    T* __restrict__ next, int64_t* __restrict__ counts) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  T clock = start[g];
  if (any_noise) {
    const T E = draws ? draws[g] : unit_exponential<T>(seed, 0, (uint32_t)g, 1u);
    clock = add_t(clock, mul_rn(mul_rn(noise[g], interval[g]), E));
  }
  next[g] = clock;
  counts[g] = 0;
}

// n_steps renewal steps from absolute step step0.  Outputs (each optional):
// spikes[k][g] (uint8) and bits, one bit per generator and step packed in
// 64-bit words (bit g & 63 of word g >> 6 of row k, rows of n_words words).
template <typename T>
__global__ void __launch_bounds__(256)
    netstim_run_kernel(int64_t n, int64_t n_steps, int64_t step0, T t0, T dt,
                       const T* __restrict__ interval, const T* __restrict__ noise,
                       const int64_t* __restrict__ number, uint64_t seed,
                       const T* __restrict__ draws, T* __restrict__ next,
                       int64_t* __restrict__ counts, uint8_t* __restrict__ spikes,
                       uint32_t* __restrict__ bits, int64_t n_words) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = g < n;
  T clock = live ? next[g] : T(0);
  int64_t count = live ? counts[g] : 0;
  const T iv = live ? interval[g] : T(0), nz = live ? noise[g] : T(0);
  const int64_t cap = (live && number) ? number[g] : INT64_MAX;
  const T a = mul_rn(iv, sub_t(T(1), nz)), b = mul_rn(iv, nz);
  for (int64_t k = 0; k < n_steps; ++k) {
    const int64_t step = step0 + k;
    const T t = add_t(t0, mul_rn((T)step, dt));
    bool fire = false;
    if (live) {
      const T E = draws ? draws[k * n + g] : unit_exponential<T>(seed, (uint64_t)step,
                                                                 (uint32_t)g, 0u);
      const bool due = t >= clock;
      fire = due && count < cap;
      const T gate = fire ? T(1) : T(0);
      const T next_interval = add_t(a, mul_rn(b, E));
      clock = add_t(clock, mul_rn(mul_rn(next_interval, gate), gate));
      count += fire ? 1 : 0;
      if (spikes) spikes[k * n + g] = fire ? 1 : 0;
    }
    if (bits) {
      // 32 generators per ballot: the low or high half of a 64-bit word
      const unsigned word = __ballot_sync(0xffffffffu, fire);
      const int64_t half = g >> 5;
      if ((threadIdx.x & 31) == 0 && half < 2 * n_words) bits[k * 2 * n_words + half] = word;
    }
  }
  if (live) {
    next[g] = clock;
    counts[g] = count;
  }
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_netstim_init(int dtype, int64_t n, const void* interval, const void* noise,
                                const void* start, int32_t any_noise, uint64_t seed,
                                const void* draws, void* next_time, int64_t* counts,
                                void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n >= 0 && n < (1ll << 32), "bad generator count");
  if (n == 0) return DGB_OK;
  DGB_REQUIRE(interval && noise && start && next_time && counts, "pointers must be non-null");
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (dtype == DGB_F32)
    netstim_init_kernel<float><<<blocks, 256, 0, as_stream(stream)>>>(
        n, (const float*)interval, (const float*)noise, (const float*)start, any_noise, seed,
        (const float*)draws, (float*)next_time, counts);
  else
    netstim_init_kernel<double><<<blocks, 256, 0, as_stream(stream)>>>(
        n, (const double*)interval, (const double*)noise, (const double*)start, any_noise, seed,
        (const double*)draws, (double*)next_time, counts);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_netstim_run(int dtype, int64_t n, int64_t n_steps, int64_t step0, double t0,
                               double dt, const void* interval, const void* noise,
                               const int64_t* number, uint64_t seed, const void* draws,
                               void* next_time, int64_t* counts, uint8_t* spikes,
                               uint64_t* bits, int64_t n_words, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n >= 0 && n < (1ll << 32) && n_steps >= 0 && step0 >= 0, "bad sizes");
  if (n == 0 || n_steps == 0) return DGB_OK;
  DGB_REQUIRE(interval && noise && next_time && counts, "pointers must be non-null");
  DGB_REQUIRE(!bits || n_words * 64 >= n, "n_words must cover every generator");
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (dtype == DGB_F32)
    netstim_run_kernel<float><<<blocks, 256, 0, as_stream(stream)>>>(
        n, n_steps, step0, (float)t0, (float)dt, (const float*)interval, (const float*)noise,
        number, seed, (const float*)draws, (float*)next_time, counts, spikes, (uint32_t*)bits,
        n_words);
  else
    netstim_run_kernel<double><<<blocks, 256, 0, as_stream(stream)>>>(
        n, n_steps, step0, t0, dt, (const double*)interval, (const double*)noise, number, seed,
        (const double*)draws, (double*)next_time, counts, spikes, (uint32_t*)bits, n_words);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}
