// Unbranched Hodgkin–Huxley cable update on sm_103a.
//
// dgb_cable_run: persistent multi-step kernel.  One warp owns one cable for
// the whole run: state (v, m, h, n) lives in registers, per-compartment
// coefficients in shared memory, and every step performs, without touching
// global memory,
//   1. the cnexp gate advance at v_old        (integrators/core.py:769-834,
//      mechanisms/_cnexp.py:96-132, mod/HH.py:24-40)
//   2. the HH affine frame G, J               (mod/HH.py:109-116)
//   3. the increment-form RHS and diagonal    (integrators/implicit.py:569-664):
//        rhs  = dt_s [ (J - G v) scale + axial(v) + axial(ve) + intra cm_inv ]
//        main = 1 - dt_s (diag_base - G scale)
//      with ve = field * I(t) evaluated on the fly (fields/analytic.py:60-62,
//      stim/waveform/implementations.py:551-558) instead of a (T,B,K) tape
//   4. the tridiagonal solve (chunk_solve.cuh) and v += dv
//   5. the rising-edge spike check (_threshold_callbacks.py:50-53) and trace
//      recording at one compartment.
// Cables are handed out through an atomic work counter in largest-first order.
//
// dgb_cable_assemble / dgb_cable_solve_update: the same step split into an
// elementwise assembly kernel (one thread per compartment, bands to global
// memory) and a ragged solve-and-update kernel: the plain per-step path.
#pragma once
// The chunk sizes compiled for each dtype.
#define DGB_CHUNK_CASES(T)                                                        \
  DGB_CASE(1) DGB_CASE(2) DGB_CASE(4) DGB_CASE(8) DGB_CASE(16)                    \
  DGB_CASE_F32(3) DGB_CASE_F32(5) DGB_CASE_F32(6) DGB_CASE_F32(7) DGB_CASE_F32(9) \
  DGB_CASE_F32(10) DGB_CASE_F32(11) DGB_CASE_F32(12) DGB_CASE_F32(13)             \
  DGB_CASE_F32(14) DGB_CASE_F32(15)
#include "chunk_solve.cuh"

namespace dgb {

template <typename T>
struct CableArgsT {
  int n_cables, n_steps, rec_every;
  const int64_t* cable_ptr;
  const int32_t* order;
  T *v, *m, *h, *n;
  const T *g_right, *g_left, *scale, *cm_inv, *field;
  const T *gnabar, *gkbar, *gl, *el;
  T ena, ek, q10, dt, dt_s;
  double dt_ms_d, t0_ms;
  int64_t step0;
  const T *ve_amp, *ve_delay, *ve_pw;
  const int32_t* in_idx;
  const T *in_amp, *in_delay, *in_pw;
  const int32_t* rec_idx;
  T* trace;
  int64_t n_rec;
  const int32_t* spk_idx;
  T spk_thr;
  int32_t *spk_below, *spk_count, *spk_first;
  int32_t* counter;
};

template <typename T>
static CableArgsT<T> typed(const dgb_cable_args* a) {
  CableArgsT<T> t;
  t.n_cables = a->n_cables;
  t.n_steps = a->n_steps;
  t.rec_every = a->rec_every > 0 ? a->rec_every : 1;
  t.cable_ptr = a->cable_ptr;
  t.order = a->order;
  t.v = (T*)a->v;
  t.m = (T*)a->m;
  t.h = (T*)a->h;
  t.n = (T*)a->n;
  t.g_right = (const T*)a->g_right;
  t.g_left = (const T*)a->g_left;
  t.scale = (const T*)a->scale;
  t.cm_inv = (const T*)a->cm_inv;
  t.field = (const T*)a->field;
  t.gnabar = (const T*)a->gnabar;
  t.gkbar = (const T*)a->gkbar;
  t.gl = (const T*)a->gl;
  t.el = (const T*)a->el;
  t.ena = (T)a->ena;
  t.ek = (T)a->ek;
  t.q10 = (T)a->q10;
  t.dt = (T)a->dt_ms;
  t.dt_s = (T)a->dt_s;
  t.dt_ms_d = a->dt_ms;
  t.t0_ms = a->t0_ms;
  t.step0 = a->step0;
  t.ve_amp = (const T*)a->ve_amp;
  t.ve_delay = (const T*)a->ve_delay;
  t.ve_pw = (const T*)a->ve_pw;
  t.in_idx = a->in_idx;
  t.in_amp = (const T*)a->in_amp;
  t.in_delay = (const T*)a->in_delay;
  t.in_pw = (const T*)a->in_pw;
  t.rec_idx = a->rec_idx;
  t.trace = (T*)a->trace;
  t.n_rec = 1 + (int64_t)a->n_steps / t.rec_every;
  t.spk_idx = a->spk_idx;
  t.spk_thr = (T)a->spk_thr;
  t.spk_below = a->spk_below;
  t.spk_count = a->spk_count;
  t.spk_first = a->spk_first;
  t.counter = a->scratch;
  return t;
}

// Per-warp shared-memory coefficient block: kNConst planes of [CH][32].
constexpr int kNConst = 8;
enum { Q_GR = 0, Q_GL, Q_SCALE, Q_FIELD, Q_GNA, Q_GK, Q_GLK, Q_EL };

template <typename T, int CH>
__device__ __forceinline__ T& sm(T* base, int q, int j, int lane) {
  return base[(q * CH + j) * 32 + lane];
}

// Select element j_sel of a register array without dynamic indexing.
template <typename T, int CH>
__device__ __forceinline__ T pick(const T (&x)[CH], int j_sel) {
  T out = x[0];
#pragma unroll
  for (int j = 1; j < CH; ++j)
    if (j == j_sel) out = x[j];
  return out;
}

template <typename T, int CH>
__device__ __noinline__ void run_cable(const CableArgsT<T>& A, int cable, T* smw) {
  const int lane = threadIdx.x & 31;
  const int64_t off = A.cable_ptr[cable];
  const int K = (int)(A.cable_ptr[cable + 1] - off);
  const bool use_ve = A.field != nullptr && A.ve_amp != nullptr;
  const T* fieldp = A.field;

  T v[CH], m[CH], h[CH], n[CH];
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int i = lane * CH + j;
    const bool in = i < K;
    const int64_t g = off + i;
    v[j] = in ? A.v[g] : T(0);
    m[j] = in ? A.m[g] : T(0);
    h[j] = in ? A.h[g] : T(0);
    n[j] = in ? A.n[g] : T(0);
    sm<T, CH>(smw, Q_GR, j, lane) = in ? A.g_right[g] : T(0);
    sm<T, CH>(smw, Q_GL, j, lane) = in ? A.g_left[g] : T(0);
    sm<T, CH>(smw, Q_SCALE, j, lane) = in ? A.scale[g] : T(0);
    sm<T, CH>(smw, Q_FIELD, j, lane) = (in && use_ve) ? fieldp[g] : T(0);
    sm<T, CH>(smw, Q_GNA, j, lane) = in ? A.gnabar[g] : T(0);
    sm<T, CH>(smw, Q_GK, j, lane) = in ? A.gkbar[g] : T(0);
    sm<T, CH>(smw, Q_GLK, j, lane) = in ? A.gl[g] : T(0);
    sm<T, CH>(smw, Q_EL, j, lane) = in ? A.el[g] : T(0);
  }
  __syncwarp();

  // Per-cable scalars.
  T ve_amp = T(0), ve_delay = T(0), ve_pw = T(0);
  if (use_ve) {
    ve_amp = A.ve_amp[cable];
    ve_delay = A.ve_delay[cable];
    ve_pw = A.ve_pw[cable];
  }
  const int in_i = A.in_idx ? A.in_idx[cable] : -1;
  T in_amp = T(0), in_delay = T(0), in_pw = T(0), in_cm = T(0);
  if (in_i >= 0 && in_i < K) {
    in_amp = A.in_amp[cable];
    in_delay = A.in_delay[cable];
    in_pw = A.in_pw[cable];
    in_cm = A.cm_inv[off + in_i];
  }
  const int in_lane = in_i >= 0 ? in_i / CH : -1, in_j = in_i >= 0 ? in_i % CH : -1;
  const int rec_i = (A.rec_idx && A.trace) ? A.rec_idx[cable] : -1;
  const int rec_lane = rec_i >= 0 ? rec_i / CH : -1, rec_j = rec_i >= 0 ? rec_i % CH : -1;
  const int spk_i = A.spk_idx ? A.spk_idx[cable] : -1;
  const int spk_lane = spk_i >= 0 ? spk_i / CH : -1, spk_j = spk_i >= 0 ? spk_i % CH : -1;
  int below = 1, count = 0, first = -1;
  if (spk_i >= 0 && lane == spk_lane) {
    below = A.spk_below[cable];
    count = A.spk_count[cable];
    first = A.spk_first[cable];
  }
  if (rec_i >= 0 && lane == rec_lane) A.trace[(int64_t)cable * A.n_rec] = pick<T, CH>(v, rec_j);

  const T dt = A.dt, dt_s = A.dt_s, q10 = A.q10, ena = A.ena, ek = A.ek;
  for (int s = 0; s < A.n_steps; ++s) {
    const T t = (T)(A.t0_ms + (double)(A.step0 + s) * A.dt_ms_d);
    const T Ive = use_ve ? rect_pulse<T>(t, ve_amp, ve_delay, ve_pw) : T(0);
    const T Iin = (in_i >= 0) ? rect_pulse<T>(t, in_amp, in_delay, in_pw) : T(0);
    // halo voltages from the neighbouring lanes
    T v_lo = shfl_up<T>(v[CH - 1], 1, 32);
    T v_hi = shfl_down<T>(v[0], 1, 32);
    T a[CH], b[CH], c[CH], d[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      const T vj = v[j];
      hh_gates<T>(vj, q10, dt, m[j], h[j], n[j]);
      T G, J;
      hh_affine<T>(m[j], h[j], n[j], sm<T, CH>(smw, Q_GNA, j, lane),
                   sm<T, CH>(smw, Q_GK, j, lane), sm<T, CH>(smw, Q_GLK, j, lane),
                   sm<T, CH>(smw, Q_EL, j, lane), ena, ek, G, J);
      const T scl = sm<T, CH>(smw, Q_SCALE, j, lane);
      const T gr = sm<T, CH>(smw, Q_GR, j, lane);
      const T glf = sm<T, CH>(smw, Q_GL, j, lane);
      const T vl = (j == 0) ? v_lo : v[j - 1];
      const T vr = (j == CH - 1) ? v_hi : v[j + 1];
      T fn = (J - G * vj) * scl;
      fn = fn + (gr * (vr - vj) - glf * (vj - vl));
      d[j] = fn;
      b[j] = T(1) - dt_s * ((-gr + -glf) - G * scl);
      a[j] = -dt_s * glf;
      c[j] = -dt_s * gr;
    }
    if (Ive != T(0)) {  // warp-uniform: the pulse is per cable
      T ve[CH];
#pragma unroll
      for (int j = 0; j < CH; ++j) ve[j] = sm<T, CH>(smw, Q_FIELD, j, lane) * Ive;
      T ve_lo = shfl_up<T>(ve[CH - 1], 1, 32);
      T ve_hi = shfl_down<T>(ve[0], 1, 32);
#pragma unroll
      for (int j = 0; j < CH; ++j) {
        const T gr = sm<T, CH>(smw, Q_GR, j, lane);
        const T glf = sm<T, CH>(smw, Q_GL, j, lane);
        const T el_ = (j == 0) ? ve_lo : ve[j - 1];
        const T er_ = (j == CH - 1) ? ve_hi : ve[j + 1];
        d[j] = d[j] + (gr * (er_ - ve[j]) - glf * (ve[j] - el_));
      }
    }
    if (Iin != T(0) && lane == in_lane) {
#pragma unroll
      for (int j = 0; j < CH; ++j)
        if (j == in_j) d[j] = d[j] + Iin * in_cm;
    }
#pragma unroll
    for (int j = 0; j < CH; ++j) d[j] = dt_s * d[j];
    chunk_solve<T, CH, 32>(a, b, c, d, lane);
#pragma unroll
    for (int j = 0; j < CH; ++j) v[j] = v[j] + d[j];
    if (spk_i >= 0 && lane == spk_lane) {
      const T vs = pick<T, CH>(v, spk_j);
      const int above = vs >= A.spk_thr;
      if (above && below) {
        if (count == 0) first = s + 1;
        count += 1;
      }
      below = !above;
    }
    if (rec_i >= 0 && lane == rec_lane && ((s + 1) % A.rec_every) == 0)
      A.trace[(int64_t)cable * A.n_rec + (s + 1) / A.rec_every] = pick<T, CH>(v, rec_j);
  }
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int i = lane * CH + j;
    if (i < K) {
      const int64_t g = off + i;
      A.v[g] = v[j];
      A.m[g] = m[j];
      A.h[g] = h[j];
      A.n[g] = n[j];
    }
  }
  if (spk_i >= 0 && lane == spk_lane) {
    A.spk_below[cable] = below;
    A.spk_count[cable] = count;
    A.spk_first[cable] = first;
  }
  __syncwarp();
}

constexpr int kCableMaxCH = 16;  // K <= 512

// float64 runs (small, latency-bound populations) use fewer chunk
// instantiations; rows past the cable end are identity rows.
template <typename T>
__device__ __forceinline__ int chunk_round(int ch) {
  if constexpr (sizeof(T) == 8) {
    return ch <= 1 ? 1 : ch <= 2 ? 2 : ch <= 4 ? 4 : ch <= 8 ? 8 : 16;
  } else {
    return ch;
  }
}

template <typename T>
__global__ void __launch_bounds__(128) cable_run_kernel(CableArgsT<T> A, int ch_max) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smw = reinterpret_cast<T*>(smem_raw) + (size_t)(threadIdx.x >> 5) * kNConst * ch_max * 32;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(A.counter, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= A.n_cables) break;
    const int cable = A.order ? A.order[idx] : idx;
    const int K = (int)(A.cable_ptr[cable + 1] - A.cable_ptr[cable]);
    const int ch = chunk_round<T>((K + 31) / 32);
    switch (ch) {
#define DGB_CASE(CHV)                  \
  case CHV:                            \
    run_cable<T, CHV>(A, cable, smw);  \
    break;
      DGB_CHUNK_CASES(T)
#undef DGB_CASE
      default:
        break;
    }
  }
}

// ---------------------------------------------------------------------------
// Plain per-step path.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void cable_assemble_kernel(CableArgsT<T> A, const int32_t* __restrict__ comp_cable,
                                      int64_t N, int32_t step, T* __restrict__ lower,
                                      T* __restrict__ mainv, T* __restrict__ upper,
                                      T* __restrict__ rhs) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= N) return;
  const int cable = comp_cable[g];
  const int64_t off = A.cable_ptr[cable];
  const int64_t K = A.cable_ptr[cable + 1] - off;
  const int64_t i = g - off;
  const T t = (T)(A.t0_ms + (double)(A.step0 + step) * A.dt_ms_d);
  const T vj = A.v[g];
  T mm = A.m[g], hh = A.h[g], nn = A.n[g];
  hh_gates<T>(vj, A.q10, A.dt, mm, hh, nn);
  A.m[g] = mm;
  A.h[g] = hh;
  A.n[g] = nn;
  T G, J;
  hh_affine<T>(mm, hh, nn, A.gnabar[g], A.gkbar[g], A.gl[g], A.el[g], A.ena, A.ek, G, J);
  const T scl = A.scale[g];
  const T gr = A.g_right[g];
  const T glf = A.g_left[g];
  const T vl = i > 0 ? A.v[g - 1] : vj;
  const T vr = i < K - 1 ? A.v[g + 1] : vj;
  T fn = (J - G * vj) * scl;
  fn = fn + (gr * (vr - vj) - glf * (vj - vl));
  if (A.field && A.ve_amp) {
    const T I = rect_pulse<T>(t, A.ve_amp[cable], A.ve_delay[cable], A.ve_pw[cable]);
    if (I != T(0)) {
      const T ve = A.field[g] * I;
      const T vel = i > 0 ? A.field[g - 1] * I : ve;
      const T ver = i < K - 1 ? A.field[g + 1] * I : ve;
      fn = fn + (gr * (ver - ve) - glf * (ve - vel));
    }
  }
  if (A.in_idx && A.in_idx[cable] == (int)i) {
    const T I = rect_pulse<T>(t, A.in_amp[cable], A.in_delay[cable], A.in_pw[cable]);
    if (I != T(0)) fn = fn + I * A.cm_inv[g];
  }
  rhs[g] = A.dt_s * fn;
  mainv[g] = T(1) - A.dt_s * ((-gr + -glf) - G * scl);
  lower[g] = -A.dt_s * glf;
  upper[g] = -A.dt_s * gr;
}

template <typename T, int CH>
__device__ __noinline__ void solve_update_cable(const CableArgsT<T>& A, int cable,
                                                const T* lower, const T* mainv,
                                                const T* upper, const T* rhs) {
  const int lane = threadIdx.x & 31;
  const int64_t off = A.cable_ptr[cable];
  const int K = (int)(A.cable_ptr[cable + 1] - off);
  T a[CH], b[CH], c[CH], d[CH];
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int i = lane * CH + j;
    const bool in = i < K;
    a[j] = in ? lower[off + i] : T(0);
    b[j] = in ? mainv[off + i] : T(1);
    c[j] = in ? upper[off + i] : T(0);
    d[j] = in ? rhs[off + i] : T(0);
  }
  chunk_solve<T, CH, 32>(a, b, c, d, lane);
#pragma unroll
  for (int j = 0; j < CH; ++j) {
    const int i = lane * CH + j;
    if (i < K) A.v[off + i] = A.v[off + i] + d[j];
  }
}

template <typename T>
__global__ void __launch_bounds__(128) cable_solve_update_kernel(CableArgsT<T> A,
                                                                 const T* lower,
                                                                 const T* mainv,
                                                                 const T* upper,
                                                                 const T* rhs) {
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < A.n_cables;
       w += warps) {
    const int cable = A.order ? A.order[w] : w;
    const int K = (int)(A.cable_ptr[cable + 1] - A.cable_ptr[cable]);
    const int ch = chunk_round<T>((K + 31) / 32);
    switch (ch) {
#define DGB_CASE(CHV)                                                      \
  case CHV:                                                                \
    solve_update_cable<T, CHV>(A, cable, lower, mainv, upper, rhs);        \
    break;
      DGB_CHUNK_CASES(T)
#undef DGB_CASE
      default:
        break;
    }
  }
}

inline int validate_cable_args(const dgb_cable_args* a) {
  DGB_REQUIRE(a != nullptr, "args must be non-null");
  DGB_REQUIRE(a->dtype == DGB_F32 || a->dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(a->n_cables >= 0 && a->n_steps >= 0, "n_cables and n_steps must be >= 0");
  DGB_REQUIRE(a->cable_ptr && a->v && a->m && a->h && a->n, "cable_ptr and v/m/h/n are required");
  DGB_REQUIRE(a->g_right && a->g_left && a->scale && a->cm_inv,
              "g_right, g_left, scale and cm_inv are required");
  DGB_REQUIRE(a->gnabar && a->gkbar && a->gl && a->el, "gnabar, gkbar, gl and el are required");
  DGB_REQUIRE(!a->in_idx || (a->in_amp && a->in_delay && a->in_pw),
              "in_idx requires in_amp, in_delay and in_pw");
  DGB_REQUIRE(!a->ve_amp || (a->field && a->ve_delay && a->ve_pw),
              "ve_amp requires field, ve_delay and ve_pw");
  DGB_REQUIRE(!a->spk_idx || (a->spk_below && a->spk_count && a->spk_first),
              "spk_idx requires spk_below, spk_count and spk_first");
  DGB_REQUIRE(!a->trace || a->rec_idx, "trace requires rec_idx");
  DGB_REQUIRE(a->rec_every >= 1, "rec_every must be >= 1");
  DGB_REQUIRE(a->lanes == 0, "lanes is reserved and must be 0");
  return DGB_OK;
}

template <typename T>
int cable_run_t(const dgb_cable_args* args, int ch_max, cudaStream_t st) {
  CableArgsT<T> A = typed<T>(args);
  const int threads = 128;
  const size_t smem = (size_t)(threads / 32) * kNConst * ch_max * 32 * sizeof(T);
  DGB_CUDA_CHECK(cudaFuncSetAttribute(cable_run_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cable_run_kernel<T>,
                                                               threads, smem));
  if (per_sm < 1) per_sm = 1;
  const int warps_needed = A.n_cables;
  int blocks = device_sm_count() * per_sm;
  const int blocks_needed = (warps_needed + 3) / 4;
  if (blocks > blocks_needed) blocks = blocks_needed;
  if (blocks < 1) blocks = 1;
  DGB_CUDA_CHECK(cudaMemsetAsync(A.counter, 0, sizeof(int32_t), st));
  cable_run_kernel<T><<<blocks, threads, smem, st>>>(A, ch_max);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T>
int cable_assemble_t(const dgb_cable_args* args, int32_t step, void* lower, void* mainv,
                     void* upper, void* rhs, cudaStream_t st) {
  const int64_t N = args->n_comp;
  const int threads = 256;
  const int64_t blocks = (N + threads - 1) / threads;
  cable_assemble_kernel<T><<<(unsigned)blocks, threads, 0, st>>>(
      typed<T>(args), args->comp_cable, N, step, (T*)lower, (T*)mainv, (T*)upper, (T*)rhs);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T>
int cable_solve_update_t(const dgb_cable_args* args, const void* lower, const void* mainv,
                         const void* upper, const void* rhs, cudaStream_t st) {
  const int threads = 128;
  int blocks = (args->n_cables + 3) / 4;
  const int cap = device_sm_count() * 16;
  if (blocks > cap) blocks = cap;
  cable_solve_update_kernel<T><<<blocks, threads, 0, st>>>(
      typed<T>(args), (const T*)lower, (const T*)mainv, (const T*)upper, (const T*)rhs);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

#define DGB_INSTANTIATE_CABLE(T)                                                         \
  template int cable_run_t<T>(const dgb_cable_args*, int, cudaStream_t);               \
  template int cable_assemble_t<T>(const dgb_cable_args*, int32_t, void*, void*, void*, \
                                   void*, cudaStream_t);                               \
  template int cable_solve_update_t<T>(const dgb_cable_args*, const void*, const void*, \
                                       const void*, const void*, cudaStream_t);

}  // namespace dgb
