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
// The per-cable work is run_rows (cable_rows.cuh).
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
#include "cable_common.cuh"
#include "cable_rows.cuh"
#include "chunk_solve.cuh"

namespace dgb {

// The order positions and lanes per cable of work item `item` (false when
// the item index is past the last item).
__device__ __forceinline__ bool item_range(int item, int n_cables, int lanes_mode, int n32,
                                           int n16, int& pos0, int& pos_end, int& lanes) {
  if (lanes_mode == 0) {
    pos0 = item;
    pos_end = n_cables;
    lanes = 32;
    return item < n_cables;
  }
  if (item < n32) {
    pos0 = item;
    pos_end = n32;
    lanes = 32;
    return true;
  }
  item -= n32;
  const int items16 = (n16 + 1) / 2;
  if (item < items16) {
    pos0 = n32 + 2 * item;
    pos_end = n32 + n16;
    lanes = 16;
    return true;
  }
  item -= items16;
  const int n8 = n_cables - n32 - n16;
  pos0 = n32 + n16 + 4 * item;
  pos_end = n_cables;
  lanes = 8;
  return item < (n8 + 3) / 4;
}

template <typename T, bool FAST, bool TAPE, bool PLANES>
__global__ void __launch_bounds__(kCableMaxWarps * 32) cable_run_kernel(CableArgsT<T> A,
                                                                        int ch_alloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  T* smw = reinterpret_cast<T*>(smem_raw) +
           (size_t)warp * RowsNQ<PLANES>::value * ch_alloc * 32;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(A.counter, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    int pos0, pos_end, lanes;
    if (!item_range(item, A.n_cables, A.lanes_mode, A.n_lanes32, A.n_lanes16, pos0, pos_end,
                    lanes))
      break;
    // rows per lane: the item's longest cable over its lanes
    const int pos = pos0 + lane / lanes;
    int K = 0;
    if (pos < pos_end) {
      const int c = A.order ? A.order[pos] : pos;
      K = (int)(A.cable_ptr[c + 1] - A.cable_ptr[c]);
    }
    const int kmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)K);
    const int ch = (kmax + lanes - 1) / lanes;
    if (ch > ch_alloc) {  // the host sized shared memory for smaller cables:
      if (lane == 0) atomicOr(A.counter + 1, kErrChunk);  // flag, never skip silently
      continue;
    }
    if (ch > 0) run_rows<T, FAST, TAPE, PLANES>(A, pos0, pos_end, lanes, ch, smw);
  }
}

// Split-gate run (DGB_CABLE_SPLIT_GATES): one 32-lane cable per CTA of
// kSplitWarps warps, the gate advance and assembly of its rows spread over
// the warps (run_rows with GW = kSplitWarps).
template <typename T, bool FAST, bool TAPE, bool PLANES>
__global__ void __launch_bounds__(kSplitWarps * 32) cable_run_split_kernel(CableArgsT<T> A,
                                                                           int ch_alloc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  T* smw = reinterpret_cast<T*>(smem_raw);
  for (;;) {
    __syncthreads();  // every warp has read the previous item
    if (threadIdx.x == 0) s_item = atomicAdd(A.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= A.n_cables) break;
    const int c = A.order ? A.order[item] : item;
    const int K = (int)(A.cable_ptr[c + 1] - A.cable_ptr[c]);
    const int ch = (K + 31) / 32;
    if (ch > ch_alloc) {  // flag, never skip silently
      if (threadIdx.x == 0) atomicOr(A.counter + 1, kErrChunk);
      continue;
    }
    if (ch > 0) run_rows<T, FAST, TAPE, PLANES, kSplitWarps>(A, item, A.n_cables, 32, ch, smw);
  }
}

// ---------------------------------------------------------------------------
// Plain per-step path.
// ---------------------------------------------------------------------------

// Chunk sizes compiled for the register-resident per-step solve: all of
// 1..16 in float32; float64 rounds up to 1, 2, 4, 8, 16 (extra rows are
// identity rows).
template <typename T>
__device__ __forceinline__ int chunk_round(int ch) {
  if constexpr (sizeof(T) == 8) {
    return ch <= 1 ? 1 : ch <= 2 ? 2 : ch <= 4 ? 4 : ch <= 8 ? 8 : 16;
  } else {
    return ch;
  }
}

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
  T fn = (J - mul_rn(G, vj)) * scl;
  fn = fn + (mul_rn(gr, vr - vj) - mul_rn(glf, vj - vl));
  if (A.field && A.ve_amp) {
    const T I = rect_pulse<T>(t, A.ve_amp[cable], A.ve_delay[cable], A.ve_pw[cable]);
    if (I != T(0)) {
      const T ve = mul_rn(A.field[g], I);
      const T vel = i > 0 ? mul_rn(A.field[g - 1], I) : ve;
      const T ver = i < K - 1 ? mul_rn(A.field[g + 1], I) : ve;
      fn = fn + (mul_rn(gr, ver - ve) - mul_rn(glf, ve - vel));
    }
  }
  if (A.in_idx && A.in_idx[cable] == (int)i) {
    const T I = rect_pulse<T>(t, A.in_amp[cable], A.in_delay[cable], A.in_pw[cable]);
    if (I != T(0)) fn = fn + I * A.cm_inv[g];
  }
  rhs[g] = A.dt_s * fn;
  mainv[g] = T(1) - A.dt_s * ((-gr + -glf) - mul_rn(G, scl));
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

template <typename T, bool FAST, bool TAPE, bool PLANES>
static int launch_cable_split(CableArgsT<T> A, int ch_max, cudaStream_t st) {
  DGB_REQUIRE(A.lanes_mode == 0, "DGB_CABLE_SPLIT_GATES needs lanes_mode 0");
  const size_t smem = (size_t)(RowsNQ<PLANES>::value + 1) * ch_max * 32 * sizeof(T);
  DGB_REQUIRE(smem <= 227 * 1024, "cable too long for shared memory (%zu bytes per cable)",
              smem);
  const int threads = kSplitWarps * 32;
  auto kern = cable_run_split_kernel<T, FAST, TAPE, PLANES>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  int blocks = device_sm_count() * per_sm;
  if (blocks > A.n_cables) blocks = A.n_cables;
  if (blocks < 1) blocks = 1;
  DGB_CUDA_CHECK(cudaMemsetAsync(A.counter, 0, 2 * sizeof(int32_t), st));
  kern<<<blocks, threads, smem, st>>>(A, ch_max);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T, bool FAST, bool TAPE, bool PLANES>
static int launch_cable_run(CableArgsT<T> A, int ch_max, cudaStream_t st) {
  // a population with at most one cable per SM: spread each cable's gate
  // work over the SM's sub-partitions
  if (A.split || (A.wpb <= 0 && A.lanes_mode == 0 && A.n_cables <= device_sm_count()))
    return launch_cable_split<T, FAST, TAPE, PLANES>(A, ch_max, st);
  // rows per lane: ch_max at 32 lanes, up to 8 on 16 or 8 lanes when split
  const int ch_alloc = (A.lanes_mode != 0 && ch_max < 8) ? 8 : ch_max;
  const size_t per_warp = (size_t)RowsNQ<PLANES>::value * ch_alloc * 32 * sizeof(T);
  int items = A.n_cables;
  if (A.lanes_mode != 0) {
    const int n8 = A.n_cables - A.n_lanes32 - A.n_lanes16;
    items = A.n_lanes32 + (A.n_lanes16 + 1) / 2 + (n8 + 3) / 4;
  }
  int wpb = persistent_wpb(A.wpb, per_warp);
  DGB_REQUIRE(wpb > 0, "cable too long for shared memory (%zu bytes per cable)", per_warp);
  if (A.wpb <= 0) {
    // default shape: a population with fewer warps of work than the device
    // has SMs x default CTA width spreads over the SMs, one CTA each
    while (wpb > 1 && (items + wpb - 1) / wpb < device_sm_count()) wpb >>= 1;
  }
  const int threads = wpb * 32;
  const size_t smem = (size_t)wpb * per_warp;
  auto kern = cable_run_kernel<T, FAST, TAPE, PLANES>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  int blocks = device_sm_count() * per_sm;
  const int blocks_needed = (items + wpb - 1) / wpb;
  if (blocks > blocks_needed) blocks = blocks_needed;
  if (blocks < 1) blocks = 1;
  DGB_CUDA_CHECK(cudaMemsetAsync(A.counter, 0, 2 * sizeof(int32_t), st));
  kern<<<blocks, threads, smem, st>>>(A, ch_alloc);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T, bool FAST, bool TAPE>
int cable_run_launch(const dgb_cable_args* args, void* tape, int ch_max, cudaStream_t st) {
  CableArgsT<T> A = typed<T>(args);
  A.tape = (T*)tape;
  const bool chan_planes = (args->flags & DGB_CABLE_UNIFORM_CHANNELS) == 0;
  const bool geo_planes = (args->flags & DGB_CABLE_UNIFORM_GEOMETRY) == 0;
  if (chan_planes || geo_planes) return launch_cable_run<T, FAST, TAPE, true>(A, ch_max, st);
  return launch_cable_run<T, FAST, TAPE, false>(A, ch_max, st);
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

// Instantiations, split so that the persistent run variants and the plain
// per-step kernels compile in parallel translation units.
#define DGB_INSTANTIATE_CABLE_RUN(T, FAST, TAPE) \
  template int cable_run_launch<T, FAST, TAPE>(const dgb_cable_args*, void*, int, cudaStream_t);
#define DGB_INSTANTIATE_CABLE_PLAIN(T)                                                   \
  template int cable_assemble_t<T>(const dgb_cable_args*, int32_t, void*, void*, void*, \
                                   void*, cudaStream_t);                               \
  template int cable_solve_update_t<T>(const dgb_cable_args*, const void*, const void*, \
                                       const void*, const void*, cudaStream_t);

}  // namespace dgb
