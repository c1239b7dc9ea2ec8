// Interpolated (differentiable) delay transport on a dense delivery ring
// queue[depth][width] on sm_103a.
//
//   dgb_two_tap_enqueue     ordered_two_tap_enqueue(_) and the two-tap branch of
//                           dense_interpolated_delay_transition
//                           (networks/_two_tap_enqueue_cpu.cpp:26-126,
//                           networks/_event_delivery.py:229-308)
//   dgb_three_tap_enqueue   the three-tap branch (_event_delivery.py:294-306)
//   dgb_two_tap_gather      delay_ring_gather_two_tap (_two_tap_enqueue_cpu.cpp:206-233)
//   dgb_two_tap_vjp         delay_ring_two_tap_vjp (:235-315) / the unfused adjoint of
//                           networks/_two_tap_enqueue.py:94-150
//   dgb_three_tap_vjp       torch autograd of the three-tap scatter (gather of the
//                           cotangent, products, tap sum in order)
//   dgb_two_tap_rollout(_vjp) many steps of the above in one launch, each
//                           block's ring columns held in shared memory
//
// Determinism: the reference's CPU op adds every edge's lower-tap value in
// edge order, then every upper-tap value in edge order, into a ring it owns
// (its CUDA path scatters with atomics).  Here one thread owns one ring column
// for the whole launch and walks that column's edges in ascending order, so
// each ring value sees exactly the reference's sequence of additions: results
// are bit-identical, with no floating-point atomics.  Every product and sum is
// rounded on its own (no FMA contraction), as the CPU op computes them.
#include <algorithm>

#include "common.cuh"

namespace dgb {

__device__ int g_delay_err = 0;

__device__ __forceinline__ void delay_fail(int code) { atomicCAS(&g_delay_err, 0, code); }

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Edge operands.  f is the upper-tap share (two taps) or the [E][3]
// coefficients (three taps); gates are indexed by pre[e] when pre is set.
template <typename T>
struct TapEdges {
  const T* w;
  const int64_t* pre;
  int64_t n_src;
  const T* f;
  int64_t n_edges;
};

// Row *slot of the ring: start = slot*width, tail = ring_size - start.
struct RingPos {
  int64_t start, tail, size;
};

__device__ __forceinline__ RingPos ring_pos(int64_t slot, int64_t width, int64_t size) {
  return RingPos{slot * width, size - slot * width, size};
}

// w[e] * gate(e).  False (and an error) for a source outside the gates.
template <typename T>
__device__ __forceinline__ bool weighted_gate(const TapEdges<T>& E, const T* __restrict__ g,
                                              int64_t e, T& wg) {
  int64_t s = e;
  if (E.pre) {
    s = E.pre[e];
    if ((uint64_t)s >= (uint64_t)E.n_src) {
      delay_fail(DGB_DELAY_ERR_SOURCE);
      return false;
    }
  }
  wg = mul_rn(E.w[e], g[s]);
  return true;
}

// Column list [j0, j1) of a plan, clamped to the edge array.
__device__ __forceinline__ bool column_range(const int64_t* __restrict__ ptr, int64_t col,
                                             int64_t n_edges, int64_t& j0, int64_t& j1) {
  j0 = ptr[col];
  j1 = ptr[col + 1];
  if (j0 < 0 || j1 < j0 || j1 > n_edges) {
    delay_fail(DGB_DELAY_ERR_PLAN);
    return false;
  }
  return true;
}

// One tap of every edge of column `col`, in list order:
//   ring[(start + addr[e]) mod size] += (w g) * (UPPER ? f : 1 - f).
// CHECK_COLUMN verifies that the address lies in this column (a plan that
// does not match its addresses would let two threads add to one value).
template <typename T, bool UPPER, bool CHECK_COLUMN>
__device__ __forceinline__ void column_taps(T* __restrict__ ring, const RingPos& P, int64_t width,
                                            int64_t col, const TapEdges<T>& E,
                                            const T* __restrict__ g,
                                            const int64_t* __restrict__ addr,
                                            const int64_t* __restrict__ ptr,
                                            const int64_t* __restrict__ edge) {
  int64_t j0, j1;
  if (!column_range(ptr, col, E.n_edges, j0, j1)) return;
  for (int64_t j = j0; j < j1; ++j) {
    const int64_t e = edge[j];
    if ((uint64_t)e >= (uint64_t)E.n_edges) {
      delay_fail(DGB_DELAY_ERR_PLAN);
      continue;
    }
    const int64_t base = addr[e];
    if ((uint64_t)base >= (uint64_t)P.size) {
      delay_fail(DGB_DELAY_ERR_ADDRESS);
      continue;
    }
    if (CHECK_COLUMN && base % width != col) {
      delay_fail(DGB_DELAY_ERR_PLAN);
      continue;
    }
    T wg;
    if (!weighted_gate(E, g, e, wg)) continue;
    const T fe = E.f[e];
    const T share = UPPER ? fe : sub_rn(T(1), fe);
    const int64_t d = base < P.tail ? P.start + base : base - P.tail;
    ring[d] = add_rn(ring[d], mul_rn(wg, share));
  }
}

// Thread = ring column.  Deliver (optional), clear, lower taps, upper taps.
template <typename T>
__global__ void __launch_bounds__(256)
    two_tap_enqueue_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                           const int64_t* __restrict__ slot_ptr, TapEdges<T> E,
                           const T* __restrict__ gates, const int64_t* __restrict__ lower,
                           const int64_t* __restrict__ upper, const int64_t* __restrict__ lo_ptr,
                           const int64_t* __restrict__ lo_edge,
                           const int64_t* __restrict__ up_ptr,
                           const int64_t* __restrict__ up_edge, T* __restrict__ payload) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= width) return;
  const int64_t slot = slot_ptr[0];
  if (slot < 0 || slot >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  const RingPos P = ring_pos(slot, width, depth * width);
  if (payload) payload[col] = ring[P.start + col];
  ring[P.start + col] = T(0);
  column_taps<T, false, true>(ring, P, width, col, E, gates, lower, lo_ptr, lo_edge);
  column_taps<T, true, true>(ring, P, width, col, E, gates, upper, up_ptr, up_edge);
}

// Thread = ring column; edges of the column in order, three taps each.
template <typename T>
__global__ void __launch_bounds__(256)
    three_tap_enqueue_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                             const int64_t* __restrict__ slot_ptr, TapEdges<T> E,
                             const T* __restrict__ gates, const int64_t* __restrict__ offsets,
                             const int64_t* __restrict__ post, const int64_t* __restrict__ ptr,
                             const int64_t* __restrict__ edge, T* __restrict__ payload) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= width) return;
  const int64_t slot = slot_ptr[0];
  if (slot < 0 || slot >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  if (payload) payload[col] = ring[slot * width + col];
  ring[slot * width + col] = T(0);
  int64_t j0, j1;
  if (!column_range(ptr, col, E.n_edges, j0, j1)) return;
  for (int64_t j = j0; j < j1; ++j) {
    const int64_t e = edge[j];
    if ((uint64_t)e >= (uint64_t)E.n_edges || post[e] != col) {
      delay_fail(DGB_DELAY_ERR_PLAN);
      continue;
    }
    T wg;
    if (!weighted_gate(E, gates, e, wg)) continue;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      int64_t r = (slot + offsets[3 * e + t]) % depth;  // remainder, made non-negative
      if (r < 0) r += depth;
      const int64_t d = r * width + col;
      ring[d] = add_rn(ring[d], mul_rn(wg, E.f[3 * e + t]));
    }
  }
}

// (base + offset) mod size, non-negative; the direct form for addresses in
// range, the general remainder otherwise.
__device__ __forceinline__ int64_t wrap_tap(int64_t base, int64_t offset, int64_t size,
                                            int64_t tail) {
  if (tail > 0 && (uint64_t)base < (uint64_t)size) return base < tail ? offset + base : base - tail;
  const int64_t r = (int64_t)((uint64_t)base + (uint64_t)offset) % size;
  return r < 0 ? r + size : r;
}

__device__ __forceinline__ int64_t tail_of(int64_t offset, int64_t size) {
  return (offset >= 0 && offset < size) ? size - offset : 0;
}

template <typename T>
__global__ void two_tap_gather_kernel(const T* __restrict__ ring, int64_t size,
                                      const int64_t* __restrict__ offset_ptr, int64_t n,
                                      const int64_t* __restrict__ lower,
                                      const int64_t* __restrict__ upper, T* __restrict__ lo_out,
                                      T* __restrict__ hi_out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int64_t offset = offset_ptr[0];
  const int64_t tail = tail_of(offset, size);
  lo_out[e] = ring[wrap_tap(lower[e], offset, size, tail)];
  hi_out[e] = ring[wrap_tap(upper[e], offset, size, tail)];
}

// Cotangents of one edge from the ring cotangent at its two taps.
template <typename T>
__device__ __forceinline__ void edge_vjp(T lo, T hi, T w, T g, T f, T& dw, T& dg, T& df) {
  const T dweighted = add_rn(mul_rn(hi, f), mul_rn(lo, sub_rn(T(1), f)));
  const T weighted = mul_rn(w, g);
  dw = mul_rn(dweighted, g);
  df = sub_rn(mul_rn(hi, weighted), mul_rn(lo, weighted));
  dg = mul_rn(dweighted, w);
}

// Gates per edge: thread = edge.
template <typename T>
__global__ void two_tap_vjp_edge_kernel(const T* __restrict__ ring, int64_t size,
                                        const int64_t* __restrict__ offset_ptr, TapEdges<T> E,
                                        const T* __restrict__ gates,
                                        const int64_t* __restrict__ lower,
                                        const int64_t* __restrict__ upper, T* __restrict__ dw,
                                        T* __restrict__ dg, T* __restrict__ df) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E.n_edges) return;
  const int64_t offset = offset_ptr[0];
  const int64_t tail = tail_of(offset, size);
  const T lo = ring[wrap_tap(lower[e], offset, size, tail)];
  const T hi = ring[wrap_tap(upper[e], offset, size, tail)];
  edge_vjp(lo, hi, E.w[e], gates[e], E.f[e], dw[e], dg[e], df[e]);
}

// Gates per source: thread = source, its edges in ascending order; the gate
// cotangent is their sum from +0 (index_select_backward's serial order).
template <typename T>
__global__ void two_tap_vjp_source_kernel(const T* __restrict__ ring, int64_t size,
                                          const int64_t* __restrict__ offset_ptr, TapEdges<T> E,
                                          const T* __restrict__ gates,
                                          const int64_t* __restrict__ lower,
                                          const int64_t* __restrict__ upper,
                                          const int64_t* __restrict__ src_ptr,
                                          const int64_t* __restrict__ src_edge,
                                          T* __restrict__ dw, T* __restrict__ dg,
                                          T* __restrict__ df) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= E.n_src) return;
  const int64_t offset = offset_ptr[0];
  const int64_t tail = tail_of(offset, size);
  T acc = T(0);
  int64_t j0, j1;
  if (column_range(src_ptr, s, E.n_edges, j0, j1)) {
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t e = src_edge[j];
      if ((uint64_t)e >= (uint64_t)E.n_edges) {
        delay_fail(DGB_DELAY_ERR_PLAN);
        continue;
      }
      int64_t se = E.pre[e];
      if (se < 0) se += E.n_src;
      if (se != s) {
        delay_fail(se < 0 || se >= E.n_src ? DGB_DELAY_ERR_SOURCE : DGB_DELAY_ERR_PLAN);
        continue;
      }
      const T lo = ring[wrap_tap(lower[e], offset, size, tail)];
      const T hi = ring[wrap_tap(upper[e], offset, size, tail)];
      T gg;
      edge_vjp(lo, hi, E.w[e], gates[s], E.f[e], dw[e], gg, df[e]);
      acc = add_rn(acc, gg);
    }
  }
  dg[s] = acc;
}

// Three taps, gates per edge: thread = edge.  Cotangents of the values
// (w g) c_t are the ring cotangent at the taps; d(w g) sums g_t c_t in tap order.
template <typename T>
__global__ void three_tap_vjp_kernel(const T* __restrict__ R, int64_t depth, int64_t width,
                                     const int64_t* __restrict__ slot_ptr, TapEdges<T> E,
                                     const T* __restrict__ gates,
                                     const int64_t* __restrict__ offsets,
                                     const int64_t* __restrict__ post, T* __restrict__ dw,
                                     T* __restrict__ dg, T* __restrict__ dc) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E.n_edges) return;
  const int64_t slot = slot_ptr[0];
  const int64_t col = post[e];
  if (slot < 0 || slot >= depth || col < 0 || col >= width) {
    delay_fail(slot < 0 || slot >= depth ? DGB_DELAY_ERR_SLOT : DGB_DELAY_ERR_ADDRESS);
    return;
  }
  const T w = E.w[e], g = gates[e];
  const T wg = mul_rn(w, g);
  T dwg = T(0);
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    int64_t r = (slot + offsets[3 * e + t]) % depth;
    if (r < 0) r += depth;
    const T gv = R[r * width + col];
    dc[3 * e + t] = mul_rn(gv, wg);
    const T p = mul_rn(gv, E.f[3 * e + t]);
    dwg = t == 0 ? p : add_rn(dwg, p);
  }
  dw[e] = mul_rn(dwg, g);
  dg[e] = mul_rn(dwg, w);
}

// ---------------------------------------------------------------------------
// Rollouts: many steps per launch, the ring on chip.
//
// One thread owns one ring column for the whole rollout: its values never
// leave the thread, so no step needs a barrier and the whole rollout is one
// launch.  A block keeps its columns' full ring depth in shared memory
// (row-major [depth][block], so a warp's accesses hit 32 distinct banks
// whatever rows its lanes touch); the ring is read from HBM once at the start
// and written once at the end, and the delivered rows leave as coalesced
// stores.  Rings too deep for shared memory run in place in HBM.  Plan: the
// column lists col_ptr / col_edge (edges ascending) and, per list position j,
// the row distances lo_row[j] / hi_row[j] in [0, depth) of the edge's taps.
// ---------------------------------------------------------------------------

// A rollout thread's column (32-bit: the host checks depth*width, n_edges and
// n_sources against 2^31).  A column with exactly one edge (n == 1) keeps that
// edge's operands in registers; others read their lists every step.  n < 0
// marks a column outside the ring or one that failed its checks (left
// untouched, error recorded).
template <typename T>
struct RollCol {
  int32_t j0, n, src, e, lo, hi;
  T w, f;
};

__device__ __forceinline__ int32_t tap_row32(int32_t slot, int32_t d, int32_t depth) {
  const int32_t r = slot + d;
  return r >= depth ? r - depth : r;
}

template <typename T>
__device__ __forceinline__ void roll_col_load(RollCol<T>& C, int64_t col, int64_t depth,
                                              int64_t width, const TapEdges<T>& E,
                                              const int64_t* __restrict__ ptr,
                                              const int64_t* __restrict__ edge,
                                              const int32_t* __restrict__ lo_row,
                                              const int32_t* __restrict__ hi_row) {
  C.n = -1;
  if (col >= width) return;
  int64_t j0, j1;
  if (!column_range(ptr, col, E.n_edges, j0, j1)) return;
  for (int64_t j = j0; j < j1; ++j) {
    const int64_t e = edge[j];
    if ((uint64_t)e >= (uint64_t)E.n_edges || (uint32_t)lo_row[j] >= (uint64_t)depth ||
        (uint32_t)hi_row[j] >= (uint64_t)depth ||
        (E.pre && (uint64_t)E.pre[e] >= (uint64_t)E.n_src)) {
      delay_fail(DGB_DELAY_ERR_PLAN);
      return;
    }
  }
  C.j0 = (int32_t)j0;
  C.n = (int32_t)(j1 - j0);
  if (C.n == 1) {
    const int64_t e = edge[j0];
    C.e = (int32_t)e;
    C.lo = lo_row[j0];
    C.hi = hi_row[j0];
    C.src = (int32_t)(E.pre ? E.pre[e] : e);
    C.w = E.w[e];
    C.f = E.f[e];
  }
}

// One edge whose taps sit at row distances lo and lo + 1 with 2 <= lo <= depth - 2:
// neither tap reaches the delivered row and consecutive steps chain through
// one cell (step k's upper-tap cell is step k + 1's lower-tap cell).
template <typename T>
__device__ __forceinline__ bool chained_taps(const RollCol<T>& C, int32_t depth) {
  return C.n == 1 && C.lo >= 2 && C.lo <= depth - 2 && C.hi == C.lo + 1;
}

// Ring column of a rollout thread: element r at rb[r * rs].
template <typename T>
struct ColRing {
  T* rb;
  int32_t rs;
  __device__ __forceinline__ T& operator[](int32_t r) const { return rb[(int64_t)r * rs]; }
};

// One step of a column with several edges: clear the delivered value, then
// both taps of every edge, lower taps in list order, then upper taps.  Out of
// line: rare, and inlined it would raise every thread's register count.
template <typename T>
__device__ __noinline__ void roll_col_generic(ColRing<T> R, int32_t slot, int32_t depth,
                                              int32_t j0, int32_t n, TapEdges<T> E,
                                              const T* __restrict__ g,
                                              const int64_t* __restrict__ edge,
                                              const int32_t* __restrict__ lo_row,
                                              const int32_t* __restrict__ hi_row) {
  R[slot] = T(0);
  for (int tap = 0; tap < 2; ++tap) {
    for (int32_t j = j0; j < j0 + n; ++j) {
      const int64_t e = edge[j];
      const T wg = mul_rn(E.w[e], g[E.pre ? E.pre[e] : e]);
      const T fe = E.f[e];
      const T share = tap ? fe : sub_rn(T(1), fe);
      T& v = R[tap_row32(slot, tap ? hi_row[j] : lo_row[j], depth)];
      v = add_rn(v, mul_rn(wg, share));
    }
  }
}

// Reverse step of a column with several edges (see the reverse kernel).  Gate
// cotangents: scratch[j * kc + k] with sources, else dgate[k * stride + e].
template <typename T, bool PRE>
__device__ __noinline__ void roll_col_generic_vjp(ColRing<T> R, int32_t slot, int32_t depth,
                                                  int32_t j0, int32_t n, TapEdges<T> E,
                                                  const T* __restrict__ g,
                                                  const int64_t* __restrict__ edge,
                                                  const int32_t* __restrict__ lo_row,
                                                  const int32_t* __restrict__ hi_row, bool first,
                                                  T* __restrict__ dw, T* __restrict__ df,
                                                  T* __restrict__ gate_out, int64_t k,
                                                  int64_t kc, int64_t stride) {
  for (int32_t j = j0; j < j0 + n; ++j) {
    const int64_t e = edge[j];
    T dwk, dgk, dfk;
    edge_vjp(R[tap_row32(slot, lo_row[j], depth)], R[tap_row32(slot, hi_row[j], depth)],
             E.w[e], g[PRE ? E.pre[e] : e], E.f[e], dwk, dgk, dfk);
    dw[e] = first ? dwk : add_rn(dw[e], dwk);
    df[e] = first ? dfk : add_rn(df[e], dfk);
    if (PRE)
      gate_out[(int64_t)j * kc + k] = dgk;
    else
      gate_out[k * stride + e] = dgk;
  }
}

// Eight consecutive values to a 32-byte-aligned group (two or four 16-byte stores).
template <typename T>
__device__ __forceinline__ void store8(T* dst, const T (&v)[8]) {
  if (sizeof(T) == 4) {
    reinterpret_cast<float4*>(dst)[0] = make_float4(v[0], v[1], v[2], v[3]);
    reinterpret_cast<float4*>(dst)[1] = make_float4(v[4], v[5], v[6], v[7]);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i)
      reinterpret_cast<double2*>(dst)[i] = make_double2(v[2 * i], v[2 * i + 1]);
  }
}

constexpr int kRollBlock = 128;
constexpr int kGateAhead = 8;  // steps per prefetch group (gates, payload cotangents)

// The thread's ring column: in shared memory (loaded from HBM, or zeros when
// the rollout starts empty) or, for deep rings, in place in HBM.
template <typename T, bool SMEM>
__device__ __forceinline__ ColRing<T> roll_ring(T* ring, int64_t width, int64_t col,
                                                int32_t depth, bool live, bool empty) {
  if (SMEM) {
    extern __shared__ __align__(16) unsigned char roll_smem[];
    ColRing<T> R{reinterpret_cast<T*>(roll_smem) + threadIdx.x, (int32_t)blockDim.x};
    if (live)
      for (int32_t r = 0; r < depth; ++r) R[r] = empty ? T(0) : ring[(int64_t)r * width + col];
    return R;
  }
  ColRing<T> R{ring + col, (int32_t)width};
  if (live && empty)
    for (int32_t r = 0; r < depth; ++r) R[r] = T(0);
  return R;
}

// n_steps steps from row *slot: deliver row slot (payload[k][col]), clear it,
// add both taps of every edge.  Thread = external column.
template <typename T, bool SMEM, bool ONE>
__global__ void __launch_bounds__(kRollBlock)
    two_tap_rollout_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                           const int64_t* __restrict__ slot_ptr, int64_t n_steps, TapEdges<T> E,
                           const T* __restrict__ gates, int64_t gate_stride,
                           const int64_t* __restrict__ ptr, const int64_t* __restrict__ edge,
                           const int32_t* __restrict__ lo_row,
                           const int32_t* __restrict__ hi_row, int flags,
                           T* __restrict__ payload) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t slot0 = slot_ptr[0];
  if (slot0 < 0 || slot0 >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  RollCol<T> C;
  roll_col_load(C, col, depth, width, E, ptr, edge, lo_row, hi_row);
  if (ONE && C.n > 1) {  // the lean variant was promised one edge per column
    delay_fail(DGB_DELAY_ERR_PLAN);
    C.n = -1;
  }
  const bool live = C.n >= 0;
  const int32_t D = (int32_t)depth;
  const ColRing<T> R =
      roll_ring<T, SMEM>(ring, width, col, D, live, (flags & DGB_ROLLOUT_EMPTY_START) != 0);
  if (!live) return;
  int32_t slot = (int32_t)slot0;
  // steps in groups of kGateAhead: the gates of the next group are loaded
  // while this group runs, so their memory latency is hidden
  T gq[kGateAhead], gn[kGateAhead];
  if (chained_taps(C, D)) {
    // One edge with taps at lo and lo + 1 (2 <= lo <= depth - 2): the cell
    // step k's upper tap updates is step k + 1's lower-tap cell, so its value
    // stays in a register (`carry`) between the two steps and reaches shared
    // memory once, after step k + 1.  The other two cells a step reads (its
    // delivered row and its upper-tap cell) are loaded one step ahead: they
    // differ from every cell the step before writes.  Values and the order of
    // operations on each value are those of the general path.
#pragma unroll
    for (int i = 0; i < kGateAhead; ++i)
      gq[i] = i < n_steps ? gates[i * gate_stride + C.src] : T(0);
    const T sh = sub_rn(T(1), C.f);
    const bool edge_hi = C.lo + 2 == D;  // upper-tap cell of step k + 1 is step k's row
    int32_t rl = tap_row32(slot, C.lo, D);
    T carry = R[rl];
    T nvs = R[slot], nvh = R[rl + 1 == D ? 0 : rl + 1];
    for (int64_t kb = 0; kb < n_steps; kb += kGateAhead) {
#pragma unroll
      for (int i = 0; i < kGateAhead; ++i) {
        const int64_t k2 = kb + kGateAhead + i;
        gn[i] = k2 < n_steps ? gates[k2 * gate_stride + C.src] : T(0);
      }
#pragma unroll
      for (int i = 0; i < kGateAhead; ++i) {
        const int64_t k = kb + i;
        if (k >= n_steps) break;
        const T vs = nvs, vh = nvh;
        const int32_t rh = rl + 1 == D ? 0 : rl + 1;
        const int32_t s1 = slot + 1 == D ? 0 : slot + 1;
        if (k + 1 < n_steps) {
          nvs = R[s1];
          nvh = edge_hi ? T(0) : R[rh + 1 == D ? 0 : rh + 1];
        }
        if (payload) payload[k * width + col] = vs;
        const T wg = mul_rn(C.w, gq[i]);
        R[slot] = T(0);
        R[rl] = add_rn(carry, mul_rn(wg, sh));
        carry = add_rn(vh, mul_rn(wg, C.f));
        slot = s1;
        rl = rh;
      }
#pragma unroll
      for (int i = 0; i < kGateAhead; ++i) gq[i] = gn[i];
    }
    R[rl] = carry;  // the last upper-tap cell
    if (SMEM && !(flags & DGB_ROLLOUT_NO_FINAL))
      for (int32_t r = 0; r < D; ++r) ring[(int64_t)r * width + col] = R[r];
    return;
  }
#pragma unroll
  for (int i = 0; i < kGateAhead; ++i)
    gq[i] = (C.n == 1 && i < n_steps) ? gates[i * gate_stride + C.src] : T(0);
  for (int64_t kb = 0; kb < n_steps; kb += kGateAhead) {
#pragma unroll
    for (int i = 0; i < kGateAhead; ++i) {
      const int64_t k2 = kb + kGateAhead + i;
      gn[i] = (C.n == 1 && k2 < n_steps) ? gates[k2 * gate_stride + C.src] : T(0);
    }
#pragma unroll
    for (int i = 0; i < kGateAhead; ++i) {
      const int64_t k = kb + i;
      if (k >= n_steps) break;
      if (C.n == 1) {
        // all three loads first, then the reference's order: clear, lower
        // tap, upper tap (a tap may land on the cleared row, or both taps on
        // one value)
        const int32_t rl = tap_row32(slot, C.lo, D), rh = tap_row32(slot, C.hi, D);
        const T vs = R[slot], vl = R[rl], vh = R[rh];
        if (payload) payload[k * width + col] = vs;
        const T wg = mul_rn(C.w, gq[i]);
        const T a = mul_rn(wg, sub_rn(T(1), C.f)), b = mul_rn(wg, C.f);
        T ns = T(0), l = vl, h = vh;
        if (rl == slot)
          ns = add_rn(ns, a);
        else
          l = add_rn(l, a);
        if (rh == slot)
          ns = add_rn(ns, b);
        else if (rh == rl)
          l = add_rn(l, b);
        else
          h = add_rn(h, b);
        R[slot] = ns;
        if (rl != slot) R[rl] = l;
        if (rh != slot && rh != rl) R[rh] = h;
      } else {
        if (payload) payload[k * width + col] = R[slot];
        if (ONE || C.n == 0)
          R[slot] = T(0);
        else
          roll_col_generic(R, slot, D, C.j0, C.n, E, gates + k * gate_stride, edge, lo_row,
                           hi_row);
      }
      if (++slot == D) slot = 0;
    }
#pragma unroll
    for (int i = 0; i < kGateAhead; ++i) gq[i] = gn[i];
  }
  if (SMEM && !(flags & DGB_ROLLOUT_NO_FINAL))
    for (int32_t r = 0; r < D; ++r) ring[(int64_t)r * width + col] = R[r];
}

// Reverse sweep of two_tap_rollout_kernel over the same steps, newest first,
// on the cotangent ring (grad_ring: in, after the rollout; out, before it).
// Per step and edge the two-tap VJP at the cotangent of the ring after the
// step; weight and share cotangents accumulate newest first (in registers for
// one-edge columns); gate cotangents go to scratch[k][j] (with sources, j =
// list position) or dgate[k][e]; then row slot_k takes the delivered row's
// cotangent gpay[k][col].
template <typename T, bool SMEM, bool PRE, bool ONE>
__global__ void __launch_bounds__(kRollBlock)
    two_tap_rollout_vjp_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                               const int64_t* __restrict__ slot_ptr, int64_t n_steps,
                               TapEdges<T> E, const T* __restrict__ gates, int64_t gate_stride,
                               const int64_t* __restrict__ ptr, const int64_t* __restrict__ edge,
                               const int32_t* __restrict__ lo_row,
                               const int32_t* __restrict__ hi_row, int flags,
                               const T* __restrict__ gpay, int accumulate, T* __restrict__ dw,
                               T* __restrict__ dgate, T* __restrict__ df,
                               T* __restrict__ scratch) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t slot0 = slot_ptr[0];
  if (slot0 < 0 || slot0 >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  RollCol<T> C;
  roll_col_load(C, col, depth, width, E, ptr, edge, lo_row, hi_row);
  if (ONE && C.n > 1) {
    delay_fail(DGB_DELAY_ERR_PLAN);
    C.n = -1;
  }
  const bool live = C.n >= 0;
  const int32_t D = (int32_t)depth;
  const ColRing<T> R =
      roll_ring<T, SMEM>(ring, width, col, D, live, (flags & DGB_ROLLOUT_EMPTY_START) != 0);
  if (!live) return;
  T aw = T(0), af = T(0);
  if (C.n == 1 && accumulate) {
    aw = dw[C.e];
    af = df[C.e];
  }
  // steps newest first in aligned groups of eight, so that a one-edge
  // column's gate cotangents leave as whole 32-byte groups of its scratch row
  // scratch[j][0..kc) (kc = n_steps rounded up to 8)
  const int64_t kc = (n_steps + 7) & ~int64_t(7);
  T* srow = PRE && C.n == 1 ? scratch + (int64_t)C.j0 * kc : nullptr;
  int32_t slot = (int32_t)((slot0 + n_steps - 1) % depth);
  const int64_t k_top = n_steps - 1;
  // the gates and delivered-row cotangents of the next group of eight steps
  // are loaded while this group runs
  T gq[8], pq[8], gn[8], pn[8];
  auto fetch = [&](int64_t base, T (&g8)[8], T (&p8)[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t k = base + i;
      const bool in = k >= 0 && k < n_steps;
      g8[i] = (C.n == 1 && in) ? gates[k * gate_stride + C.src] : T(0);
      p8[i] = (gpay && in) ? gpay[k * width + col] : T(0);
    }
  };
  fetch(k_top & ~int64_t(7), gq, pq);
  if (chained_taps(C, D) && n_steps > 0) {
    // Reverse of the chained forward: step k reads the cells at lo and lo + 1
    // and then replaces its delivered row; step k - 1's upper-tap cell is step
    // k's lower-tap cell, unchanged in between, so that value is carried in a
    // register, and step k - 1's lower-tap cell is loaded one step ahead (it
    // is not step k's delivered row, as lo >= 2).
    int32_t rl = tap_row32(slot, C.lo, D);
    T vl = R[rl], vh = R[rl + 1 == D ? 0 : rl + 1];
    for (int64_t gb = k_top & ~int64_t(7); gb >= 0; gb -= 8) {
      fetch(gb - 8, gn, pn);
      T buf[8];
#pragma unroll
      for (int i = 7; i >= 0; --i) {
        const int64_t k = gb + i;
        buf[i] = T(0);
        if (k >= n_steps) continue;
        const int32_t rl0 = rl == 0 ? D - 1 : rl - 1;
        const T vl0 = k > 0 ? R[rl0] : T(0);  // step k - 1's lower-tap cell
        const bool first = (k == k_top) && !accumulate;
        T dwk, dgk, dfk;
        edge_vjp(vl, vh, C.w, gq[i], C.f, dwk, dgk, dfk);
        aw = first ? dwk : add_rn(aw, dwk);
        af = first ? dfk : add_rn(af, dfk);
        if (PRE)
          buf[i] = dgk;
        else
          dgate[k * gate_stride + C.e] = dgk;
        R[slot] = pq[i];
        slot = slot == 0 ? D - 1 : slot - 1;
        vh = vl;
        vl = vl0;
        rl = rl0;
      }
      if (srow) store8(srow + gb, buf);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        gq[i] = gn[i];
        pq[i] = pn[i];
      }
    }
    dw[C.e] = aw;
    df[C.e] = af;
    if (SMEM && !(flags & DGB_ROLLOUT_NO_FINAL))
      for (int32_t r = 0; r < D; ++r) ring[(int64_t)r * width + col] = R[r];
    return;
  }
  for (int64_t gb = k_top & ~int64_t(7); gb >= 0; gb -= 8) {
    fetch(gb - 8, gn, pn);
    T buf[8];
#pragma unroll
    for (int i = 7; i >= 0; --i) {
      const int64_t k = gb + i;
      buf[i] = T(0);
      if (k >= n_steps) continue;
      const bool first = (k == k_top) && !accumulate;
      if (C.n == 1) {
        T dwk, dgk, dfk;
        edge_vjp(R[tap_row32(slot, C.lo, D)], R[tap_row32(slot, C.hi, D)], C.w, gq[i], C.f,
                 dwk, dgk, dfk);
        aw = first ? dwk : add_rn(aw, dwk);
        af = first ? dfk : add_rn(af, dfk);
        if (PRE)
          buf[i] = dgk;
        else
          dgate[k * gate_stride + C.e] = dgk;
      } else if (!ONE && C.n > 1) {
        roll_col_generic_vjp<T, PRE>(R, slot, D, C.j0, C.n, E, gates + k * gate_stride, edge,
                                     lo_row, hi_row, first, dw, df, PRE ? scratch : dgate, k, kc,
                                     gate_stride);
      }
      R[slot] = pq[i];
      slot = slot == 0 ? D - 1 : slot - 1;
    }
    if (srow) store8(srow + gb, buf);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      gq[i] = gn[i];
      pq[i] = pn[i];
    }
  }
  if (C.n == 1 && n_steps > 0) {
    dw[C.e] = aw;
    df[C.e] = af;
  }
  if (SMEM && !(flags & DGB_ROLLOUT_NO_FINAL))
    for (int32_t r = 0; r < D; ++r) ring[(int64_t)r * width + col] = R[r];
}

// dgate[k][s] = sum over the source's edges, in ascending edge order from +0,
// of scratch[pos][k] (pos = the edge's list position; rows of kc values, k
// contiguous).  Thread = (source, step), steps fastest: a warp reads 32
// consecutive steps of one scratch row per edge.
template <typename T>
__global__ void source_sum_kernel(const T* __restrict__ scratch, int64_t n_steps, int64_t kc,
                                  int64_t n_edges, int64_t n_src,
                                  const int64_t* __restrict__ src_ptr,
                                  const int64_t* __restrict__ src_pos, T* __restrict__ dgate) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_steps * n_src) return;
  const int64_t s = i / n_steps, k = i - s * n_steps;
  T acc = T(0);
  int64_t j0, j1;
  if (column_range(src_ptr, s, n_edges, j0, j1)) {
    // eight loads in flight, then their additions in order
    for (int64_t jb = j0; jb < j1; jb += 8) {
      T v[8];
      bool ok[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int64_t j = jb + q;
        const int64_t pos = j < j1 ? src_pos[j] : 0;
        ok[q] = j < j1 && (uint64_t)pos < (uint64_t)n_edges;
        if (j < j1 && !ok[q]) delay_fail(DGB_DELAY_ERR_PLAN);
        v[q] = ok[q] ? scratch[pos * kc + k] : T(0);
      }
#pragma unroll
      for (int q = 0; q < 8; ++q)
        if (ok[q]) acc = add_rn(acc, v[q]);
    }
  }
  dgate[k * n_src + s] = acc;
}

// ---------------------------------------------------------------------------
// Direct rollouts: columns with one edge whose taps sit at row distances lo
// and lo + 1, 1 <= lo <= depth - 2 (every connection of a transition whose
// ring is deeper than its longest delay).  Such a column's cell delivered at
// step k was cleared at step k - depth (or holds its initial value, for
// k < depth) and then received exactly two additions, the upper tap of step
// k - lo - 1 and the lower tap of step k - lo, in that order.  So
//   payload[k] = (c0 + (w g[k-lo-1]) f) + (w g[k-lo]) (1 - f)
// with the same roundings as the step-by-step ring, and every step is
// independent: each thread streams its column through time with no ring
// state at all.  The reverse sweep iterates over delivery steps m: the
// cotangent delivered at m is the lower-tap cotangent of step m - lo and the
// upper-tap cotangent of step m - lo - 1, so its reads are whole rows.
// Gates are read per source from gT[s][k] (steps contiguous, rows of kc), so
// a thread's consecutive steps share cache sectors.
// ---------------------------------------------------------------------------

// gT[s][k] = gates[k][s] (k < n; rows of kc values); 32 x 32 tiles.
template <typename T>
__global__ void gates_by_source_kernel(const T* __restrict__ g, T* __restrict__ gT, int64_t n,
                                       int64_t S, int64_t kc) {
  __shared__ T tile[32][33];
  const int64_t k0 = (int64_t)blockIdx.x * 32, s0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t k = k0 + r, s = s0 + threadIdx.x;
    if (k < n && s < S) tile[r][threadIdx.x] = g[k * S + s];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t s = s0 + r, k = k0 + threadIdx.x;
    if (s < S && k < n) gT[s * kc + k] = tile[threadIdx.x][r];
  }
}

// A direct-rollout column: -1 outside the ring or failing the checks, else
// its edge count (0 or 1) and, for one edge, its operands.
template <typename T>
__device__ __forceinline__ int direct_col_load(int64_t col, int64_t depth, int64_t width,
                                               const TapEdges<T>& E,
                                               const int64_t* __restrict__ ptr,
                                               const int64_t* __restrict__ edge,
                                               const int32_t* __restrict__ lo_row,
                                               const int32_t* __restrict__ hi_row, int32_t& lo,
                                               int64_t& src, int64_t& e, T& w, T& f) {
  if (col >= width) return -1;
  int64_t j0, j1;
  if (!column_range(ptr, col, E.n_edges, j0, j1)) return -1;
  if (j1 == j0) return 0;
  e = j1 - j0 == 1 ? edge[j0] : -1;
  if (e < 0 || e >= E.n_edges || lo_row[j0] < 1 || lo_row[j0] > depth - 2 ||
      hi_row[j0] != lo_row[j0] + 1 || (E.pre && (uint64_t)E.pre[e] >= (uint64_t)E.n_src)) {
    delay_fail(DGB_DELAY_ERR_PLAN);
    return -1;
  }
  lo = lo_row[j0];
  src = E.pre ? E.pre[e] : e;
  w = E.w[e];
  f = E.f[e];
  return 1;
}

// Gate of step k of the thread's source: gT[src][k] (GT) or gates[k][src].
template <typename T, bool GT>
__device__ __forceinline__ T gate_at(const T* __restrict__ g, int64_t k, int64_t src,
                                     int64_t stride, int64_t g_kc) {
  return GT ? g[src * g_kc + k] : g[k * stride + src];
}

template <typename T, bool GT>
__global__ void __launch_bounds__(128)
    two_tap_direct_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                          const int64_t* __restrict__ slot_ptr, int64_t n_steps, TapEdges<T> E,
                          const T* __restrict__ gates, int64_t gate_stride, int64_t g_kc,
                          const int64_t* __restrict__ ptr, const int64_t* __restrict__ edge,
                          const int32_t* __restrict__ lo_row,
                          const int32_t* __restrict__ hi_row, int flags,
                          T* __restrict__ payload) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t slot0 = slot_ptr[0];
  if (slot0 < 0 || slot0 >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  int32_t lo = 0;
  int64_t src = 0, e = 0;
  T w = T(0), f = T(0);
  const int ne = direct_col_load(col, depth, width, E, ptr, edge, lo_row, hi_row, lo, src, e, w, f);
  if (ne < 0) return;
  const bool empty = (flags & DGB_ROLLOUT_EMPTY_START) != 0;
  const T share = sub_rn(T(1), f);
  const int32_t D = (int32_t)depth;
  // value of the cell delivered at (virtual) step k, from steps < n_steps
  auto cell = [&](int64_t k, int32_t row, T gj, T gj1) -> T {
    T v = (k < D && !empty) ? ring[(int64_t)row * width + col] : T(0);
    if (ne == 1) {
      const int64_t j = k - lo;
      if (j - 1 >= 0 && j - 1 < n_steps) v = add_rn(v, mul_rn(mul_rn(w, gj1), f));
      if (j >= 0 && j < n_steps) v = add_rn(v, mul_rn(mul_rn(w, gj), share));
    }
    return v;
  };
  int32_t row = (int32_t)slot0;
  // gates one group ahead: gq holds steps kb - lo .. kb - lo + 7
  T gq[8], gn[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t j = (int64_t)i - lo;
    gq[i] = (ne == 1 && j >= 0 && j < n_steps) ? gate_at<T, GT>(gates, j, src, gate_stride, g_kc)
                                               : T(0);
  }
  // the upper-tap term of step k is the lower-tap product of step k - 1:
  // (w g[j-1]) is carried, and each delivered value is
  //   ((c0 + wg_prev f) + wg (1 - f)),  terms present once their step exists
  T wg_prev = T(0);
  T* out = payload ? payload + col : nullptr;
  const T* init = ring + (int64_t)row * width + col;
  for (int64_t kb = 0; kb < n_steps; kb += 8) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t j = kb + 8 + i - lo;
      gn[i] = (ne == 1 && j >= 0 && j < n_steps) ? gate_at<T, GT>(gates, j, src, gate_stride, g_kc)
                                                 : T(0);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t k = kb + i;
      if (k >= n_steps) break;
      T v = (k < D && !empty) ? *init : T(0);
      const int64_t j = k - lo;
      const T wg = mul_rn(w, gq[i]);
      if (ne == 1) {
        if (j >= 1) v = add_rn(v, mul_rn(wg_prev, f));
        if (j >= 0) v = add_rn(v, mul_rn(wg, share));
      }
      wg_prev = wg;
      if (out) {
        *out = v;
        out += width;
      }
      if (++row == D) {
        row = 0;
        init = ring + col;
      } else {
        init += width;
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) gq[i] = gn[i];
  }
  if (flags & DGB_ROLLOUT_NO_FINAL) return;
  // the ring after the rollout: row of (virtual) step n + d, d < depth, holds
  // the value that step would deliver from steps before n (read before write)
  for (int32_t d = 0; d < D; ++d) {
    const int64_t k = n_steps + d;
    const int64_t j = k - lo;
    const T gj = (ne == 1 && j >= 0 && j < n_steps)
                     ? gate_at<T, GT>(gates, j, src, gate_stride, g_kc) : T(0);
    const T gj1 = (ne == 1 && j - 1 >= 0 && j - 1 < n_steps)
                      ? gate_at<T, GT>(gates, j - 1, src, gate_stride, g_kc) : T(0);
    const T v = cell(k, row, gj, gj1);
    ring[(int64_t)row * width + col] = v;
    if (++row == D) row = 0;
  }
}

// Reverse sweep of two_tap_direct_kernel on the cotangent ring (in place: in,
// after the rollout, out, before it), over delivery steps m newest first.
// cot(m) = grad_payload[m] (m < n) or the ring cotangent of m's row; step
// k = m - lo takes lower-tap cotangent cot(m) and upper-tap cotangent
// cot(m + 1).  Gate cotangents: scratch[j0][k] in aligned groups of eight
// (a shift register) with sources, else dgate[k][e].
template <typename T, bool GT, bool PRE>
__global__ void __launch_bounds__(128)
    two_tap_direct_vjp_kernel(T* __restrict__ R, int64_t depth, int64_t width,
                              const int64_t* __restrict__ slot_ptr, int64_t n_steps,
                              TapEdges<T> E, const T* __restrict__ gates, int64_t gate_stride,
                              int64_t g_kc, const int64_t* __restrict__ ptr,
                              const int64_t* __restrict__ edge,
                              const int32_t* __restrict__ lo_row,
                              const int32_t* __restrict__ hi_row, int flags,
                              const T* __restrict__ gpay, int accumulate, T* __restrict__ dw,
                              T* __restrict__ dgate, T* __restrict__ df,
                              T* __restrict__ scratch) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t slot0 = slot_ptr[0];
  if (slot0 < 0 || slot0 >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  int32_t lo = 0;
  int64_t src = 0, e = 0;
  T w = T(0), f = T(0);
  const int ne = direct_col_load(col, depth, width, E, ptr, edge, lo_row, hi_row, lo, src, e, w, f);
  if (ne < 0) return;
  const bool empty = (flags & DGB_ROLLOUT_EMPTY_START) != 0;
  const int32_t D = (int32_t)depth;
  const int64_t n = n_steps;
  if (ne == 1) {
    T aw = accumulate ? dw[e] : T(0), af = accumulate ? df[e] : T(0);
    const int64_t kc = (n + 7) & ~int64_t(7);  // scratch row length
    T* srow = PRE ? scratch + (ptr[col] * kc) : nullptr;
    T sh[8];  // gate cotangents of steps k .. k + 7 once k reaches a multiple of 8
#pragma unroll
    for (int i = 0; i < 8; ++i) sh[i] = T(0);
    // delivery steps m from n + depth - 1 down to 0, the same for every lane
    // (step k = m - lo is this lane's when 0 <= k < n), in aligned groups of
    // eight; the cotangents and gates of the next group are loaded while a
    // group runs, the cotangents past L1 (each is read once)
    const int64_t m_hi = n + D - 1;
    auto cot = [&](int64_t m, int32_t row) -> T {
      if (m < n) return gpay ? __ldcg(gpay + m * width + col) : T(0);
      return empty ? T(0) : __ldcg(R + (int64_t)row * width + col);
    };
    auto fetch = [&](int64_t gb, T (&c8)[8], T (&g8)[8]) {
      int32_t row = (int32_t)((slot0 + gb) % depth);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int64_t m = gb + i, k = m - lo;
        c8[i] = (gb >= 0 && m <= m_hi) ? cot(m, row) : T(0);
        g8[i] = (gb >= 0 && k >= 0 && k < n) ? gate_at<T, GT>(gates, k, src, gate_stride, g_kc)
                                             : T(0);
        if (++row == D) row = 0;
      }
    };
    T cq[8], gq[8], cn[8], gn[8];
    const int64_t g_top = m_hi & ~int64_t(7);
    fetch(g_top, cq, gq);
    T c_next = T(0);  // cot(m + 1)
    for (int64_t gb = g_top; gb >= 0; gb -= 8) {
      fetch(gb - 8, cn, gn);
#pragma unroll
      for (int i = 7; i >= 0; --i) {
        const int64_t m = gb + i, k = m - lo;
        if (m > m_hi) continue;
        if (k >= 0 && k < n) {
          T dwk, dgk, dfk;
          edge_vjp(cq[i], c_next, w, gq[i], f, dwk, dgk, dfk);
          const bool first = (k == n - 1) && !accumulate;
          aw = first ? dwk : add_rn(aw, dwk);
          af = first ? dfk : add_rn(af, dfk);
          if (PRE) {
#pragma unroll
            for (int q = 7; q > 0; --q) sh[q] = sh[q - 1];
            sh[0] = dgk;
            if ((k & 7) == 0) store8(srow + k, sh);
          } else {
            dgate[k * gate_stride + e] = dgk;
          }
        }
        c_next = cq[i];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        cq[i] = cn[i];
        gq[i] = gn[i];
      }
    }
    if (n > 0) {
      dw[e] = aw;
      df[e] = af;
    }
  }
  // the ring cotangent before the rollout: row of step d takes the cotangent
  // of its first delivery (d < n) or passes through
  int32_t row = (int32_t)slot0;
  for (int32_t d = 0; d < D; ++d) {
    if (d < n)
      R[(int64_t)row * width + col] = gpay ? gpay[(int64_t)d * width + col] : T(0);
    else if (empty)
      R[(int64_t)row * width + col] = T(0);
    if (++row == D) row = 0;
  }
}

inline unsigned blocks_for(int64_t n, int th) { return (unsigned)((n + th - 1) / th); }

template <typename T>
TapEdges<T> tap_edges(const void* w, const int64_t* pre, int64_t n_src, const void* f,
                      int64_t n_edges) {
  return TapEdges<T>{(const T*)w, pre, n_src, (const T*)f, n_edges};
}

}  // namespace dgb

using namespace dgb;

#define DGB_DELAY_DISPATCH(dtype, ...)        \
  do {                                        \
    if ((dtype) == DGB_F32) {                 \
      using T = float;                        \
      __VA_ARGS__;                            \
    } else {                                  \
      using T = double;                       \
      __VA_ARGS__;                            \
    }                                         \
  } while (0)

static int check_ring(int dtype, const void* queue, int64_t depth, int64_t width,
                      const int64_t* slot, int64_t n_edges, const void* weights, const void* gates,
                      const int64_t* pre_idx, int64_t n_sources, const void* f) {
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(depth >= 1 && width >= 0 && n_edges >= 0, "bad ring sizes");
  DGB_REQUIRE(width > 0 || n_edges == 0, "Empty ring cannot receive edges");
  DGB_REQUIRE(!pre_idx || n_sources >= 1 || n_edges == 0, "n_sources must be >= 1 with pre_idx");
  DGB_REQUIRE(queue && slot, "queue and slot must be non-null");
  DGB_REQUIRE(n_edges == 0 || (weights && gates && f), "edge operands must be non-null");
  return DGB_OK;
}

extern "C" int dgb_two_tap_enqueue(int dtype, void* queue, int64_t depth, int64_t width,
                                   const int64_t* slot, int64_t n_edges, const void* weights,
                                   const void* gates, const int64_t* pre_idx, int64_t n_sources,
                                   const void* fraction, const int64_t* lower,
                                   const int64_t* upper, const int64_t* lower_ptr,
                                   const int64_t* lower_edge, const int64_t* upper_ptr,
                                   const int64_t* upper_edge, void* payload, void* stream) {
  clear_error();
  int rc = check_ring(dtype, queue, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, fraction);
  if (rc) return rc;
  if (width == 0) return DGB_OK;
  DGB_REQUIRE(lower_ptr && upper_ptr && (n_edges == 0 || (lower && upper && lower_edge &&
                                                          upper_edge)),
              "addresses and column plans must be non-null");
  DGB_DELAY_DISPATCH(dtype, two_tap_enqueue_kernel<T><<<blocks_for(width, 256), 256, 0,
                                                        as_stream(stream)>>>(
                                (T*)queue, depth, width, slot,
                                tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges),
                                (const T*)gates, lower, upper, lower_ptr, lower_edge, upper_ptr,
                                upper_edge, (T*)payload));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_three_tap_enqueue(int dtype, void* queue, int64_t depth, int64_t width,
                                     const int64_t* slot, int64_t n_edges, const void* weights,
                                     const void* gates, const int64_t* pre_idx,
                                     int64_t n_sources, const void* coeff,
                                     const int64_t* offsets, const int64_t* post_idx,
                                     const int64_t* post_ptr, const int64_t* post_edge,
                                     void* payload, void* stream) {
  clear_error();
  int rc = check_ring(dtype, queue, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, coeff);
  if (rc) return rc;
  if (width == 0) return DGB_OK;
  DGB_REQUIRE(post_ptr && (n_edges == 0 || (offsets && post_idx && post_edge)),
              "offsets, post_idx and the column plan must be non-null");
  DGB_DELAY_DISPATCH(dtype, three_tap_enqueue_kernel<T><<<blocks_for(width, 256), 256, 0,
                                                          as_stream(stream)>>>(
                                (T*)queue, depth, width, slot,
                                tap_edges<T>(weights, pre_idx, n_sources, coeff, n_edges),
                                (const T*)gates, offsets, post_idx, post_ptr, post_edge,
                                (T*)payload));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_two_tap_gather(int dtype, const void* ring, int64_t ring_size,
                                  const int64_t* offset, int64_t n_edges, const int64_t* lower,
                                  const int64_t* upper, void* lower_values, void* upper_values,
                                  void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(ring_size > 0, "Two-tap gather requires a nonempty ring");
  DGB_REQUIRE(n_edges >= 0, "bad edge count");
  if (n_edges == 0) return DGB_OK;
  DGB_REQUIRE(ring && offset && lower && upper && lower_values && upper_values,
              "pointers must be non-null");
  DGB_DELAY_DISPATCH(dtype, two_tap_gather_kernel<T><<<blocks_for(n_edges, 256), 256, 0,
                                                       as_stream(stream)>>>(
                                (const T*)ring, ring_size, offset, n_edges, lower, upper,
                                (T*)lower_values, (T*)upper_values));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_two_tap_vjp(int dtype, const void* ring, int64_t ring_size,
                               const int64_t* offset, int64_t n_edges, const void* weights,
                               const void* gates, const int64_t* pre_idx, int64_t n_sources,
                               const void* fraction, const int64_t* lower, const int64_t* upper,
                               const int64_t* source_ptr, const int64_t* source_edge,
                               void* grad_weights, void* grad_gates, void* grad_fraction,
                               void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(ring_size > 0, "Two-tap VJP requires a nonempty ring");
  DGB_REQUIRE(n_edges >= 0 && (!pre_idx || n_sources >= 0), "bad sizes");
  DGB_REQUIRE(ring && offset, "ring and offset must be non-null");
  const bool from_source = pre_idx != nullptr;
  if (n_edges == 0 && !(from_source && n_sources > 0)) return DGB_OK;
  DGB_REQUIRE(n_edges == 0 || (weights && gates && fraction && lower && upper && grad_weights &&
                                grad_fraction),
              "operands must be non-null");
  DGB_REQUIRE(grad_gates, "grad_gates must be non-null");
  DGB_REQUIRE(!from_source || (source_ptr && (n_edges == 0 || source_edge)),
              "the source plan must be non-null with pre_idx");
  cudaStream_t st = as_stream(stream);
  if (from_source) {
    DGB_DELAY_DISPATCH(dtype, two_tap_vjp_source_kernel<T><<<blocks_for(n_sources, 256), 256, 0,
                                                             st>>>(
                                  (const T*)ring, ring_size, offset,
                                  tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges),
                                  (const T*)gates, lower, upper, source_ptr, source_edge,
                                  (T*)grad_weights, (T*)grad_gates, (T*)grad_fraction));
  } else {
    DGB_DELAY_DISPATCH(dtype, two_tap_vjp_edge_kernel<T><<<blocks_for(n_edges, 256), 256, 0,
                                                           st>>>(
                                  (const T*)ring, ring_size, offset,
                                  tap_edges<T>(weights, nullptr, 0, fraction, n_edges),
                                  (const T*)gates, lower, upper, (T*)grad_weights,
                                  (T*)grad_gates, (T*)grad_fraction));
  }
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_three_tap_vjp(int dtype, const void* ring, int64_t depth, int64_t width,
                                 const int64_t* slot, int64_t n_edges, const void* weights,
                                 const void* gates, const void* coeff, const int64_t* offsets,
                                 const int64_t* post_idx, void* grad_weights, void* grad_gates,
                                 void* grad_coeff, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(depth >= 1 && width >= 0 && n_edges >= 0, "bad ring sizes");
  if (n_edges == 0) return DGB_OK;
  DGB_REQUIRE(width > 0, "Empty ring cannot receive edges");
  DGB_REQUIRE(ring && slot && weights && gates && coeff && offsets && post_idx && grad_weights &&
                  grad_gates && grad_coeff,
              "pointers must be non-null");
  DGB_DELAY_DISPATCH(dtype, three_tap_vjp_kernel<T><<<blocks_for(n_edges, 256), 256, 0,
                                                      as_stream(stream)>>>(
                                (const T*)ring, depth, width, slot,
                                tap_edges<T>(weights, nullptr, 0, coeff, n_edges),
                                (const T*)gates, offsets, post_idx, (T*)grad_weights,
                                (T*)grad_gates, (T*)grad_coeff));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

// Rollout launch: the ring in shared memory when a 128-column block's ring
// fits (opt-in size), else in place in HBM.
template <typename K>
static int roll_smem_setup(K kernel, size_t bytes) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 0;
  if (bytes > (size_t)optin) return 0;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) ==
         cudaSuccess;
}

template <typename T, bool ONE>
static void launch_rollout(T* ring, int64_t depth, int64_t width, const int64_t* slot,
                           int64_t n_steps, TapEdges<T> E, const T* gates, int64_t stride,
                           int64_t g_kc, const int64_t* ptr, const int64_t* edge,
                           const int32_t* lo, const int32_t* hi, int flags, T* payload,
                           cudaStream_t st) {
  const unsigned blocks = blocks_for(width, kRollBlock);
  if (flags & DGB_ROLLOUT_CHAINED) {
    if (flags & DGB_ROLLOUT_GATES_BY_SOURCE)
      two_tap_direct_kernel<T, true><<<blocks, kRollBlock, 0, st>>>(
          ring, depth, width, slot, n_steps, E, gates, stride, g_kc, ptr, edge, lo, hi, flags,
          payload);
    else
      two_tap_direct_kernel<T, false><<<blocks, kRollBlock, 0, st>>>(
          ring, depth, width, slot, n_steps, E, gates, stride, g_kc, ptr, edge, lo, hi, flags,
          payload);
    return;
  }
  const size_t bytes = (size_t)kRollBlock * depth * sizeof(T);
  if (roll_smem_setup(two_tap_rollout_kernel<T, true, ONE>, bytes))
    two_tap_rollout_kernel<T, true, ONE><<<blocks, kRollBlock, bytes, st>>>(
        ring, depth, width, slot, n_steps, E, gates, stride, ptr, edge, lo, hi, flags, payload);
  else
    two_tap_rollout_kernel<T, false, ONE><<<blocks, kRollBlock, 0, st>>>(
        ring, depth, width, slot, n_steps, E, gates, stride, ptr, edge, lo, hi, flags, payload);
}

template <typename T, bool PRE, bool ONE>
static void launch_rollout_vjp(T* ring, int64_t depth, int64_t width, const int64_t* slot,
                               int64_t n_steps, TapEdges<T> E, const T* gates, int64_t stride,
                               int64_t g_kc, const int64_t* ptr, const int64_t* edge,
                               const int32_t* lo, const int32_t* hi, int flags, const T* gpay,
                               int accumulate, T* dw, T* dgate, T* df, T* scratch,
                               cudaStream_t st) {
  const unsigned blocks = blocks_for(width, kRollBlock);
  if (flags & DGB_ROLLOUT_CHAINED) {
    if (flags & DGB_ROLLOUT_GATES_BY_SOURCE)
      two_tap_direct_vjp_kernel<T, true, PRE><<<blocks, kRollBlock, 0, st>>>(
          ring, depth, width, slot, n_steps, E, gates, stride, g_kc, ptr, edge, lo, hi, flags,
          gpay, accumulate, dw, dgate, df, scratch);
    else
      two_tap_direct_vjp_kernel<T, false, PRE><<<blocks, kRollBlock, 0, st>>>(
          ring, depth, width, slot, n_steps, E, gates, stride, g_kc, ptr, edge, lo, hi, flags,
          gpay, accumulate, dw, dgate, df, scratch);
    return;
  }
  const size_t bytes = (size_t)kRollBlock * depth * sizeof(T);
  if (roll_smem_setup(two_tap_rollout_vjp_kernel<T, true, PRE, ONE>, bytes))
    two_tap_rollout_vjp_kernel<T, true, PRE, ONE><<<blocks, kRollBlock, bytes, st>>>(
        ring, depth, width, slot, n_steps, E, gates, stride, ptr, edge, lo, hi, flags, gpay,
        accumulate, dw, dgate, df, scratch);
  else
    two_tap_rollout_vjp_kernel<T, false, PRE, ONE><<<blocks, kRollBlock, 0, st>>>(
        ring, depth, width, slot, n_steps, E, gates, stride, ptr, edge, lo, hi, flags, gpay,
        accumulate, dw, dgate, df, scratch);
}

static int check_rollout_flags(int32_t flags, const int64_t* pre_idx, int64_t n_steps,
                               int64_t gate_row) {
  if (flags & DGB_ROLLOUT_GATES_BY_SOURCE) {
    DGB_REQUIRE(pre_idx != nullptr && (flags & DGB_ROLLOUT_CHAINED),
                "gates by source need pre_idx and a chained plan");
    DGB_REQUIRE(gate_row >= n_steps, "gate_row must cover n_steps");
  }
  return DGB_OK;
}

extern "C" int dgb_gates_by_source(int dtype, int64_t n_steps, int64_t n_sources,
                                   const void* gates, void* gates_t, int64_t gate_row,
                                   void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n_steps >= 0 && n_sources >= 0 && gate_row >= n_steps, "bad sizes");
  if (n_steps == 0 || n_sources == 0) return DGB_OK;
  DGB_REQUIRE(gates && gates_t && gates != gates_t, "gates and gates_t must be distinct");
  DGB_REQUIRE((n_steps + 31) / 32 < (1ll << 31) && (n_sources + 31) / 32 < 65536,
              "too many steps or sources for one launch");
  const dim3 grid((unsigned)((n_steps + 31) / 32), (unsigned)((n_sources + 31) / 32));
  DGB_DELAY_DISPATCH(dtype, gates_by_source_kernel<T><<<grid, dim3(32, 8), 0,
                                                        as_stream(stream)>>>(
                                (const T*)gates, (T*)gates_t, n_steps, n_sources, gate_row));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_two_tap_rollout(int dtype, void* ring, int64_t depth, int64_t width,
                                   const int64_t* slot, int64_t n_steps, int64_t n_edges,
                                   const void* weights, const void* gates, int64_t gate_row,
                                   const int64_t* pre_idx, int64_t n_sources,
                                   const void* fraction, const int64_t* col_ptr,
                                   const int64_t* col_edge, const int32_t* lower_row,
                                   const int32_t* upper_row, int32_t flags, void* payload,
                                   void* stream) {
  clear_error();
  int rc = check_ring(dtype, ring, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, fraction);
  if (rc) return rc;
  DGB_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (width == 0 || n_steps == 0) return DGB_OK;
  DGB_REQUIRE(col_ptr && (n_edges == 0 || (col_edge && lower_row && upper_row)),
              "the rollout plan must be non-null");
  DGB_REQUIRE(depth * width < (1ll << 31) && n_edges < (1ll << 31) &&
                  n_sources < (1ll << 31),
              "rollout ring size, edge and source counts must be below 2^31");
  rc = check_rollout_flags(flags, pre_idx, n_steps, gate_row);
  if (rc) return rc;
  const int64_t stride = pre_idx ? n_sources : n_edges;
  const bool one = (flags & DGB_ROLLOUT_ONE_EDGE) != 0;
  cudaStream_t st = as_stream(stream);
  DGB_DELAY_DISPATCH(dtype, {
    const TapEdges<T> E = tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges);
    if (one)
      launch_rollout<T, true>((T*)ring, depth, width, slot, n_steps, E, (const T*)gates, stride,
                              gate_row, col_ptr, col_edge, lower_row, upper_row, flags,
                              (T*)payload, st);
    else
      launch_rollout<T, false>((T*)ring, depth, width, slot, n_steps, E, (const T*)gates,
                               stride, gate_row, col_ptr, col_edge, lower_row, upper_row, flags,
                               (T*)payload, st);
  });
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_two_tap_rollout_vjp(int dtype, void* grad_ring, int64_t depth, int64_t width,
                                       const int64_t* slot, int64_t n_steps, int64_t n_edges,
                                       const void* weights, const void* gates, int64_t gate_row,
                                       const int64_t* pre_idx, int64_t n_sources,
                                       const void* fraction, const int64_t* col_ptr,
                                       const int64_t* col_edge, const int32_t* lower_row,
                                       const int32_t* upper_row, int32_t flags,
                                       const int64_t* source_ptr, const int64_t* source_pos,
                                       const void* grad_payload, int32_t accumulate,
                                       void* grad_weights, void* grad_gates, void* grad_fraction,
                                       void* edge_scratch, void* stream) {
  clear_error();
  int rc = check_ring(dtype, grad_ring, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, fraction);
  if (rc) return rc;
  DGB_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (width == 0 || n_steps == 0) return DGB_OK;
  DGB_REQUIRE(col_ptr && (n_edges == 0 || (col_edge && lower_row && upper_row)),
              "the rollout plan must be non-null");
  DGB_REQUIRE(depth * width < (1ll << 31) && n_edges < (1ll << 31) &&
                  n_sources < (1ll << 31),
              "rollout ring size, edge and source counts must be below 2^31");
  rc = check_rollout_flags(flags, pre_idx, n_steps, gate_row);
  if (rc) return rc;
  DGB_REQUIRE(n_edges == 0 || (grad_weights && grad_fraction), "gradients must be non-null");
  DGB_REQUIRE(grad_gates || (pre_idx ? n_sources : n_edges) == 0, "grad_gates must be non-null");
  const bool pre = pre_idx != nullptr;
  DGB_REQUIRE(!pre || (source_ptr && (n_edges == 0 || (source_pos && edge_scratch))),
              "the source plan and edge_scratch must be non-null with pre_idx");
  const int64_t stride = pre ? n_sources : n_edges;
  const bool one = (flags & DGB_ROLLOUT_ONE_EDGE) != 0;
  cudaStream_t st = as_stream(stream);
  DGB_DELAY_DISPATCH(dtype, {
    const TapEdges<T> E = tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges);
    T* R = (T*)grad_ring;
    T* gw = (T*)grad_weights;
    T* gf = (T*)grad_fraction;
    const T* gg = (const T*)gates;
    const T* gp = (const T*)grad_payload;
    if (pre && one)
      launch_rollout_vjp<T, true, true>(R, depth, width, slot, n_steps, E, gg, stride, gate_row,
                                        col_ptr, col_edge, lower_row, upper_row, flags, gp,
                                        accumulate, gw, nullptr, gf, (T*)edge_scratch, st);
    else if (pre)
      launch_rollout_vjp<T, true, false>(R, depth, width, slot, n_steps, E, gg, stride,
                                         gate_row, col_ptr, col_edge, lower_row, upper_row,
                                         flags, gp, accumulate, gw, nullptr, gf,
                                         (T*)edge_scratch, st);
    else if (one)
      launch_rollout_vjp<T, false, true>(R, depth, width, slot, n_steps, E, gg, stride,
                                         gate_row, col_ptr, col_edge, lower_row, upper_row,
                                         flags, gp, accumulate, gw, (T*)grad_gates, gf, nullptr,
                                         st);
    else
      launch_rollout_vjp<T, false, false>(R, depth, width, slot, n_steps, E, gg, stride,
                                          gate_row, col_ptr, col_edge, lower_row, upper_row,
                                          flags, gp, accumulate, gw, (T*)grad_gates, gf, nullptr,
                                          st);
  });
  DGB_LAUNCH_CHECK();
  if (pre && n_sources > 0) {
    const int64_t kc = (n_steps + 7) & ~int64_t(7);
    DGB_DELAY_DISPATCH(dtype, source_sum_kernel<T><<<blocks_for(n_steps * n_sources, 256), 256,
                                                     0, st>>>(
                                  (const T*)edge_scratch, n_steps, kc, n_edges, n_sources,
                                  source_ptr, source_pos, (T*)grad_gates));
    DGB_LAUNCH_CHECK();
  }
  return DGB_OK;
}

extern "C" int dgb_delay_status(void* stream) {
  clear_error();
  DGB_CUDA_CHECK(cudaStreamSynchronize(as_stream(stream)));
  int h = 0;
  DGB_CUDA_CHECK(cudaMemcpyFromSymbol(&h, g_delay_err, sizeof(int)));
  if (h) {
    const int zero = 0;
    DGB_CUDA_CHECK(cudaMemcpyToSymbol(g_delay_err, &zero, sizeof(int)));
  }
  return h;
}
