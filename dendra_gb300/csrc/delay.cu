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
//   dgb_two_tap_window(_vjp) many steps of the above in one launch (rollouts)
//
// Determinism: the reference's CPU op adds every edge's lower-tap value in
// edge order, then every upper-tap value in edge order, into a ring it owns
// (its CUDA path scatters with atomics).  Here one thread owns one ring column
// for the whole launch and walks that column's edges in ascending order, so
// each ring value sees exactly the reference's sequence of additions: results
// are bit-identical, with no floating-point atomics.  Every product and sum is
// rounded on its own (no FMA contraction), as the CPU op computes them.
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

// n_steps enqueue steps, thread = column (consistent plan: both taps of an
// edge in its column).  Columns never touch each other, so no step needs a
// grid-wide barrier; the addresses are checked against the column once.
template <typename T>
__global__ void __launch_bounds__(256)
    two_tap_window_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                          const int64_t* __restrict__ slot_ptr, int64_t n_steps, TapEdges<T> E,
                          const T* __restrict__ gates, int64_t gate_stride,
                          const int64_t* __restrict__ lower, const int64_t* __restrict__ upper,
                          const int64_t* __restrict__ ptr, const int64_t* __restrict__ edge,
                          T* __restrict__ payload) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= width) return;
  int64_t slot = slot_ptr[0];
  if (slot < 0 || slot >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  const int64_t size = depth * width;
  {  // the column's addresses, once
    int64_t j0, j1;
    if (!column_range(ptr, col, E.n_edges, j0, j1)) return;
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t e = edge[j];
      if ((uint64_t)e >= (uint64_t)E.n_edges || (uint64_t)lower[e] >= (uint64_t)size ||
          (uint64_t)upper[e] >= (uint64_t)size || lower[e] % width != col ||
          upper[e] % width != col) {
        delay_fail(DGB_DELAY_ERR_PLAN);
        return;
      }
    }
  }
  for (int64_t k = 0; k < n_steps; ++k) {
    const RingPos P = ring_pos(slot, width, size);
    const T* g = gates + k * gate_stride;
    if (payload) payload[k * width + col] = ring[P.start + col];
    ring[P.start + col] = T(0);
    column_taps<T, false, false>(ring, P, width, col, E, g, lower, ptr, edge);
    column_taps<T, true, false>(ring, P, width, col, E, g, upper, ptr, edge);
    if (++slot == depth) slot = 0;
  }
}

// Reverse of two_tap_window_kernel, thread = column, steps newest first.
template <typename T, bool PRE>
__global__ void __launch_bounds__(256)
    two_tap_window_vjp_kernel(T* __restrict__ R, int64_t depth, int64_t width,
                              const int64_t* __restrict__ slot_ptr, int64_t n_steps,
                              TapEdges<T> E, const T* __restrict__ gates, int64_t gate_stride,
                              const int64_t* __restrict__ lower,
                              const int64_t* __restrict__ upper,
                              const int64_t* __restrict__ ptr, const int64_t* __restrict__ edge,
                              const T* __restrict__ gpay, int accumulate, T* __restrict__ dw,
                              T* __restrict__ dgate, T* __restrict__ df,
                              T* __restrict__ scratch) {
  const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= width) return;
  const int64_t slot0 = slot_ptr[0];
  if (slot0 < 0 || slot0 >= depth) {
    if (col == 0) delay_fail(DGB_DELAY_ERR_SLOT);
    return;
  }
  const int64_t size = depth * width;
  int64_t j0, j1;
  if (!column_range(ptr, col, E.n_edges, j0, j1)) return;
  for (int64_t j = j0; j < j1; ++j) {
    const int64_t e = edge[j];
    if ((uint64_t)e >= (uint64_t)E.n_edges || (uint64_t)lower[e] >= (uint64_t)size ||
        (uint64_t)upper[e] >= (uint64_t)size || lower[e] % width != col ||
        upper[e] % width != col ||
        (PRE && (uint64_t)E.pre[e] >= (uint64_t)E.n_src)) {
      delay_fail(DGB_DELAY_ERR_PLAN);
      return;
    }
  }
  int64_t slot = (slot0 + n_steps - 1) % depth;
  for (int64_t k = n_steps - 1; k >= 0; --k) {
    const RingPos P = ring_pos(slot, width, size);
    const T* g = gates + k * gate_stride;
    const bool store = (k == n_steps - 1) && !accumulate;
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t e = edge[j];
      const int64_t bl = lower[e], bu = upper[e];
      const T lo = R[bl < P.tail ? P.start + bl : bl - P.tail];
      const T hi = R[bu < P.tail ? P.start + bu : bu - P.tail];
      const int64_t s = PRE ? E.pre[e] : e;
      T dwk, dgk, dfk;
      edge_vjp(lo, hi, E.w[e], g[s], E.f[e], dwk, dgk, dfk);
      dw[e] = store ? dwk : add_rn(dw[e], dwk);
      df[e] = store ? dfk : add_rn(df[e], dfk);
      if (PRE)
        scratch[k * E.n_edges + e] = dgk;
      else
        dgate[k * gate_stride + e] = dgk;
    }
    R[P.start + col] = gpay ? gpay[k * width + col] : T(0);
    slot = slot == 0 ? depth - 1 : slot - 1;
  }
}

// dgate[k][s] = sum of scratch[k][e] over the source's edges, ascending, from +0.
template <typename T>
__global__ void source_sum_kernel(const T* __restrict__ scratch, int64_t n_steps,
                                  int64_t n_edges, int64_t n_src,
                                  const int64_t* __restrict__ src_ptr,
                                  const int64_t* __restrict__ src_edge, T* __restrict__ dgate) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_steps * n_src) return;
  const int64_t k = i / n_src, s = i - k * n_src;
  T acc = T(0);
  int64_t j0, j1;
  if (column_range(src_ptr, s, n_edges, j0, j1)) {
    for (int64_t j = j0; j < j1; ++j) {
      const int64_t e = src_edge[j];
      if ((uint64_t)e >= (uint64_t)n_edges) {
        delay_fail(DGB_DELAY_ERR_PLAN);
        continue;
      }
      acc = add_rn(acc, scratch[k * n_edges + e]);
    }
  }
  dgate[i] = acc;
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

extern "C" int dgb_two_tap_window(int dtype, void* queue, int64_t depth, int64_t width,
                                  const int64_t* slot, int64_t n_steps, int64_t n_edges,
                                  const void* weights, const void* gates,
                                  const int64_t* pre_idx, int64_t n_sources,
                                  const void* fraction, const int64_t* lower,
                                  const int64_t* upper, const int64_t* col_ptr,
                                  const int64_t* col_edge, void* payload, void* stream) {
  clear_error();
  int rc = check_ring(dtype, queue, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, fraction);
  if (rc) return rc;
  DGB_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (width == 0 || n_steps == 0) return DGB_OK;
  DGB_REQUIRE(col_ptr && (n_edges == 0 || (lower && upper && col_edge)),
              "addresses and the column plan must be non-null");
  const int64_t stride = pre_idx ? n_sources : n_edges;
  DGB_DELAY_DISPATCH(dtype, two_tap_window_kernel<T><<<blocks_for(width, 256), 256, 0,
                                                       as_stream(stream)>>>(
                                (T*)queue, depth, width, slot, n_steps,
                                tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges),
                                (const T*)gates, stride, lower, upper, col_ptr, col_edge,
                                (T*)payload));
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_two_tap_window_vjp(int dtype, void* grad_queue, int64_t depth, int64_t width,
                                      const int64_t* slot, int64_t n_steps, int64_t n_edges,
                                      const void* weights, const void* gates,
                                      const int64_t* pre_idx, int64_t n_sources,
                                      const void* fraction, const int64_t* lower,
                                      const int64_t* upper, const int64_t* col_ptr,
                                      const int64_t* col_edge, const int64_t* source_ptr,
                                      const int64_t* source_edge, const void* grad_payload,
                                      int32_t accumulate, void* grad_weights, void* grad_gates,
                                      void* grad_fraction, void* edge_scratch, void* stream) {
  clear_error();
  int rc = check_ring(dtype, grad_queue, depth, width, slot, n_edges, weights, gates, pre_idx,
                      n_sources, fraction);
  if (rc) return rc;
  DGB_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  if (width == 0 || n_steps == 0) return DGB_OK;
  DGB_REQUIRE(col_ptr && (n_edges == 0 || (lower && upper && col_edge)),
              "addresses and the column plan must be non-null");
  DGB_REQUIRE(n_edges == 0 || (grad_weights && grad_fraction), "gradients must be non-null");
  DGB_REQUIRE(grad_gates || (pre_idx ? n_sources : n_edges) == 0, "grad_gates must be non-null");
  const bool pre = pre_idx != nullptr;
  DGB_REQUIRE(!pre || (source_ptr && (n_edges == 0 || (source_edge && edge_scratch))),
              "the source plan and edge_scratch must be non-null with pre_idx");
  const int64_t stride = pre ? n_sources : n_edges;
  cudaStream_t st = as_stream(stream);
  if (pre) {
    DGB_DELAY_DISPATCH(dtype, two_tap_window_vjp_kernel<T, true><<<blocks_for(width, 256), 256,
                                                                   0, st>>>(
                                  (T*)grad_queue, depth, width, slot, n_steps,
                                  tap_edges<T>(weights, pre_idx, n_sources, fraction, n_edges),
                                  (const T*)gates, stride, lower, upper, col_ptr, col_edge,
                                  (const T*)grad_payload, accumulate, (T*)grad_weights, nullptr,
                                  (T*)grad_fraction, (T*)edge_scratch));
    DGB_LAUNCH_CHECK();
    if (n_sources > 0)
      DGB_DELAY_DISPATCH(dtype, source_sum_kernel<T><<<blocks_for(n_steps * n_sources, 256), 256,
                                                       0, st>>>(
                                    (const T*)edge_scratch, n_steps, n_edges, n_sources,
                                    source_ptr, source_edge, (T*)grad_gates));
  } else {
    DGB_DELAY_DISPATCH(dtype, two_tap_window_vjp_kernel<T, false><<<blocks_for(width, 256), 256,
                                                                    0, st>>>(
                                  (T*)grad_queue, depth, width, slot, n_steps,
                                  tap_edges<T>(weights, nullptr, 0, fraction, n_edges),
                                  (const T*)gates, stride, lower, upper, col_ptr, col_edge,
                                  (const T*)grad_payload, accumulate, (T*)grad_weights,
                                  (T*)grad_gates, (T*)grad_fraction, nullptr));
  }
  DGB_LAUNCH_CHECK();
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
