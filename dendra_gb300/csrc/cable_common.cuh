// Pieces shared by the forward cable kernels (cable_impl.cuh) and their
// adjoint (cable_adjoint_impl.cuh): the typed argument block, the
// shared-memory plane addressing and the state tape row walk.
#pragma once
#include "cable_decl.cuh"

namespace dgb {

constexpr int kCableWarps = 4;     // default warps (cables in flight) per block
constexpr int kCableMaxWarps = 4;  // largest accepted warps_per_block
// warps of one cable in the split-gate run: one per SM sub-partition (one
// warp alone leaves most of an SM's arithmetic rate unused)
constexpr int kSplitWarps = 4;

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
  const int32_t* spk_idx2;
  int32_t* spk_below2;
  int stop_on_spike;
  int32_t* counter;
  T* tape;         // (n_steps + 1, 4, n_comp) state tape, nullptr = none
  int64_t n_comp;  // total compartments (tape plane stride)
  int wpb;         // requested warps per block (0 = default)
  int split;       // DGB_CABLE_SPLIT_GATES: one cable per CTA, gates on kSplitWarps warps
  int n_rast, rast_cap;
  const int32_t* rast_idx;
  int32_t *rast_below, *rast_count;
  int64_t* rast_steps;
  int lanes_mode, n_lanes32, n_lanes16;
  T* trace_all;
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
  t.spk_idx2 = a->spk_idx2;
  t.spk_below2 = a->spk_below2;
  t.stop_on_spike = (a->flags & DGB_CABLE_STOP_ON_SPIKE) ? 1 : 0;
  t.counter = a->scratch;
  t.tape = nullptr;
  t.n_comp = a->n_comp;
  t.wpb = a->warps_per_block;
  t.split = (a->flags & DGB_CABLE_SPLIT_GATES) ? 1 : 0;
  t.n_rast = a->rast_idx ? a->n_rast : 0;
  t.rast_cap = a->rast_cap;
  t.rast_idx = a->rast_idx;
  t.rast_below = a->rast_below;
  t.rast_count = a->rast_count;
  t.rast_steps = a->rast_steps;
  t.lanes_mode = a->lanes_mode;
  t.n_lanes32 = a->n_lanes32;
  t.n_lanes16 = a->n_lanes16;
  t.trace_all = (T*)a->trace_all;
  return t;
}

// error bits of scratch[1]
constexpr int kErrChunk = 1;

// Shared-memory planes of one warp (one cable).  Plane q holds row j of lane r
// at [(q * ch + j) * 32 + r]: the 32 lanes touch 32 consecutive words, so
// every access is bank-conflict free for any chunk size ch.  Planes 0..6 are
// always present; the rest only when a coefficient varies along the cable.
enum { P_V = 0, P_M, P_H, P_N, P_AP, P_CP, P_DP, P_FIXED };

struct PlaneLayout {
  int n_planes;
  int q_geo;   // g_right, g_left, scale planes (-1: uniform per cable)
  int q_fld;   // extracellular lead field (-1: no ve)
  int q_chan;  // gnabar, gkbar, gl, el planes (-1: uniform per cable)
};

__host__ __device__ inline PlaneLayout plane_layout(bool geo_planes, bool field, bool chan_planes) {
  PlaneLayout L;
  int q = P_FIXED;
  L.q_geo = geo_planes ? q : -1;
  q += geo_planes ? 3 : 0;
  L.q_fld = field ? q : -1;
  q += field ? 1 : 0;
  L.q_chan = chan_planes ? q : -1;
  q += chan_planes ? 4 : 0;
  L.n_planes = q;
  return L;
}

template <typename T>
struct Planes {
  T* base;
  int ch;
  __device__ __forceinline__ T& at(int q, int j, int r) const {
    return base[(q * ch + j) * 32 + r];
  }
};

// Division policy: exact IEEE division, or the approximate reciprocal in the
// float32 fast-math variant.
template <typename T, bool FAST>
__device__ __forceinline__ T dv(T a, T b) {
  if constexpr (FAST) {
    return __fdividef(a, b);
  } else {
    return a / b;
  }
}

// Pivot reciprocal and division of the persistent run's solve: dv's policy in
// float32; in float64 the Newton-refined reciprocal (rcp_nr64), within about
// an ulp of the correctly rounded quotient (pivots of the diagonally dominant
// cable systems are normal and far from zero).
template <typename T, bool FAST>
__device__ __forceinline__ T srcp(T b) {
  if constexpr (sizeof(T) == 8) {
    return rcp_nr64(b);
  } else {
    return dv<T, FAST>(T(1), b);
  }
}
template <typename T, bool FAST>
__device__ __forceinline__ T sdv(T a, T b) {
  if constexpr (sizeof(T) == 8) {
    return a * rcp_nr64(b);
  } else {
    return dv<T, FAST>(a, b);
  }
}

// Row i of a cable lives in lane i / ch, slot i % ch of the planes.  The
// tape stores rows contiguously, so lane r visits rows r, r + 32, ... with
// (lane, slot) advanced incrementally: 32 = (32 / ch) * ch + 32 % ch.
struct RowWalk {
  int i, lane, j;
  int dl, dj, ch;
  __device__ __forceinline__ RowWalk(int r, int ch_) : i(r), lane(r / ch_), j(r % ch_),
      dl(32 / ch_), dj(32 % ch_), ch(ch_) {}
  __device__ __forceinline__ void next() {
    i += 32;
    lane += dl;
    j += dj;
    if (j >= ch) {
      j -= ch;
      ++lane;
    }
  }
};

// Warps per block for a persistent launch: the requested count (default
// kCableWarps), halved while the block's shared memory exceeds 227 KB.
// Returns 0 when even one warp does not fit.
inline int persistent_wpb(int requested, size_t per_warp) {
  int wpb = requested > 0 ? requested : kCableWarps;
  while (wpb > 1 && (size_t)wpb * per_warp > 227 * 1024) wpb >>= 1;
  return (size_t)wpb * per_warp <= 227 * 1024 ? wpb : 0;
}

// Copy planes q_v, q_m, q_h, q_n of one cable to dst[q * N + i] (coalesced).
template <typename T>
__device__ __forceinline__ void tape_store(const Planes<T>& P, int K, int ch, int q_v, int q_m,
                                           int q_h, int q_n, T* dst, int64_t N) {
  for (RowWalk w(threadIdx.x & 31, ch); w.i < K; w.next()) {
    dst[w.i] = P.at(q_v, w.j, w.lane);
    dst[N + w.i] = P.at(q_m, w.j, w.lane);
    dst[2 * N + w.i] = P.at(q_h, w.j, w.lane);
    dst[3 * N + w.i] = P.at(q_n, w.j, w.lane);
  }
}

}  // namespace dgb
