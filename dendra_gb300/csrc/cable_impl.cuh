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
#include "cable_common.cuh"
#include "chunk_solve.cuh"

namespace dgb {

// One cable, all steps, one warp.  ch = rows per lane (runtime), rows of lane
// r are i = r*ch + j.  Rows with i >= K are identity rows with zero
// coefficients and zero state.
template <typename T, bool FAST, bool TAPE>
__device__ void run_cable(const CableArgsT<T>& A, int cable, T* smw, int ch,
                          const PlaneLayout& lay) {
  const int r = threadIdx.x & 31;
  const int64_t off = A.cable_ptr[cable];
  const int K = (int)(A.cable_ptr[cable + 1] - off);
  Planes<T> P{smw, ch};
  const bool use_ve = lay.q_fld >= 0;

  for (int j = 0; j < ch; ++j) {
    const int i = r * ch + j;
    const bool in = i < K;
    const int64_t g = off + i;
    P.at(P_V, j, r) = in ? A.v[g] : T(0);
    P.at(P_M, j, r) = in ? A.m[g] : T(0);
    P.at(P_H, j, r) = in ? A.h[g] : T(0);
    P.at(P_N, j, r) = in ? A.n[g] : T(0);
    if (lay.q_geo >= 0) {
      P.at(lay.q_geo + 0, j, r) = in ? A.g_right[g] : T(0);
      P.at(lay.q_geo + 1, j, r) = in ? A.g_left[g] : T(0);
      P.at(lay.q_geo + 2, j, r) = in ? A.scale[g] : T(0);
    }
    if (use_ve) P.at(lay.q_fld, j, r) = in ? A.field[g] : T(0);
    if (lay.q_chan >= 0) {
      P.at(lay.q_chan + 0, j, r) = in ? A.gnabar[g] : T(0);
      P.at(lay.q_chan + 1, j, r) = in ? A.gkbar[g] : T(0);
      P.at(lay.q_chan + 2, j, r) = in ? A.gl[g] : T(0);
      P.at(lay.q_chan + 3, j, r) = in ? A.el[g] : T(0);
    }
  }
  // uniform coefficients: the cable's values, identical on every compartment
  // (interior edges for g_right / g_left), so reading them once is exact
  T gna_c = T(0), gk_c = T(0), gl_c = T(0), el_c = T(0);
  if (lay.q_chan < 0) {
    gna_c = A.gnabar[off];
    gk_c = A.gkbar[off];
    gl_c = A.gl[off];
    el_c = A.el[off];
  }
  T gr_c = T(0), glf_c = T(0), sc_c = T(0);
  if (lay.q_geo < 0) {
    gr_c = K > 1 ? A.g_right[off] : T(0);
    glf_c = K > 1 ? A.g_left[off + 1] : T(0);
    sc_c = A.scale[off];
  }
  __syncwarp();

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
  const int rec_i = (A.rec_idx && A.trace) ? A.rec_idx[cable] : -1;
  const int spk_i = A.spk_idx ? A.spk_idx[cable] : -1;
  const int spk_i2 = A.spk_idx2 ? A.spk_idx2[cable] : -1;
  // the count and first step live in lane 0; each detection compartment keeps
  // its latch in the lane that owns it
  int below = 1, below2 = 1, count = 0, first = -1;
  if (spk_i >= 0 && r == 0) {
    count = A.spk_count[cable];
    first = A.spk_first[cable];
  }
  if (spk_i >= 0 && r == spk_i / ch) below = A.spk_below[cable];
  if (spk_i2 >= 0 && r == spk_i2 / ch) below2 = A.spk_below2[cable];
  if (rec_i >= 0 && r == rec_i / ch) A.trace[(int64_t)cable * A.n_rec] = P.at(P_V, rec_i % ch, r);
  if constexpr (TAPE) {
    if (A.tape) {
      tape_store<T>(P, K, ch, P_V, P_M, P_H, P_N, A.tape + off, A.n_comp);
      __syncwarp();
    }
  }

  const T dt = A.dt, dt_s = A.dt_s, q10 = A.q10, ena = A.ena, ek = A.ek;
  const int last = ch - 1;
  for (int s = 0; s < A.n_steps; ++s) {
    const T t = (T)(A.t0_ms + (double)(A.step0 + s) * A.dt_ms_d);
    const T Ive = use_ve ? rect_pulse<T>(t, ve_amp, ve_delay, ve_pw) : T(0);
    const T Iin = (in_i >= 0) ? rect_pulse<T>(t, in_amp, in_delay, in_pw) : T(0);
    const bool ve_on = Ive != T(0);  // per cable: warp-uniform

    // ---- phase A: gates, membrane frame, row assembly fused with the
    //      forward sweep of the chunk elimination (chunk_solve.cuh, step 1)
    T As = T(0), Bs = T(1), Cs = T(0), Ds = T(0);
    T ap = T(0), cp = T(0), dp = T(0);
    T v_prev = (r > 0) ? P.at(P_V, last, r - 1) : T(0);
    T vj = P.at(P_V, 0, r);
    T f_prev = T(0), fj = T(0);
    if (ve_on) {
      f_prev = (r > 0) ? P.at(lay.q_fld, last, r - 1) : T(0);
      fj = P.at(lay.q_fld, 0, r);
    }
    for (int j = 0; j < ch; ++j) {
      const T v_next = (j < last) ? P.at(P_V, j + 1, r) : ((r < 31) ? P.at(P_V, 0, r + 1) : T(0));
      T m = P.at(P_M, j, r), h = P.at(P_H, j, r), n = P.at(P_N, j, r);
      if constexpr (FAST) {
        hh_gates_fast(vj, q10, dt, m, h, n);
      } else {
        hh_gates<T>(vj, q10, dt, m, h, n);
      }
      P.at(P_M, j, r) = m;
      P.at(P_H, j, r) = h;
      P.at(P_N, j, r) = n;
      T G, J;
      if (lay.q_chan >= 0) {
        hh_affine<T>(m, h, n, P.at(lay.q_chan, j, r), P.at(lay.q_chan + 1, j, r),
                     P.at(lay.q_chan + 2, j, r), P.at(lay.q_chan + 3, j, r), ena, ek, G, J);
      } else {
        hh_affine<T>(m, h, n, gna_c, gk_c, gl_c, el_c, ena, ek, G, J);
      }
      T scl, gr, glf;
      if (lay.q_geo >= 0) {
        gr = P.at(lay.q_geo, j, r);
        glf = P.at(lay.q_geo + 1, j, r);
        scl = P.at(lay.q_geo + 2, j, r);
      } else {
        const int i = r * ch + j;
        gr = i < K - 1 ? gr_c : T(0);
        glf = (i >= 1 && i < K) ? glf_c : T(0);
        scl = i < K ? sc_c : T(0);
      }
      // row i couples to i-1 through glf and to i+1 through gr; at a cable
      // end (or past it) that coefficient is exactly zero
      T fn = (J - mul_rn(G, vj)) * scl;
      fn = fn + (mul_rn(gr, v_next - vj) - mul_rn(glf, vj - v_prev));
      if (ve_on) {
        const T f_next = (j < last) ? P.at(lay.q_fld, j + 1, r)
                                    : ((r < 31) ? P.at(lay.q_fld, 0, r + 1) : T(0));
        // ve values are rounded before they are differenced, as the reference
        // materialises its ve tape; a fused field*I - ve would skip that rounding
        const T ve_l = mul_rn(f_prev, Ive), ve_c = mul_rn(fj, Ive), ve_r = mul_rn(f_next, Ive);
        fn = fn + (mul_rn(gr, ve_r - ve_c) - mul_rn(glf, ve_c - ve_l));
        f_prev = fj;
        fj = f_next;
      }
      if (r * ch + j == in_i) fn = fn + Iin * in_cm;
      const T b = T(1) - dt_s * ((-gr + -glf) - mul_rn(G, scl));
      const T a = -dt_s * glf;
      const T c = -dt_s * gr;
      const T d = dt_s * fn;
      if (j == 0) {
        As = a;
        Bs = b;
        Cs = c;
        Ds = d;
      } else if (j == 1) {
        const T rinv = dv<T, FAST>(T(1), b);
        ap = a * rinv;
        cp = c * rinv;
        dp = d * rinv;
      } else {
        const T rinv = dv<T, FAST>(T(1), b - a * cp);
        ap = -a * ap * rinv;
        dp = (d - a * dp) * rinv;
        cp = c * rinv;
      }
      if (j >= 1) {
        P.at(P_AP, j, r) = ap;
        P.at(P_CP, j, r) = cp;
        P.at(P_DP, j, r) = dp;
      }
      v_prev = vj;
      vj = v_next;
    }
    // ---- phase B: backward sweep (rows ch-3 .. 1) and the reduced row
    T al, be, ga, de, Ae = ap, Ce = cp, De = dp;
    if (ch == 1) {
      al = As;
      be = Bs;
      ga = Cs;
      de = Ds;
    } else {
      T a2 = ap, c2 = cp, d2 = dp;  // row ch-2 after the loop below
      if (ch >= 3) {
        a2 = P.at(P_AP, ch - 2, r);
        c2 = P.at(P_CP, ch - 2, r);
        d2 = P.at(P_DP, ch - 2, r);
        for (int j = ch - 3; j >= 1; --j) {
          const T cj = P.at(P_CP, j, r);
          d2 = P.at(P_DP, j, r) - cj * d2;
          a2 = P.at(P_AP, j, r) - cj * a2;
          c2 = -cj * c2;
          P.at(P_AP, j, r) = a2;
          P.at(P_CP, j, r) = c2;
          P.at(P_DP, j, r) = d2;
        }
      }
      T Bs2 = Bs, Cs2 = Cs, Ds2 = Ds;
      if (ch >= 3) {
        Bs2 = Bs - Cs * a2;
        Cs2 = -Cs * c2;
        Ds2 = Ds - Cs * d2;
      }
      T Ae_l = shfl_up<T>(Ae, 1, 32), Ce_l = shfl_up<T>(Ce, 1, 32), De_l = shfl_up<T>(De, 1, 32);
      if (r == 0) {
        Ae_l = T(0);
        Ce_l = T(0);
        De_l = T(0);
      }
      al = -As * Ae_l;
      be = Bs2 - As * Ce_l - Cs2 * Ae;
      ga = -Cs2 * Ce;
      de = Ds2 - As * De_l - Cs2 * De;
    }
    // ---- phase C: PCR across the 32 lanes, then back-substitution
#pragma unroll
    for (int sh = 1; sh < 32; sh <<= 1) {
      T al_l = shfl_up<T>(al, sh, 32), be_l = shfl_up<T>(be, sh, 32);
      T ga_l = shfl_up<T>(ga, sh, 32), de_l = shfl_up<T>(de, sh, 32);
      T al_r = shfl_down<T>(al, sh, 32), be_r = shfl_down<T>(be, sh, 32);
      T ga_r = shfl_down<T>(ga, sh, 32), de_r = shfl_down<T>(de, sh, 32);
      const bool hl = r >= sh;
      const bool hr = r + sh < 32;
      T k1 = hl ? dv<T, FAST>(al, be_l) : T(0);
      T k2 = hr ? dv<T, FAST>(ga, be_r) : T(0);
      T al_n = hl ? -k1 * al_l : T(0);
      T ga_n = hr ? -k2 * ga_r : T(0);
      be = be - (hl ? k1 * ga_l : T(0)) - (hr ? k2 * al_r : T(0));
      de = de - (hl ? k1 * de_l : T(0)) - (hr ? k2 * de_r : T(0));
      al = al_n;
      ga = ga_n;
    }
    const T xs = dv<T, FAST>(de, be);
    T xe = xs;
    if (ch > 1) {
      T xs_next = shfl_down<T>(xs, 1, 32);
      if (r == 31) xs_next = T(0);
      xe = De - Ae * xs - Ce * xs_next;
    }
    __syncwarp();  // every lane has read its neighbours' v for this step
    P.at(P_V, 0, r) = P.at(P_V, 0, r) + xs;
    for (int j = 1; j < last; ++j)
      P.at(P_V, j, r) = P.at(P_V, j, r) + (P.at(P_DP, j, r) - P.at(P_AP, j, r) * xs -
                                           P.at(P_CP, j, r) * xe);
    if (ch > 1) P.at(P_V, last, r) = P.at(P_V, last, r) + xe;
    if (spk_i >= 0) {
      int edge = 0;
      if (r == spk_i / ch) {
        const int above = P.at(P_V, spk_i % ch, r) >= A.spk_thr;
        edge = above && below;
        below = !above;
      }
      int edge2 = 0;
      if (spk_i2 >= 0 && r == spk_i2 / ch) {
        const int above = P.at(P_V, spk_i2 % ch, r) >= A.spk_thr;
        edge2 = above && below2;
        below2 = !above;
      }
      const unsigned fired = __ballot_sync(0xffffffffu, edge || edge2);
      if (fired && r == 0) {
        if (count == 0) first = s + 1;
        count += 1;
      }
      if (A.stop_on_spike && fired) {
        if (rec_i >= 0 && r == rec_i / ch && ((s + 1) % A.rec_every) == 0)
          A.trace[(int64_t)cable * A.n_rec + (s + 1) / A.rec_every] = P.at(P_V, rec_i % ch, r);
        __syncwarp();
        break;
      }
    }
    if (rec_i >= 0 && r == rec_i / ch && ((s + 1) % A.rec_every) == 0)
      A.trace[(int64_t)cable * A.n_rec + (s + 1) / A.rec_every] = P.at(P_V, rec_i % ch, r);
    __syncwarp();  // new v visible to the neighbouring lanes
    if constexpr (TAPE) {
      if (A.tape) {
        tape_store<T>(P, K, ch, P_V, P_M, P_H, P_N,
                      A.tape + (int64_t)(s + 1) * 4 * A.n_comp + off, A.n_comp);
        __syncwarp();  // the next step rewrites rows other lanes just read
      }
    }
  }
  for (int j = 0; j < ch; ++j) {
    const int i = r * ch + j;
    if (i < K) {
      const int64_t g = off + i;
      A.v[g] = P.at(P_V, j, r);
      A.m[g] = P.at(P_M, j, r);
      A.h[g] = P.at(P_H, j, r);
      A.n[g] = P.at(P_N, j, r);
    }
  }
  if (spk_i >= 0 && r == 0) {
    A.spk_count[cable] = count;
    A.spk_first[cable] = first;
  }
  if (spk_i >= 0 && r == spk_i / ch) A.spk_below[cable] = below;
  if (spk_i2 >= 0 && r == spk_i2 / ch) A.spk_below2[cable] = below2;
  __syncwarp();
}

template <typename T, bool FAST, bool TAPE>
__global__ void __launch_bounds__(kCableMaxWarps * 32) cable_run_kernel(CableArgsT<T> A, int ch_max,
                                                                     PlaneLayout lay) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5;
  T* smw = reinterpret_cast<T*>(smem_raw) + (size_t)warp * lay.n_planes * ch_max * 32;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(A.counter, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= A.n_cables) break;
    const int cable = A.order ? A.order[idx] : idx;
    const int K = (int)(A.cable_ptr[cable + 1] - A.cable_ptr[cable]);
    const int ch = (K + 31) / 32;
    if (ch > ch_max) {  // the host sized shared memory for smaller cables: flag, never skip silently
      if (lane == 0) atomicOr(A.counter + 1, kErrChunk);
      continue;
    }
    run_cable<T, FAST, TAPE>(A, cable, smw, ch, lay);
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

template <typename T, bool FAST, bool TAPE = false>
static int launch_cable_run(CableArgsT<T> A, int ch_max, const PlaneLayout& lay,
                            cudaStream_t st) {
  // one warp per cable in flight; long cables get fewer warps per block so
  // the block's planes fit the 227 KB shared-memory limit
  const size_t per_warp = (size_t)lay.n_planes * ch_max * 32 * sizeof(T);
  const int wpb = persistent_wpb(A.wpb, per_warp);
  DGB_REQUIRE(wpb > 0, "cable too long for shared memory (%zu bytes per cable)", per_warp);
  const int threads = wpb * 32;
  const size_t smem = (size_t)wpb * per_warp;
  auto kern = cable_run_kernel<T, FAST, TAPE>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  int blocks = device_sm_count() * per_sm;
  const int blocks_needed = (A.n_cables + wpb - 1) / wpb;
  if (blocks > blocks_needed) blocks = blocks_needed;
  if (blocks < 1) blocks = 1;
  DGB_CUDA_CHECK(cudaMemsetAsync(A.counter, 0, 2 * sizeof(int32_t), st));
  kern<<<blocks, threads, smem, st>>>(A, ch_max, lay);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T>
int cable_run_t(const dgb_cable_args* args, int ch_max, cudaStream_t st) {
  CableArgsT<T> A = typed<T>(args);
  const bool field = args->field != nullptr && args->ve_amp != nullptr;
  const bool chan_planes = (args->flags & DGB_CABLE_UNIFORM_CHANNELS) == 0;
  const bool geo_planes = (args->flags & DGB_CABLE_UNIFORM_GEOMETRY) == 0;
  const PlaneLayout lay = plane_layout(geo_planes, field, chan_planes);
  if constexpr (sizeof(T) == 4) {
    if (args->flags & DGB_CABLE_FAST_MATH) return launch_cable_run<T, true>(A, ch_max, lay, st);
  }
  return launch_cable_run<T, false>(A, ch_max, lay, st);
}

template <typename T>
int cable_run_taped_t(const dgb_cable_args* args, void* tape, int ch_max, cudaStream_t st) {
  CableArgsT<T> A = typed<T>(args);
  A.tape = (T*)tape;
  const bool field = args->field != nullptr && args->ve_amp != nullptr;
  const bool chan_planes = (args->flags & DGB_CABLE_UNIFORM_CHANNELS) == 0;
  const bool geo_planes = (args->flags & DGB_CABLE_UNIFORM_GEOMETRY) == 0;
  const PlaneLayout lay = plane_layout(geo_planes, field, chan_planes);
  if constexpr (sizeof(T) == 4) {
    if (args->flags & DGB_CABLE_FAST_MATH) return launch_cable_run<T, true, true>(A, ch_max, lay, st);
  }
  return launch_cable_run<T, false, true>(A, ch_max, lay, st);
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
  template int cable_run_taped_t<T>(const dgb_cable_args*, void*, int, cudaStream_t);   \
  template int cable_assemble_t<T>(const dgb_cable_args*, int32_t, void*, void*, void*, \
                                   void*, cudaStream_t);                               \
  template int cable_solve_update_t<T>(const dgb_cable_args*, const void*, const void*, \
                                       const void*, const void*, cudaStream_t);

}  // namespace dgb
