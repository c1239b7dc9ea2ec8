// Persistent cable update of dgb_cable_run: one work item is one cable on 32
// lanes, two cables on 16 lanes or four cables on 8 lanes (P lanes per cable:
// the Thomas/PCR split).  Lane r of a cable owns rows r*ch .. r*ch+ch-1.  Per
// step and row, fused (integrators/core.py:769-834,
// integrators/implicit.py:569-664): gates at v_old (mechanisms/_cnexp.py:
// 96-132, mod/HH.py:24-40) -> G, J (mod/HH.py:109-116) -> increment RHS and
// diagonal -> the forward sweep of the lane's chunk elimination; then the
// backward sweep, PCR across the P lanes by shuffles (chunk_solve.cuh), back
// substitution and v += dv, spike checks and recording.
//
// Shared memory of a warp: ch_alloc rows of NQ planes, row-interleaved,
//   element (row j, plane q, lane L) at [(j * NQ + q) * 32 + L]
// so one row pointer reaches every plane of its row at a compile-time offset
// (q * 32 elements) and a warp's access to one (j, q) touches 32 consecutive
// words (conflict free).  The row loop is not unrolled: the kernel's code
// stays small enough for the instruction cache while warps of different
// cable lengths share an SM.
//   planes 0..6   v, m, h, n, and the elimination's a', c', d'
//   plane  7      extracellular axial term (constant while a pulse is on)
//   planes 8..10  g_right, g_left, scale   (only when geometry varies)
//   planes 11..14 gnabar, gkbar, gl, el    (only when channels vary)
//   one more plane after those with split gates: the assembled diagonal b
//   (a, c, d go to planes 4..6, which the forward sweep then overwrites)
// Rows past a cable's end (i >= K, padding of the last lanes) run the same
// update with the cable's own membrane and axial coefficients but no
// extracellular or clamp drive: the last real row has exactly zero coupling to
// them (g_right = 0 there), so they never change a real row's value, and they
// stay finite (undriven HH compartments; a NaN there would reach real rows
// through 0 * NaN in the reduction).  With per-compartment planes they read
// zero coefficients.
#pragma once
#include "cable_common.cuh"
#include "chunk_solve.cuh"

namespace dgb {

enum {
  Q_V = 0, Q_M, Q_H, Q_N, Q_AP, Q_CP, Q_DP, Q_VAX,
  Q_GR, Q_GL, Q_SC, Q_GNA, Q_GK, Q_GLK, Q_EL,
  Q_BASE = 8,  // planes without per-compartment coefficients
  Q_ALL = 15   // with geometry and channel planes
};

// Planes per row for a launch: per-compartment geometry or channels need all 15
// (both sets are then read from planes).
template <bool PLANES>
struct RowsNQ {
  static constexpr int value = PLANES ? Q_ALL : Q_BASE;
};

template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

// Coalesced copy between global rows [0, K) of one cable and its plane q:
// the group's P lanes visit rows r, r + P, ... (row i lives in group lane
// i / ch, slot i % ch).
template <typename T>
__device__ __forceinline__ void rows_load(T* wsm, int NQ, int q, int ch, int lane0, int P, int r,
                                          const T* __restrict__ src, int K) {
  for (int i = r; i < P * ch; i += P) {
    const int j = i % ch, L = lane0 + i / ch;
    wsm[(j * NQ + q) * 32 + L] = i < K ? src[i] : T(0);
  }
}
template <typename T>
__device__ __forceinline__ void rows_store(const T* wsm, int NQ, int q, int ch, int lane0, int P,
                                           int r, T* dst, int K) {
  for (int i = r; i < K; i += P) {
    const int j = i % ch, L = lane0 + i / ch;
    dst[i] = wsm[(j * NQ + q) * 32 + L];
  }
}
// The per-step state tape: planes v, m, h, n to dst[i], dst[N + i],
// dst[2N + i], dst[3N + i] in one walk over rows r, r + P, ..., advancing
// (lane, slot) by (P / ch, P % ch) with one carry (P % ch < ch): two integer
// divisions per store instead of two per row and plane.
template <typename T>
__device__ __forceinline__ void rows_store_state(const T* wsm, int NQ, int ch, int lane0, int P,
                                                 int r, T* dst, int64_t N, int K) {
  int L = lane0 + r / ch, j = r % ch;
  const int dl = P / ch, dj = P % ch;
  for (int i = r; i < K; i += P) {
    const T* w = wsm + j * NQ * 32 + L;
    dst[i] = w[0 * 32];
    dst[N + i] = w[1 * 32];
    dst[2 * N + i] = w[2 * 32];
    dst[3 * N + i] = w[3 * 32];
    L += dl;
    j += dj;
    if (j >= ch) {
      j -= ch;
      ++L;
    }
  }
}

// First step s in [0, n_steps] whose stimulus time t(s) = T(t0 + (step0 + s) dt)
// is >= tb (n_steps when none).  t(s) never decreases with s, so a rectangular
// pulse on [delay, delay + pw) is on exactly for s in
// [first_step_at(delay), first_step_at(delay + pw)): the same steps as testing
// t(s) every step, found once per cable instead of per step.
template <typename T>
__device__ __forceinline__ int first_step_at(const CableArgsT<T>& A, T tb) {
  int lo = 0, hi = A.n_steps;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const T t = (T)(A.t0_ms + (double)(A.step0 + mid) * A.dt_ms_d);
    if (t >= tb) {
      hi = mid;
    } else {
      lo = mid + 1;
    }
  }
  return lo;
}

// Steps [s0, s1) during which the pulse (amp on [delay, delay + pw)) is nonzero.
template <typename T>
__device__ __forceinline__ void pulse_steps(const CableArgsT<T>& A, T amp, T delay, T pw,
                                            int& s0, int& s1) {
  const T stop = delay + pw;
  s0 = s1 = 0;
  if (!(amp != T(0)) || stop != stop || delay != delay) return;
  s0 = first_step_at<T>(A, delay);
  s1 = first_step_at<T>(A, stop);
  if (s1 < s0) s1 = s0;
}

// GW > 1 (split gates): the CTA's GW warps share one 32-lane cable.  Warp w
// advances the gates and assembles rows j = w, w + GW, ... of every lane into
// planes a -> Q_AP, b -> Q_B, c -> Q_CP, d / dt_s -> Q_DP; after a CTA barrier warp 0
// runs the forward sweep over those rows (the same operations, in the same
// order, as the fused sweep) and the rest of the step alone.  Warp 0 also does
// every global load and store of the cable.
template <typename T, bool FAST, bool TAPE, bool PLANES, int GW = 1>
__device__ __forceinline__ void run_rows(const CableArgsT<T>& A, int pos0, int pos_end, int P,
                                         int ch, T* wsm) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int NQ = RowsNQ<PLANES>::value + (GW > 1 ? 1 : 0);
  constexpr int Q_B = RowsNQ<PLANES>::value;  // split gates: the assembled diagonal
  constexpr int rs = NQ * 32;  // elements from one row to the next
  const int gw = GW > 1 ? (int)(threadIdx.x >> 5) : 0;
  const bool solver = gw == 0;
  const int lane = threadIdx.x & 31;
  const int grp = lane / P;
  const int r = lane - grp * P;
  const int lane0 = grp * P;
  const int pos = pos0 + grp;
  const int cable = pos < pos_end ? (A.order ? A.order[pos] : pos) : -1;
  const int64_t off = cable >= 0 ? A.cable_ptr[cable] : 0;
  const int K = cable >= 0 ? (int)(A.cable_ptr[cable + 1] - off) : 0;
  const int row0 = r * ch;
  T* const p0 = wsm + lane;  // this lane's row 0
  const bool use_ve = A.field != nullptr && A.ve_amp != nullptr;

  // ---- load state and coefficients (rows past K start at zero)
  if (solver) {
    rows_load<T>(wsm, NQ, Q_V, ch, lane0, P, r, A.v + off, K);
    rows_load<T>(wsm, NQ, Q_M, ch, lane0, P, r, A.m + off, K);
    rows_load<T>(wsm, NQ, Q_H, ch, lane0, P, r, A.h + off, K);
    rows_load<T>(wsm, NQ, Q_N, ch, lane0, P, r, A.n + off, K);
    if constexpr (PLANES) {
      rows_load<T>(wsm, NQ, Q_GR, ch, lane0, P, r, A.g_right + off, K);
      rows_load<T>(wsm, NQ, Q_GL, ch, lane0, P, r, A.g_left + off, K);
      rows_load<T>(wsm, NQ, Q_SC, ch, lane0, P, r, A.scale + off, K);
      rows_load<T>(wsm, NQ, Q_GNA, ch, lane0, P, r, A.gnabar + off, K);
      rows_load<T>(wsm, NQ, Q_GK, ch, lane0, P, r, A.gkbar + off, K);
      rows_load<T>(wsm, NQ, Q_GLK, ch, lane0, P, r, A.gl + off, K);
      rows_load<T>(wsm, NQ, Q_EL, ch, lane0, P, r, A.el + off, K);
    }
    if (use_ve) rows_load<T>(wsm, NQ, Q_VAX, ch, lane0, P, r, A.field + off, K);
  }
  __syncwarp();
  // uniform coefficients: the cable's values, identical on every compartment
  // (interior edges for g_right / g_left), so reading them once is exact
  T gna_c = T(0), gk_c = T(0), gl_c = T(0), el_c = T(0);
  T gr_c = T(0), glf_c = T(0), sc_c = T(0);
  if (!PLANES && K > 0) {
    gna_c = A.gnabar[off];
    gk_c = A.gkbar[off];
    gl_c = A.gl[off];
    el_c = A.el[off];
    gr_c = K > 1 ? A.g_right[off] : T(0);
    glf_c = K > 1 ? A.g_left[off + 1] : T(0);
    sc_c = A.scale[off];
  }
  const T glel_c = mul_rn(gl_c, el_c);  // the leak's reversal term, rounded as per row
  // row j of this lane is the cable's last row (no right coupling)
  const int j_last = K - 1 - row0;
  // coefficients of row j (pointer pr); the first row has no left coupling
  auto coef = [&](const T* pr, int j, T& gr, T& glf, T& scl) {
    if constexpr (PLANES) {  // planes hold 0 past K, and 0 at the ends by contract
      gr = pr[Q_GR * 32];
      glf = pr[Q_GL * 32];
      scl = pr[Q_SC * 32];
    } else {
      gr = j == j_last ? T(0) : gr_c;
      glf = (j == 0 && r == 0) ? T(0) : glf_c;
      scl = sc_c;
    }
  };

  // extracellular drive: the axial ve term at ve = field * amp, evaluated
  // once with the rounded operations of the per-step form (the field rows are
  // replaced by the term in place, after every lane has read its neighbours)
  T ve_amp = T(0), ve_delay = T(0), ve_pw = T(0);
  if (use_ve && K > 0) {
    ve_amp = A.ve_amp[cable];
    ve_delay = A.ve_delay[cable];
    ve_pw = A.ve_pw[cable];
  }
  if (use_ve && solver) {
    T f_prev = r > 0 ? wsm[((ch - 1) * NQ + Q_VAX) * 32 + lane - 1] : T(0);
    T f_hi = r < P - 1 ? wsm[Q_VAX * 32 + lane + 1] : T(0);
    T fj = p0[Q_VAX * 32];
    __syncwarp();
    T* pr = p0;
    for (int j = 0; j < ch; ++j, pr += rs) {
      const T f_next = j < ch - 1 ? pr[rs + Q_VAX * 32] : f_hi;
      T gr, glf, scl;
      coef(pr, j, gr, glf, scl);
      const T ve_l = mul_rn(f_prev, ve_amp), ve_c = mul_rn(fj, ve_amp);
      const T ve_r = mul_rn(f_next, ve_amp);
      // zero on rows past the end: they must not be driven (see the header)
      pr[Q_VAX * 32] = row0 + j < K ? mul_rn(gr, ve_r - ve_c) - mul_rn(glf, ve_c - ve_l) : T(0);
      f_prev = fj;
      fj = f_next;
    }
    __syncwarp();
  }
  const int in_i = (A.in_idx && K > 0) ? A.in_idx[cable] : -1;
  T in_amp = T(0), in_delay = T(0), in_pw = T(0), in_cm = T(0);
  int in_j = -1;  // this lane's row of the clamp
  if (in_i >= 0 && in_i < K) {
    in_amp = A.in_amp[cable];
    in_delay = A.in_delay[cable];
    in_pw = A.in_pw[cable];
    in_cm = A.cm_inv[off + in_i];
    if (in_i / ch == r) in_j = in_i % ch;
  }
  // pulse steps of the extracellular drive and of the clamp
  int ve_s0 = 0, ve_s1 = 0, in_s0 = 0, in_s1 = 0;
  if (use_ve && K > 0) pulse_steps<T>(A, ve_amp, ve_delay, ve_pw, ve_s0, ve_s1);
  if (in_j >= 0) pulse_steps<T>(A, in_amp, in_delay, in_pw, in_s0, in_s1);
  // single-compartment trace and Active-style detection (count, first step);
  // v of compartment i sits at vofs(i) of the warp's planes
  auto vofs = [&](int i) { return ((i % ch) * NQ + Q_V) * 32 + lane0 + i / ch; };
  const int rec_i = (A.rec_idx && A.trace && K > 0) ? A.rec_idx[cable] : -1;
  const int spk_i = (A.spk_idx && K > 0) ? A.spk_idx[cable] : -1;
  const int spk_i2 = (A.spk_idx2 && spk_i >= 0) ? A.spk_idx2[cable] : -1;
  const int rec_o = rec_i >= 0 ? vofs(rec_i) : 0;
  const int spk_o = spk_i >= 0 ? vofs(spk_i) : 0;
  const int spk_o2 = spk_i2 >= 0 ? vofs(spk_i2) : 0;
  int below = 1, below2 = 1, count = 0, first = -1;
  if (spk_i >= 0 && r == 0) {
    count = A.spk_count[cable];
    first = A.spk_first[cable];
    below = A.spk_below[cable];
    if (spk_i2 >= 0) below2 = A.spk_below2[cable];
  }
  // raster: group lane q < n_rast keeps check q
  int r_idx = -1, r_latch = 1, r_count = 0, r_o = 0;
  if (r < A.n_rast && K > 0) {
    r_idx = A.rast_idx[(int64_t)cable * A.n_rast + r];
    if (r_idx >= K) r_idx = -1;
    if (r_idx >= 0) {
      r_o = vofs(r_idx);
      r_latch = A.rast_below[(int64_t)cable * A.n_rast + r];
      r_count = A.rast_count[(int64_t)cable * A.n_rast + r];
    }
  }
  if (solver && rec_i >= 0 && r == 0) A.trace[(int64_t)cable * A.n_rec] = wsm[rec_o];
  if (solver && A.trace_all) rows_store<T>(wsm, NQ, Q_V, ch, lane0, P, r, A.trace_all + off, K);
  if constexpr (TAPE) {
    if (solver && A.tape) {
      T* tp = A.tape + off;
      rows_store_state<T>(wsm, NQ, ch, lane0, P, r, tp, A.n_comp, K);
    }
  }
  __syncwarp();  // the first step rewrites rows other lanes just stored
  if constexpr (GW > 1) __syncthreads();  // the planes are loaded for every warp

  bool live = K > 0;  // this group's cable is still advancing
  int rec_left = A.rec_every, rec_k = 0;  // steps to the next record, records so far
  const T dt = A.dt, dt_s = A.dt_s, q10 = A.q10, ena = A.ena, ek = A.ek;
  for (int s = 0; s < A.n_steps; ++s) {
    const bool ve_on = s >= ve_s0 && s < ve_s1;
    const T Iin = (s >= in_s0 && s < in_s1) ? in_amp : T(0);

    // ---- gates, membrane frame, row assembly fused with the forward sweep.
    // Row 0 keeps its row (As, Bs, Cs, Ds); rows j >= 1 are eliminated against
    // the previous one, x_j + a'_j x_s + c'_j x_{j+1} = d'_j, starting from
    // (a', c', d') = (-1, 0, 0), which reproduces row 1's own division.
    T As = T(0), Bs = T(1), Cs = T(0), Ds = T(0);
    T ap = T(-1), cp = T(0), dp = T(0);
    {
      // the neighbouring lanes' boundary values
      const T v_hi = r < P - 1 ? wsm[Q_V * 32 + lane + 1] : T(0);
      const T v_lo = r > 0 ? wsm[((ch - 1) * NQ + Q_V) * 32 + lane - 1] : T(0);
      // one row: gates advanced in place, returns the row's a, b, c, d
      auto assemble = [&](T* pr, int j, T v_prev, T vj, T v_next, auto ve_tag, T& a, T& b,
                          T& c, T& d) {
        T m = pr[Q_M * 32], h = pr[Q_H * 32], n = pr[Q_N * 32];
        if constexpr (FAST) {
          hh_gates_fast_warp(vj, q10, dt, m, h, n);
        } else {
          hh_gates<T>(vj, q10, dt, m, h, n);
        }
        pr[Q_M * 32] = m;
        pr[Q_H * 32] = h;
        pr[Q_N * 32] = n;
        T G, J;
        if constexpr (PLANES) {
          hh_affine<T>(m, h, n, pr[Q_GNA * 32], pr[Q_GK * 32], pr[Q_GLK * 32], pr[Q_EL * 32],
                       ena, ek, G, J);
        } else {
          hh_affine_glel<T>(m, h, n, gna_c, gk_c, gl_c, glel_c, ena, ek, G, J);
        }
        T gr, glf, scl;
        coef(pr, j, gr, glf, scl);
        // row i couples to i-1 through glf and to i+1 through gr
        T fn = (J - mul_rn(G, vj)) * scl;
        fn = fn + (mul_rn(gr, v_next - vj) - mul_rn(glf, vj - v_prev));
        if constexpr (decltype(ve_tag)::value) fn = fn + pr[Q_VAX * 32];
        if (j == in_j) fn = fn + Iin * in_cm;
        b = T(1) - dt_s * ((-gr + -glf) - mul_rn(G, scl));
        a = -dt_s * glf;
        c = -dt_s * gr;
        // split gates: fn itself, scaled where the sweep uses it, so that the
        // product dt_s * fn contracts with the sweep's operations exactly as
        // in the fused sweep
        if constexpr (GW > 1) {
          d = fn;
        } else {
          d = dt_s * fn;
        }
      };
      auto sweep = [&](auto ve_tag) {
        T* pr = p0;
        T vj = pr[Q_V * 32];
        T v_next = ch > 1 ? pr[rs + Q_V * 32] : v_hi;
        assemble(pr, 0, v_lo, vj, v_next, ve_tag, As, Bs, Cs, Ds);
        T v_prev = vj;
        vj = v_next;
        for (int j = 1; j < ch; ++j) {
          pr += rs;
          v_next = j < ch - 1 ? pr[rs + Q_V * 32] : v_hi;
          T a, b, c, d;
          assemble(pr, j, v_prev, vj, v_next, ve_tag, a, b, c, d);
          const T rinv = srcp<T, FAST>(b - a * cp);
          ap = -a * ap * rinv;
          dp = (d - a * dp) * rinv;
          cp = c * rinv;
          pr[Q_AP * 32] = ap;
          pr[Q_CP * 32] = cp;
          pr[Q_DP * 32] = dp;
          v_prev = vj;
          vj = v_next;
        }
      };
      if constexpr (GW == 1) {
        if (ve_on) {
          sweep(BoolTag<true>{});
        } else {
          sweep(BoolTag<false>{});
        }
      } else {
        auto rows = [&](auto ve_tag) {
          for (int j = gw; j < ch; j += GW) {
            T* pr = p0 + j * rs;
            const T vj = pr[Q_V * 32];
            const T v_prev = j > 0 ? pr[Q_V * 32 - rs] : v_lo;
            const T v_next = j < ch - 1 ? pr[rs + Q_V * 32] : v_hi;
            T a, b, c, d;
            assemble(pr, j, v_prev, vj, v_next, ve_tag, a, b, c, d);
            pr[Q_AP * 32] = a;
            pr[Q_B * 32] = b;
            pr[Q_CP * 32] = c;
            pr[Q_DP * 32] = d;
          }
        };
        if (ve_on) {
          rows(BoolTag<true>{});
        } else {
          rows(BoolTag<false>{});
        }
        __syncthreads();  // every row assembled
        if (solver) {
          T* pr = p0;
          As = pr[Q_AP * 32];
          Bs = pr[Q_B * 32];
          Cs = pr[Q_CP * 32];
          Ds = dt_s * pr[Q_DP * 32];
          for (int j = 1; j < ch; ++j) {
            pr += rs;
            const T a = pr[Q_AP * 32], b = pr[Q_B * 32], c = pr[Q_CP * 32];
            const T d = dt_s * pr[Q_DP * 32];
            const T rinv = srcp<T, FAST>(b - a * cp);
            ap = -a * ap * rinv;
            dp = (d - a * dp) * rinv;
            cp = c * rinv;
            pr[Q_AP * 32] = ap;
            pr[Q_CP * 32] = cp;
            pr[Q_DP * 32] = dp;
          }
        }
      }
    }
    bool done = false;  // stop on spike: no cable of the warp advances further
    if (solver) {
      // ---- backward sweep (rows ch-3 .. 1) and the lane's reduced row
      T al, be, ga, de;
      const T Ae = ap, Ce = cp, De = dp;  // row ch-1 (forward form)
      if (ch == 1) {
        al = As;
        be = Bs;
        ga = Cs;
        de = Ds;
      } else {
        T a2 = ap, c2 = cp, d2 = dp;  // row 1 once the loop below has run
        if (ch >= 3) {
          T* q = p0 + (ch - 2) * rs;
          a2 = q[Q_AP * 32];
          c2 = q[Q_CP * 32];
          d2 = q[Q_DP * 32];
          for (int j = ch - 3; j >= 1; --j) {
            q -= rs;
            const T cj = q[Q_CP * 32];
            d2 = q[Q_DP * 32] - cj * d2;
            a2 = q[Q_AP * 32] - cj * a2;
            c2 = -cj * c2;
            q[Q_AP * 32] = a2;
            q[Q_CP * 32] = c2;
            q[Q_DP * 32] = d2;
          }
        }
        T Bs2 = Bs, Cs2 = Cs, Ds2 = Ds;
        if (ch >= 3) {
          Bs2 = Bs - Cs * a2;
          Cs2 = -Cs * c2;
          Ds2 = Ds - Cs * d2;
        }
        T Ae_l = shfl_up<T>(Ae, 1, P), Ce_l = shfl_up<T>(Ce, 1, P), De_l = shfl_up<T>(De, 1, P);
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
      // ---- PCR across the P lanes, then back substitution
#pragma unroll
      for (int sh = 1; sh < 32; sh <<= 1) {
        if (sh >= P) break;
        // float64: each lane's pivot reciprocal, shuffled to both neighbours
        T pv = be;
        if constexpr (sizeof(T) == 8) pv = srcp<T, FAST>(be);
        T al_l = shfl_up<T>(al, sh, P), pv_l = shfl_up<T>(pv, sh, P);
        T ga_l = shfl_up<T>(ga, sh, P), de_l = shfl_up<T>(de, sh, P);
        T al_r = shfl_down<T>(al, sh, P), pv_r = shfl_down<T>(pv, sh, P);
        T ga_r = shfl_down<T>(ga, sh, P), de_r = shfl_down<T>(de, sh, P);
        const bool hl = r >= sh;
        const bool hr = r + sh < P;
        T k1, k2;
        if constexpr (sizeof(T) == 8) {
          k1 = hl ? al * pv_l : T(0);
          k2 = hr ? ga * pv_r : T(0);
        } else {
          k1 = hl ? dv<T, FAST>(al, pv_l) : T(0);
          k2 = hr ? dv<T, FAST>(ga, pv_r) : T(0);
        }
        T al_n = hl ? -k1 * al_l : T(0);
        T ga_n = hr ? -k2 * ga_r : T(0);
        be = be - (hl ? k1 * ga_l : T(0)) - (hr ? k2 * al_r : T(0));
        de = de - (hl ? k1 * de_l : T(0)) - (hr ? k2 * de_r : T(0));
        al = al_n;
        ga = ga_n;
      }
      const T xs = sdv<T, FAST>(de, be);
      T xe = xs;
      if (ch > 1) {
        T xs_next = shfl_down<T>(xs, 1, P);
        if (r == P - 1) xs_next = T(0);
        xe = De - Ae * xs - Ce * xs_next;
      }
      __syncwarp();  // every lane has read its neighbours' v for this step
      p0[Q_V * 32] = p0[Q_V * 32] + xs;
      {
        T* q = p0;
        for (int j = 1; j < ch - 1; ++j) {
          q += rs;
          q[Q_V * 32] = q[Q_V * 32] + (q[Q_DP * 32] - q[Q_AP * 32] * xs - q[Q_CP * 32] * xe);
        }
      }
      if (ch > 1) p0[(ch - 1) * rs + Q_V * 32] = p0[(ch - 1) * rs + Q_V * 32] + xe;
      __syncwarp();  // new v visible to every lane of the group

      // ---- detection (group lane 0), raster (group lanes < n_rast), recording
      bool stop_now = false;
      if (A.spk_idx) {
        int edge = 0;
        if (live && spk_i >= 0 && r == 0) {
          const int above = wsm[spk_o] >= A.spk_thr;
          edge = above && below;
          below = !above;
          if (spk_i2 >= 0) {
            const int above2 = wsm[spk_o2] >= A.spk_thr;
            edge = edge || (above2 && below2);
            below2 = !above2;
          }
          if (edge) {
            if (count == 0) first = s + 1;
            count += 1;
          }
        }
        stop_now = A.stop_on_spike && __shfl_sync(FULL, edge, lane0) && live;
      }
      if (live && r_idx >= 0) {
        const int above = wsm[r_o] >= A.spk_thr;
        if (above && r_latch) {
          if (r_count < A.rast_cap)
            A.rast_steps[((int64_t)cable * A.n_rast + r) * A.rast_cap + r_count] = A.step0 + s + 1;
          r_count += 1;
        }
        r_latch = !above;
      }
      // record every rec_every steps (a countdown: no division per step)
      const bool rec_due = --rec_left == 0;
      if (rec_due) {
        rec_left = A.rec_every;
        ++rec_k;
        if (live && rec_i >= 0 && r == 0) A.trace[(int64_t)cable * A.n_rec + rec_k] = wsm[rec_o];
        if (A.trace_all)
          rows_store<T>(wsm, NQ, Q_V, ch, lane0, P, r, A.trace_all + (int64_t)rec_k * A.n_comp + off,
                        live ? K : 0);
      }
      if constexpr (TAPE) {
        if (A.tape) {
          T* tp = A.tape + (int64_t)(s + 1) * 4 * A.n_comp + off;
          rows_store_state<T>(wsm, NQ, ch, lane0, P, r, tp, A.n_comp, K);
        }
      }
      if (A.stop_on_spike) {
        // a cable that fired stops here: its state is written now and frozen
        if (stop_now) {
          rows_store<T>(wsm, NQ, Q_V, ch, lane0, P, r, A.v + off, K);
          rows_store<T>(wsm, NQ, Q_M, ch, lane0, P, r, A.m + off, K);
          rows_store<T>(wsm, NQ, Q_H, ch, lane0, P, r, A.h + off, K);
          rows_store<T>(wsm, NQ, Q_N, ch, lane0, P, r, A.n + off, K);
          live = false;
        }
        done = !__any_sync(FULL, live);
      }
    }  // solver
    if constexpr (GW == 1) {
      if (done) break;
      __syncwarp();  // the next step rewrites rows other lanes just read
    } else {
      __shared__ int s_done;
      if (threadIdx.x == 0) s_done = done;
      __syncthreads();  // the new v is visible to every warp
      if (s_done) break;
    }
  }
  // ---- write back the state of cables still advancing, and the counters
  if (!solver) return;
  if (live) {
    rows_store<T>(wsm, NQ, Q_V, ch, lane0, P, r, A.v + off, K);
    rows_store<T>(wsm, NQ, Q_M, ch, lane0, P, r, A.m + off, K);
    rows_store<T>(wsm, NQ, Q_H, ch, lane0, P, r, A.h + off, K);
    rows_store<T>(wsm, NQ, Q_N, ch, lane0, P, r, A.n + off, K);
  }
  if (spk_i >= 0 && r == 0) {
    A.spk_count[cable] = count;
    A.spk_first[cable] = first;
    A.spk_below[cable] = below;
    if (spk_i2 >= 0) A.spk_below2[cable] = below2;
  }
  if (r_idx >= 0) {
    A.rast_below[(int64_t)cable * A.n_rast + r] = r_latch;
    A.rast_count[(int64_t)cable * A.n_rast + r] = r_count;
  }
  __syncwarp();
}

}  // namespace dgb
