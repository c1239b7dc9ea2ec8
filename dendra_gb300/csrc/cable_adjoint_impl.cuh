// Adjoint (reverse mode) of the unbranched HH cable update, one segment of
// steps at a time, from the state tape written by dgb_cable_run_taped.
//
// Forward step s, per compartment i (cable_impl.cuh):
//   m' = cnexp(m, a_m(v), b_m(v))  (and h', n')                      gates at v_old
//   G  = gl + gnabar m'^3 h' + gkbar n'^4,  J = gl el + gna ena + gk ek
//   fn = (J - G v) scl + gr (v_{i+1} - v) - glf (v - v_{i-1}) + [ve terms] + Iin cm_inv
//   M x = dt_s fn,  M = tridiag(a = -dt_s glf, b = 1 + dt_s (gr + glf + G scl), c = -dt_s gr)
//   v' = v + x
// Reverse of that step for the adjoints (lv', lm', lh', ln') of the state after it:
//   M^T mu = lv'                         (transposed chunked solve)
//   lfn = dt_s mu,  lb = -mu x_i,  la = -mu x_{i-1},  lc = -mu x_{i+1}
//   lgr  = dt_s (lb - lc) + (dv_r + dve_r) lfn,  lglf = dt_s (lb - la) - (dv_l + dve_l) lfn
//   lG = dt_s scl lb - v scl lfn,  lJ = scl lfn
//   gnabar += m'^3 h' (lG + ena lJ),  gkbar += n'^4 (lG + ek lJ),  gl += lG + el lJ,
//   axial += lgr gr + lglf glf                    (per compartment)
//   lm' += 3 gnabar m'^2 h' (lG + ena lJ) ...; lm = dm'/dm lm' ...
//   lv = lv' - (G scl + gr + glf) lfn_i + gr_{i-1} lfn_{i-1} + glf_{i+1} lfn_{i+1}
//        + dm'/dv lm' + dh'/dv lh' + dn'/dv ln'
// The reference gets the same numbers from torch autograd through
// integrators/implicit.py:569-664 and the transpose solve of
// ThomasSolve.backward (triton/t_kernel_thomas.py:147-189).
#pragma once
#include "adjoint.cuh"
#include "cable_common.cuh"
#include "chunk_solve.cuh"

namespace dgb {

template <typename T>
struct AdjArgsT {
  const T* tape;
  const T* trace_grad;
  int64_t trace_len;
  T *lam_v, *lam_m, *lam_h, *lam_n;
  T *g_gna, *g_gk, *g_gl, *g_ax;
};

// Planes of one warp in the adjoint: tape state (V and VN swap roles every
// step), adjoint state, solve scratch, gradient accumulators, and what phase 1
// keeps for phase 3 (G and the six gate partials).  Geometry, lead field and
// channel planes follow when they vary along the cable, as in the forward.
enum {
  Q_V0 = 0, Q_V1, Q_M, Q_H, Q_N, Q_LV, Q_LM, Q_LH, Q_LN, Q_MU, Q_AP, Q_CP, Q_DP,
  Q_GNA, Q_GK, Q_GL, Q_GAX, Q_G, Q_DMM, Q_DMV, Q_DHH, Q_DHV, Q_DNN, Q_DNV, Q_FIXED
};

__host__ __device__ inline PlaneLayout adjoint_layout(bool geo_planes, bool field,
                                                      bool chan_planes) {
  PlaneLayout L;
  int q = Q_FIXED;
  L.q_geo = geo_planes ? q : -1;
  q += geo_planes ? 3 : 0;
  L.q_fld = field ? q : -1;
  q += field ? 1 : 0;
  L.q_chan = chan_planes ? q : -1;
  q += chan_planes ? 4 : 0;
  L.n_planes = q;
  return L;
}

// Chunked tridiagonal solve of one warp's system held in shared-memory
// planes: rows i = r*ch + j, coefficients from row(j, a, b, c, d); the
// solution goes to plane qx.  Same elimination as the forward's fused solve
// (local sweep per lane, reduced row per lane, PCR across the 32 lanes).
template <typename T, bool FAST, class Row>
__device__ __forceinline__ void plane_solve(const Planes<T>& P, int ch, int qx, Row row) {
  const int r = threadIdx.x & 31;
  const int last = ch - 1;
  T As = T(0), Bs = T(1), Cs = T(0), Ds = T(0);
  T ap = T(0), cp = T(0), dp = T(0);
  for (int j = 0; j < ch; ++j) {
    T a, b, c, d;
    row(j, a, b, c, d);
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
      P.at(Q_AP, j, r) = ap;
      P.at(Q_CP, j, r) = cp;
      P.at(Q_DP, j, r) = dp;
    }
  }
  T al, be, ga, de, Ae = ap, Ce = cp, De = dp;
  if (ch == 1) {
    al = As;
    be = Bs;
    ga = Cs;
    de = Ds;
  } else {
    T a2 = ap, c2 = cp, d2 = dp;
    if (ch >= 3) {
      a2 = P.at(Q_AP, ch - 2, r);
      c2 = P.at(Q_CP, ch - 2, r);
      d2 = P.at(Q_DP, ch - 2, r);
      for (int j = ch - 3; j >= 1; --j) {
        const T cj = P.at(Q_CP, j, r);
        d2 = P.at(Q_DP, j, r) - cj * d2;
        a2 = P.at(Q_AP, j, r) - cj * a2;
        c2 = -cj * c2;
        P.at(Q_AP, j, r) = a2;
        P.at(Q_CP, j, r) = c2;
        P.at(Q_DP, j, r) = d2;
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
  P.at(qx, 0, r) = xs;
  for (int j = 1; j < last; ++j)
    P.at(qx, j, r) = P.at(Q_DP, j, r) - P.at(Q_AP, j, r) * xs - P.at(Q_CP, j, r) * xe;
  if (ch > 1) P.at(qx, last, r) = xe;
}

// Value of plane q at row i - 1 / i + 1 of lane r's slot j (0 past the cable).
template <typename T>
__device__ __forceinline__ T row_prev(const Planes<T>& P, int q, int j, int r, int last) {
  return j > 0 ? P.at(q, j - 1, r) : (r > 0 ? P.at(q, last, r - 1) : T(0));
}
template <typename T>
__device__ __forceinline__ T row_next(const Planes<T>& P, int q, int j, int r, int last) {
  return j < last ? P.at(q, j + 1, r) : (r < 31 ? P.at(q, 0, r + 1) : T(0));
}

template <typename T, bool FAST>
__device__ void adjoint_cable(const CableArgsT<T>& A, const AdjArgsT<T>& D, int cable, T* smw,
                              int ch, const PlaneLayout& lay) {
  const int r = threadIdx.x & 31;
  const int64_t off = A.cable_ptr[cable];
  const int K = (int)(A.cable_ptr[cable + 1] - off);
  const int64_t N = A.n_comp;
  Planes<T> P{smw, ch};
  const bool use_ve = lay.q_fld >= 0;
  const int last = ch - 1;

  for (int j = 0; j < ch; ++j) {
    const int i = r * ch + j;
    const bool in = i < K;
    const int64_t g = off + i;
    P.at(Q_LV, j, r) = in ? D.lam_v[g] : T(0);
    P.at(Q_LM, j, r) = in ? D.lam_m[g] : T(0);
    P.at(Q_LH, j, r) = in ? D.lam_h[g] : T(0);
    P.at(Q_LN, j, r) = in ? D.lam_n[g] : T(0);
    // the accumulators continue from their values after the later segments
    P.at(Q_GNA, j, r) = in ? D.g_gna[g] : T(0);
    P.at(Q_GK, j, r) = in ? D.g_gk[g] : T(0);
    P.at(Q_GL, j, r) = in ? D.g_gl[g] : T(0);
    P.at(Q_GAX, j, r) = in ? D.g_ax[g] : T(0);
    // padding rows keep zero state: their gates stay finite and their
    // adjoints stay zero (every coupling coefficient is zero there)
    P.at(Q_V0, j, r) = T(0);
    P.at(Q_V1, j, r) = T(0);
    P.at(Q_M, j, r) = T(0);
    P.at(Q_H, j, r) = T(0);
    P.at(Q_N, j, r) = T(0);
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
  T ve_amp = T(0), ve_delay = T(0), ve_pw = T(0);
  if (use_ve) {
    ve_amp = A.ve_amp[cable];
    ve_delay = A.ve_delay[cable];
    ve_pw = A.ve_pw[cable];
  }
  const int rec_i = (A.rec_idx && D.trace_grad) ? A.rec_idx[cable] : -1;
  __syncwarp();
  const int S = A.n_steps;
  int qv = Q_V0, qvn = Q_V1;
  // v after the segment
  {
    const T* src = D.tape + (int64_t)S * 4 * N + off;
    for (RowWalk w(r, ch); w.i < K; w.next()) P.at(qvn, w.j, w.lane) = src[w.i];
  }
  const T dt = A.dt, dt_s = A.dt_s, q10 = A.q10, ena = A.ena, ek = A.ek;
  // per-row coefficients (uniform values or planes)
  auto geo = [&](int j, T& gr, T& glf, T& scl) {
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
  };
  // g_right of row i - 1 and g_left of row i + 1 (the transposed couplings)
  auto gr_prev = [&](int j) -> T {
    if (lay.q_geo >= 0) return row_prev<T>(P, lay.q_geo, j, r, last);
    const int i = r * ch + j;
    return (i >= 1 && i <= K - 1) ? gr_c : T(0);
  };
  auto glf_next = [&](int j) -> T {
    if (lay.q_geo >= 0) return row_next<T>(P, lay.q_geo + 1, j, r, last);
    const int i = r * ch + j;
    return (i + 1 < K) ? glf_c : T(0);
  };
  for (int s = S - 1; s >= 0; --s) {
    {
      const T* src = D.tape + (int64_t)s * 4 * N + off;
      for (RowWalk w(r, ch); w.i < K; w.next()) {
        P.at(qv, w.j, w.lane) = src[w.i];
        P.at(Q_M, w.j, w.lane) = src[N + w.i];
        P.at(Q_H, w.j, w.lane) = src[2 * N + w.i];
        P.at(Q_N, w.j, w.lane) = src[3 * N + w.i];
      }
    }
    // the trace sample recorded after this step
    const int64_t gstep = A.step0 + s + 1;
    if (rec_i >= 0 && r == rec_i / ch && gstep % A.rec_every == 0 &&
        gstep / A.rec_every < D.trace_len)
      P.at(Q_LV, rec_i % ch, r) += D.trace_grad[(int64_t)cable * D.trace_len + gstep / A.rec_every];
    __syncwarp();
    const T t = (T)(A.t0_ms + (double)(A.step0 + s) * A.dt_ms_d);
    const T Ive = use_ve ? rect_pulse<T>(t, ve_amp, ve_delay, ve_pw) : T(0);
    const bool ve_on = Ive != T(0);

    // ---- phase 1: gates with partials at v_old, conductance G
    for (int j = 0; j < ch; ++j) {
      const T v = P.at(qv, j, r);
      T m = P.at(Q_M, j, r), h = P.at(Q_H, j, r), n = P.at(Q_N, j, r);
      T dmm, dmv, dhh, dhv, dnn, dnv;
      if constexpr (FAST) {
        hh_gates_partials_fast(v, q10, dt, m, h, n, dmm, dmv, dhh, dhv, dnn, dnv);
      } else {
        hh_gates_partials<T>(v, q10, dt, m, h, n, dmm, dmv, dhh, dhv, dnn, dnv);
      }
      P.at(Q_M, j, r) = m;
      P.at(Q_H, j, r) = h;
      P.at(Q_N, j, r) = n;
      P.at(Q_DMM, j, r) = dmm;
      P.at(Q_DMV, j, r) = dmv;
      P.at(Q_DHH, j, r) = dhh;
      P.at(Q_DHV, j, r) = dhv;
      P.at(Q_DNN, j, r) = dnn;
      P.at(Q_DNV, j, r) = dnv;
      T gna = gna_c, gk = gk_c, gl = gl_c;
      if (lay.q_chan >= 0) {
        gna = P.at(lay.q_chan, j, r);
        gk = P.at(lay.q_chan + 1, j, r);
        gl = P.at(lay.q_chan + 2, j, r);
      }
      const T m3 = m * m * m;
      const T n2 = n * n;
      P.at(Q_G, j, r) = gl + gna * m3 * h + gk * (n2 * n2);
    }
    // ---- phase 2: M^T mu = lv'
    plane_solve<T, FAST>(P, ch, Q_MU, [&](int j, T& a, T& b, T& c, T& d) {
      T gr, glf, scl;
      geo(j, gr, glf, scl);
      b = T(1) - dt_s * ((-gr + -glf) - mul_rn(P.at(Q_G, j, r), scl));
      a = -dt_s * gr_prev(j);
      c = -dt_s * glf_next(j);
      d = P.at(Q_LV, j, r);
    });
    __syncwarp();  // mu of the neighbouring rows

    // ---- phase 3: adjoints of the state before the step, parameter gradients
    T f_prev = T(0), fj = T(0);
    if (ve_on) {
      f_prev = (r > 0) ? P.at(lay.q_fld, last, r - 1) : T(0);
      fj = P.at(lay.q_fld, 0, r);
    }
    for (int j = 0; j < ch; ++j) {
      const T mu = P.at(Q_MU, j, r);
      const T mu_p = row_prev<T>(P, Q_MU, j, r, last);
      const T mu_n = row_next<T>(P, Q_MU, j, r, last);
      const T v = P.at(qv, j, r);
      const T v_p = row_prev<T>(P, qv, j, r, last);
      const T v_n = row_next<T>(P, qv, j, r, last);
      const T x = P.at(qvn, j, r) - v;
      const T x_p = row_prev<T>(P, qvn, j, r, last) - v_p;
      const T x_n = row_next<T>(P, qvn, j, r, last) - v_n;
      T gr, glf, scl;
      geo(j, gr, glf, scl);
      T dvr = v_n - v, dvl = v - v_p;
      if (ve_on) {
        const T f_next = row_next<T>(P, lay.q_fld, j, r, last);
        const T ve_l = mul_rn(f_prev, Ive), ve_c = mul_rn(fj, Ive), ve_r = mul_rn(f_next, Ive);
        dvr = dvr + (ve_r - ve_c);
        dvl = dvl + (ve_c - ve_l);
        f_prev = fj;
        fj = f_next;
      }
      const T lfn = dt_s * mu;
      const T lb = -mu * x;
      const T la = -mu * x_p;
      const T lc = -mu * x_n;
      const T lgr = dt_s * (lb - lc) + dvr * lfn;
      const T lglf = dt_s * (lb - la) - dvl * lfn;
      P.at(Q_GAX, j, r) += lgr * gr + lglf * glf;
      const T G = P.at(Q_G, j, r);
      const T lG = dt_s * scl * lb - v * scl * lfn;
      const T lJ = scl * lfn;
      T gna = gna_c, gk = gk_c, el = el_c;
      if (lay.q_chan >= 0) {
        gna = P.at(lay.q_chan, j, r);
        gk = P.at(lay.q_chan + 1, j, r);
        el = P.at(lay.q_chan + 3, j, r);
      }
      const T m = P.at(Q_M, j, r), h = P.at(Q_H, j, r), n = P.at(Q_N, j, r);
      const T m2 = m * m, n2 = n * n;
      const T m3 = m2 * m, n3 = n2 * n;
      const T lgna = lG + ena * lJ;
      const T lgk = lG + ek * lJ;
      P.at(Q_GNA, j, r) += m3 * h * lgna;
      P.at(Q_GK, j, r) += (n2 * n2) * lgk;
      P.at(Q_GL, j, r) += lG + el * lJ;
      const T lm = P.at(Q_LM, j, r) + T(3) * gna * m2 * h * lgna;
      const T lh = P.at(Q_LH, j, r) + gna * m3 * lgna;
      const T ln = P.at(Q_LN, j, r) + T(4) * gk * n3 * lgk;
      const T lv = P.at(Q_LV, j, r) - (G * scl + gr + glf) * lfn + gr_prev(j) * (dt_s * mu_p) +
                   glf_next(j) * (dt_s * mu_n) + P.at(Q_DMV, j, r) * lm +
                   P.at(Q_DHV, j, r) * lh + P.at(Q_DNV, j, r) * ln;
      P.at(Q_LM, j, r) = P.at(Q_DMM, j, r) * lm;
      P.at(Q_LH, j, r) = P.at(Q_DHH, j, r) * lh;
      P.at(Q_LN, j, r) = P.at(Q_DNN, j, r) * ln;
      P.at(Q_LV, j, r) = lv;
    }
    __syncwarp();  // every lane is done with this step's rows before the next load
    const int tq = qv;
    qv = qvn;
    qvn = tq;
  }
  // the initial state's trace sample (recorded before the first step)
  if (rec_i >= 0 && A.step0 == 0 && r == rec_i / ch && D.trace_len > 0)
    P.at(Q_LV, rec_i % ch, r) += D.trace_grad[(int64_t)cable * D.trace_len];
  __syncwarp();
  for (int j = 0; j < ch; ++j) {
    const int i = r * ch + j;
    if (i < K) {
      const int64_t g = off + i;
      D.lam_v[g] = P.at(Q_LV, j, r);
      D.lam_m[g] = P.at(Q_LM, j, r);
      D.lam_h[g] = P.at(Q_LH, j, r);
      D.lam_n[g] = P.at(Q_LN, j, r);
      D.g_gna[g] = P.at(Q_GNA, j, r);
      D.g_gk[g] = P.at(Q_GK, j, r);
      D.g_gl[g] = P.at(Q_GL, j, r);
      D.g_ax[g] = P.at(Q_GAX, j, r);
    }
  }
  __syncwarp();
}

template <typename T, bool FAST>
__global__ void __launch_bounds__(kCableMaxWarps * 32)
    cable_adjoint_kernel(CableArgsT<T> A, AdjArgsT<T> D, int ch_max, PlaneLayout lay) {
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
    if (ch > ch_max) {
      if (lane == 0) atomicOr(A.counter + 1, kErrChunk);
      continue;
    }
    adjoint_cable<T, FAST>(A, D, cable, smw, ch, lay);
  }
}

template <typename T, bool FAST>
static int launch_adjoint(const CableArgsT<T>& A, const AdjArgsT<T>& D, int ch_max,
                          const PlaneLayout& lay, cudaStream_t st) {
  const size_t per_warp = (size_t)lay.n_planes * ch_max * 32 * sizeof(T);
  const int wpb = persistent_wpb(A.wpb, per_warp);
  if (wpb == 0) {
    set_error("cable too long for the adjoint's shared memory (%zu bytes per cable, limit %d)",
              per_warp, 227 * 1024);
    return DGB_ERANGE;
  }
  const int threads = wpb * 32;
  const size_t smem = (size_t)wpb * per_warp;
  auto kern = cable_adjoint_kernel<T, FAST>;
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
  kern<<<blocks, threads, smem, st>>>(A, D, ch_max, lay);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

template <typename T>
int cable_adjoint_t(const dgb_cable_args* args, const dgb_cable_adjoint_args* adj, int ch_max,
                    cudaStream_t st) {
  CableArgsT<T> A = typed<T>(args);
  AdjArgsT<T> D;
  D.tape = (const T*)adj->tape;
  D.trace_grad = (const T*)adj->trace_grad;
  D.trace_len = adj->trace_len;
  D.lam_v = (T*)adj->lam_v;
  D.lam_m = (T*)adj->lam_m;
  D.lam_h = (T*)adj->lam_h;
  D.lam_n = (T*)adj->lam_n;
  D.g_gna = (T*)adj->grad_gnabar;
  D.g_gk = (T*)adj->grad_gkbar;
  D.g_gl = (T*)adj->grad_gl;
  D.g_ax = (T*)adj->grad_axial;
  const bool field = args->field != nullptr && args->ve_amp != nullptr;
  const bool chan_planes = (args->flags & DGB_CABLE_UNIFORM_CHANNELS) == 0;
  const bool geo_planes = (args->flags & DGB_CABLE_UNIFORM_GEOMETRY) == 0;
  const PlaneLayout lay = adjoint_layout(geo_planes, field, chan_planes);
  if constexpr (sizeof(T) == 4) {
    if (args->flags & DGB_CABLE_FAST_MATH) return launch_adjoint<T, true>(A, D, ch_max, lay, st);
  }
  return launch_adjoint<T, false>(A, D, ch_max, lay, st);
}

#define DGB_INSTANTIATE_CABLE_ADJOINT(T)                                                \
  template int cable_adjoint_t<T>(const dgb_cable_args*, const dgb_cable_adjoint_args*, \
                                  int, cudaStream_t);

}  // namespace dgb
