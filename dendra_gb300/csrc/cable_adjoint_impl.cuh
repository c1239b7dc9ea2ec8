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
#include "bulk.cuh"
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

// Error bit of scratch[1]: a tape-stage wait gave up; the warp drained its
// copies and stopped (the segment's results are then incomplete).
constexpr int kErrTapeWait = 4;
constexpr uint32_t kTapeWaitLimit = 1u << 22;  // polls before a stage wait gives up
// Polls of the first wait on a tape stage: kTapeWaitLimit unless the
// diagnostic dgb_cable_adjoint_set_wait_limit lowered it (the drain after a
// give-up always uses kTapeWaitLimit).  One copy per dtype's translation
// unit; the setter writes both.
static __device__ uint32_t g_tape_wait_limit = kTapeWaitLimit;

// Row-interleaved planes of one warp (one cable), as in the forward kernel:
// element (row j, plane q, lane L) at [(j * NQ + q) * 32 + L], so one row
// pointer reaches every plane of its row at a compile-time offset and the 32
// lanes of an access touch 32 consecutive words.  Lane r owns compartments
// r*ch .. r*ch+ch-1.
//   LV..LN   adjoint state          MU          transposed solve's solution
//   AP..DP   elimination scratch    GNA..GAX    gradient accumulators
//   G        conductance (phase 1 -> 3)  DMM..DNV  gate partials (1 -> 3)
//   GR..CEL  geometry, lead field, channels (only when they vary, PLANES)
enum {
  R_LV = 0, R_LM, R_LH, R_LN, R_MU, R_AP, R_CP, R_DP, R_GNA, R_GK, R_GL, R_GAX, R_G,
  R_DMM, R_DMV, R_DHH, R_DHV, R_DNN, R_DNV,
  R_BASE = 19,  // uniform geometry and channels, no lead field
  R_GR = 19, R_GLF, R_SC, R_FLD, R_CNA, R_CK, R_CL, R_CEL,
  R_ALL = 27
};

template <bool PLANES>
struct AdjNQ {
  static constexpr int value = PLANES ? R_ALL : R_BASE;
};

// Tape stages: the 4 tape planes (v, m, h, n) of one step in natural order,
// brought by cp.async.bulk; plane q of stage b is a region of `cap` elements
// whose compartment i sits at sh[q] + i (the copy starts at the 16-byte
// boundary below the plane's first compartment; the last partial 16 bytes
// come by plain loads).  Then v of the step after the current one (vn, cap
// elements, natural order).
template <typename T>
__host__ __device__ inline int64_t tape_stage_cap(int ch_max) {
  constexpr int64_t E = 16 / sizeof(T);
  return ((int64_t)32 * ch_max + E - 1 + E - 1) / E * E;
}

template <typename T, bool PLANES>
__host__ __device__ inline size_t adjoint_warp_smem(int ch_max, int nstage) {
  return ((size_t)AdjNQ<PLANES>::value * ch_max * 32 +
          (size_t)(4 * nstage + 1) * tape_stage_cap<T>(ch_max)) * sizeof(T);
}

// Post the copies of tape step s (planes v, m, h, n of compartments
// [off, off + K)) into stage `st`; lane 0 posts the bulk copies, lanes 0..3
// load the partial last 16 bytes of planes 0..3.
template <typename T>
__device__ __forceinline__ void tape_issue(const T* tape, int64_t N, int64_t off, int K, int s,
                                           T* st, int64_t cap, uint32_t bar, int lane) {
  constexpr int64_t E = 16 / sizeof(T);
  if (lane == 0) {
    uint32_t bytes = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t lo = (int64_t)s * 4 * N + q * N + off;
      const int64_t lo16 = lo & ~(E - 1), hi16 = (lo + K) & ~(E - 1);
      if (hi16 > lo16) bytes += (uint32_t)((hi16 - lo16) * (int64_t)sizeof(T));
    }
    bulk::bar_expect(bar, bytes);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t lo = (int64_t)s * 4 * N + q * N + off;
      const int64_t lo16 = lo & ~(E - 1), hi16 = (lo + K) & ~(E - 1);
      if (hi16 > lo16)
        bulk::load(bulk::smem_addr(st + q * cap), tape + lo16,
                   (uint32_t)((hi16 - lo16) * (int64_t)sizeof(T)), bar);
    }
  }
  if (lane < 4) {
    const int64_t lo = (int64_t)s * 4 * N + lane * N + off, hi = lo + K;
    const int64_t lo16 = lo & ~(E - 1);
    int64_t e = hi & ~(E - 1);
    if (e < lo) e = lo;
    for (; e < hi; ++e) st[lane * cap + (e - lo16)] = tape[e];
  }
}

template <typename T, bool FAST, bool PLANES>
__device__ bool adjoint_rows(const CableArgsT<T>& A, const AdjArgsT<T>& D, int cable, T* wsm,
                             T* stg, int64_t cap, int nstage, int ch, uint32_t* bars,
                             uint32_t& par) {
  constexpr int NQ = AdjNQ<PLANES>::value;
  constexpr int rs = NQ * 32;
  const uint32_t wait_limit = g_tape_wait_limit;
  constexpr int64_t E = 16 / sizeof(T);
  const int r = threadIdx.x & 31;
  const int64_t off = A.cable_ptr[cable];
  const int K = (int)(A.cable_ptr[cable + 1] - off);
  const int64_t N = A.n_comp;
  const int last = ch - 1;
  const int row0 = r * ch;
  T* const p0 = wsm + r;
  T* const vn = stg + 4 * nstage * cap;  // v after the current step, natural order
  const bool use_ve = PLANES && A.field != nullptr && A.ve_amp != nullptr;
  // compartment i of tape plane q sits at stage + q * cap + sh_q + i (4N is a
  // multiple of 16 bytes, so the shift does not depend on the step)
  int sh[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) sh[q] = (int)((q * N + off) & (E - 1));

  // ---- state, accumulators and coefficient planes (lane r: its own rows)
  {
    T* pr = p0;
    for (int j = 0; j < ch; ++j, pr += rs) {
      const int i = row0 + j;
      const bool in = i < K;
      const int64_t g = off + i;
      pr[R_LV * 32] = in ? D.lam_v[g] : T(0);
      pr[R_LM * 32] = in ? D.lam_m[g] : T(0);
      pr[R_LH * 32] = in ? D.lam_h[g] : T(0);
      pr[R_LN * 32] = in ? D.lam_n[g] : T(0);
      pr[R_GNA * 32] = in ? D.g_gna[g] : T(0);
      pr[R_GK * 32] = in ? D.g_gk[g] : T(0);
      pr[R_GL * 32] = in ? D.g_gl[g] : T(0);
      pr[R_GAX * 32] = in ? D.g_ax[g] : T(0);
      if constexpr (PLANES) {  // zero past K and at the cable's ends by contract
        pr[R_GR * 32] = in ? A.g_right[g] : T(0);
        pr[R_GLF * 32] = in ? A.g_left[g] : T(0);
        pr[R_SC * 32] = in ? A.scale[g] : T(0);
        pr[R_FLD * 32] = (in && use_ve) ? A.field[g] : T(0);
        pr[R_CNA * 32] = in ? A.gnabar[g] : T(0);
        pr[R_CK * 32] = in ? A.gkbar[g] : T(0);
        pr[R_CL * 32] = in ? A.gl[g] : T(0);
        pr[R_CEL * 32] = in ? A.el[g] : T(0);
      }
    }
  }
  T gna_c = T(0), gk_c = T(0), gl_c = T(0), el_c = T(0), gr_c = T(0), glf_c = T(0), sc_c = T(0);
  if constexpr (!PLANES) {
    gna_c = A.gnabar[off];
    gk_c = A.gkbar[off];
    gl_c = A.gl[off];
    el_c = A.el[off];
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
  const int S = A.n_steps;
  // v after the segment
  for (int i = r; i < K; i += 32) vn[i] = D.tape[(int64_t)S * 4 * N + off + i];
  __syncwarp();
  bulk::fence_async_smem();  // earlier generic use of the stages before the copies
  if (S >= 1) tape_issue<T>(D.tape, N, off, K, S - 1, stg + ((S - 1) & (nstage - 1)) * 4 * cap,
                            cap, bars[(S - 1) & (nstage - 1)], r);
  const T dt = A.dt, dt_s = A.dt_s, q10 = A.q10, ena = A.ena, ek = A.ek;

  // per-row coefficients of row j (compartment i): uniform values or planes
  auto geo = [&](const T* pr, int i, T& gr, T& glf, T& scl) {
    if constexpr (PLANES) {
      gr = pr[R_GR * 32];
      glf = pr[R_GLF * 32];
      scl = pr[R_SC * 32];
    } else {
      gr = i < K - 1 ? gr_c : T(0);
      glf = (i >= 1 && i < K) ? glf_c : T(0);
      scl = i < K ? sc_c : T(0);
    }
  };
  // the transposed couplings: g_right of compartment i - 1, g_left of i + 1
  // (PLANES: neighbouring rows, across the lane boundary at a chunk's ends)
  auto gr_prev = [&](const T* pr, int j, int i) -> T {
    if constexpr (PLANES) {
      return j > 0 ? pr[-rs + R_GR * 32] : (r > 0 ? wsm[(last * NQ + R_GR) * 32 + r - 1] : T(0));
    } else {
      return (i >= 1 && i <= K - 1) ? gr_c : T(0);
    }
  };
  auto glf_next = [&](const T* pr, int j, int i) -> T {
    if constexpr (PLANES) {
      return j < last ? pr[rs + R_GLF * 32] : (r < 31 ? wsm[R_GLF * 32 + r + 1] : T(0));
    } else {
      return (i + 1 < K) ? glf_c : T(0);
    }
  };

  for (int s = S - 1; s >= 0; --s) {
    const int b = s & (nstage - 1);
    T* const st = stg + b * 4 * cap;
    if (nstage == 2 && s >= 1) {
      // prefetch the next (earlier) step into the other stage, which every
      // lane finished reading at the end of the previous step
      tape_issue<T>(D.tape, N, off, K, s - 1, stg + ((s - 1) & 1) * 4 * cap, cap,
                    bars[(s - 1) & 1], r);
    }
    // wait for this step's tape (phases alternate per stage use)
    const uint32_t parity = (par >> b) & 1u;
    const bool landed = bulk::bar_wait(bars[b], parity, wait_limit);
    if (!__all_sync(0xffffffffu, landed)) {
      if (r == 0) {
        atomicOr(A.counter + 1, kErrTapeWait);
        // drain: this stage, and the prefetch posted into the other one
        bulk::bar_wait(bars[b], parity, kTapeWaitLimit);
        if (nstage == 2 && s >= 1)
          bulk::bar_wait(bars[b ^ 1], (par >> (b ^ 1)) & 1u, kTapeWaitLimit);
      }
      __syncwarp();
      return false;
    }
    par ^= 1u << b;
    __syncwarp();  // the plain tail loads of this stage
    const T* sv = st + sh[0];
    T* sm = st + cap + sh[1];
    T* shh = st + 2 * cap + sh[2];
    T* sn = st + 3 * cap + sh[3];
    // the trace sample recorded after this step
    const int64_t gstep = A.step0 + s + 1;
    if (rec_i >= 0 && r == rec_i / ch && gstep % A.rec_every == 0 &&
        gstep / A.rec_every < D.trace_len)
      p0[(rec_i % ch) * rs + R_LV * 32] +=
          D.trace_grad[(int64_t)cable * D.trace_len + gstep / A.rec_every];
    __syncwarp();
    const T t = (T)(A.t0_ms + (double)(A.step0 + s) * A.dt_ms_d);
    const T Ive = use_ve ? rect_pulse<T>(t, ve_amp, ve_delay, ve_pw) : T(0);
    const bool ve_on = Ive != T(0);

    // ---- phases 1 + 2a: gates with partials at v_old, conductance G, fused
    // with the forward sweep of the transposed solve M^T mu = lv
    T As = T(0), Bs = T(1), Cs = T(0), Ds = T(0);
    T ap = T(0), cp = T(0), dp = T(0);
    {
      T* pr = p0;
      for (int j = 0; j < ch; ++j, pr += rs) {
        const int i = row0 + j;
        const bool in = i < K;
        // padding rows keep zero state: their gates stay finite and their
        // adjoints stay zero (every coupling coefficient is zero there)
        const T v = in ? sv[i] : T(0);
        T m = in ? sm[i] : T(0), h = in ? shh[i] : T(0), n = in ? sn[i] : T(0);
        T dmm, dmv, dhh, dhv, dnn, dnv;
        if constexpr (FAST) {
          hh_gates_partials_fast(v, q10, dt, m, h, n, dmm, dmv, dhh, dhv, dnn, dnv);
        } else {
          hh_gates_partials<T>(v, q10, dt, m, h, n, dmm, dmv, dhh, dhv, dnn, dnv);
        }
        if (in) {  // the advanced gates replace the tape's in the stage
          sm[i] = m;
          shh[i] = h;
          sn[i] = n;
        }
        pr[R_DMM * 32] = dmm;
        pr[R_DMV * 32] = dmv;
        pr[R_DHH * 32] = dhh;
        pr[R_DHV * 32] = dhv;
        pr[R_DNN * 32] = dnn;
        pr[R_DNV * 32] = dnv;
        T gna = gna_c, gk = gk_c, gl = gl_c;
        if constexpr (PLANES) {
          gna = pr[R_CNA * 32];
          gk = pr[R_CK * 32];
          gl = pr[R_CL * 32];
        }
        const T m3 = m * m * m;
        const T n2 = n * n;
        const T G = gl + gna * m3 * h + gk * (n2 * n2);
        pr[R_G * 32] = G;
        T gr, glf, scl;
        geo(pr, i, gr, glf, scl);
        const T bb = T(1) - dt_s * ((-gr + -glf) - mul_rn(G, scl));
        const T aa = -dt_s * gr_prev(pr, j, i);
        const T cc = -dt_s * glf_next(pr, j, i);
        const T dd = pr[R_LV * 32];
        if (j == 0) {
          As = aa;
          Bs = bb;
          Cs = cc;
          Ds = dd;
        } else {
          if (j == 1) {
            const T rinv = dv<T, FAST>(T(1), bb);
            ap = aa * rinv;
            cp = cc * rinv;
            dp = dd * rinv;
          } else {
            const T rinv = dv<T, FAST>(T(1), bb - aa * cp);
            ap = -aa * ap * rinv;
            dp = (dd - aa * dp) * rinv;
            cp = cc * rinv;
          }
          pr[R_AP * 32] = ap;
          pr[R_CP * 32] = cp;
          pr[R_DP * 32] = dp;
        }
      }
    }
    // ---- phase 2b: backward sweep, reduced row, PCR across the lanes, mu
    {
      T al, be, ga, de;
      const T Ae = ap, Ce = cp, De = dp;
      if (ch == 1) {
        al = As;
        be = Bs;
        ga = Cs;
        de = Ds;
      } else {
        T a2 = ap, c2 = cp, d2 = dp;
        if (ch >= 3) {
          T* q = p0 + (ch - 2) * rs;
          a2 = q[R_AP * 32];
          c2 = q[R_CP * 32];
          d2 = q[R_DP * 32];
          for (int j = ch - 3; j >= 1; --j) {
            q -= rs;
            const T cj = q[R_CP * 32];
            d2 = q[R_DP * 32] - cj * d2;
            a2 = q[R_AP * 32] - cj * a2;
            c2 = -cj * c2;
            q[R_AP * 32] = a2;
            q[R_CP * 32] = c2;
            q[R_DP * 32] = d2;
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
      for (int sh2 = 1; sh2 < 32; sh2 <<= 1) {
        T al_l = shfl_up<T>(al, sh2, 32), be_l = shfl_up<T>(be, sh2, 32);
        T ga_l = shfl_up<T>(ga, sh2, 32), de_l = shfl_up<T>(de, sh2, 32);
        T al_r = shfl_down<T>(al, sh2, 32), be_r = shfl_down<T>(be, sh2, 32);
        T ga_r = shfl_down<T>(ga, sh2, 32), de_r = shfl_down<T>(de, sh2, 32);
        const bool hl = r >= sh2;
        const bool hr = r + sh2 < 32;
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
      p0[R_MU * 32] = xs;
      T* q = p0;
      for (int j = 1; j < last; ++j) {
        q += rs;
        q[R_MU * 32] = q[R_DP * 32] - q[R_AP * 32] * xs - q[R_CP * 32] * xe;
      }
      if (ch > 1) p0[last * rs + R_MU * 32] = xe;
    }
    __syncwarp();  // mu of the neighbouring rows

    // ---- phase 3: adjoints of the state before the step, parameter gradients
    {
      // sliding windows over compartments i-1, i, i+1: mu (row planes, the
      // chunk's ends from the neighbouring lanes), v and v_next (natural order)
      T mu_p = r > 0 ? wsm[(last * NQ + R_MU) * 32 + r - 1] : T(0);
      T mu_c = p0[R_MU * 32];
      const T mu_hi = r < 31 ? wsm[R_MU * 32 + r + 1] : T(0);
      auto vat = [&](const T* a, int i) -> T { return (i >= 0 && i < K) ? a[i] : T(0); };
      T v_p = vat(sv, row0 - 1), v_c = vat(sv, row0);
      T x_p = vat(vn, row0 - 1) - v_p, x_c = vat(vn, row0) - v_c;
      T f_prev = T(0), fj = T(0);
      if (PLANES && ve_on) {
        f_prev = r > 0 ? wsm[(last * NQ + R_FLD) * 32 + r - 1] : T(0);
        fj = p0[R_FLD * 32];
      }
      T* pr = p0;
      for (int j = 0; j < ch; ++j, pr += rs) {
        const int i = row0 + j;
        const T mu_n = j < last ? pr[rs + R_MU * 32] : mu_hi;
        const T v_n = vat(sv, i + 1);
        const T x_n = vat(vn, i + 1) - v_n;
        const T mu = mu_c, v = v_c, x = x_c;
        T gr, glf, scl;
        geo(pr, i, gr, glf, scl);
        T dvr = v_n - v, dvl = v - v_p;
        if (PLANES && ve_on) {
          const T f_next = j < last ? pr[rs + R_FLD * 32] : (r < 31 ? wsm[R_FLD * 32 + r + 1] : T(0));
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
        pr[R_GAX * 32] += lgr * gr + lglf * glf;
        const T G = pr[R_G * 32];
        const T lG = dt_s * scl * lb - v * scl * lfn;
        const T lJ = scl * lfn;
        T gna = gna_c, gk = gk_c, el = el_c;
        if constexpr (PLANES) {
          gna = pr[R_CNA * 32];
          gk = pr[R_CK * 32];
          el = pr[R_CEL * 32];
        }
        const bool in = i < K;
        const T m = in ? sm[i] : T(0), h = in ? shh[i] : T(0), n = in ? sn[i] : T(0);
        const T m2 = m * m, n2 = n * n;
        const T m3 = m2 * m, n3 = n2 * n;
        const T lgna = lG + ena * lJ;
        const T lgk = lG + ek * lJ;
        pr[R_GNA * 32] += m3 * h * lgna;
        pr[R_GK * 32] += (n2 * n2) * lgk;
        pr[R_GL * 32] += lG + el * lJ;
        const T lm = pr[R_LM * 32] + T(3) * gna * m2 * h * lgna;
        const T lh = pr[R_LH * 32] + gna * m3 * lgna;
        const T ln = pr[R_LN * 32] + T(4) * gk * n3 * lgk;
        const T lv = pr[R_LV * 32] - (G * scl + gr + glf) * lfn + gr_prev(pr, j, i) * (dt_s * mu_p) +
                     glf_next(pr, j, i) * (dt_s * mu_n) + pr[R_DMV * 32] * lm +
                     pr[R_DHV * 32] * lh + pr[R_DNV * 32] * ln;
        pr[R_LM * 32] = pr[R_DMM * 32] * lm;
        pr[R_LH * 32] = pr[R_DHH * 32] * lh;
        pr[R_LN * 32] = pr[R_DNN * 32] * ln;
        pr[R_LV * 32] = lv;
        mu_p = mu;
        mu_c = mu_n;
        v_p = v;
        v_c = v_n;
        x_p = x;
        x_c = x_n;
      }
    }
    __syncwarp();  // every lane is done with vn and this stage
    // v of this step is v_next of the step before it
    for (int i = r; i < K; i += 32) vn[i] = sv[i];
    __syncwarp();
    bulk::fence_async_smem();  // this step's generic accesses before later copies
    if (nstage == 1 && s >= 1)
      tape_issue<T>(D.tape, N, off, K, s - 1, stg, cap, bars[0], r);
  }
  // the initial state's trace sample (recorded before the first step)
  if (rec_i >= 0 && A.step0 == 0 && r == rec_i / ch && D.trace_len > 0)
    p0[(rec_i % ch) * rs + R_LV * 32] += D.trace_grad[(int64_t)cable * D.trace_len];
  __syncwarp();
  {
    const T* pr = p0;
    for (int j = 0; j < ch; ++j, pr += rs) {
      const int i = row0 + j;
      if (i < K) {
        const int64_t g = off + i;
        D.lam_v[g] = pr[R_LV * 32];
        D.lam_m[g] = pr[R_LM * 32];
        D.lam_h[g] = pr[R_LH * 32];
        D.lam_n[g] = pr[R_LN * 32];
        D.g_gna[g] = pr[R_GNA * 32];
        D.g_gk[g] = pr[R_GK * 32];
        D.g_gl[g] = pr[R_GL * 32];
        D.g_ax[g] = pr[R_GAX * 32];
      }
    }
  }
  __syncwarp();
  return true;
}

template <typename T, bool FAST, bool PLANES>
__global__ void __launch_bounds__(kCableMaxWarps * 32)
    cable_adjoint_kernel(CableArgsT<T> A, AdjArgsT<T> D, int ch_max, int nstage) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars_all[kCableMaxWarps * 2];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  constexpr int NQ = AdjNQ<PLANES>::value;
  const int64_t cap = tape_stage_cap<T>(ch_max);
  T* wsm = reinterpret_cast<T*>(smem_raw +
                                (size_t)warp * adjoint_warp_smem<T, PLANES>(ch_max, nstage));
  T* stg = wsm + (size_t)NQ * ch_max * 32;
  uint32_t bars[2] = {bulk::smem_addr(&bars_all[warp * 2]), bulk::smem_addr(&bars_all[warp * 2 + 1])};
  if (lane == 0) {
    bulk::bar_init(bars[0], 1);
    bulk::bar_init(bars[1], 1);
    bulk::bar_init_fence();
  }
  __syncwarp();
  uint32_t par = 0;  // parity of the next phase of each stage's barrier
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
    if (!adjoint_rows<T, FAST, PLANES>(A, D, cable, wsm, stg, cap, nstage, ch, bars, par)) break;
  }
}

template <typename T, bool FAST, bool PLANES>
static int launch_adjoint(const CableArgsT<T>& A, const AdjArgsT<T>& D, int ch_max,
                          cudaStream_t st) {
  // two tape stages (the next step's copy overlaps this step) when they fit,
  // else one (the copy is waited for at once)
  int nstage = 2;
  int wpb = persistent_wpb(A.wpb, adjoint_warp_smem<T, PLANES>(ch_max, 2));
  if (wpb == 0) {
    nstage = 1;
    wpb = persistent_wpb(A.wpb, adjoint_warp_smem<T, PLANES>(ch_max, 1));
  }
  if (wpb == 0) {
    set_error("cable too long for the adjoint's shared memory (%zu bytes per cable, limit %d)",
              adjoint_warp_smem<T, PLANES>(ch_max, 1), 227 * 1024);
    return DGB_ERANGE;
  }
  const int threads = wpb * 32;
  const size_t smem = (size_t)wpb * adjoint_warp_smem<T, PLANES>(ch_max, nstage);
  auto kern = cable_adjoint_kernel<T, FAST, PLANES>;
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
  kern<<<blocks, threads, smem, st>>>(A, D, ch_max, nstage);
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
  if ((reinterpret_cast<uintptr_t>(adj->tape) & 15u) != 0) {
    set_error("the adjoint's tape must be 16-byte aligned");
    return DGB_EINVAL;
  }
  const bool field = args->field != nullptr && args->ve_amp != nullptr;
  const bool chan_planes = (args->flags & DGB_CABLE_UNIFORM_CHANNELS) == 0;
  const bool geo_planes = (args->flags & DGB_CABLE_UNIFORM_GEOMETRY) == 0;
  const bool planes = field || chan_planes || geo_planes;
  if constexpr (sizeof(T) == 4) {
    if (args->flags & DGB_CABLE_FAST_MATH)
      return planes ? launch_adjoint<T, true, true>(A, D, ch_max, st)
                    : launch_adjoint<T, true, false>(A, D, ch_max, st);
  }
  return planes ? launch_adjoint<T, false, true>(A, D, ch_max, st)
                : launch_adjoint<T, false, false>(A, D, ch_max, st);
}

// Sets this translation unit's tape-stage wait limit (polls < 0: the default).
template <typename T>
int cable_adjoint_wait_limit_t(int64_t polls) {
  const uint32_t v = polls < 0 ? kTapeWaitLimit
                               : (uint32_t)(polls > 0xffffffffll ? 0xffffffffll : polls);
  DGB_CUDA_CHECK(cudaMemcpyToSymbol(g_tape_wait_limit, &v, sizeof v));
  return DGB_OK;
}

#define DGB_INSTANTIATE_CABLE_ADJOINT(T)                                                \
  template int cable_adjoint_t<T>(const dgb_cable_args*, const dgb_cable_adjoint_args*, \
                                  int, cudaStream_t);                                   \
  template int cable_adjoint_wait_limit_t<T>(int64_t);

}  // namespace dgb
