/*
 * CPU oracle for the Dendra cable update — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithms, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker
 * and CPU timing baseline.  It is never part of the product path.
 *
 * This file is included twice by oracle.c, once with REAL=double (suffix
 * _f64) and once with REAL=float (suffix _f32), so that both precisions
 * follow the reference's dtype-specific branches exactly.  It is compiled
 * with -ffp-contract=off so each operation rounds like the reference's
 * elementwise PyTorch kernels.
 *
 * Reference files (Dendra v0.30.1, paths relative to its source tree):
 *   rates   dendra/models/mod/HH.py:24-40, dendra/models/mechanisms/ops.py:13-125
 *   cnexp   dendra/models/mechanisms/_cnexp.py:46-132 (via ode.py:51-73)
 *   current dendra/models/mod/HH.py:109-116
 *   update  dendra/models/integrators/implicit.py:484-522 and :569-664
 *   thomas  dendra/models/integrators/tridiag/pcr.py:125-183
 *   pcr     dendra/models/integrators/tridiag/pcr.py:4-96
 *   dhs     dendra/models/integrators/triton/dhs_kernel.py:14-112
 *   pulse   dendra/models/stim/waveform/implementations.py:551-558,
 *           dendra/models/stim/waveform/_gates.py:50-65
 *   spikes  dendra/models/_threshold_callbacks.py:50-53
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define F(name) CAT(name, SFX)

/* Reciprocal-exprel even series (ops.py:13-44). */
static REAL F(even_series)(REAL q) {
  REAL q2 = q * q;
  REAL value;
  if (IS_F64) {
    value = q2 * (REAL)(43867.0 / 5109094217170944000.0) - (REAL)(3617.0 / 10670622842880000.0);
    value = value * q2 + (REAL)(1.0 / 74724249600.0);
    value = value * q2 - (REAL)(691.0 / 1307674368000.0);
    value = value * q2 + (REAL)(1.0 / 47900160.0);
  } else {
    value = q2 * (REAL)(-691.0 / 1307674368000.0) + (REAL)(1.0 / 47900160.0);
  }
  value = value * q2 - (REAL)(1.0 / 1209600.0);
  value = value * q2 + (REAL)(1.0 / 30240.0);
  value = value * q2 - (REAL)(1.0 / 720.0);
  value = value * q2 + (REAL)(1.0 / 12.0);
  return value;
}

/* vtrap(x, y) = x / (exp(x/y) - 1) with the local Bernoulli branch (ops.py:47-112). */
REAL F(orc_vtrap)(REAL x, REAL y) {
  REAL q = x / y;
  REAL thr = IS_F64 ? (REAL)0.5 : (REAL)1.0;
  if (FABS(q) <= thr) {
    REAL even = F(even_series)(q);
    return (y - x / (REAL)2) + x * (q * even);
  }
  return x / (EXP(q) - (REAL)1);
}

/* expm1(z)/z by Horner Taylor series for |z| <= 0.5 (_cnexp.py:46-93). */
REAL F(orc_phi1)(REAL z) {
  REAL value;
  if (IS_F64) {
    value = z * (REAL)(1.0 / 355687428096000.0) + (REAL)(1.0 / 20922789888000.0);
    value = value * z + (REAL)(1.0 / 1307674368000.0);
    value = value * z + (REAL)(1.0 / 87178291200.0);
    value = value * z + (REAL)(1.0 / 6227020800.0);
    value = value * z + (REAL)(1.0 / 479001600.0);
    value = value * z + (REAL)(1.0 / 39916800.0);
    value = value * z + (REAL)(1.0 / 3628800.0);
    value = value * z + (REAL)(1.0 / 362880.0);
  } else {
    value = z * (REAL)(1.0 / 3628800.0) + (REAL)(1.0 / 362880.0);
  }
  value = value * z + (REAL)(1.0 / 40320.0);
  value = value * z + (REAL)(1.0 / 5040.0);
  value = value * z + (REAL)(1.0 / 720.0);
  value = value * z + (REAL)(1.0 / 120.0);
  value = value * z + (REAL)(1.0 / 24.0);
  value = value * z + (REAL)(1.0 / 6.0);
  value = value * z + (REAL)(1.0 / 2.0);
  value = value * z + (REAL)1;
  return value;
}

/* Rate constants am1=0.1, ah1=0.07, an1=0.01 are held by the reference as
   float32 values even in a float64 model (its GLOBAL buffers are created in
   float32 and widened), so the oracle uses the float32-rounded values. */
#define AM1 ((REAL)0.1f)
#define AH1 ((REAL)0.07f)
#define AN1 ((REAL)0.01f)

/* HH rate pairs (source a, decay b) for m, h, n at voltage v (HH.py:24-40). */
void F(orc_hh_rates)(REAL v, REAL q10, REAL* out6) {
  REAL alpha_m = AM1 * F(orc_vtrap)(-(v + (REAL)40), (REAL)10);
  REAL beta_m = (REAL)4.0 * EXP(-(v + (REAL)65) / (REAL)18);
  REAL alpha_h = AH1 * EXP(-(v + (REAL)65) / (REAL)20);
  REAL beta_h = (REAL)1.0 / (EXP(-(v + (REAL)35) / (REAL)10) + (REAL)1);
  REAL alpha_n = AN1 * F(orc_vtrap)(-(v + (REAL)55), (REAL)10);
  REAL beta_n = (REAL)0.125 * EXP(-(v + (REAL)65) / (REAL)80);
  out6[0] = q10 * alpha_m;
  out6[1] = q10 * (alpha_m + beta_m);
  out6[2] = q10 * alpha_h;
  out6[3] = q10 * (alpha_h + beta_h);
  out6[4] = q10 * alpha_n;
  out6[5] = q10 * (alpha_n + beta_n);
}

/* Steady-state gates at v (HH.py:42-56). */
void F(orc_hh_steady)(REAL v, REAL* mhn) {
  REAL alpha_m = AM1 * F(orc_vtrap)(-(v + (REAL)40), (REAL)10);
  REAL beta_m = (REAL)4.0 * EXP(-(v + (REAL)65) / (REAL)18);
  REAL alpha_h = AH1 * EXP(-(v + (REAL)65) / (REAL)20);
  REAL beta_h = (REAL)1.0 / (EXP(-(v + (REAL)35) / (REAL)10) + (REAL)1);
  REAL alpha_n = AN1 * F(orc_vtrap)(-(v + (REAL)55), (REAL)10);
  REAL beta_n = (REAL)0.125 * EXP(-(v + (REAL)65) / (REAL)80);
  mhn[0] = alpha_m / (alpha_m + beta_m);
  mhn[1] = alpha_h / (alpha_h + beta_h);
  mhn[2] = alpha_n / (alpha_n + beta_n);
}

/* cnexp exact affine step of x' = a - b x over dt (_cnexp.py:96-132). */
REAL F(orc_cnexp)(REAL x, REAL a, REAL b, REAL dt) {
  REAL rate = a - b * x;
  REAL coef = -b;
  REAL z = coef * dt;
  if (FABS(z) <= (REAL)0.5) {
    return x + dt * rate * F(orc_phi1)(z);
  }
  REAL eq = -a / coef;
  return eq + (x - eq) * EXP(z);
}

/* Functional Thomas solve of one system (pcr.py:125-183).  a,c: K-1; b,d,x: K. */
void F(orc_thomas)(int64_t K, const REAL* a, const REAL* b, const REAL* c,
                   const REAL* d, REAL* x, REAL* work) {
  if (K == 1) {
    x[0] = d[0] / b[0];
    return;
  }
  REAL* cp = work;
  REAL* dp = work + K;
  REAL denom0 = b[0];
  cp[0] = c[0] / denom0;
  dp[0] = d[0] / denom0;
  for (int64_t i = 1; i < K; ++i) {
    REAL denom = b[i] - a[i - 1] * cp[i - 1];
    if (i < K - 1) cp[i] = c[i] / denom;
    dp[i] = (d[i] - a[i - 1] * dp[i - 1]) / denom;
  }
  x[K - 1] = dp[K - 1];
  for (int64_t i = K - 2; i >= 0; --i) x[i] = dp[i] - cp[i] * x[i + 1];
}

/* Batched Thomas over B row-major systems. */
void F(orc_thomas_batched)(int64_t B, int64_t K, const REAL* a, const REAL* b,
                           const REAL* c, const REAL* d, REAL* x) {
#pragma omp parallel
  {
    REAL* work = (REAL*)malloc(sizeof(REAL) * 2 * (size_t)(K > 0 ? K : 1));
#pragma omp for schedule(static)
    for (int64_t i = 0; i < B; ++i) {
      F(orc_thomas)(K, a + i * (K - 1), b + i * K, c + i * (K - 1), d + i * K,
                    x + i * K, work);
    }
    free(work);
  }
}

/* Parallel cyclic reduction with zero-padded shifted bands (pcr.py:4-96). */
void F(orc_pcr)(int64_t K, const REAL* a_in, const REAL* b_in, const REAL* c_in,
                const REAL* d_in, REAL* x) {
  if (K == 1) {
    x[0] = d_in[0] / b_in[0];
    return;
  }
  REAL* buf = (REAL*)malloc(sizeof(REAL) * 8 * (size_t)K);
  REAL *a = buf, *b = buf + K, *c = buf + 2 * K, *d = buf + 3 * K;
  REAL *an = buf + 4 * K, *bn = buf + 5 * K, *cn = buf + 6 * K, *dn = buf + 7 * K;
  a[0] = 0;
  for (int64_t i = 1; i < K; ++i) a[i] = a_in[i - 1];
  for (int64_t i = 0; i < K - 1; ++i) c[i] = c_in[i];
  c[K - 1] = 0;
  for (int64_t i = 0; i < K; ++i) {
    b[i] = b_in[i];
    d[i] = d_in[i];
  }
  for (int64_t s = 1; s < K; s <<= 1) {
    for (int64_t i = 0; i < K; ++i) {
      REAL alpha = (i >= s) ? -a[i] / b[i - s] : (REAL)0;
      REAL beta = (i + s < K) ? -c[i] / b[i + s] : (REAL)0;
      REAL a_left = (i >= s) ? a[i - s] : (REAL)0;
      REAL c_left = (i >= s) ? c[i - s] : (REAL)0;
      REAL d_left = (i >= s) ? d[i - s] : (REAL)0;
      REAL a_right = (i + s < K) ? a[i + s] : (REAL)0;
      REAL c_right = (i + s < K) ? c[i + s] : (REAL)0;
      REAL d_right = (i + s < K) ? d[i + s] : (REAL)0;
      an[i] = alpha * a_left;
      bn[i] = b[i] + alpha * c_left + beta * a_right;
      cn[i] = beta * c_right;
      dn[i] = d[i] + alpha * d_left + beta * d_right;
    }
    REAL* t;
    t = a; a = an; an = t;
    t = b; b = bn; bn = t;
    t = c; c = cn; cn = t;
    t = d; d = dn; dn = t;
  }
  for (int64_t i = 0; i < K; ++i) x[i] = d[i] / b[i];
  free(buf);
}

/* 3x3 inverse by cofactors over the determinant. */
static void F(inv3)(const REAL* a, REAL* v) {
  REAL c0 = a[4] * a[8] - a[5] * a[7];
  REAL c3 = a[5] * a[6] - a[3] * a[8];
  REAL c6 = a[3] * a[7] - a[4] * a[6];
  REAL det = a[0] * c0 + a[1] * c3 + a[2] * c6;
  REAL r = (REAL)1 / det;
  v[0] = c0 * r;
  v[1] = (a[2] * a[7] - a[1] * a[8]) * r;
  v[2] = (a[1] * a[5] - a[2] * a[4]) * r;
  v[3] = c3 * r;
  v[4] = (a[0] * a[8] - a[2] * a[6]) * r;
  v[5] = (a[2] * a[3] - a[0] * a[5]) * r;
  v[6] = c6 * r;
  v[7] = (a[1] * a[6] - a[0] * a[7]) * r;
  v[8] = (a[0] * a[4] - a[1] * a[3]) * r;
}

/* Block Thomas for 3x3 main blocks and diagonal off-diagonal blocks, the
 * algorithm of the reference's thomas_bt3_kernel (triton/bt_kernel.py:38-170):
 *   P_k = main_k - diag(lower_{k-1}) P_{k-1}^{-1} diag(upper_{k-1}),
 *   r_k = rhs_k - diag(lower_{k-1}) P_{k-1}^{-1} r_{k-1},
 *   x_k = P_k^{-1} (r_k - diag(upper_k) x_{k+1}).
 * lower, upper (B, K-1, 3); main (B, K, 3, 3); rhs, x (B, K, 3). */
void F(orc_block3_thomas)(int64_t B, int64_t K, const REAL* lower, const REAL* mainb,
                          const REAL* upper, const REAL* rhs, REAL* x) {
#pragma omp parallel
  {
    REAL* pinv = (REAL*)malloc(sizeof(REAL) * 9 * (size_t)K);
    REAL* r = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)K);
#pragma omp for schedule(static)
    for (int64_t b = 0; b < B; ++b) {
      const REAL* lo = lower + b * (K - 1) * 3;
      const REAL* up = upper + b * (K - 1) * 3;
      const REAL* mb = mainb + b * K * 9;
      const REAL* rb = rhs + b * K * 3;
      REAL* xb = x + b * K * 3;
      F(inv3)(mb, pinv);
      for (int q = 0; q < 3; ++q) r[q] = rb[q];
      for (int64_t k = 1; k < K; ++k) {
        const REAL* pp = pinv + (k - 1) * 9;
        REAL m[9];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j)
            m[i * 3 + j] = mb[k * 9 + i * 3 + j] - lo[(k - 1) * 3 + i] * (pp[i * 3 + j] * up[(k - 1) * 3 + j]);
        for (int i = 0; i < 3; ++i) {
          REAL w = pp[i * 3] * r[(k - 1) * 3] + pp[i * 3 + 1] * r[(k - 1) * 3 + 1] +
                   pp[i * 3 + 2] * r[(k - 1) * 3 + 2];
          r[k * 3 + i] = rb[k * 3 + i] - lo[(k - 1) * 3 + i] * w;
        }
        F(inv3)(m, pinv + k * 9);
      }
      for (int64_t k = K - 1; k >= 0; --k) {
        REAL d[3];
        for (int i = 0; i < 3; ++i)
          d[i] = r[k * 3 + i] - (k + 1 < K ? up[k * 3 + i] * xb[(k + 1) * 3 + i] : (REAL)0);
        const REAL* pp = pinv + k * 9;
        for (int i = 0; i < 3; ++i)
          xb[k * 3 + i] = pp[i * 3] * d[0] + pp[i * 3 + 1] * d[1] + pp[i * 3 + 2] * d[2];
      }
    }
    free(r);
    free(pinv);
  }
}

/* Rectangular pulse gate on [delay, delay+pw) at time t (_gates.py:50-65).
   The reference forms the time grid and delay+pw in the state dtype, so a
   float64 reference run of a float32 run evaluates the gate in float32 (gate_f32). */
static REAL F(rect)(double t0_ms, int32_t s, double dt_ms, REAL amp, REAL delay, REAL pw,
                    int32_t gate_f32) {
  if (gate_f32) {
    float t = (float)(t0_ms + (double)s * dt_ms);
    float d = (float)delay, stop = (float)delay + (float)pw;
    return (t >= d && t < stop) ? amp : (REAL)0;
  }
  REAL t = (REAL)(t0_ms + (double)s * dt_ms);
  REAL stop = delay + pw;
  return (t >= delay && t < stop) ? amp : (REAL)0;
}

/* Read-only description of a packed cable problem (mirrors dgb_cable_args). */
typedef struct {
  const int64_t* cable_ptr;
  const REAL *g_right, *g_left, *scale, *cm_inv, *field;
  const REAL *gnabar, *gkbar, *gl, *el;
  REAL ena, ek, q10, dt, dt_s;
  double dt_ms_d, t0_ms;
  const REAL *ve_amp, *ve_delay, *ve_pw;
  const int32_t* in_idx;
  const REAL *in_amp, *in_delay, *in_pw;
  int32_t gate_f32;
} F(cable_prob);

/* One backward-Euler step of cable c (the update of implicit.py:569-664 after
   the gate advance of integrators/core.py:769-834).  w: 10*kmax workspace. */
static void F(cable_step)(const F(cable_prob)* P, int32_t c, int32_t s, REAL* vv, REAL* mm,
                          REAL* hh, REAL* nn, REAL* w, int64_t kmax) {
  const int64_t o = P->cable_ptr[c];
  const int64_t K = P->cable_ptr[c + 1] - o;
  const REAL *g_right = P->g_right, *g_left = P->g_left, *scale = P->scale;
  REAL* lower = w;
  REAL* mainv = w + kmax;
  REAL* upper = w + 2 * kmax;
  REAL* rhs = w + 3 * kmax;
  REAL* x = w + 4 * kmax;
  REAL* fn = w + 5 * kmax;
  REAL* G = w + 6 * kmax;
  REAL* ve = w + 7 * kmax;
  REAL* work = w + 8 * kmax;
  const REAL dt = P->dt, dt_s = P->dt_s;
  /* stimulus time of this step: binary64 grid cast to the state dtype */
  const int use_ve = P->field && P->ve_amp;
  if (use_ve) {
    REAL I = F(rect)(P->t0_ms, s, P->dt_ms_d, P->ve_amp[c], P->ve_delay[c], P->ve_pw[c],
                     P->gate_f32);
    for (int64_t i = 0; i < K; ++i) ve[i] = P->field[o + i] * I;
  }
  for (int64_t i = 0; i < K; ++i) {
    REAL vi = vv[i];
    REAL r[6];
    F(orc_hh_rates)(vi, P->q10, r);
    mm[i] = F(orc_cnexp)(mm[i], r[0], r[1], dt);
    hh[i] = F(orc_cnexp)(hh[i], r[2], r[3], dt);
    nn[i] = F(orc_cnexp)(nn[i], r[4], r[5], dt);
    REAL m3 = mm[i] * mm[i] * mm[i];
    REAL n4 = (nn[i] * nn[i]) * (nn[i] * nn[i]);
    REAL gna = P->gnabar[o + i] * m3 * hh[i];
    REAL gk = P->gkbar[o + i] * n4;
    REAL Gi = P->gl[o + i] + gna + gk;
    REAL Ji = P->gl[o + i] * P->el[o + i] + gna * P->ena + gk * P->ek;
    G[i] = Gi;
    fn[i] = (Ji - Gi * vi) * scale[o + i];
  }
  if (K > 1) {
    for (int64_t i = 0; i < K; ++i) {
      REAL ax = (REAL)0;
      if (i == 0) {
        ax = g_right[o] * (vv[1] - vv[0]);
      } else if (i == K - 1) {
        ax = -(g_left[o + i] * (vv[i] - vv[i - 1]));
      } else {
        ax = g_right[o + i] * (vv[i + 1] - vv[i]) - g_left[o + i] * (vv[i] - vv[i - 1]);
      }
      fn[i] = fn[i] + ax;
    }
    if (use_ve) {
      for (int64_t i = 0; i < K; ++i) {
        REAL ex;
        if (i == 0) {
          ex = g_right[o] * (ve[1] - ve[0]);
        } else if (i == K - 1) {
          ex = -(g_left[o + i] * (ve[i] - ve[i - 1]));
        } else {
          ex = g_right[o + i] * (ve[i + 1] - ve[i]) - g_left[o + i] * (ve[i] - ve[i - 1]);
        }
        fn[i] = fn[i] + ex;
      }
    }
  }
  if (P->in_idx && P->in_amp && P->in_idx[c] >= 0) {
    int32_t ii = P->in_idx[c];
    REAL I = F(rect)(P->t0_ms, s, P->dt_ms_d, P->in_amp[c], P->in_delay[c], P->in_pw[c],
                     P->gate_f32);
    for (int64_t i = 0; i < K; ++i) {
      REAL inj = (i == ii) ? I : (REAL)0;
      fn[i] = fn[i] + inj * P->cm_inv[o + i];
    }
  }
  for (int64_t i = 0; i < K; ++i) {
    REAL diag_base = -g_right[o + i] + -g_left[o + i];
    rhs[i] = dt_s * fn[i];
    mainv[i] = (REAL)1 - dt_s * (diag_base - G[i] * scale[o + i]);
    if (i < K - 1) upper[i] = -dt_s * g_right[o + i];
    if (i > 0) lower[i - 1] = -dt_s * g_left[o + i];
  }
  if (K == 1) {
    x[0] = rhs[0] / mainv[0];
  } else {
    F(orc_thomas)(K, lower, mainv, upper, rhs, x, work);
  }
  for (int64_t i = 0; i < K; ++i) vv[i] = vv[i] + x[i];
}

static int64_t F(max_cable)(int32_t n_cables, const int64_t* cable_ptr) {
  int64_t kmax = 1;
  for (int32_t c = 0; c < n_cables; ++c) {
    int64_t K = cable_ptr[c + 1] - cable_ptr[c];
    if (K > kmax) kmax = K;
  }
  return kmax;
}

/*
 * Multi-step backward-Euler HH cable run, all cables packed by cable_ptr.
 * Arguments mirror dgb_cable_args.
 */
void F(orc_cable_run)(int32_t n_cables, int32_t n_steps, int32_t rec_every,
                      const int64_t* cable_ptr, REAL* v, REAL* m, REAL* h, REAL* n,
                      const REAL* g_right, const REAL* g_left, const REAL* scale,
                      const REAL* cm_inv, const REAL* field, const REAL* gnabar,
                      const REAL* gkbar, const REAL* gl, const REAL* el, double ena_d,
                      double ek_d, double q10_d, double dt_ms_d, double dt_s_d,
                      double t0_ms, const REAL* ve_amp, const REAL* ve_delay,
                      const REAL* ve_pw, const int32_t* in_idx, const REAL* in_amp,
                      const REAL* in_delay, const REAL* in_pw, const int32_t* rec_idx,
                      REAL* trace, const int32_t* spk_idx, double spk_thr_d,
                      int32_t* spk_below, int32_t* spk_count, int32_t* spk_first,
                      int32_t gate_f32, const int32_t* spk_idx2, int32_t* spk_below2,
                      REAL* trace_all, int32_t n_rast, const int32_t* rast_idx,
                      int32_t* rast_below, int32_t* rast_count, int32_t rast_cap,
                      int64_t* rast_steps, int64_t step0) {
  const F(cable_prob) P = {cable_ptr, g_right, g_left, scale, cm_inv, field, gnabar, gkbar, gl,
                           el, (REAL)ena_d, (REAL)ek_d, (REAL)q10_d, (REAL)dt_ms_d,
                           (REAL)dt_s_d, dt_ms_d, t0_ms, ve_amp, ve_delay, ve_pw, in_idx,
                           in_amp, in_delay, in_pw, gate_f32};
  const REAL thr = (REAL)spk_thr_d;
  const int64_t n_rec = 1 + (int64_t)n_steps / (rec_every > 0 ? rec_every : 1);
  const int64_t kmax = F(max_cable)(n_cables, cable_ptr);
#pragma omp parallel
  {
    REAL* w = (REAL*)malloc(sizeof(REAL) * 10 * (size_t)kmax);
#pragma omp for schedule(dynamic, 1)
    for (int32_t c = 0; c < n_cables; ++c) {
      const int64_t o = cable_ptr[c];
      REAL* vv = v + o;
      REAL *mm = m + o, *hh = h + o, *nn = n + o;
      const int32_t ri = rec_idx ? rec_idx[c] : -1;
      const int32_t si = spk_idx ? spk_idx[c] : -1;
      const int32_t si2 = spk_idx2 ? spk_idx2[c] : -1;
      if (trace && ri >= 0) trace[(int64_t)c * n_rec] = vv[ri];
      const int64_t Kc = cable_ptr[c + 1] - o;
      if (trace_all)
        for (int64_t i = 0; i < Kc; ++i) trace_all[o + i] = vv[i];
      for (int32_t s = 0; s < n_steps; ++s) {
        F(cable_step)(&P, c, s, vv, mm, hh, nn, w, kmax);
        if (si >= 0) {
          /* a rising edge at either detection compartment counts once */
          int above = vv[si] >= thr;
          int edge = above && spk_below[c];
          spk_below[c] = !above;
          if (si2 >= 0) {
            int above2 = vv[si2] >= thr;
            edge = edge || (above2 && spk_below2[c]);
            spk_below2[c] = !above2;
          }
          if (edge) {
            if (spk_count[c] == 0) spk_first[c] = s + 1;
            spk_count[c] += 1;
          }
        }
        if (trace && ri >= 0 && ((s + 1) % rec_every) == 0)
          trace[(int64_t)c * n_rec + (s + 1) / rec_every] = vv[ri];
        /* Raster / threshold_crossing: every upward crossing at each checked
           compartment, with its absolute step */
        for (int32_t q = 0; q < n_rast; ++q) {
          const int64_t e = (int64_t)c * n_rast + q;
          const int32_t ci = rast_idx[e];
          if (ci < 0 || ci >= Kc) continue;
          const int above = vv[ci] >= thr;
          if (above && rast_below[e]) {
            if (rast_count[e] < rast_cap) rast_steps[e * rast_cap + rast_count[e]] = step0 + s + 1;
            rast_count[e] += 1;
          }
          rast_below[e] = !above;
        }
        if (trace_all && ((s + 1) % rec_every) == 0) {
          REAL* row = trace_all + (int64_t)((s + 1) / rec_every) * cable_ptr[n_cables] + o;
          for (int64_t i = 0; i < Kc; ++i) row[i] = vv[i];
        }
      }
    }
    free(w);
  }
}

/* ---- reverse mode -------------------------------------------------------
 * Derivatives of the gate advance on the branch the forward takes (the same
 * branch tests as orc_vtrap, orc_phi1 and orc_cnexp).  The reference obtains
 * them by torch autograd through those operations. */

/* d/du of the even series (u = q^2). */
static REAL F(even_series_du)(REAL q) {
  REAL u = q * q;
  REAL value;
  if (IS_F64) {
    value = u * (REAL)(8.0 * 43867.0 / 5109094217170944000.0)
            - (REAL)(7.0 * 3617.0 / 10670622842880000.0);
    value = value * u + (REAL)(6.0 / 74724249600.0);
    value = value * u - (REAL)(5.0 * 691.0 / 1307674368000.0);
    value = value * u + (REAL)(4.0 / 47900160.0);
  } else {
    value = u * (REAL)(-5.0 * 691.0 / 1307674368000.0) + (REAL)(4.0 / 47900160.0);
  }
  value = value * u - (REAL)(3.0 / 1209600.0);
  value = value * u + (REAL)(2.0 / 30240.0);
  value = value * u - (REAL)(1.0 / 720.0);
  return value;
}

static REAL F(vtrap_dx)(REAL x, REAL y) {
  REAL q = x / y;
  REAL thr = IS_F64 ? (REAL)0.5 : (REAL)1.0;
  if (FABS(q) <= thr) {
    REAL u = q * q;
    return (REAL)-0.5 + (REAL)2 * q * F(even_series)(q) + (REAL)2 * q * u * F(even_series_du)(q);
  }
  REAL e = EXP(q);
  REAL em1 = e - (REAL)1;
  return (em1 - x * e / y) / (em1 * em1);
}

/* d/dz of the phi1 Taylor polynomial: sum_k k z^(k-1) / (k+1)!. */
static REAL F(phi1_dz)(REAL z) {
  const int N = IS_F64 ? 16 : 9;
  double inv[18];
  inv[0] = 1.0;
  for (int k = 1; k <= 17; ++k) inv[k] = inv[k - 1] / (double)k; /* 1/k! */
  REAL value = (REAL)(N * inv[N + 1]);
  for (int k = N - 1; k >= 1; --k) value = value * z + (REAL)(k * inv[k + 1]);
  return value;
}

/* x' = cnexp(x, a, b, dt) with dx'/dx, dx'/da, dx'/db. */
static REAL F(cnexp_d)(REAL x, REAL a, REAL b, REAL dt, REAL* dx, REAL* da, REAL* db) {
  REAL rate = a - b * x;
  REAL coef = -b;
  REAL z = coef * dt;
  if (FABS(z) <= (REAL)0.5) {
    REAL ph = F(orc_phi1)(z);
    *dx = (REAL)1 - dt * b * ph;
    *da = dt * ph;
    *db = dt * (-x) * ph - dt * rate * F(phi1_dz)(z) * dt;
    return x + dt * rate * ph;
  }
  REAL E = EXP(z);
  REAL eq = -a / coef;
  *dx = E;
  *da = ((REAL)1 - E) / b;
  *db = -(a / (b * b)) * ((REAL)1 - E) - (x - eq) * E * dt;
  return eq + (x - eq) * E;
}

/* Gate advance at v with partials d(new)/d(old) (dg[0..2]) and d(new)/dv (dg[3..5]). */
static void F(gates_d)(REAL v, REAL q10, REAL dt, REAL* mhn, REAL* dg) {
  REAL xm = -(v + (REAL)40), xn = -(v + (REAL)55);
  REAL alpha_m = AM1 * F(orc_vtrap)(xm, (REAL)10);
  REAL beta_m = (REAL)4.0 * EXP(-(v + (REAL)65) / (REAL)18);
  REAL alpha_h = AH1 * EXP(-(v + (REAL)65) / (REAL)20);
  REAL eh = EXP(-(v + (REAL)35) / (REAL)10);
  REAL beta_h = (REAL)1.0 / (eh + (REAL)1);
  REAL alpha_n = AN1 * F(orc_vtrap)(xn, (REAL)10);
  REAL beta_n = (REAL)0.125 * EXP(-(v + (REAL)65) / (REAL)80);
  REAL d_am = -AM1 * F(vtrap_dx)(xm, (REAL)10), d_bm = -beta_m / (REAL)18;
  REAL d_ah = -alpha_h / (REAL)20, d_bh = eh / ((REAL)10 * (eh + (REAL)1) * (eh + (REAL)1));
  REAL d_an = -AN1 * F(vtrap_dx)(xn, (REAL)10), d_bn = -beta_n / (REAL)80;
  REAL a[3] = {q10 * alpha_m, q10 * alpha_h, q10 * alpha_n};
  REAL b[3] = {q10 * (alpha_m + beta_m), q10 * (alpha_h + beta_h), q10 * (alpha_n + beta_n)};
  REAL da_v[3] = {q10 * d_am, q10 * d_ah, q10 * d_an};
  REAL db_v[3] = {q10 * (d_am + d_bm), q10 * (d_ah + d_bh), q10 * (d_an + d_bn)};
  for (int k = 0; k < 3; ++k) {
    REAL dx, da, db;
    mhn[k] = F(cnexp_d)(mhn[k], a[k], b[k], dt, &dx, &da, &db);
    dg[k] = dx;
    dg[3 + k] = da * da_v[k] + db * db_v[k];
  }
}

/*
 * Gradient of a recorded trace functional: runs the forward of orc_cable_run
 * keeping the whole state tape in memory, then the reverse sweep.
 *   trace_grad: (n_cables, n_rec) dLoss/dtrace for the trace orc_cable_run
 *               records with the same arguments.
 *   out: lam_v/m/h/n (n_comp) adjoint of the initial state; g_gna, g_gk, g_gl
 *        (n_comp) dLoss/d(gnabar, gkbar, gl); g_ax (n_comp) lam_g * g over
 *        both axial bands of each row.  v/m/h/n are left at the final state.
 */
void F(orc_cable_grad)(int32_t n_cables, int32_t n_steps, int32_t rec_every,
                       const int64_t* cable_ptr, REAL* v, REAL* m, REAL* h, REAL* n,
                       const REAL* g_right, const REAL* g_left, const REAL* scale,
                       const REAL* cm_inv, const REAL* field, const REAL* gnabar,
                       const REAL* gkbar, const REAL* gl, const REAL* el, double ena_d,
                       double ek_d, double q10_d, double dt_ms_d, double dt_s_d,
                       double t0_ms, const REAL* ve_amp, const REAL* ve_delay,
                       const REAL* ve_pw, const int32_t* in_idx, const REAL* in_amp,
                       const REAL* in_delay, const REAL* in_pw, const int32_t* rec_idx,
                       const REAL* trace_grad, int32_t gate_f32, REAL* lam_v, REAL* lam_m,
                       REAL* lam_h, REAL* lam_n, REAL* g_gna, REAL* g_gk, REAL* g_gl,
                       REAL* g_ax) {
  const F(cable_prob) P = {cable_ptr, g_right, g_left, scale, cm_inv, field, gnabar, gkbar, gl,
                           el, (REAL)ena_d, (REAL)ek_d, (REAL)q10_d, (REAL)dt_ms_d,
                           (REAL)dt_s_d, dt_ms_d, t0_ms, ve_amp, ve_delay, ve_pw, in_idx,
                           in_amp, in_delay, in_pw, gate_f32};
  const REAL dt = P.dt, dt_s = P.dt_s, ena = P.ena, ek = P.ek;
  const int64_t n_rec = 1 + (int64_t)n_steps / (rec_every > 0 ? rec_every : 1);
  const int64_t kmax = F(max_cable)(n_cables, cable_ptr);
#pragma omp parallel
  {
    REAL* w = (REAL*)malloc(sizeof(REAL) * 20 * (size_t)kmax);
    REAL* tape = (REAL*)malloc(sizeof(REAL) * 4 * (size_t)kmax * ((size_t)n_steps + 1));
#pragma omp for schedule(dynamic, 1)
    for (int32_t c = 0; c < n_cables; ++c) {
      const int64_t o = cable_ptr[c];
      const int64_t K = cable_ptr[c + 1] - o;
      REAL *vv = v + o, *mm = m + o, *hh = h + o, *nn = n + o;
      for (int32_t s = 0; s <= n_steps; ++s) {
        REAL* t = tape + (size_t)s * 4 * K;
        if (s > 0) F(cable_step)(&P, c, s - 1, vv, mm, hh, nn, w, kmax);
        for (int64_t i = 0; i < K; ++i) {
          t[i] = vv[i];
          t[K + i] = mm[i];
          t[2 * K + i] = hh[i];
          t[3 * K + i] = nn[i];
        }
      }
      REAL *lv = lam_v + o, *lm = lam_m + o, *lh = lam_h + o, *ln = lam_n + o;
      REAL *gga = g_gna + o, *ggk = g_gk + o, *ggl = g_gl + o;
      REAL* gax = g_ax + o;
      for (int64_t i = 0; i < K; ++i)
        lv[i] = lm[i] = lh[i] = ln[i] = gga[i] = ggk[i] = ggl[i] = gax[i] = 0;
      REAL *mu = w, *bb = w + kmax, *lo = w + 2 * kmax, *up = w + 3 * kmax, *G = w + 4 * kmax;
      REAL *gm = w + 5 * kmax, *gh = w + 6 * kmax, *gn = w + 7 * kmax, *dg = w + 8 * kmax;
      REAL *ve = w + 14 * kmax, *work = w + 15 * kmax, *lfn = w + 17 * kmax;
      const int32_t ri = rec_idx ? rec_idx[c] : -1;
      const int use_ve = field && ve_amp;
      for (int32_t s = n_steps - 1; s >= 0; --s) {
        const REAL* t = tape + (size_t)s * 4 * K;
        const REAL* vn = tape + (size_t)(s + 1) * 4 * K;
        if (trace_grad && ri >= 0 && ((s + 1) % rec_every) == 0)
          lv[ri] += trace_grad[(int64_t)c * n_rec + (s + 1) / rec_every];
        REAL I = 0;
        if (use_ve) {
          I = F(rect)(t0_ms, s, dt_ms_d, ve_amp[c], ve_delay[c], ve_pw[c], gate_f32);
          for (int64_t i = 0; i < K; ++i) ve[i] = field[o + i] * I;
        }
        for (int64_t i = 0; i < K; ++i) {
          REAL mhn[3] = {t[K + i], t[2 * K + i], t[3 * K + i]};
          REAL d6[6];
          F(gates_d)(t[i], P.q10, dt, mhn, d6);
          gm[i] = mhn[0];
          gh[i] = mhn[1];
          gn[i] = mhn[2];
          for (int k = 0; k < 6; ++k) dg[k * kmax + i] = d6[k];
          REAL m3 = mhn[0] * mhn[0] * mhn[0];
          REAL n4 = (mhn[2] * mhn[2]) * (mhn[2] * mhn[2]);
          G[i] = gl[o + i] + gnabar[o + i] * m3 * mhn[1] + gkbar[o + i] * n4;
          bb[i] = (REAL)1 - dt_s * ((-g_right[o + i] + -g_left[o + i]) - G[i] * scale[o + i]);
        }
        /* transposed bands: row i couples to i-1 through the forward's upper
           band of row i-1 and to i+1 through the lower band of row i+1 */
        for (int64_t i = 0; i + 1 < K; ++i) {
          lo[i] = -dt_s * g_right[o + i];
          up[i] = -dt_s * g_left[o + i + 1];
        }
        if (K == 1) {
          mu[0] = lv[0] / bb[0];
        } else {
          F(orc_thomas)(K, lo, bb, up, lv, mu, work);
        }
        for (int64_t i = 0; i < K; ++i) lfn[i] = dt_s * mu[i];
        for (int64_t i = 0; i < K; ++i) {
          const REAL vi = t[i];
          const REAL x = vn[i] - vi;
          const REAL v_p = i > 0 ? t[i - 1] : (REAL)0, v_n = i + 1 < K ? t[i + 1] : (REAL)0;
          const REAL x_p = i > 0 ? vn[i - 1] - v_p : (REAL)0;
          const REAL x_n = i + 1 < K ? vn[i + 1] - v_n : (REAL)0;
          const REAL gr = g_right[o + i], glf = g_left[o + i], scl = scale[o + i];
          REAL dvr = v_n - vi, dvl = vi - v_p;
          if (use_ve) {
            const REAL ve_l = i > 0 ? ve[i - 1] : (REAL)0, ve_r = i + 1 < K ? ve[i + 1] : (REAL)0;
            dvr = dvr + (ve_r - ve[i]);
            dvl = dvl + (ve[i] - ve_l);
          }
          const REAL lb = -mu[i] * x, la = -mu[i] * x_p, lc = -mu[i] * x_n;
          const REAL lgr = dt_s * (lb - lc) + dvr * lfn[i];
          const REAL lglf = dt_s * (lb - la) - dvl * lfn[i];
          gax[i] += lgr * gr + lglf * glf;
          const REAL lG = dt_s * scl * lb - vi * scl * lfn[i];
          const REAL lJ = scl * lfn[i];
          const REAL mq = gm[i], hq = gh[i], nq = gn[i];
          const REAL lgna = lG + ena * lJ, lgk = lG + ek * lJ;
          gga[i] += mq * mq * mq * hq * lgna;
          ggk[i] += (nq * nq) * (nq * nq) * lgk;
          ggl[i] += lG + el[o + i] * lJ;
          const REAL lmq = lm[i] + (REAL)3 * gnabar[o + i] * mq * mq * hq * lgna;
          const REAL lhq = lh[i] + gnabar[o + i] * mq * mq * mq * lgna;
          const REAL lnq = ln[i] + (REAL)4 * gkbar[o + i] * nq * nq * nq * lgk;
          REAL lvi = lv[i] - (G[i] * scl + gr + glf) * lfn[i];
          if (i > 0) lvi += g_right[o + i - 1] * lfn[i - 1];
          if (i + 1 < K) lvi += g_left[o + i + 1] * lfn[i + 1];
          lvi += dg[3 * kmax + i] * lmq + dg[4 * kmax + i] * lhq + dg[5 * kmax + i] * lnq;
          lm[i] = dg[i] * lmq;
          lh[i] = dg[kmax + i] * lhq;
          ln[i] = dg[2 * kmax + i] * lnq;
          lv[i] = lvi;
        }
      }
      if (trace_grad && ri >= 0) lv[ri] += trace_grad[(int64_t)c * n_rec];
    }
    free(tape);
    free(w);
  }
}

/*
 * Sequential DHS/Hines solve of one tree in solver order: layers
 * layer_ptr[0..L] list nodes deepest first; parent[] uses the same indices
 * (dhs_kernel.py:45-112, executed one node at a time).
 */
void F(orc_dhs_solve)(int64_t K, const REAL* d_in, const REAL* a, const REAL* b_in,
                      const int32_t* parent, const int32_t* order,
                      const int32_t* layer_ptr, int32_t n_layers, REAL* x) {
  REAL* D = (REAL*)malloc(sizeof(REAL) * 2 * (size_t)K);
  REAL* Bv = D + K;
  for (int64_t i = 0; i < K; ++i) {
    D[i] = d_in[i];
    Bv[i] = b_in[i];
  }
  for (int32_t l = 0; l < n_layers; ++l) {
    for (int32_t o = layer_ptr[l]; o < layer_ptr[l + 1]; ++o) {
      int32_t i = order[o];
      REAL g = a[i];
      REAL old_d = D[i];
      REAL di = old_d + g;
      D[i] = di;
      int32_t p = parent[i];
      if (p >= 0) {
        REAL fac = -g * ((REAL)1 / di);
        D[p] = D[p] + (-fac * old_d);
        Bv[p] = Bv[p] + (-fac * Bv[i]);
      }
    }
  }
  for (int32_t l = n_layers - 1; l >= 0; --l) {
    for (int32_t o = layer_ptr[l]; o < layer_ptr[l + 1]; ++o) {
      int32_t i = order[o];
      int32_t p = parent[i];
      REAL vp = p >= 0 ? x[p] : (REAL)0;
      x[i] = (Bv[i] + a[i] * vp) / D[i];
    }
  }
  free(D);
}

void F(orc_dhs_solve_batched)(int64_t B, int64_t K, const REAL* d, const REAL* a,
                              const REAL* b, const int32_t* parent, const int32_t* order,
                              const int32_t* layer_ptr, int32_t n_layers, REAL* x) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < B; ++i)
    F(orc_dhs_solve)(K, d + i * K, a + i * K, b + i * K, parent, order, layer_ptr,
                     n_layers, x + i * K);
}


/*
 * Network of branched cells, one step at a time (networks/net.py:214-240,
 * netcon.py:5183-5205, integrators/tree.py:1202-1357):
 *   deliver ring row slot into Exp2Syn A, B (A += w factor, B += w factor) and
 *   clear it; background event adds bg_weight to synapse bg_syn; detect the
 *   soma rising edge on v; enqueue weight at (slot + delay) % depth for every
 *   connection of a spiking source (connection order); decay A, B; soma HH
 *   gates; assemble f = (J - G v) area - axial flows, main = cm/dt + G area;
 *   sequential DHS solve; v += dv.  Arrays follow dgb_net_args (host memory).
 */
void F(orc_net_run)(int32_t n_cells, int32_t n_steps, int64_t step0, int64_t depth,
                    int64_t* slot_io, int64_t n_syn, const int64_t* node_ptr,
                    const int32_t* plan_of, const int64_t* plan_node_ptr,
                    const int64_t* plan_layer_off, const int32_t* parent, const int32_t* order,
                    const int32_t* layer_ptr, const int32_t* child_ptr, const int32_t* child_idx,
                    REAL* v, const REAL* area, const REAL* cm_dt, const REAL* a_geom,
                    const REAL* gl, const REAL* el, REAL* m, REAL* h, REAL* n, double gnabar_d,
                    double gkbar_d, double ena_d, double ek_d, double q10_d, double dt_d,
                    double thr_d, const int64_t* syn_ptr, const int32_t* node_syn_ptr,
                    REAL* syn_A, REAL* syn_B, const REAL* syn_factor, const REAL* decay_A,
                    const REAL* decay_B, double e_syn_d, REAL* ring, const uint64_t* bg_bits,
                    int64_t bg_words, int32_t bg_syn, double bg_weight_d, int64_t n_conn,
                    const int64_t* conn_pre, const int64_t* conn_post, const int64_t* conn_delay,
                    const REAL* conn_weight, uint8_t* below, int32_t* spike_count,
                    uint8_t* raster /* [n_steps][n_cells] or NULL */,
                    const REAL* ve_field, const REAL* ve_amp, const REAL* ve_delay,
                    const REAL* ve_pw, const int32_t* in_node, const REAL* in_amp,
                    const REAL* in_delay, const REAL* in_pw, double t0_ms) {
  const REAL gnabar = (REAL)gnabar_d, gkbar = (REAL)gkbar_d, ena = (REAL)ena_d, ek = (REAL)ek_d;
  const REAL q10 = (REAL)q10_d, dt = (REAL)dt_d, thr = (REAL)thr_d, e_syn = (REAL)e_syn_d;
  const REAL bg_weight = (REAL)bg_weight_d;
  int64_t kmax = 1;
  for (int32_t c = 0; c < n_cells; ++c)
    if (node_ptr[c + 1] - node_ptr[c] > kmax) kmax = node_ptr[c + 1] - node_ptr[c];
  REAL* main_ = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)kmax);
  REAL* rhs = main_ + kmax;
  REAL* x = rhs + kmax;
  uint8_t* spiked = (uint8_t*)malloc((size_t)(n_cells > 0 ? n_cells : 1));
  int64_t slot = *slot_io;
  for (int32_t s = 0; s < n_steps; ++s) {
    const int64_t g = step0 + s;
    REAL* row = ring + slot * n_syn;
    /* 1. deliver */
    for (int32_t c = 0; c < n_cells; ++c) {
      const int bg = bg_bits && ((bg_bits[g * bg_words + (c >> 6)] >> (c & 63)) & 1ull);
      for (int64_t k = syn_ptr[c]; k < syn_ptr[c + 1]; ++k) {
        REAL w = row[k];
        row[k] = (REAL)0;
        if (bg && k - syn_ptr[c] == bg_syn) w = w + bg_weight;
        if (w != (REAL)0) {
          REAL inc = w * syn_factor[k];
          syn_A[k] = syn_A[k] + inc;
          syn_B[k] = syn_B[k] + inc;
        }
      }
    }
    /* 2. detect on the previous step's soma v, enqueue in connection order */
    for (int32_t c = 0; c < n_cells; ++c) {
      int above = v[node_ptr[c]] >= thr;
      spiked[c] = (uint8_t)(above && below[c]);
      below[c] = (uint8_t)!above;
      if (spiked[c]) spike_count[c] += 1;
      if (raster) raster[(int64_t)s * n_cells + c] = spiked[c];
    }
    for (int64_t e = 0; e < n_conn; ++e) {
      if (!spiked[conn_pre[e]]) continue;
      int64_t r = (slot + conn_delay[e]) % depth;
      ring[r * n_syn + conn_post[e]] = ring[r * n_syn + conn_post[e]] + conn_weight[e];
    }
    /* 3-4. advance and solve every cell */
    for (int32_t c = 0; c < n_cells; ++c) {
      const int64_t base = node_ptr[c];
      const int32_t K = (int32_t)(node_ptr[c + 1] - base);
      const int32_t p = plan_of ? plan_of[c] : c;
      const int64_t pn = plan_node_ptr[p], pl = plan_layer_off[p];
      const int32_t* par = parent + pn;
      const int32_t* cptr = child_ptr + pn + p;
      const int32_t* cidx = child_idx + pn;
      const int32_t* nsp = node_syn_ptr + base + c;
      const int64_t s0 = syn_ptr[c];
      for (int64_t k = syn_ptr[c]; k < syn_ptr[c + 1]; ++k) {
        syn_A[k] = syn_A[k] * decay_A[k];
        syn_B[k] = syn_B[k] * decay_B[k];
      }
      {
        REAL r6[6];
        F(orc_hh_rates)(v[base], q10, r6);
        m[c] = F(orc_cnexp)(m[c], r6[0], r6[1], dt);
        h[c] = F(orc_cnexp)(h[c], r6[2], r6[3], dt);
        n[c] = F(orc_cnexp)(n[c], r6[4], r6[5], dt);
      }
      for (int32_t i = 0; i < K; ++i) {
        const REAL vi = v[base + i];
        REAL G, J;
        if (i == 0) {
          REAL m3 = m[c] * m[c] * m[c];
          REAL n2 = n[c] * n[c];
          REAL gna = gnabar * m3 * h[c];
          REAL gk = gkbar * (n2 * n2);
          G = gl[base] + gna + gk;
          J = gl[base] * el[base] + gna * ena + gk * ek;
        } else {
          G = gl[base + i];
          J = gl[base + i] * el[base + i];
        }
        const REAL ar = area[base + i];
        for (int32_t k = nsp[i]; k < nsp[i + 1]; ++k) {
          REAL gs = (syn_B[s0 + k] - syn_A[s0 + k]) / ((REAL)1e6 * ar);
          G = G + gs;
          J = J + gs * e_syn;
        }
        REAL f = (J - G * vi) * ar;
        if (par[i] >= 0) f = f - a_geom[base + i] * (vi - v[base + par[i]]);
        for (int32_t k = cptr[i]; k < cptr[i + 1]; ++k) {
          int32_t ch = cidx[k];
          f = f + a_geom[base + ch] * (v[base + ch] - vi);
        }
        /* extracellular edge currents g (ve_child - ve_parent), summed on
           their own, then the injected current (tree.py:1262-1302) */
        if (ve_field && ve_amp) {
          const REAL I = F(rect)(t0_ms, g, dt_d, ve_amp[c], ve_delay[c], ve_pw[c], 0);
          if (I != (REAL)0) {
            const REAL vei = ve_field[base + i] * I;
            REAL S = (REAL)0;
            if (par[i] >= 0) S = S - a_geom[base + i] * (vei - ve_field[base + par[i]] * I);
            for (int32_t k = cptr[i]; k < cptr[i + 1]; ++k) {
              int32_t ch = cidx[k];
              S = S + a_geom[base + ch] * (ve_field[base + ch] * I - vei);
            }
            f = f + S;
          }
        }
        if (in_node && in_amp && in_node[c] == i)
          f = f + F(rect)(t0_ms, g, dt_d, in_amp[c], in_delay[c], in_pw[c], 0);
        rhs[i] = f;
        main_[i] = cm_dt[base + i] + G * ar;
      }
      F(orc_dhs_solve)(K, main_, a_geom + base, rhs, par, order + pn, layer_ptr + pl,
                       (int32_t)(plan_layer_off[p + 1] - pl - 1), x);
      for (int32_t i = 0; i < K; ++i) v[base + i] = v[base + i] + x[i];
    }
    slot = (slot + 1) % depth;
  }
  *slot_io = slot;
  free(main_);
  free(spiked);
}

/* ---------------------------------------------------------------------------
 * Interpolated delay transport on a dense ring [depth][width]:
 *   enqueue  networks/_two_tap_enqueue_cpu.cpp:26-126 (ordered_two_tap_enqueue)
 *            and networks/_event_delivery.py:229-308 (taps 2 and 3)
 *   vjp      networks/_two_tap_enqueue_cpu.cpp:235-315 / _two_tap_enqueue.py:94-150
 * ------------------------------------------------------------------------- */

/* Gate of edge e (pre: per source, else per edge); -1 for a bad source. */
static int F(tap_gate)(const REAL* g, const int64_t* pre, int64_t n_src, int64_t e, REAL* out) {
  int64_t s = e;
  if (pre) {
    s = pre[e];
    if (s < 0 || s >= n_src) return -1;
  }
  *out = g[s];
  return 0;
}

/* One step in place.  Row slot -> payload (if non-null), cleared; every edge in
 * order adds (w g)(1 - f) at (slot*width + lower) mod size, then every edge in
 * order (w g) f at its upper address.  Returns 0, or -1 when an address, a
 * source index or the slot is out of range (the reference's TORCH_CHECKs). */
int F(orc_two_tap_enqueue)(int64_t depth, int64_t width, REAL* ring, int64_t slot,
                           int64_t n_edges, const REAL* w, const REAL* g, const int64_t* pre,
                           int64_t n_src, const REAL* f, const int64_t* lower,
                           const int64_t* upper, REAL* payload) {
  const int64_t size = depth * width;
  if (slot < 0 || slot >= depth) return -1;
  const int64_t start = slot * width, tail = size - start;
  for (int64_t c = 0; c < width; ++c) {
    if (payload) payload[c] = ring[start + c];
    ring[start + c] = 0;
  }
  for (int tap = 0; tap < 2; ++tap) {
    const int64_t* addr = tap ? upper : lower;
    for (int64_t e = 0; e < n_edges; ++e) {
      const int64_t base = addr[e];
      REAL ge;
      if (base < 0 || base >= size || F(tap_gate)(g, pre, n_src, e, &ge)) return -1;
      const int64_t d = base < tail ? start + base : base - tail;
      const REAL wg = w[e] * ge;
      const REAL share = tap ? f[e] : (REAL)1 - f[e];
      ring[d] = ring[d] + wg * share;
    }
  }
  return 0;
}

/* Three taps: every edge in order, taps 0..2, at
 * ((slot + offsets[e][t]) mod depth) * width + post[e], value (w g) coeff[e][t]. */
int F(orc_three_tap_enqueue)(int64_t depth, int64_t width, REAL* ring, int64_t slot,
                             int64_t n_edges, const REAL* w, const REAL* g, const int64_t* pre,
                             int64_t n_src, const REAL* coeff, const int64_t* offsets,
                             const int64_t* post, REAL* payload) {
  if (slot < 0 || slot >= depth) return -1;
  for (int64_t c = 0; c < width; ++c) {
    if (payload) payload[c] = ring[slot * width + c];
    ring[slot * width + c] = 0;
  }
  for (int64_t e = 0; e < n_edges; ++e) {
    REAL ge;
    if (post[e] < 0 || post[e] >= width || F(tap_gate)(g, pre, n_src, e, &ge)) return -1;
    const REAL wg = w[e] * ge;
    for (int t = 0; t < 3; ++t) {
      int64_t r = (slot + offsets[3 * e + t]) % depth;
      if (r < 0) r += depth;
      const int64_t d = r * width + post[e];
      ring[d] = ring[d] + wg * coeff[3 * e + t];
    }
  }
  return 0;
}

static int64_t F(wrap_tap)(int64_t base, int64_t offset, int64_t size) {
  int64_t r = (int64_t)((uint64_t)base + (uint64_t)offset) % size;
  return r < 0 ? r + size : r;
}

/* Cotangents of weights, gates and fractions from the ring cotangent R read
 * at the two taps (offset = slot*width).  With pre, dg[s] sums its edges'
 * values in edge order from +0. */
void F(orc_two_tap_vjp)(int64_t size, const REAL* R, int64_t offset, int64_t n_edges,
                        const REAL* w, const REAL* g, const int64_t* pre, int64_t n_src,
                        const REAL* f, const int64_t* lower, const int64_t* upper, REAL* dw,
                        REAL* dg, REAL* df) {
  if (pre)
    for (int64_t s = 0; s < n_src; ++s) dg[s] = 0;
  for (int64_t e = 0; e < n_edges; ++e) {
    int64_t s = e;
    if (pre) {
      s = pre[e];
      if (s < 0) s += n_src;
    }
    const REAL lo = R[F(wrap_tap)(lower[e], offset, size)];
    const REAL hi = R[F(wrap_tap)(upper[e], offset, size)];
    const REAL dweighted = hi * f[e] + lo * ((REAL)1 - f[e]);
    const REAL weighted = w[e] * g[s];
    dw[e] = dweighted * g[s];
    df[e] = hi * weighted - lo * weighted;
    const REAL gg = dweighted * w[e];
    if (pre)
      dg[s] = dg[s] + gg;
    else
      dg[e] = gg;
  }
}

/* n_steps enqueue steps from slot0, gates[k] of stride n_src (pre) or n_edges,
 * payload[k][width]. */
int F(orc_two_tap_rollout)(int64_t depth, int64_t width, REAL* ring, int64_t slot0,
                           int64_t n_steps, int64_t n_edges, const REAL* w, const REAL* gates,
                           const int64_t* pre, int64_t n_src, const REAL* f,
                           const int64_t* lower, const int64_t* upper, REAL* payload) {
  const int64_t stride = pre ? n_src : n_edges;
  for (int64_t k = 0; k < n_steps; ++k) {
    if (F(orc_two_tap_enqueue)(depth, width, ring, (slot0 + k) % depth, n_edges, w,
                               gates + k * stride, pre, n_src, f, lower, upper,
                               payload ? payload + k * width : 0))
      return -1;
  }
  return 0;
}

/* Reverse of orc_two_tap_rollout, newest step first: per step the VJP at the
 * cotangent R of the ring after the step (dw, df accumulated newest first,
 * stored at the newest step), then R[row slot_k] = gpay[k]. */
void F(orc_two_tap_rollout_vjp)(int64_t depth, int64_t width, REAL* R, int64_t slot0,
                                int64_t n_steps, int64_t n_edges, const REAL* w,
                                const REAL* gates, const int64_t* pre, int64_t n_src,
                                const REAL* f, const int64_t* lower, const int64_t* upper,
                                const REAL* gpay, REAL* dw, REAL* dgates, REAL* df) {
  const int64_t stride = pre ? n_src : n_edges;
  REAL* tw = (REAL*)malloc(sizeof(REAL) * (size_t)(n_edges + 1));
  REAL* tf = (REAL*)malloc(sizeof(REAL) * (size_t)(n_edges + 1));
  for (int64_t k = n_steps - 1; k >= 0; --k) {
    const int64_t slot = (slot0 + k) % depth;
    F(orc_two_tap_vjp)(depth * width, R, slot * width, n_edges, w, gates + k * stride, pre,
                       n_src, f, lower, upper, tw, dgates + k * stride, tf);
    for (int64_t e = 0; e < n_edges; ++e) {
      dw[e] = (k == n_steps - 1) ? tw[e] : dw[e] + tw[e];
      df[e] = (k == n_steps - 1) ? tf[e] : df[e] + tf[e];
    }
    for (int64_t c = 0; c < width; ++c) R[slot * width + c] = gpay ? gpay[k * width + c] : 0;
  }
  free(tw);
  free(tf);
}

/* ---------------------------------------------------------------------------
 * NetStim renewal (networks/_netstim_renewal.py:70-159) with counter-based
 * draws: Philox4x32-10 (Salmon et al., SC'11), E = -ln(U) by the atanh series
 * in double precision with rounded operations only (same draws as the GPU).
 * ------------------------------------------------------------------------- */
static void F(philox4x32_10)(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = (uint32_t)p1;
    c[2] = n2;
    c[3] = (uint32_t)p0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

void F(orc_philox4x32_10)(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  for (int i = 0; i < 4; ++i) out[i] = ctr[i];
  F(philox4x32_10)(out, key[0], key[1]);
}

double F(orc_series_log)(double x) {
  int e = 0;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  const double s = (m - 1.0) / (m + 1.0);
  const double s2 = s * s;
  double p = 1.0 / 23.0;
  p = p * s2 + 1.0 / 21.0;
  p = p * s2 + 1.0 / 19.0;
  p = p * s2 + 1.0 / 17.0;
  p = p * s2 + 1.0 / 15.0;
  p = p * s2 + 1.0 / 13.0;
  p = p * s2 + 1.0 / 11.0;
  p = p * s2 + 1.0 / 9.0;
  p = p * s2 + 1.0 / 7.0;
  p = p * s2 + 1.0 / 5.0;
  p = p * s2 + 1.0 / 3.0;
  p = p * s2 + 1.0;
  const double lm = (2.0 * s) * p;
  return (double)e * 0.69314718055994530942 + lm;
}

REAL F(orc_unit_exponential)(uint64_t seed, uint64_t step, uint32_t gen, uint32_t stream) {
  uint32_t c[4] = {(uint32_t)step, gen, stream, (uint32_t)(step >> 32)};
  F(philox4x32_10)(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  double u;
  if (IS_F64) {
    const uint64_t b = ((uint64_t)c[0] << 21) ^ (uint64_t)(c[1] >> 11);
    u = ((double)(b & ((1ull << 53) - 1)) + 0.5) * 1.1102230246251565e-16;
  } else {
    u = ((double)(c[0] >> 8) + 0.5) * 5.9604644775390625e-08;
  }
  return (REAL)(-F(orc_series_log)(u));
}

void F(orc_netstim_init)(int64_t n, const REAL* interval, const REAL* noise, const REAL* start,
                         int32_t any_noise, uint64_t seed, const REAL* draws, REAL* next,
                         int64_t* counts) {
  for (int64_t g = 0; g < n; ++g) {
    REAL clock = start[g];
    if (any_noise) {
      const REAL E = draws ? draws[g] : F(orc_unit_exponential)(seed, 0, (uint32_t)g, 1u);
      clock = clock + (noise[g] * interval[g]) * E;
    }
    next[g] = clock;
    counts[g] = 0;
  }
}

void F(orc_netstim_run)(int64_t n, int64_t n_steps, int64_t step0, double t0, double dt,
                        const REAL* interval, const REAL* noise, const int64_t* number,
                        uint64_t seed, const REAL* draws, REAL* next, int64_t* counts,
                        uint8_t* spikes) {
  const REAL T0 = (REAL)t0, DT = (REAL)dt;
  for (int64_t g = 0; g < n; ++g) {
    REAL clock = next[g];
    int64_t count = counts[g];
    const int64_t cap = number ? number[g] : INT64_MAX;
    const REAL a = interval[g] * ((REAL)1 - noise[g]), b = interval[g] * noise[g];
    for (int64_t k = 0; k < n_steps; ++k) {
      const int64_t step = step0 + k;
      const REAL t = T0 + (REAL)step * DT;
      const REAL E = draws ? draws[k * n + g]
                           : F(orc_unit_exponential)(seed, (uint64_t)step, (uint32_t)g, 0u);
      const int fire = (t >= clock) && count < cap;
      const REAL gate = fire ? (REAL)1 : (REAL)0;
      const REAL nxt = a + b * E;
      clock = clock + (nxt * gate) * gate;
      count += fire;
      if (spikes) spikes[k * n + g] = (uint8_t)fire;
    }
    next[g] = clock;
    counts[g] = count;
  }
}

#undef AM1
#undef AH1
#undef AN1
#undef F
