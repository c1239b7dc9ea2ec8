// Register-resident tridiagonal solve for one system spread over a group of
// P lanes (P divides 32) with CH consecutive rows per lane.
//
// Lane r of the group owns rows [r*CH, r*CH + CH).  Row i reads
//   a_i x_{i-1} + b_i x_i + c_i x_{i+1} = d_i
// with a_0 = 0 and c_{last} = 0; rows past the end of a system are identity
// rows (a = c = 0, b = 1, d = 0).
//
// Algorithm (sub-structured Thomas + parallel cyclic reduction):
//  1. each lane eliminates its chunk sequentially, expressing every interior
//     row as x_j = d''_j - a''_j x_s - c''_j x_e in terms of its first (x_s)
//     and last (x_e) unknowns;
//  2. substituting the x_e rows leaves one tridiagonal row per lane in the
//     x_s unknowns, which the group solves by PCR with warp shuffles
//     (log2 P stages, no shared memory, no barriers);
//  3. x_e and the interior rows follow by back-substitution.
// The reference's sequential Thomas (tridiag/pcr.py:125-183,
// triton/t_kernel_thomas.py:13-80) and PCR (tridiag/pcr.py:4-96,
// triton/pcr_kernel_thomas.py:15-97) solve the same systems; results agree to
// rounding for the diagonally dominant cable matrices.
#pragma once

#include "common.cuh"

namespace dgb {

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int delta, int width) {
  return __shfl_up_sync(0xffffffffu, v, delta, width);
}
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int delta, int width) {
  return __shfl_down_sync(0xffffffffu, v, delta, width);
}

// Solve in place: on return d[j] holds x for the lane's rows.  a, b, c are
// clobbered.  All 32 lanes of the warp must call this together (groups of P).
// FAST selects the reciprocal (solve_rcp) and, in the reduction, multiplies
// by the neighbours' reciprocal pivots instead of dividing by their pivots.
template <typename T, int CH, int P, bool FAST = false>
__device__ __forceinline__ void chunk_solve(T (&a)[CH], T (&b)[CH], T (&c)[CH], T (&d)[CH],
                                            int r) {
  T As, Bs, Cs, Ds;  // reduced row of x_s
  T Ae, Ce, De;      // forward-form row of x_e (its diagonal is 1)
  if constexpr (CH == 1) {
    As = a[0];
    Bs = b[0];
    Cs = c[0];
    Ds = d[0];
    Ae = T(0);
    Ce = T(0);
    De = T(0);
  } else {
    // Forward sweep over rows 1..CH-1, in terms of x_s:
    //   x_j + ap_j x_s + cp_j x_{j+1} = dp_j   (stored in a, c, d)
    {
      T rinv = solve_rcp<T, FAST>(b[1]);
      a[1] = a[1] * rinv;
      c[1] = c[1] * rinv;
      d[1] = d[1] * rinv;
    }
#pragma unroll
    for (int j = 2; j < CH; ++j) {
      T rinv = solve_rcp<T, FAST>(b[j] - a[j] * c[j - 1]);
      T aj = a[j];
      a[j] = -aj * a[j - 1] * rinv;
      d[j] = (d[j] - aj * d[j - 1]) * rinv;
      c[j] = c[j] * rinv;
    }
    Ae = a[CH - 1];
    Ce = c[CH - 1];
    De = d[CH - 1];
    // Backward sweep over rows CH-3..1, in terms of x_s and x_e:
    //   x_j = d''_j - a''_j x_s - c''_j x_e   (stored in d, a, c)
#pragma unroll
    for (int j = CH - 3; j >= 1; --j) {
      T cj = c[j];
      d[j] = d[j] - cj * d[j + 1];
      a[j] = a[j] - cj * a[j + 1];
      c[j] = -cj * c[j + 1];
    }
    As = a[0];
    if constexpr (CH == 2) {
      Bs = b[0];
      Cs = c[0];
      Ds = d[0];
    } else {
      Bs = b[0] - c[0] * a[1];
      Cs = -c[0] * c[1];
      Ds = d[0] - c[0] * d[1];
    }
  }
  T al, be, ga, de;
  if constexpr (CH == 1) {
    // one row per lane: it already couples only the neighbouring lanes' rows
    al = As;
    be = Bs;
    ga = Cs;
    de = Ds;
    (void)Ae;
    (void)Ce;
    (void)De;
  } else {
    // Eliminate the x_e unknowns: one row per lane in x_s.
    T Ae_l = shfl_up<T>(Ae, 1, P);
    T Ce_l = shfl_up<T>(Ce, 1, P);
    T De_l = shfl_up<T>(De, 1, P);
    if (r == 0) {
      Ae_l = T(0);
      Ce_l = T(0);
      De_l = T(0);
    }
    al = -As * Ae_l;
    be = Bs - As * Ce_l - Cs * Ae;
    ga = -Cs * Ce;
    de = Ds - As * De_l - Cs * De;
  }
  // Parallel cyclic reduction across the P lanes.
#pragma unroll
  for (int s = 1; s < P; s <<= 1) {
    // FAST: the neighbours' pivots travel as reciprocals (one per lane)
    const T piv = FAST ? solve_rcp<T, FAST>(be) : be;
    T al_l = shfl_up<T>(al, s, P), be_l = shfl_up<T>(piv, s, P);
    T ga_l = shfl_up<T>(ga, s, P), de_l = shfl_up<T>(de, s, P);
    T al_r = shfl_down<T>(al, s, P), be_r = shfl_down<T>(piv, s, P);
    T ga_r = shfl_down<T>(ga, s, P), de_r = shfl_down<T>(de, s, P);
    const bool hl = r >= s;
    const bool hr = r + s < P;
    T k1 = hl ? (FAST ? al * be_l : al / be_l) : T(0);
    T k2 = hr ? (FAST ? ga * be_r : ga / be_r) : T(0);
    T al_n = hl ? -k1 * al_l : T(0);
    T ga_n = hr ? -k2 * ga_r : T(0);
    be = be - (hl ? k1 * ga_l : T(0)) - (hr ? k2 * al_r : T(0));
    de = de - (hl ? k1 * de_l : T(0)) - (hr ? k2 * de_r : T(0));
    al = al_n;
    ga = ga_n;
  }
  T xs = FAST ? de * solve_rcp<T, FAST>(be) : de / be;
  if constexpr (CH == 1) {
    d[0] = xs;
  } else {
    T xs_next = shfl_down<T>(xs, 1, P);
    if (r == P - 1) xs_next = T(0);
    T xe = De - Ae * xs - Ce * xs_next;
    d[0] = xs;
#pragma unroll
    for (int j = 1; j < CH - 1; ++j) d[j] = d[j] - a[j] * xs - c[j] * xe;
    d[CH - 1] = xe;
  }
}

}  // namespace dgb
