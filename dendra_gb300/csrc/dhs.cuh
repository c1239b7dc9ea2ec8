// Deterministic DHS / Hines elimination of one tree by one warp.
//
// Row i of the tree system (nodes in solver order, parent p(i), axial
// conductance g_i to the parent, g_root = 0 acts as extra diagonal):
//   (d_i + g_i + sum_{c child of i} g_c) x_i - g_i x_p(i) - sum_c g_c x_c = b_i
// Elimination leaves -> root by depth layers (layer_ptr over order, deepest
// layer first), back substitution root -> leaves.  The reference kernel
// (triton/dhs_kernel.py:14-112) pushes each child's Schur contribution into
// its parent with floating-point atomics; here every node pulls its
// children's contributions in a fixed child order, so results are
// deterministic and need no atomics:
//   D_i = d_i + sum_c (g_c / (D_c + g_c)) D_c,  B_i = b_i + sum_c (g_c / (D_c + g_c)) B_c
//   x_i = (B_i + g_i x_p(i)) / (D_i + g_i)
// D and B live in shared memory (2 K values per tree); x overwrites B.
#pragma once

#include "common.cuh"

namespace dgb {

template <typename I>
struct TreeTopoT {
  const I* parent;     // [K] local parent (root: -1 for int32, 0xFFFF for uint16)
  const I* order;      // [K] nodes, deepest layer first
  const I* layer_ptr;  // [L+1] layer boundaries in order
  const I* child_ptr;  // [K+1] children CSR
  const I* child_idx;  // [K-1]
  int32_t K, L;
};
using TreeTopo = TreeTopoT<int32_t>;

__device__ __forceinline__ bool has_parent(int32_t p) { return p >= 0; }
__device__ __forceinline__ bool has_parent(uint16_t p) { return p != 0xFFFFu; }

// Synchronisation of the threads that solve one tree: a warp, or a group of
// warps meeting at named barrier `id` (1..15) with `count` threads.
struct WarpSync {
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
struct GroupSync {
  int id, count;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};


// sD, sB: shared arrays of K values holding d and b on entry; g: axial
// conductances of this tree (global or shared).  On return sB holds x.
// FAST (float only): solve_rcp reciprocals, x = (b + g x_p) * rcp(d + g) in
// the substitution, exactly as the FAST chain schedule below computes them.
template <typename T, typename I, int W = 32, class Sync = WarpSync, bool FAST = false>
__device__ __forceinline__ void dhs_eliminate(const TreeTopoT<I>& t, const T* g, T* sD, T* sB,
                                              int lane, Sync sync = Sync()) {
  for (int l = 0; l < t.L; ++l) {
    const int lo = t.layer_ptr[l], hi = t.layer_ptr[l + 1];
    for (int o = lo + lane; o < hi; o += W) {
      const int i = t.order[o];
      T D = sD[i], Bv = sB[i];
      const int c0 = t.child_ptr[i], c1 = t.child_ptr[i + 1];
      for (int k = c0; k < c1; ++k) {
        const int c = t.child_idx[k];
        const T gc = g[c];
        const T Dc = sD[c];
        const T f = gc * solve_rcp<T, FAST>(Dc + gc);
        D = D + f * Dc;
        Bv = Bv + f * sB[c];
      }
      sD[i] = D;
      sB[i] = Bv;
    }
    sync();
  }
}

template <typename T, typename I, int W = 32, class Sync = WarpSync, bool FAST = false>
__device__ __forceinline__ void dhs_substitute(const TreeTopoT<I>& t, const T* g, T* sD, T* sB,
                                               int lane, Sync sync = Sync()) {
  for (int l = t.L - 1; l >= 0; --l) {
    const int lo = t.layer_ptr[l], hi = t.layer_ptr[l + 1];
    for (int o = lo + lane; o < hi; o += W) {
      const int i = t.order[o];
      const I p = t.parent[i];
      const T gi = g[i];
      const T xp = has_parent(p) ? sB[p] : T(0);
      sB[i] = FAST ? (sB[i] + gi * xp) * solve_rcp<T, FAST>(sD[i] + gi)
                   : (sB[i] + gi * xp) / (sD[i] + gi);
    }
    sync();
  }
}

// Chain schedule of the same elimination.  A chain is a maximal unbranched
// path: its top is the root or a child of a branch node, every node above its
// bottom has exactly one child (the next node down), and its bottom is a leaf
// or a branch node.  Chains are listed bottom -> top (nodes), chain after
// chain (chain_ptr), grouped by level (level_ptr): a level-0 chain ends in a
// leaf, a level-l chain ends in a branch node whose child chains all have
// lower levels.  One lane eliminates a whole chain with the recurrence in
// registers (no shared-memory round trip or warp synchronisation per node);
// the warp synchronises once per level.  Every node performs exactly the
// operations of dhs_eliminate / dhs_substitute, so the results are identical.
template <typename I>
struct ChainTopoT {
  const I* nodes;      // [K]
  const I* chain_ptr;  // [n_chains + 1]
  const I* level_ptr;  // [n_levels + 1]
  int32_t n_levels;
};

// lane: index of the thread among the W threads solving this tree.  FAST
// (float only) takes the reciprocals as solve_rcp's refined approximation and,
// in the substitution, multiplies by the next node's reciprocal pivot, which
// is formed one node ahead, off the recurrence's critical path.
template <typename T, typename I, int W = 32, class Sync = WarpSync, bool FAST = false>
__device__ __forceinline__ void chain_eliminate(const TreeTopoT<I>& t, const ChainTopoT<I>& c,
                                                const T* g, T* sD, T* sB, int lane,
                                                Sync sync = Sync()) {
  for (int l = 0; l < c.n_levels; ++l) {
    const int c1 = c.level_ptr[l + 1];
    for (int ch = c.level_ptr[l] + lane; ch < c1; ch += W) {
      const int p = c.chain_ptr[ch], e = c.chain_ptr[ch + 1];
      int i = c.nodes[p];
      // the walk's first node j (the bottom's parent) and the index after it,
      // with j's values, are loaded before the bottom's own work: the bottom
      // writes only itself, so they do not wait on it (chains are disjoint)
      int q = p + 1;
      int j = q < e ? c.nodes[q] : 0;
      int jn = q + 1 < e ? c.nodes[q + 1] : 0;
      T dj = T(0), bj = T(0), gj = T(0);
      if (q < e) {
        dj = sD[j];
        bj = sB[j];
        gj = g[j];
      }
      T gc = g[i];
      T D = sD[i], Bv = sB[i];
      const int k0 = t.child_ptr[i], k1 = t.child_ptr[i + 1];
      // the bottom's children (the tops of lower chains): the first two are
      // loaded together, so their divisions overlap; the sums keep the child
      // order
      if (k1 > k0) {
        const bool two = k1 > k0 + 1;
        const int ca = t.child_idx[k0];
        const int cb = two ? t.child_idx[k0 + 1] : ca;
        const T ga = g[ca], Da = sD[ca], Ba = sB[ca];
        const T gb = g[cb], Db = sD[cb], Bb = sB[cb];
        const T fa = ga * solve_rcp<T, FAST>(Da + ga);
        const T fb = gb * solve_rcp<T, FAST>(Db + gb);
        D = D + fa * Da;
        Bv = Bv + fa * Ba;
        if (two) {
          D = D + fb * Db;
          Bv = Bv + fb * Bb;
        }
        for (int k = k0 + 2; k < k1; ++k) {
          const int cc = t.child_idx[k];
          const T gc = g[cc];
          const T Dc = sD[cc];
          const T f = gc * solve_rcp<T, FAST>(Dc + gc);
          D = D + f * Dc;
          Bv = Bv + f * sB[cc];
        }
      }
      sD[i] = D;
      sB[i] = Bv;
      // up the chain (the single child of node j is the node below it); the
      // next node's values and the index after it are loaded ahead, before
      // this node's division and stores, so neither load waits on the other
      for (; q < e; ++q) {
        const int jnn = q + 2 < e ? c.nodes[q + 2] : 0;
        T dn = T(0), bn = T(0), gn = T(0);
        if (q + 1 < e) {
          dn = sD[jn];
          bn = sB[jn];
          gn = g[jn];
        }
        const T f = gc * solve_rcp<T, FAST>(D + gc);
        D = dj + f * D;
        Bv = bj + f * Bv;
        sD[j] = D;
        sB[j] = Bv;
        gc = gj;
        j = jn;
        jn = jnn;
        dj = dn;
        bj = bn;
        gj = gn;
      }
    }
    sync();
  }
}

template <typename T, typename I, int W = 32, class Sync = WarpSync, bool FAST = false>
__device__ __forceinline__ void chain_substitute(const TreeTopoT<I>& t, const ChainTopoT<I>& c,
                                                 const T* g, T* sD, T* sB, int lane,
                                                 Sync sync = Sync()) {
  for (int l = c.n_levels - 1; l >= 0; --l) {
    const int c1 = c.level_ptr[l + 1];
    for (int ch = c.level_ptr[l] + lane; ch < c1; ch += W) {
      const int p = c.chain_ptr[ch], e = c.chain_ptr[ch + 1];
      const I par = t.parent[c.nodes[e - 1]];
      T xp = has_parent(par) ? sB[par] : T(0);
      // down the chain from its top: the next node's values and the index
      // after it loaded ahead
      int j = c.nodes[e - 1];
      int jn = e - 2 >= p ? c.nodes[e - 2] : 0;
      T bj = sB[j], dj = sD[j], gj = g[j];
      T rj = FAST ? solve_rcp<T, FAST>(dj + gj) : T(0);
      for (int q = e - 1; q >= p; --q) {
        const int jnn = q - 2 >= p ? c.nodes[q - 2] : 0;
        T bn = T(0), dn = T(0), gn = T(0);
        if (q > p) {
          bn = sB[jn];
          dn = sD[jn];
          gn = g[jn];
        }
        const T rn = FAST ? solve_rcp<T, FAST>(dn + gn) : T(0);
        xp = FAST ? (bj + gj * xp) * rj : (bj + gj * xp) / (dj + gj);
        sB[j] = xp;
        j = jn;
        jn = jnn;
        bj = bn;
        dj = dn;
        gj = gn;
        rj = rn;
      }
    }
    sync();
  }
}

}  // namespace dgb
