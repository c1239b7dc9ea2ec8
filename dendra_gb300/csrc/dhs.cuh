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

// sD, sB: shared arrays of K values holding d and b on entry; g: axial
// conductances of this tree (global or shared).  On return sB holds x.
template <typename T, typename I>
__device__ __forceinline__ void dhs_eliminate(const TreeTopoT<I>& t, const T* g, T* sD, T* sB,
                                              int lane) {
  for (int l = 0; l < t.L; ++l) {
    const int lo = t.layer_ptr[l], hi = t.layer_ptr[l + 1];
    for (int o = lo + lane; o < hi; o += 32) {
      const int i = t.order[o];
      T D = sD[i], Bv = sB[i];
      const int c0 = t.child_ptr[i], c1 = t.child_ptr[i + 1];
      for (int k = c0; k < c1; ++k) {
        const int c = t.child_idx[k];
        const T gc = g[c];
        const T Dc = sD[c];
        const T f = gc * (T(1) / (Dc + gc));
        D = D + f * Dc;
        Bv = Bv + f * sB[c];
      }
      sD[i] = D;
      sB[i] = Bv;
    }
    __syncwarp();
  }
}

template <typename T, typename I>
__device__ __forceinline__ void dhs_substitute(const TreeTopoT<I>& t, const T* g, T* sD, T* sB,
                                               int lane) {
  for (int l = t.L - 1; l >= 0; --l) {
    const int lo = t.layer_ptr[l], hi = t.layer_ptr[l + 1];
    for (int o = lo + lane; o < hi; o += 32) {
      const int i = t.order[o];
      const I p = t.parent[i];
      const T gi = g[i];
      const T xp = has_parent(p) ? sB[p] : T(0);
      sB[i] = (sB[i] + gi * xp) / (sD[i] + gi);
    }
    __syncwarp();
  }
}

}  // namespace dgb
