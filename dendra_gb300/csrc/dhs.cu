// Tree (DHS/Hines) solves: dgb_dhs_solve (one topology, B trees) and
// dgb_dhs_solve_forest (many topologies, one launch).
//
// Replaces dhs_solve_cuda (triton/dhs_kernel.py:634-651, kernels :14-212) and
// dhs_solve_multi_cuda (triton/dhs_kernel_multi.py:831-888).  One warp per
// tree; a tree's D/B accumulators live in shared memory; elimination and
// back substitution follow dhs.cuh (deterministic, no atomics).
#include "dhs.cuh"

namespace dgb {

struct ForestArgsT {
  int32_t n_trees;
  // single shared topology (dgb_dhs_solve): every tree uses the plan arrays
  // directly, trees packed at t * shared_k, shared_l layers
  int32_t shared_k, shared_l;
  const int64_t* node_ptr;
  const int32_t* plan_of;
  const int64_t* plan_node_ptr;
  const int64_t* plan_layer_off;
  const int32_t* parent;
  const int32_t* order;
  const int32_t* layer_ptr;
  const int32_t* child_ptr;
  const int32_t* child_idx;
  // optional per-tree node counts (row-padded planes: tree t's K_t nodes
  // start at node_ptr[t]); NULL: K_t = node_ptr[t+1] - node_ptr[t]
  const int32_t* tree_k;
  // optional chain schedule of every plan (dgb_forest's chain arrays)
  const int64_t* plan_chain_off;
  const int64_t* plan_clevel_off;
  const int32_t* chain_nodes;
  const int32_t* chain_ptr;
  const int32_t* chain_level;
};

__device__ __forceinline__ TreeTopo forest_topo(const ForestArgsT& F, int plan, int K) {
  TreeTopo t;
  if (F.shared_k > 0) {
    t.parent = F.parent;
    t.order = F.order;
    t.layer_ptr = F.layer_ptr;
    t.child_ptr = F.child_ptr;
    t.child_idx = F.child_idx;
    t.K = K;
    t.L = F.shared_l;
    return t;
  }
  const int64_t pn = F.plan_node_ptr[plan];
  const int64_t pl = F.plan_layer_off[plan];
  t.parent = F.parent + pn;
  t.order = F.order + pn;
  t.layer_ptr = F.layer_ptr + pl;
  t.child_ptr = F.child_ptr + pn + plan;  // K+1 entries per plan
  t.child_idx = F.child_idx + pn;
  t.K = K;
  t.L = (int)(F.plan_layer_off[plan + 1] - pl - 1);
  return t;
}

template <typename T>
__global__ void __launch_bounds__(128) dhs_forest_kernel(ForestArgsT F, const T* __restrict__ d,
                                                         const T* __restrict__ g,
                                                         const T* __restrict__ b, T* __restrict__ x,
                                                         int kmax, T* __restrict__ work) {
  // work == nullptr: the accumulators in shared memory; else each warp's
  // 2*kmax values in the global workspace (trees too large for shared memory)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  T* sD = (work ? work + (size_t)blockIdx.x * wpb * 2 * kmax : reinterpret_cast<T*>(smem_raw)) +
          (size_t)warp * 2 * kmax;
  T* sB = sD + kmax;
  for (int tree = blockIdx.x * wpb + warp; tree < F.n_trees; tree += gridDim.x * wpb) {
    const int64_t base = F.shared_k > 0 ? (int64_t)tree * F.shared_k : F.node_ptr[tree];
    const int K = F.shared_k > 0 ? F.shared_k
                  : (F.tree_k ? F.tree_k[tree] : (int)(F.node_ptr[tree + 1] - base));
    const int plan = F.shared_k > 0 ? 0 : (F.plan_of ? F.plan_of[tree] : tree);
    const TreeTopo t = forest_topo(F, plan, K);
    for (int i = lane; i < K; i += 32) {
      sD[i] = d[base + i];
      sB[i] = b[base + i];
    }
    __syncwarp();
    if (F.chain_nodes && F.shared_k == 0) {
      // chain schedule: one lane per unbranched chain, a sync per chain level
      // (the same operations per node as the layer schedule)
      const int64_t pn = F.plan_node_ptr[plan];
      const int64_t cp0 = F.plan_chain_off[plan], cl0 = F.plan_clevel_off[plan];
      const ChainTopoT<int32_t> ct{F.chain_nodes + pn, F.chain_ptr + cp0, F.chain_level + cl0,
                                   (int32_t)(F.plan_clevel_off[plan + 1] - cl0 - 1)};
      chain_eliminate<T, int32_t>(t, ct, g + base, sD, sB, lane);
      chain_substitute<T, int32_t>(t, ct, g + base, sD, sB, lane);
    } else {
      dhs_eliminate<T, int32_t>(t, g + base, sD, sB, lane);
      dhs_substitute<T, int32_t>(t, g + base, sD, sB, lane);
    }
    for (int i = lane; i < K; i += 32) x[base + i] = sB[i];
    __syncwarp();
  }
}

template <typename T>
static int forest_launch(const ForestArgsT& F, int kmax, const void* d, const void* g,
                         const void* b, void* x, cudaStream_t st) {
  const size_t per_warp = (size_t)2 * kmax * sizeof(T);
  int wpb = 4;
  while (wpb > 1 && wpb * per_warp > 227 * 1024) wpb >>= 1;
  // a tree too large for shared memory: the same program on a stream-ordered
  // global workspace, four warps per block, four blocks per SM
  const bool global = wpb * per_warp > 227 * 1024;
  if (global) wpb = 4;
  const size_t smem = global ? 0 : wpb * per_warp;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(dhs_forest_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dhs_forest_kernel<T>,
                                                               wpb * 32, smem));
  if (per_sm < 1) per_sm = 1;
  if (global) per_sm = 4;
  int blocks = device_sm_count() * per_sm;
  const int need = (F.n_trees + wpb - 1) / wpb;
  if (blocks > need) blocks = need;
  T* work = nullptr;
  if (global) DGB_CUDA_CHECK(cudaMallocAsync((void**)&work, (size_t)blocks * wpb * per_warp, st));
  dhs_forest_kernel<T><<<blocks, wpb * 32, smem, st>>>(F, (const T*)d, (const T*)g, (const T*)b,
                                                       (T*)x, kmax, work);
  DGB_LAUNCH_CHECK();
  if (global) DGB_CUDA_CHECK(cudaFreeAsync(work, st));
  return DGB_OK;
}

static int forest_dispatch(int dtype, const ForestArgsT& F, int kmax, const void* d,
                           const void* g, const void* b, void* x, void* stream) {
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  if (F.n_trees == 0) return DGB_OK;
  DGB_REQUIRE(d && g && b && x, "d, a, b and x must be non-null");
  DGB_REQUIRE(F.parent && F.order && F.layer_ptr && F.child_ptr && F.child_idx,
              "tree plan arrays must be non-null");
  DGB_REQUIRE(F.shared_k > 0 || (F.node_ptr && F.plan_node_ptr && F.plan_layer_off),
              "forest offsets (node_ptr, plan_node_ptr, plan_layer_off) must be non-null");
  DGB_REQUIRE(kmax >= 1, "trees must have at least one node");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32) return forest_launch<float>(F, kmax, d, g, b, x, st);
  return forest_launch<double>(F, kmax, d, g, b, x, st);
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_dhs_solve_forest(int dtype, const dgb_forest* forest, const void* d,
                                    const void* a, const void* b, void* x, void* stream) {
  clear_error();
  DGB_REQUIRE(forest != nullptr, "forest must be non-null");
  DGB_REQUIRE(forest->n_trees >= 0, "n_trees must be >= 0");
  ForestArgsT F{forest->n_trees, 0, 0, forest->node_ptr, forest->plan_of, forest->plan_node_ptr,
                forest->plan_layer_off, forest->parent, forest->order, forest->layer_ptr,
                forest->child_ptr, forest->child_idx, forest->tree_k,
                forest->plan_chain_off, forest->plan_clevel_off, forest->chain_nodes,
                forest->chain_ptr, forest->chain_level};
  DGB_REQUIRE(!F.chain_nodes || (F.chain_ptr && F.chain_level && F.plan_chain_off &&
                                 F.plan_clevel_off),
              "the chain schedule needs chain_ptr, chain_level and their plan offsets");
  return forest_dispatch(dtype, F, forest->max_k, d, a, b, x, stream);
}

extern "C" int dgb_dhs_solve(int dtype, int64_t B, int64_t K, const void* d, const void* a,
                             const void* b, const int32_t* parent, const int32_t* order,
                             const int32_t* layer_ptr, int32_t n_layers,
                             const int32_t* child_ptr, const int32_t* child_idx, void* x,
                             void* stream) {
  clear_error();
  DGB_REQUIRE(B >= 0 && K >= 1, "B and K must both be >= 1 (got B=%lld K=%lld)", (long long)B,
              (long long)K);
  DGB_REQUIRE(n_layers >= 1, "layer_ptr must contain at least two entries");
  DGB_REQUIRE(B <= INT32_MAX && K <= INT32_MAX, "too many trees or nodes");
  ForestArgsT F{(int32_t)B, (int32_t)K, n_layers, nullptr, nullptr, nullptr, nullptr,
                parent,     order,      layer_ptr, child_ptr, child_idx, nullptr,
                nullptr,    nullptr,    nullptr,   nullptr,   nullptr};
  return forest_dispatch(dtype, F, (int)K, d, a, b, x, stream);
}
