// Tree (DHS/Hines) solves with 3x3 blocks on sm_103a: the multi-layer
// extracellular tree systems of the reference's _dhs_bt integrator
// (integrators/tree_bt.py), drop-in for dhs_bt_solve_cuda
// (triton/dhs_kernel_bt.py:465-479, kernel :39-240).
//
// Node i of a tree (solver order; B trees share one topology) has a 3x3 block
// D_i and an edge to its parent E_i = diag(g_i); the matrix has
//   A_ii = D_i + E_i + sum over children c of E_c,   A_ic = A_ci = -E_c
// (a root's E_i only adds to its diagonal).  Elimination runs leaves -> root
// by depth layers, every node pulling its children in CSR order
// (deterministic; the reference adds them to the parent with atomics):
//   M_i = D_i + E_i + sum_c (E_c - E_c M_c^-1 E_c)
//   y_i = M_i^-1 (b_i + sum_c E_c y_c)
// and back substitution runs root -> leaves: x_i = y_i + M_i^-1 E_i x_parent.
// One warp per tree; M^-1 and y (then x) of every node stay in shared memory
// (12 values per node).  transpose = 1 solves with D_i^T: the adjoint system
// (the edge blocks are diagonal, hence symmetric).
#include "common.cuh"
#include "m3.cuh"

namespace dgb {

// work == nullptr: scratch in shared memory; else each block uses its slice
// of 12*K values of the global workspace (trees too large for shared memory).
template <typename T, bool TR>
__global__ void __launch_bounds__(32)
    dhs_block3_kernel(int64_t B, int32_t K, int32_t L, const T* __restrict__ D,
                      const T* __restrict__ G, const T* __restrict__ rhs,
                      const int32_t* __restrict__ parent, const int32_t* __restrict__ order,
                      const int32_t* __restrict__ layer_ptr,
                      const int32_t* __restrict__ child_ptr,
                      const int32_t* __restrict__ child_idx, T* __restrict__ x,
                      T* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sMinv = work ? work + (size_t)blockIdx.x * 12 * K
                  : reinterpret_cast<T*>(smem_raw);  // [K][9]
  T* sY = sMinv + (size_t)9 * K;              // [K][3]: y, then x
  const int lane = threadIdx.x;
  for (int64_t tree = blockIdx.x; tree < B; tree += gridDim.x) {
    const T* Dt = D + tree * (int64_t)K * 9;
    const T* Gt = G + tree * (int64_t)K * 3;
    const T* bt = rhs + tree * (int64_t)K * 3;
    for (int l = 0; l < L; ++l) {
      const int o1 = layer_ptr[l + 1];
      for (int o = layer_ptr[l] + lane; o < o1; o += 32) {
        const int i = order[o];
        M3<T> M;
#pragma unroll
        for (int q = 0; q < 9; ++q) M.a[q] = TR ? Dt[i * 9 + (q % 3) * 3 + q / 3] : Dt[i * 9 + q];
        T bv[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          M.a[r * 4] = M.a[r * 4] + Gt[i * 3 + r];
          bv[r] = bt[i * 3 + r];
        }
        const int c1 = child_ptr[i + 1];
        for (int k = child_ptr[i]; k < c1; ++k) {
          const int c = child_idx[k];
          T gc[3];
#pragma unroll
          for (int r = 0; r < 3; ++r) gc[r] = Gt[c * 3 + r];
          const T* Mc = sMinv + (size_t)c * 9;
          const T* yc = sY + (size_t)c * 3;
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            M.a[r * 4] = M.a[r * 4] + gc[r];
#pragma unroll
            for (int s = 0; s < 3; ++s) M.a[r * 3 + s] = M.a[r * 3 + s] - gc[r] * Mc[r * 3 + s] * gc[s];
            bv[r] = bv[r] + gc[r] * yc[r];
          }
        }
        const M3<T> Mi = inv3(M);
        T y[3];
        mv(Mi, bv, y);
#pragma unroll
        for (int q = 0; q < 9; ++q) sMinv[(size_t)i * 9 + q] = Mi.a[q];
#pragma unroll
        for (int r = 0; r < 3; ++r) sY[(size_t)i * 3 + r] = y[r];
      }
      __syncwarp();
    }
    for (int l = L - 1; l >= 0; --l) {
      const int o1 = layer_ptr[l + 1];
      for (int o = layer_ptr[l] + lane; o < o1; o += 32) {
        const int i = order[o];
        const int p = parent[i];
        if (p < 0) continue;  // a root keeps x = y
        T e[3], d[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) e[r] = Gt[i * 3 + r] * sY[(size_t)p * 3 + r];
        M3<T> Mi;
#pragma unroll
        for (int q = 0; q < 9; ++q) Mi.a[q] = sMinv[(size_t)i * 9 + q];
        mv(Mi, e, d);
#pragma unroll
        for (int r = 0; r < 3; ++r) sY[(size_t)i * 3 + r] = sY[(size_t)i * 3 + r] + d[r];
      }
      __syncwarp();
    }
    T* xt = x + tree * (int64_t)K * 3;
    for (int q = lane; q < 3 * K; q += 32) xt[q] = sY[q];
    __syncwarp();
  }
}

template <typename T>
static int launch_dhs_block3(int64_t B, int32_t K, int32_t L, const void* D, const void* G,
                             const void* rhs, const int32_t* parent, const int32_t* order,
                             const int32_t* layer_ptr, const int32_t* child_ptr,
                             const int32_t* child_idx, void* x, int transpose,
                             cudaStream_t st) {
  const size_t scratch = (size_t)12 * K * sizeof(T);
  int dev = 0, optin = 0, sms = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  // trees whose scratch does not fit on chip: a stream-ordered workspace of
  // 16 trees per SM in flight
  const bool global = scratch > (size_t)optin;
  const int64_t cap = global ? (int64_t)sms * 16 : (int64_t)65535 * 32;
  const unsigned blocks = (unsigned)(B < cap ? B : cap);
  const size_t smem = global ? 0 : scratch;
  T* work = nullptr;
  if (global) DGB_CUDA_CHECK(cudaMallocAsync((void**)&work, (size_t)blocks * scratch, st));
  if (transpose) {
    DGB_CUDA_CHECK(cudaFuncSetAttribute(dhs_block3_kernel<T, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dhs_block3_kernel<T, true><<<blocks, 32, smem, st>>>(
        B, K, L, (const T*)D, (const T*)G, (const T*)rhs, parent, order, layer_ptr, child_ptr,
        child_idx, (T*)x, work);
  } else {
    DGB_CUDA_CHECK(cudaFuncSetAttribute(dhs_block3_kernel<T, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dhs_block3_kernel<T, false><<<blocks, 32, smem, st>>>(
        B, K, L, (const T*)D, (const T*)G, (const T*)rhs, parent, order, layer_ptr, child_ptr,
        child_idx, (T*)x, work);
  }
  DGB_LAUNCH_CHECK();
  if (global) DGB_CUDA_CHECK(cudaFreeAsync(work, st));
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_dhs_block3_solve(int dtype, int64_t B, int64_t K, const void* main_blocks,
                                    const void* edge, const void* rhs, const int32_t* parent,
                                    const int32_t* order, const int32_t* layer_ptr,
                                    int32_t n_layers, const int32_t* child_ptr,
                                    const int32_t* child_idx, void* x, int32_t transpose,
                                    void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(B >= 1 && K >= 1, "B and K must both be >= 1");
  DGB_REQUIRE(K <= INT32_MAX / 12 && n_layers >= 1, "bad tree size or layer count");
  DGB_REQUIRE(main_blocks && edge && rhs && x && parent && order && layer_ptr && child_ptr &&
                  (K == 1 || child_idx),
              "pointers must be non-null");
  DGB_REQUIRE(x != rhs, "x must not alias rhs");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32)
    return launch_dhs_block3<float>(B, (int32_t)K, n_layers, main_blocks, edge, rhs, parent,
                                    order, layer_ptr, child_ptr, child_idx, x, transpose, st);
  return launch_dhs_block3<double>(B, (int32_t)K, n_layers, main_blocks, edge, rhs, parent,
                                   order, layer_ptr, child_ptr, child_idx, x, transpose, st);
}
