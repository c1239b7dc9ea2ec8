// Tree contraction solve on sm_103a: drop-in for the reference's CUDA tree
// contraction (models/integrators/triton/tree_contraction.py, kernels
// :14-480, solve :748-768) on a plan of dendra_gb300/contraction.py.
//
// Scalar Hines systems in conductance form: shunt d_i, conductance g_i to the
// parent (a root's g a second shunt).  One warp per batch row; every scratch
// value of the row lives in shared memory:
//   saved/pivot/bridge  [3][n_interior]  segment elimination, for recovery
//   summary             [5][n_segments]  ancestor shunt/value, child
//                                        shunt/value, bridge
//   shunt/value         [2][R + U]       state slots (SSA: update u writes R+u)
//   edge                [R + n_bridges]  edge slots
//   xr                  [R]              solution of the retained nodes
// Phases, separated by __syncwarp: condense segments (lane per segment, top
// to bottom), gather the retained nodes' reduced state, contraction rounds
// (lane per update; each update pulls its removed neighbours in plan order),
// root solves, recovery rounds in reverse, retained x to HBM, segment
// recovery (lane per segment, bottom to top; reads the endpoints' x back from
// HBM, written by this warp before the barrier).
// Only correctly rounded single operations (no contraction into FMA), so the
// numpy restatement of the same plan reproduces every bit.
#include "common.cuh"

namespace dgb {

__device__ __forceinline__ float tc_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double tc_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float tc_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double tc_div(double a, double b) { return __ddiv_rn(a, b); }

// small * (large / pivot) of the pair, ordered by magnitude
template <typename T>
__device__ __forceinline__ T schur(T left, T right, T pivot) {
  const bool left_small = fabs(left) < fabs(right);
  const T small = left_small ? left : right;
  const T large = left_small ? right : left;
  return mul_rn(small, tc_div(large, pivot));
}

struct TcCounts {
  int K, S, I, R, U, P, NR, NB;
};

static __host__ __device__ __forceinline__ int64_t tc_row_values(const TcCounts& c) {
  return 3ll * c.I + 5ll * c.S + 2ll * (c.R + c.U) + 2ll * c.R + c.NB;
}

template <typename T>
__global__ void __launch_bounds__(128)
    tree_contract_kernel(dgb_contract_plan p, TcCounts c, int64_t B, const T* __restrict__ d,
                         const T* __restrict__ g, const T* __restrict__ rhs, T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  T* saved = reinterpret_cast<T*>(smem_raw) + (size_t)warp * tc_row_values(c);
  T* pivots = saved + c.I;
  T* bridges = pivots + c.I;
  T* summ = bridges + c.I;        // [5][S]
  T* st_s = summ + 5 * c.S;       // [R+U]
  T* st_r = st_s + (c.R + c.U);   // [R+U]
  T* edge = st_r + (c.R + c.U);   // [R+NB]
  T* xr = edge + (c.R + c.NB);    // [R]
  const int32_t* seg_anc = p.seg;
  const int32_t* seg_child = p.seg + c.S;
  const int32_t* seg_a0 = p.seg + 2 * c.S;
  const int32_t* seg_a1 = p.seg + 3 * c.S;
  const int32_t* ret_node = p.retained;
  const int32_t* ret_in = p.retained + c.R;
  const int32_t* ret_e0 = p.retained + 2 * c.R;
  const int32_t* ret_ne = p.retained + 3 * c.R;
  const int NE = p.n_endpoints, Q = p.n_incidence, NRT = p.n_roots;
  for (int64_t row = (int64_t)blockIdx.x * wpb + warp; row < B; row += (int64_t)gridDim.x * wpb) {
    const T* dr = d + row * c.K;
    const T* gr = g + row * c.K;
    const T* br = rhs + row * c.K;
    T* xo = x + row * c.K;
    // 1. segment condensation, top to bottom
    for (int s = lane; s < c.S; s += 32) {
      const int child = seg_child[s], a0 = seg_a0[s], a1 = seg_a1[s];
      T near = gr[p.interior[a0]];
      T left_d = T(0), left_r = T(0), carry_d = T(0), carry_r = T(0);
      for (int pos = a0; pos < a1; ++pos) {
        const int node = p.interior[pos];
        const int succ = pos + 1 < a1 ? p.interior[pos + 1] : child;
        const T far = gr[succ];
        const T shunt = tc_add(dr[node], carry_d);
        const T value = tc_add(br[node], carry_r);
        const T pivot = tc_add(shunt, tc_add(near, far));
        saved[pos] = value;
        pivots[pos] = pivot;
        bridges[pos] = near;
        left_d = tc_add(left_d, schur(near, shunt, pivot));
        left_r = tc_add(left_r, mul_rn(tc_div(near, pivot), value));
        carry_d = schur(far, shunt, pivot);
        carry_r = mul_rn(tc_div(far, pivot), value);
        near = schur(near, far, pivot);
      }
      summ[s] = left_d;
      summ[c.S + s] = left_r;
      summ[2 * c.S + s] = carry_d;
      summ[3 * c.S + s] = carry_r;
      summ[4 * c.S + s] = near;
    }
    __syncwarp();
    // 2. reduced state of the retained nodes
    for (int r = lane; r < c.R; r += 32) {
      const int node = ret_node[r], in = ret_in[r], e0 = ret_e0[r], ne = ret_ne[r];
      T diag = dr[node], val = br[node];
      for (int e = e0; e < e0 + ne; ++e) {
        const int s = p.endpoint[e], side = p.endpoint[NE + e];
        diag = tc_add(diag, summ[2 * side * c.S + s]);
        val = tc_add(val, summ[(2 * side + 1) * c.S + s]);
      }
      st_s[r] = diag;
      st_r[r] = val;
      edge[r] = in >= 0 ? summ[4 * c.S + in] : gr[node];
    }
    __syncwarp();
    // 3. contraction rounds
    for (int ph = 0; ph < c.P; ++ph) {
      const int u1 = p.round_ptr[ph + 1];
      for (int u = p.round_ptr[ph] + lane; u < u1; u += 32) {
        const int src = p.update[u], q0 = p.update[c.U + u], nq = p.update[2 * c.U + u];
        T diag = st_s[src], val = st_r[src];
        for (int q = q0; q < q0 + nq; ++q) {
          const int m = p.incidence[q], ns = p.incidence[Q + q];
          const int fs = p.incidence[2 * Q + q], dest = p.incidence[3 * Q + q];
          const T shunt = st_s[m], value = st_r[m], near = edge[ns];
          const T far = fs >= 0 ? edge[fs] : T(0);
          const T pivot = tc_add(shunt, tc_add(near, far));
          diag = tc_add(diag, schur(near, shunt, pivot));
          val = tc_add(val, mul_rn(tc_div(near, pivot), value));
          if (dest >= 0) edge[dest] = schur(near, far, pivot);
        }
        st_s[c.R + u] = diag;
        st_r[c.R + u] = val;
      }
      __syncwarp();
    }
    // 4. roots
    for (int k = lane; k < NRT; k += 32) {
      const int r = p.roots[k], st = p.roots[NRT + k];
      xr[r] = tc_div(st_r[st], tc_add(st_s[st], edge[r]));
    }
    __syncwarp();
    // 5. recovery rounds, last round first
    const int32_t* rp = p.round_ptr + (c.P + 1);
    for (int ph = c.P - 1; ph >= 0; --ph) {
      const int e1 = rp[ph + 1];
      for (int e = rp[ph] + lane; e < e1; e += 32) {
        const int node = p.recovery[e], st = p.recovery[c.NR + e];
        const int a = p.recovery[2 * c.NR + e], ch = p.recovery[3 * c.NR + e];
        const int ns = p.recovery[4 * c.NR + e], fs = p.recovery[5 * c.NR + e];
        const T near = edge[ns];
        const T far = fs >= 0 ? edge[fs] : T(0);
        const T xc = ch >= 0 ? xr[ch] : T(0);
        const T pivot = tc_add(st_s[st], tc_add(near, far));
        xr[node] = tc_div(tc_add(tc_add(st_r[st], mul_rn(near, xr[a])), mul_rn(far, xc)), pivot);
      }
      __syncwarp();
    }
    // 6. retained nodes to HBM
    for (int r = lane; r < c.R; r += 32) xo[ret_node[r]] = xr[r];
    __syncwarp();
    // 7. segment recovery, bottom to top
    for (int s = lane; s < c.S; s += 32) {
      int succ = seg_child[s];
      const T xa = xo[seg_anc[s]];
      T xs = xo[succ];
      for (int pos = seg_a1[s] - 1; pos >= seg_a0[s]; --pos) {
        const int node = p.interior[pos];
        const T v = tc_div(tc_add(tc_add(saved[pos], mul_rn(bridges[pos], xa)),
                                  mul_rn(gr[succ], xs)),
                           pivots[pos]);
        xo[node] = v;
        succ = node;
        xs = v;
      }
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void single_node_kernel(int64_t B, const T* __restrict__ d, const T* __restrict__ g,
                                   const T* __restrict__ rhs, T* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < B) x[i] = tc_div(rhs[i], tc_add(d[i], g[i]));
}

template <typename T>
static int launch_contract(int64_t B, const dgb_contract_plan& p, const void* d, const void* g,
                           const void* rhs, void* x, cudaStream_t st) {
  if (p.size == 1) {
    single_node_kernel<T><<<(unsigned)((B + 255) / 256), 256, 0, st>>>(
        B, (const T*)d, (const T*)g, (const T*)rhs, (T*)x);
    DGB_LAUNCH_CHECK();
    return DGB_OK;
  }
  const TcCounts c{p.size, p.n_segments, p.n_interior, p.n_retained,
                   p.n_updates, p.n_rounds, p.n_eliminated, p.n_bridges};
  const size_t row_bytes = (size_t)tc_row_values(c) * sizeof(T);
  int dev = 0, optin = 0, sms = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (row_bytes > (size_t)optin) {
    set_error("tree contraction scratch of %zu bytes per row exceeds shared memory", row_bytes);
    return DGB_ERANGE;
  }
  // up to 4 rows (warps) per block while the scratch fits comfortably
  int wpb = 4;
  while (wpb > 1 && (size_t)wpb * row_bytes > 96 * 1024) wpb >>= 1;
  const size_t smem = (size_t)wpb * row_bytes;
  const int64_t need = (B + wpb - 1) / wpb;
  const int64_t cap = (int64_t)sms * 64;
  const unsigned blocks = (unsigned)(need < cap ? need : cap);
  DGB_CUDA_CHECK(cudaFuncSetAttribute(tree_contract_kernel<T>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tree_contract_kernel<T><<<blocks, 32 * wpb, smem, st>>>(p, c, B, (const T*)d, (const T*)g,
                                                          (const T*)rhs, (T*)x);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_tree_contract_solve(int dtype, int64_t B, const dgb_contract_plan* plan,
                                       const void* d, const void* g, const void* rhs, void* x,
                                       void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(plan != nullptr, "plan must be non-null");
  const dgb_contract_plan& p = *plan;
  DGB_REQUIRE(B >= 0 && p.size >= 1, "bad batch or plan size");
  if (B == 0) return DGB_OK;
  DGB_REQUIRE(d && g && rhs && x, "pointers must be non-null");
  DGB_REQUIRE(x != rhs && x != d && x != g, "x must not alias an input");
  DGB_REQUIRE(B <= INT64_MAX / p.size, "batch too large");
  if (p.size > 1) {
    DGB_REQUIRE(p.n_segments >= 0 && p.n_interior >= 0 && p.n_retained >= 1 &&
                    p.n_retained + p.n_interior == p.size && p.n_rounds >= 0 &&
                    p.n_updates >= 0 && p.n_incidence >= 0 && p.n_roots >= 1 &&
                    p.n_eliminated == p.n_retained - p.n_roots && p.n_bridges >= 0 &&
                    p.n_endpoints == 2 * p.n_segments,
                "inconsistent contraction plan counts");
    DGB_REQUIRE(p.retained && p.round_ptr && p.roots &&
                    (p.n_segments == 0 || (p.seg && p.interior && p.endpoint)) &&
                    (p.n_updates == 0 || (p.update && p.incidence)) &&
                    (p.n_eliminated == 0 || p.recovery),
                "plan table pointers must be non-null");
  }
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32) return launch_contract<float>(B, p, d, g, rhs, x, st);
  return launch_contract<double>(B, p, d, g, rhs, x, st);
}

extern "C" size_t dgb_contract_plan_size(void) { return sizeof(dgb_contract_plan); }
