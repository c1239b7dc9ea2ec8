// Tree contraction solve on sm_103a: drop-in for the reference's CUDA tree
// contraction (models/integrators/triton/tree_contraction.py, kernels
// :14-480, solve :748-768) on a plan of dendra_gb300/contraction.py.
//
// Scalar Hines systems in conductance form: shunt d_i, conductance g_i to the
// parent (a root's g a second shunt).  One block (32-256 threads) per batch
// row; the row and every scratch value live in shared memory:
//   d, g, rhs           [3][K]           the row, loaded coalesced; an
//                                        interior node's pivot and reduced
//                                        value overwrite its d and rhs when
//                                        it is eliminated, and x overwrites
//                                        rhs when it is recovered
//   bridge              [n_interior]     segment elimination, for recovery
//   summary             [5][n_segments]  ancestor shunt/value, child
//                                        shunt/value, bridge
//   shunt/value         [2][R + U]       state slots (SSA: update u writes R+u)
//   edge                [R + n_bridges]  edge slots
//   xr                  [R]              x of the retained nodes
// Phases, separated by block barriers: load the row, condense
// segments (thread per segment, top to bottom), gather the retained nodes'
// reduced state, contraction rounds (thread per update; each update pulls its
// removed neighbours in plan order), root solves, recovery rounds in reverse,
// segment recovery (thread per segment, bottom to top), store x coalesced.
// Only correctly rounded single operations (no contraction into FMA), so the
// numpy restatement of the same plan reproduces every bit.
#include "common.cuh"

namespace dgb {

__device__ __forceinline__ float tc_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double tc_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float tc_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double tc_div(double a, double b) { return __ddiv_rn(a, b); }

// small * (large / pivot) of the pair (a, b), ordered by magnitude, given
// the rounded quotients qa = a / pivot and qb = b / pivot: the same value as
// dividing the larger factor inside the product.
template <typename T>
__device__ __forceinline__ T schur_q(T a, T qa, T b, T qb) {
  return fabs(a) < fabs(b) ? mul_rn(a, qb) : mul_rn(b, qa);
}

struct TcCounts {
  int K, S, I, R, U, P, NR, NB;
};

static __host__ __device__ __forceinline__ int64_t tc_row_values(const TcCounts& c) {
  return 3ll * c.K + c.I + 5ll * c.S + 2ll * (c.R + c.U) + 2ll * c.R + c.NB;
}

// One CTA of TPR threads per batch row (grid-stride over rows); phases are
// separated by __syncthreads.
template <typename T, int TPR>
__global__ void __launch_bounds__(TPR, (TPR >= 256 && sizeof(T) == 4) ? 5 : 1)
    tree_contract_kernel(dgb_contract_plan p, TcCounts c, int64_t B, const T* __restrict__ d,
                         const T* __restrict__ g, const T* __restrict__ rhs, T* __restrict__ x) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  T* sd = reinterpret_cast<T*>(smem_raw);  // [K]: d, then interior pivots
  T* sg = sd + c.K;                          // [K]
  T* sb = sg + c.K;                          // [K]: rhs, interior values, then x
  T* bridges = sb + c.K;                     // [I]
  T* summ = bridges + c.I;                   // [5][S]
  T* st_s = summ + 5 * c.S;                  // [R+U]
  T* st_r = st_s + (c.R + c.U);              // [R+U]
  T* edge = st_r + (c.R + c.U);              // [R+NB]
  T* xr = edge + (c.R + c.NB);               // [R]
  const int32_t* seg_anc = p.seg;
  const int32_t* seg_child = p.seg + c.S;
  const int32_t* seg_a0 = p.seg + 2 * c.S;
  const int32_t* seg_a1 = p.seg + 3 * c.S;
  const int32_t* ret_node = p.retained;
  const int32_t* ret_in = p.retained + c.R;
  const int32_t* ret_e0 = p.retained + 2 * c.R;
  const int32_t* ret_ne = p.retained + 3 * c.R;
  const int NE = p.n_endpoints, NRT = p.n_roots;
  for (int64_t row = blockIdx.x; row < B; row += gridDim.x) {
    {  // 0. stage the row: four loads per array in flight per thread
      const T* dr = d + row * c.K;
      const T* gr = g + row * c.K;
      const T* br = rhs + row * c.K;
      for (int i0 = tid; i0 < c.K; i0 += 4 * TPR) {
        T vd[4], vg[4], vb[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int i = i0 + k * TPR;
          if (i < c.K) {
            vd[k] = __ldcs(dr + i);
            vg[k] = __ldcs(gr + i);
            vb[k] = __ldcs(br + i);
          }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int i = i0 + k * TPR;
          if (i < c.K) {
            sd[i] = vd[k];
            sg[i] = vg[k];
            sb[i] = vb[k];
          }
        }
      }
    }
    __syncthreads();
    {  // the next row of this block into L2 while this one computes
      const int64_t nrow = row + gridDim.x;
      if (nrow < B) {
        const int lines = (int)(((int64_t)c.K * sizeof(T) + 127) / 128);
        const char* pd = reinterpret_cast<const char*>(d + nrow * c.K);
        const char* pg = reinterpret_cast<const char*>(g + nrow * c.K);
        const char* pb = reinterpret_cast<const char*>(rhs + nrow * c.K);
        for (int l = tid; l < lines; l += TPR) {
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pd + 128 * (int64_t)l));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pg + 128 * (int64_t)l));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pb + 128 * (int64_t)l));
        }
      }
    }
    // 1. segment condensation, top to bottom
    for (int s = tid; s < c.S; s += TPR) {
      const int child = ret_node[seg_child[s]], a0 = seg_a0[s], a1 = seg_a1[s];
      int node = p.interior[a0];
      int succ = a0 + 1 < a1 ? p.interior[a0 + 1] : child;
      T near = sg[node];
      T left_d = T(0), left_r = T(0), carry_d = T(0), carry_r = T(0);
      for (int pos = a0; pos < a1; ++pos) {
        // the index after next is loaded while this step computes
        const int next = pos + 2 < a1 ? p.interior[pos + 2] : child;
        const T far = sg[succ];
        const T shunt = tc_add(sd[node], carry_d);
        const T value = tc_add(sb[node], carry_r);
        const T pivot = tc_add(shunt, tc_add(near, far));
        const T qn = tc_div(near, pivot), qf = tc_div(far, pivot);
        const T as = fabs(shunt);
        const T qs = (fabs(near) < as || fabs(far) < as) ? tc_div(shunt, pivot) : T(0);
        sb[node] = value;  // this node's d and rhs are read only here
        sd[node] = pivot;
        bridges[pos] = near;
        left_d = tc_add(left_d, schur_q(near, qn, shunt, qs));
        left_r = tc_add(left_r, mul_rn(qn, value));
        carry_d = schur_q(far, qf, shunt, qs);
        carry_r = mul_rn(qf, value);
        near = schur_q(near, qn, far, qf);
        node = succ;
        succ = next;
      }
      summ[s] = left_d;
      summ[c.S + s] = left_r;
      summ[2 * c.S + s] = carry_d;
      summ[3 * c.S + s] = carry_r;
      summ[4 * c.S + s] = near;
    }
    __syncthreads();
    // 2. reduced state of the retained nodes
    for (int r = tid; r < c.R; r += TPR) {
      const int node = ret_node[r], in = ret_in[r], e0 = ret_e0[r], ne = ret_ne[r];
      T diag = sd[node], val = sb[node];
      for (int e = e0; e < e0 + ne; ++e) {
        const int s = p.endpoint[e], side = p.endpoint[NE + e];
        diag = tc_add(diag, summ[2 * side * c.S + s]);
        val = tc_add(val, summ[(2 * side + 1) * c.S + s]);
      }
      st_s[r] = diag;
      st_r[r] = val;
      edge[r] = in >= 0 ? summ[4 * c.S + in] : sg[node];
    }
    __syncthreads();
    // 3. contraction rounds
    for (int ph = 0; ph < c.P; ++ph) {
      const int u1 = p.round_ptr[ph + 1];
      for (int u = p.round_ptr[ph] + tid; u < u1; u += TPR) {
        const int4 up = __ldg(reinterpret_cast<const int4*>(p.update) + u);
        const int src = up.x, q0 = up.y, nq = up.z;
        T diag = st_s[src], val = st_r[src];
        for (int q = q0; q < q0 + nq; ++q) {
          const int4 in = __ldg(reinterpret_cast<const int4*>(p.incidence) + q);
          const int m = in.x, ns = in.y, fs = in.z, dest = in.w;
          const T shunt = st_s[m], value = st_r[m], near = edge[ns];
          const T far = fs >= 0 ? edge[fs] : T(0);
          const T pivot = tc_add(shunt, tc_add(near, far));
          const T qn = tc_div(near, pivot);
          const T qs = fabs(near) < fabs(shunt) ? tc_div(shunt, pivot) : T(0);
          diag = tc_add(diag, schur_q(near, qn, shunt, qs));
          val = tc_add(val, mul_rn(qn, value));
          if (dest >= 0) {
            const T qf = fabs(far) <= fabs(near) ? T(0) : tc_div(far, pivot);
            edge[dest] = schur_q(near, qn, far, qf);
          }
        }
        st_s[c.R + u] = diag;
        st_r[c.R + u] = val;
      }
      __syncthreads();
    }
    // 4. roots
    for (int k = tid; k < NRT; k += TPR) {
      const int r = p.roots[k], st = p.roots[NRT + k];
      xr[r] = tc_div(st_r[st], tc_add(st_s[st], edge[r]));
    }
    __syncthreads();
    // 5. recovery rounds, last round first
    const int32_t* rp = p.round_ptr + (c.P + 1);
    for (int ph = c.P - 1; ph >= 0; --ph) {
      const int e1 = rp[ph + 1];
      for (int e = rp[ph] + tid; e < e1; e += TPR) {
        const int4 r0 = __ldg(reinterpret_cast<const int4*>(p.recovery) + 2 * e);
        const int4 r1 = __ldg(reinterpret_cast<const int4*>(p.recovery) + 2 * e + 1);
        const int node = r0.x, st = r0.y, a = r0.z, ch = r0.w, ns = r1.x, fs = r1.y;
        const T near = edge[ns];
        const T far = fs >= 0 ? edge[fs] : T(0);
        const T xc = ch >= 0 ? xr[ch] : T(0);
        const T pivot = tc_add(st_s[st], tc_add(near, far));
        xr[node] = tc_div(tc_add(tc_add(st_r[st], mul_rn(near, xr[a])), mul_rn(far, xc)), pivot);
      }
      __syncthreads();
    }
    // 6. retained x into the row (their rhs is dead after the gather)
    for (int r = tid; r < c.R; r += TPR) sb[ret_node[r]] = xr[r];
    // 7. segment recovery, bottom to top (endpoint x from xr)
    for (int s = tid; s < c.S; s += TPR) {
      int succ = ret_node[seg_child[s]];
      const T xa = xr[seg_anc[s]];
      T xs = xr[seg_child[s]];
      const int a0 = seg_a0[s];
      int node = p.interior[seg_a1[s] - 1];
      for (int pos = seg_a1[s] - 1; pos >= a0; --pos) {
        const int prev = pos > a0 ? p.interior[pos - 1] : 0;  // loaded ahead
        const T v = tc_div(tc_add(tc_add(sb[node], mul_rn(bridges[pos], xa)),
                                  mul_rn(sg[succ], xs)),
                           sd[node]);
        sb[node] = v;
        succ = node;
        xs = v;
        node = prev;
      }
    }
    __syncthreads();
    // 8. x to HBM, coalesced
    T* xrow = x + row * c.K;
    for (int i = tid; i < c.K; i += TPR) __stcs(xrow + i, sb[i]);
    __syncthreads();
  }
}

template <typename T>
__global__ void single_node_kernel(int64_t B, const T* __restrict__ d, const T* __restrict__ g,
                                   const T* __restrict__ rhs, T* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < B) x[i] = tc_div(rhs[i], tc_add(d[i], g[i]));
}

template <typename T, int TPR>
static int launch_tpr(int64_t B, const dgb_contract_plan& p, const TcCounts& c, size_t smem,
                      int sms, const void* d, const void* g, const void* rhs, void* x,
                      cudaStream_t st) {
  auto kern = tree_contract_kernel<T, TPR>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPR, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t cap = (int64_t)sms * per_sm;
  const unsigned blocks = (unsigned)(B < cap ? B : cap);
  kern<<<blocks, TPR, smem, st>>>(p, c, B, (const T*)d, (const T*)g, (const T*)rhs, (T*)x);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
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
  const size_t smem = (size_t)tc_row_values(c) * sizeof(T);
  int dev = 0, optin = 0, sms = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (smem > (size_t)optin) {
    set_error("tree contraction scratch of %zu bytes per row exceeds shared memory", smem);
    return DGB_ERANGE;
  }
  int tpr = p.threads;
  if (tpr == 0) {  // about one thread per two items of the widest phase, at most 256
    const int wide = c.S > c.R ? c.S : c.R;
    tpr = wide > 160 ? 256 : (wide > 80 ? 128 : (wide > 40 ? 64 : 32));
  }
  switch (tpr) {
    case 32: return launch_tpr<T, 32>(B, p, c, smem, sms, d, g, rhs, x, st);
    case 64: return launch_tpr<T, 64>(B, p, c, smem, sms, d, g, rhs, x, st);
    case 128: return launch_tpr<T, 128>(B, p, c, smem, sms, d, g, rhs, x, st);
    case 256: return launch_tpr<T, 256>(B, p, c, smem, sms, d, g, rhs, x, st);
    default:
      set_error("threads per row must be 0, 32, 64, 128 or 256; got %d", tpr);
      return DGB_EINVAL;
  }
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
  DGB_REQUIRE((p.n_updates == 0 || ((uintptr_t)p.update & 15) == 0) &&
                  (p.n_incidence == 0 || ((uintptr_t)p.incidence & 15) == 0) &&
                  (p.n_eliminated == 0 || ((uintptr_t)p.recovery & 15) == 0),
              "update, incidence and recovery tables must be 16-byte aligned");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32) return launch_contract<float>(B, p, d, g, rhs, x, st);
  return launch_contract<double>(B, p, d, g, rhs, x, st);
}

extern "C" size_t dgb_contract_plan_size(void) { return sizeof(dgb_contract_plan); }
