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

// Node of interior position pos of a segment: arithmetic when the run's ids
// are consecutive (stride +1/-1), else from the interior table.
__device__ __forceinline__ int seg_node(const int32_t* __restrict__ interior, int first,
                                        int stride, int a0, int pos) {
  return stride != 0 ? first + stride * (pos - a0) : __ldg(interior + pos);
}

// One CTA of TPR threads per batch row (grid-stride over rows); phases are
// separated by __syncthreads.  Plan tables are records (vector loads); the
// records of a thread's next contraction or recovery round are loaded while
// the current round computes.
//
// GW = true keeps the row's values in a global workspace (one slice of
// tc_row_values(c) per block) instead of shared memory: the same program for
// trees whose scratch does not fit on chip.
template <typename T, int TPR, bool GW>
__global__ void __launch_bounds__(TPR, (TPR >= 256 && sizeof(T) == 4) ? 5 : 1)
    tree_contract_kernel(dgb_contract_plan p, TcCounts c, int64_t B, const T* __restrict__ d,
                         const T* __restrict__ g, const T* __restrict__ rhs, T* __restrict__ x,
                         T* __restrict__ work) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  T* sd = GW ? work + (size_t)blockIdx.x * tc_row_values(c)
             : reinterpret_cast<T*>(smem_raw);  // [K]: d, then interior pivots
  T* sg = sd + c.K;                          // [K]
  T* sb = sg + c.K;                          // [K]: rhs, interior values, then x
  T* bridges = sb + c.K;                     // [I]
  T* summ = bridges + c.I;                   // [5][S]
  T* st_s = summ + 5 * c.S;                  // [R+U]
  T* st_r = st_s + (c.R + c.U);              // [R+U]
  T* edge = st_r + (c.R + c.U);              // [R+NB]
  T* xr = edge + (c.R + c.NB);               // [R]
  const int4* seg4 = reinterpret_cast<const int4*>(p.seg);        // 2 per segment
  const int4* ret4 = reinterpret_cast<const int4*>(p.retained);   // 2 per retained node
  const int2* end2 = reinterpret_cast<const int2*>(p.endpoint);   // 1 per endpoint
  const int4* upd4 = reinterpret_cast<const int4*>(p.update);
  const int4* inc4 = reinterpret_cast<const int4*>(p.incidence);
  const int4* rec4 = reinterpret_cast<const int4*>(p.recovery);   // 2 per record
  const int NRT = p.n_roots;
  // round offsets and roots: read on every round's critical path, so kept in
  // shared memory for the block's lifetime
  int32_t* s_int = GW ? reinterpret_cast<int32_t*>(smem_raw) : reinterpret_cast<int32_t*>(xr + c.R);
  for (int i = tid; i < 2 * (c.P + 1); i += TPR) s_int[i] = __ldg(p.round_ptr + i);
  for (int i = tid; i < 2 * NRT; i += TPR) s_int[2 * (c.P + 1) + i] = __ldg(p.roots + i);
  const int32_t* rp_upd = s_int;
  const int32_t* rp_rec = s_int + (c.P + 1);
  const int32_t* roots = s_int + 2 * (c.P + 1);
  __syncthreads();
  for (int64_t row = blockIdx.x; row < B; row += gridDim.x) {
    {  // 0. stage the row: UNR loads per array in flight per thread
      constexpr int UNR = TPR >= 256 ? 2 : 4;
      const T* dr = d + row * c.K;
      const T* gr = g + row * c.K;
      const T* br = rhs + row * c.K;
      for (int i0 = tid; i0 < c.K; i0 += UNR * TPR) {
        T vd[UNR], vg[UNR], vb[UNR];
#pragma unroll
        for (int k = 0; k < UNR; ++k) {
          const int i = i0 + k * TPR;
          if (i < c.K) {
            vd[k] = __ldcs(dr + i);
            vg[k] = __ldcs(gr + i);
            vb[k] = __ldcs(br + i);
          }
        }
#pragma unroll
        for (int k = 0; k < UNR; ++k) {
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
      const int4 h = __ldg(seg4 + 2 * s), h2 = __ldg(seg4 + 2 * s + 1);
      const int a0 = h.z, a1 = h.w, first = h2.x, stride = h2.y, child = h2.z;
      int node = first;
      int succ = a0 + 1 < a1 ? seg_node(p.interior, first, stride, a0, a0 + 1) : child;
      T near = sg[node];
      T left_d = T(0), left_r = T(0), carry_d = T(0), carry_r = T(0);
      for (int pos = a0; pos < a1; ++pos) {
        // the index after next is loaded while this step computes
        const int next = pos + 2 < a1 ? seg_node(p.interior, first, stride, a0, pos + 2) : child;
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
    // records of this thread's first contraction round, fetched before the barrier
    int4 up_next = make_int4(-1, 0, 0, 0), in_next = make_int4(0, 0, -1, -1);
    if (c.P > 0) {
      const int u = rp_upd[0] + tid;
      if (u < rp_upd[1]) {
        up_next = __ldg(upd4 + u);
        in_next = __ldg(inc4 + up_next.y);
      }
    }
    __syncthreads();
    // 2. reduced state of the retained nodes
    for (int r = tid; r < c.R; r += TPR) {
      const int4 rr = __ldg(ret4 + 2 * r), codes = __ldg(ret4 + 2 * r + 1);
      const int node = rr.x, in = rr.y, e0 = rr.z, ne = rr.w;
      T diag = sd[node], val = sb[node];
      for (int k = 0; k < ne; ++k) {
        int sg_, side;
        if (k < 4) {
          const int code = k == 0 ? codes.x : k == 1 ? codes.y : k == 2 ? codes.z : codes.w;
          sg_ = code >> 1;
          side = code & 1;
        } else {
          const int2 ep = __ldg(end2 + e0 + k);
          sg_ = ep.x;
          side = ep.y;
        }
        diag = tc_add(diag, summ[2 * side * c.S + sg_]);
        val = tc_add(val, summ[(2 * side + 1) * c.S + sg_]);
      }
      st_s[r] = diag;
      st_r[r] = val;
      edge[r] = in >= 0 ? summ[4 * c.S + in] : sg[node];
    }
    __syncthreads();
    // 3. contraction rounds
    for (int ph = 0; ph < c.P; ++ph) {
      const int u0 = rp_upd[ph], u1 = rp_upd[ph + 1];
      const int4 up_first = up_next, in_first = in_next;
      up_next = make_int4(-1, 0, 0, 0);
      if (ph + 1 < c.P) {  // prefetch the next round's first record of this thread
        const int un = u1 + tid;
        if (un < rp_upd[ph + 2]) {
          up_next = __ldg(upd4 + un);
          in_next = __ldg(inc4 + up_next.y);
        }
      }
      for (int u = u0 + tid; u < u1; u += TPR) {
        const int4 up = u == u0 + tid ? up_first : __ldg(upd4 + u);
        const int src = up.x, q0 = up.y, nq = up.z;
        T diag = st_s[src], val = st_r[src];
        for (int q = q0; q < q0 + nq; ++q) {
          const int4 in = (u == u0 + tid && q == q0) ? in_first : __ldg(inc4 + q);
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
    // records of this thread's first recovery round (the last round)
    int4 rc_a = make_int4(-1, 0, 0, 0), rc_b = make_int4(0, 0, 0, 0);
    if (c.P > 0) {
      const int e = rp_rec[c.P - 1] + tid;
      if (e < rp_rec[c.P]) {
        rc_a = __ldg(rec4 + 2 * e);
        rc_b = __ldg(rec4 + 2 * e + 1);
      }
    }
    // 4. roots
    for (int k = tid; k < NRT; k += TPR) {
      const int r = roots[k], st = roots[NRT + k];
      xr[r] = tc_div(st_r[st], tc_add(st_s[st], edge[r]));
    }
    __syncthreads();
    // 5. recovery rounds, last round first
    for (int ph = c.P - 1; ph >= 0; --ph) {
      const int e0 = rp_rec[ph], e1 = rp_rec[ph + 1];
      const int4 fa = rc_a, fb = rc_b;
      rc_a = make_int4(-1, 0, 0, 0);
      if (ph > 0) {
        const int en = rp_rec[ph - 1] + tid;
        if (en < e0) {
          rc_a = __ldg(rec4 + 2 * en);
          rc_b = __ldg(rec4 + 2 * en + 1);
        }
      }
      for (int e = e0 + tid; e < e1; e += TPR) {
        const bool mine = e == e0 + tid;
        const int4 r0 = mine ? fa : __ldg(rec4 + 2 * e);
        const int4 r1 = mine ? fb : __ldg(rec4 + 2 * e + 1);
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
    for (int r = tid; r < c.R; r += TPR) sb[__ldg(ret4 + 2 * r).x] = xr[r];
    // 7. segment recovery, bottom to top (endpoint x from xr)
    for (int s = tid; s < c.S; s += TPR) {
      const int4 h = __ldg(seg4 + 2 * s), h2 = __ldg(seg4 + 2 * s + 1);
      const int a0 = h.z, a1 = h.w, first = h2.x, stride = h2.y;
      int succ = h2.z;
      const T xa = xr[h.x];
      T xs = xr[h.y];
      int node = seg_node(p.interior, first, stride, a0, a1 - 1);
      for (int pos = a1 - 1; pos >= a0; --pos) {
        const int prev = pos > a0 ? seg_node(p.interior, first, stride, a0, pos - 1) : 0;
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

// Blocks of the global-workspace variant per SM (its workspace is sized by
// blocks x the row's values).
constexpr int kGwBlocksPerSm = 4;

template <typename T, int TPR, bool GW>
static int launch_tpr(int64_t B, const dgb_contract_plan& p, const TcCounts& c, size_t smem,
                      int sms, const void* d, const void* g, const void* rhs, void* x,
                      void* work, cudaStream_t st) {
  auto kern = tree_contract_kernel<T, TPR, GW>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TPR, smem));
  if (per_sm < 1) per_sm = 1;
  if (GW) per_sm = kGwBlocksPerSm;  // the workspace holds exactly this many rows per SM
  const int64_t cap = (int64_t)sms * per_sm;
  const unsigned blocks = (unsigned)(B < cap ? B : cap);
  kern<<<blocks, TPR, smem, st>>>(p, c, B, (const T*)d, (const T*)g, (const T*)rhs, (T*)x,
                                  (T*)work);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

static size_t tc_int_bytes(const dgb_contract_plan& p) {
  return 4 * (2 * ((size_t)p.n_rounds + 1) + 2 * (size_t)p.n_roots);
}

static TcCounts tc_counts(const dgb_contract_plan& p) {
  return TcCounts{p.size, p.n_segments, p.n_interior, p.n_retained,
                  p.n_updates, p.n_rounds, p.n_eliminated, p.n_bridges};
}

// Workspace bytes of the global variant for B rows; 0 when the row's scratch
// fits in shared memory (or the tree is a single node).
static int tc_work_bytes(int dtype, const dgb_contract_plan& p, int64_t B, size_t* bytes) {
  *bytes = 0;
  if (p.size == 1 || B == 0) return DGB_OK;
  const size_t elem = dtype == DGB_F32 ? 4 : 8;
  const size_t row = (size_t)tc_row_values(tc_counts(p)) * elem;
  int dev = 0, optin = 0, sms = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (row + tc_int_bytes(p) <= (size_t)optin) return DGB_OK;
  const int64_t cap = (int64_t)sms * kGwBlocksPerSm;
  *bytes = (size_t)(B < cap ? B : cap) * row;
  return DGB_OK;
}

template <typename T>
static int launch_contract(int64_t B, const dgb_contract_plan& p, const void* d, const void* g,
                           const void* rhs, void* x, void* work, size_t work_bytes,
                           cudaStream_t st) {
  if (p.size == 1) {
    single_node_kernel<T><<<(unsigned)((B + 255) / 256), 256, 0, st>>>(
        B, (const T*)d, (const T*)g, (const T*)rhs, (T*)x);
    DGB_LAUNCH_CHECK();
    return DGB_OK;
  }
  const TcCounts c = tc_counts(p);
  size_t need = 0;
  const int rc = tc_work_bytes(sizeof(T) == 4 ? DGB_F32 : DGB_F64, p, B, &need);
  if (rc != DGB_OK) return rc;
  const bool gw = need > 0;
  if (gw && (work == nullptr || work_bytes < need)) {
    set_error("tree contraction needs a %zu-byte workspace (dgb_tree_contract_work_size)", need);
    return DGB_EINVAL;
  }
  if (gw && ((uintptr_t)work % sizeof(T)) != 0) {
    set_error("workspace must be aligned to the element size");
    return DGB_EINVAL;
  }
  const size_t smem = gw ? tc_int_bytes(p) : (size_t)tc_row_values(c) * sizeof(T) + tc_int_bytes(p);
  int dev = 0, sms = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int tpr = p.threads;
  if (tpr == 0) {  // by the widest phase: 128 threads from 80 items, 256 from 640
    const int wide = c.S > c.R ? c.S : c.R;
    tpr = wide > 640 ? 256 : (wide > 80 ? 128 : (wide > 40 ? 64 : 32));
  }
  if (gw) {
    if (tpr == 256) return launch_tpr<T, 256, true>(B, p, c, smem, sms, d, g, rhs, x, work, st);
    if (tpr == 32 || tpr == 64 || tpr == 128)
      return launch_tpr<T, 128, true>(B, p, c, smem, sms, d, g, rhs, x, work, st);
  } else {
    switch (tpr) {
      case 32: return launch_tpr<T, 32, false>(B, p, c, smem, sms, d, g, rhs, x, nullptr, st);
      case 64: return launch_tpr<T, 64, false>(B, p, c, smem, sms, d, g, rhs, x, nullptr, st);
      case 128: return launch_tpr<T, 128, false>(B, p, c, smem, sms, d, g, rhs, x, nullptr, st);
      case 256: return launch_tpr<T, 256, false>(B, p, c, smem, sms, d, g, rhs, x, nullptr, st);
      default: break;
    }
  }
  set_error("threads per row must be 0, 32, 64, 128 or 256; got %d", tpr);
  return DGB_EINVAL;
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_tree_contract_solve(int dtype, int64_t B, const dgb_contract_plan* plan,
                                       const void* d, const void* g, const void* rhs, void* x,
                                       void* work, size_t work_bytes, void* stream) {
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
  DGB_REQUIRE(p.size == 1 ||
                  (((uintptr_t)p.retained & 15) == 0 &&
                   (p.n_segments == 0 ||
                    (((uintptr_t)p.seg & 15) == 0 && ((uintptr_t)p.endpoint & 7) == 0)) &&
                   (p.n_updates == 0 || ((uintptr_t)p.update & 15) == 0) &&
                   (p.n_incidence == 0 || ((uintptr_t)p.incidence & 15) == 0) &&
                   (p.n_eliminated == 0 || ((uintptr_t)p.recovery & 15) == 0)),
              "plan record tables must be 16-byte aligned (endpoint 8-byte)");
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32) return launch_contract<float>(B, p, d, g, rhs, x, work, work_bytes, st);
  return launch_contract<double>(B, p, d, g, rhs, x, work, work_bytes, st);
}

extern "C" size_t dgb_tree_contract_work_size(int dtype, const dgb_contract_plan* plan,
                                              int64_t B) {
  clear_error();
  if (plan == nullptr || B < 0 || (dtype != DGB_F32 && dtype != DGB_F64)) return 0;
  size_t bytes = 0;
  if (tc_work_bytes(dtype, *plan, B, &bytes) != DGB_OK) return 0;
  return bytes;
}

extern "C" size_t dgb_contract_plan_size(void) { return sizeof(dgb_contract_plan); }
