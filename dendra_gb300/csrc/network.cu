// Spiking network of branched cells: window-persistent tree update and
// deterministic event enqueue (sm_103a).
//
// dgb_net_window advances every cell by W consecutive steps in one launch.
// Because every connection delay is at least W steps (the network's minimum
// delay), no event emitted inside the window is due inside it, so cells are
// independent for the whole window.  One warp owns one cell; per step, in the
// reference's phase order (networks/net.py:214-240, netcon.py:5183-5205):
//   1. deliver today's ring row into the cell's Exp2Syn states
//      (A += w*factor, B += w*factor; mod/EXP2SYN.py:154-156) and clear it,
//      plus the pre-generated background (NetStim) events;
//   2. rising-edge detection at the soma on v from the previous step
//      (networks/spiking.py:7-10); spikes are recorded in a 64-bit window mask;
//   3. state advance: A, B exact decay, soma HH gates by cnexp at v_old;
//   4. tree system (integrators/tree.py:1202-1357): f = (J - G v) area, axial
//      flows between child and parent, main = cm/dt + G area; DHS solve
//      (dhs.cuh; float cells take the chain sweeps' reciprocals in fast mode,
//      as the reference's Triton tree solve divides with the approximate
//      float division); v += dv.
// dgb_net_enqueue then scatters the window's spikes into the delay ring,
// one thread per target synapse, in connection then step order.
#include <stdint.h>
#include <type_traits>

#include "dhs.cuh"

namespace dgb {

template <typename T>
struct NetArgsT {
  int32_t n_cells, n_steps;
  int64_t step0, depth, slot0, n_syn;
  // forest
  const int64_t* node_ptr;
  const int32_t* plan_of;
  const int64_t* plan_node_ptr;
  const int64_t* plan_layer_off;
  const int32_t *parent, *order, *layer_ptr, *child_ptr, *child_idx;
  // chain schedule (chain_nodes == nullptr: layer schedule)
  const int64_t *plan_chain_off, *plan_clevel_off;
  const int32_t *chain_nodes, *chain_ptr, *chain_level;
  // per node
  T* v;
  const T *area, *cm_dt, *a_geom, *gl, *el;
  // soma HH, per cell
  T *m, *h, *n;
  T gnabar, gkbar, ena, ek, q10, dt, thr;
  // synapses
  const int64_t* syn_ptr;       // [n_cells+1]
  const int32_t* node_syn_ptr;  // [N + n_cells]: per cell K+1 entries (local synapse ranges per node)
  T *syn_A, *syn_B;
  const T *syn_factor, *syn_decay_A, *syn_decay_B;
  T e_syn;
  T* ring;                      // [depth][n_syn]
  // background events
  const unsigned long long* bg_bits;  // [steps][bg_words]
  int64_t bg_words;
  int32_t bg_syn;               // local synapse receiving background events
  T bg_weight;
  // extracellular and injected drive (nullptr: none)
  const T *ve_field, *ve_amp, *ve_delay, *ve_pw;
  const int32_t* in_node;
  const T *in_amp, *in_delay, *in_pw;
  double t0_ms, dt_d;
  // spikes
  uint8_t* below;
  unsigned long long* spike_bits;  // [n_cells] for this window
  int32_t* spike_count;
  // subset of cells (nullptr: all n_cells)
  const int32_t* cell_list;
  int32_t n_list;
};

// Shared memory of one warp (one cell): values sV, sD, sB, sG (axial
// conductance) of kmax entries in T, then the cell's plan as 16-bit indices
// (order or chain nodes, parent, child_ptr, child_idx, and layer_ptr or
// chain_ptr + chain levels), staged once per window so that the index chains
// of the DHS sweeps stay on chip.
template <typename T>
__host__ __device__ inline size_t net_warp_smem(int kmax) {
  const size_t vals = (size_t)4 * kmax * sizeof(T);
  const size_t idx = (size_t)2 * (6 * (size_t)kmax + 3);
  return (vals + idx + 15) & ~(size_t)15;
}

// A group of TPC threads (one warp, or 2 or 4 warps meeting at a named
// barrier) advances one cell; lane is the thread's index in the group.  Wider
// groups spread every per-cell loop (nodes, chains of a level, synapses) over
// more threads with the same shared memory per cell.
template <typename T, int TPC>
__device__ __forceinline__ void cell_sync(int group) {
  if constexpr (TPC == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(group + 1), "r"(TPC) : "memory");
  }
}

template <typename T, int TPC>
__global__ void __launch_bounds__(TPC > 128 ? TPC : 128) net_window_kernel(NetArgsT<T> A,
                                                                          int kmax) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int group = threadIdx.x / TPC, lane = threadIdx.x % TPC;
  const int cpb = blockDim.x / TPC;  // cells in flight per block
  unsigned char* wbase = smem_raw + (size_t)group * net_warp_smem<T>(kmax);
  using Sync = typename std::conditional<TPC == 32, WarpSync, GroupSync>::type;
  Sync sync;
  if constexpr (TPC != 32) sync = Sync{group + 1, TPC};
  T* sV = reinterpret_cast<T*>(wbase);
  T* sD = sV + kmax;
  T* sB = sD + kmax;
  T* sG = sB + kmax;
  uint16_t* sOrder = reinterpret_cast<uint16_t*>(sG + kmax);
  uint16_t* sParent = sOrder + kmax;
  uint16_t* sCptr = sParent + kmax;
  uint16_t* sCidx = sCptr + kmax + 1;
  uint16_t* sLptr = sCidx + kmax;      // layer_ptr, or chain_ptr then chain levels
  const bool chains = A.chain_nodes != nullptr;
  const int n_items = A.cell_list ? A.n_list : A.n_cells;
  for (int item = blockIdx.x * cpb + group; item < n_items; item += gridDim.x * cpb) {
    const int cell = A.cell_list ? A.cell_list[item] : item;
    const int64_t base = A.node_ptr[cell];
    const int K = (int)(A.node_ptr[cell + 1] - base);
    if (K > kmax) {  // the list's size bound was wrong: flag the cell, never overrun
      if (lane == 0) A.spike_count[cell] = INT32_MIN;
      continue;
    }
    const int plan = A.plan_of ? A.plan_of[cell] : cell;
    const int64_t pn = A.plan_node_ptr[plan], pl = A.plan_layer_off[plan];
    const int L = (int)(A.plan_layer_off[plan + 1] - pl - 1);
    // stage the plan (16-bit) and the axial conductances
    for (int i = lane; i < K; i += TPC) {
      sOrder[i] = (uint16_t)A.order[pn + i];
      const int32_t p = A.parent[pn + i];
      sParent[i] = p >= 0 ? (uint16_t)p : (uint16_t)0xFFFFu;
      sCptr[i] = (uint16_t)A.child_ptr[pn + plan + i];
      sCidx[i] = (uint16_t)A.child_idx[pn + i];
      sG[i] = A.a_geom[base + i];
      sV[i] = A.v[base + i];
    }
    if (lane == 0) sCptr[K] = (uint16_t)A.child_ptr[pn + plan + K];
    TreeTopoT<uint16_t> t{sParent, sOrder, sLptr, sCptr, sCidx, K, L};
    ChainTopoT<uint16_t> ct{sOrder, sLptr, sLptr, 0};
    if (chains) {
      // chain nodes replace the order; chain_ptr and the chain levels follow
      const int64_t cp0 = A.plan_chain_off[plan], cl0 = A.plan_clevel_off[plan];
      const int NC = (int)(A.plan_chain_off[plan + 1] - cp0 - 1);
      const int NL = (int)(A.plan_clevel_off[plan + 1] - cl0 - 1);
      uint16_t* sLev = sLptr + NC + 1;
      for (int i = lane; i < K; i += TPC) sOrder[i] = (uint16_t)A.chain_nodes[pn + i];
      for (int c = lane; c <= NC; c += TPC) sLptr[c] = (uint16_t)A.chain_ptr[cp0 + c];
      for (int l = lane; l <= NL; l += TPC) sLev[l] = (uint16_t)A.chain_level[cl0 + l];
      ct = ChainTopoT<uint16_t>{sOrder, sLptr, sLev, NL};
    } else {
      for (int l = lane; l <= L; l += TPC) sLptr[l] = (uint16_t)A.layer_ptr[pl + l];
    }
    const int32_t* nsp = A.node_syn_ptr + base + cell;  // K+1 entries
    const int64_t s0 = A.syn_ptr[cell];
    const int S = (int)(A.syn_ptr[cell + 1] - s0);
    const T* area = A.area + base;
    const T* cmdt = A.cm_dt + base;
    const T* gl = A.gl + base;
    const T* el = A.el + base;
    // local node of the cell's injected current (-1: none)
    const int in_i = (A.in_node && A.in_amp) ? A.in_node[cell] : -1;
    T m = T(0), h = T(0), nn = T(0);
    int below = 1, count = 0;
    if (lane == 0) {
      m = A.m[cell];
      h = A.h[cell];
      nn = A.n[cell];
      below = A.below[cell];
      count = A.spike_count[cell];
    }
    unsigned long long bits = 0ull;
    cell_sync<T, TPC>(group);
    for (int s = 0; s < A.n_steps; ++s) {
      const int64_t g = A.step0 + s;
      const int64_t slot = (A.slot0 + s) % A.depth;
      T* row = A.ring + slot * A.n_syn + s0;
      // this step's drive (uniform over the cell)
      T Ive = T(0), Iin = T(0);
      if (A.ve_field || in_i >= 0) {
        const T t = (T)(A.t0_ms + (double)g * A.dt_d);
        if (A.ve_field) Ive = rect_pulse<T>(t, A.ve_amp[cell], A.ve_delay[cell], A.ve_pw[cell]);
        if (in_i >= 0) Iin = rect_pulse<T>(t, A.in_amp[cell], A.in_delay[cell], A.in_pw[cell]);
      }
      const bool ve_on = Ive != T(0);
      // 1. deliver today's events (and clear the row)
      const bool bg = A.bg_bits && ((A.bg_bits[g * A.bg_words + (cell >> 6)] >> (cell & 63)) & 1ull);
      // (with 3. the synapse decay, in the same pass: A = (A + w factor) decay_A;
      // the spike detection between them reads only v)
      for (int k = lane; k < S; k += TPC) {
        T w = row[k];
        if (w != T(0)) {
          row[k] = T(0);
        }
        if (bg && k == A.bg_syn) w = w + A.bg_weight;
        T sa = A.syn_A[s0 + k], sb = A.syn_B[s0 + k];
        if (w != T(0)) {
          const T inc = w * A.syn_factor[s0 + k];
          sa = sa + inc;
          sb = sb + inc;
        }
        A.syn_A[s0 + k] = sa * A.syn_decay_A[s0 + k];
        A.syn_B[s0 + k] = sb * A.syn_decay_B[s0 + k];
      }
      // 2. rising edge at the soma on the previous step's v
      if (lane == 0) {
        const bool above = sV[0] >= A.thr;
        if (above && below) {
          bits |= 1ull << s;
          count += 1;
        }
        below = above ? 0 : 1;
      }
      // 3. state advance: soma gates at v_old (the synapse decay ran above)
      if (lane == 0) hh_gates<T>(sV[0], A.q10, A.dt, m, h, nn);
      cell_sync<T, TPC>(group);
      // 4. assemble the tree system into sD (main) and sB (rhs); two nodes per
      // pass, their global loads issued together
      auto assemble = [&](int i, T gli, T eli, T ar, T cmi, int k0, int k1) {
        const T vi = sV[i];
        T G, J;
        if (i == 0) {
          hh_affine<T>(m, h, nn, A.gnabar, A.gkbar, gli, eli, A.ena, A.ek, G, J);
        } else {
          G = gli;
          J = mul_rn(gli, eli);
        }
        for (int k = k0; k < k1; ++k) {
          // Exp2Syn: g = B - A (uS) -> density g / (1e6 area) (S/cm^2)
          const T gs = (A.syn_B[s0 + k] - A.syn_A[s0 + k]) / (T(1e6) * ar);
          G = G + gs;
          J = J + mul_rn(gs, A.e_syn);
        }
        T f = (J - mul_rn(G, vi)) * ar;
        const uint16_t p = sParent[i];
        if (has_parent(p)) f = f - mul_rn(sG[i], vi - sV[p]);
        for (int k = sCptr[i]; k < sCptr[i + 1]; ++k) {
          const int c = sCidx[k];
          f = f + mul_rn(sG[c], sV[c] - vi);
        }
        if (ve_on) {  // extracellular edge currents, summed on their own
          const T* fld = A.ve_field + base;
          const T vei = mul_rn(fld[i], Ive);
          T S = T(0);
          if (has_parent(p)) S = S - mul_rn(sG[i], vei - mul_rn(fld[p], Ive));
          for (int k = sCptr[i]; k < sCptr[i + 1]; ++k) {
            const int c = sCidx[k];
            S = S + mul_rn(sG[c], mul_rn(fld[c], Ive) - vei);
          }
          f = f + S;
        }
        if (i == in_i) f = f + Iin;
        sB[i] = f;
        sD[i] = cmi + mul_rn(G, ar);
      };
      for (int i0 = lane; i0 < K; i0 += 2 * TPC) {
        const int i1 = i0 + TPC;
        const bool two = i1 < K;
        const T gl0 = gl[i0], el0 = el[i0], ar0 = area[i0], cm0 = cmdt[i0];
        const int a0 = nsp[i0], b0 = nsp[i0 + 1];
        T gl1 = T(0), el1 = T(0), ar1 = T(1), cm1 = T(0);
        int a1 = 0, b1 = 0;
        if (two) {
          gl1 = gl[i1];
          el1 = el[i1];
          ar1 = area[i1];
          cm1 = cmdt[i1];
          a1 = nsp[i1];
          b1 = nsp[i1 + 1];
        }
        assemble(i0, gl0, el0, ar0, cm0, a0, b0);
        if (two) assemble(i1, gl1, el1, ar1, cm1, a1, b1);
      }
      cell_sync<T, TPC>(group);
      if (chains) {
        chain_eliminate<T, uint16_t, TPC, Sync, kFastRcp<T>>(t, ct, sG, sD, sB, lane, sync);
        chain_substitute<T, uint16_t, TPC, Sync, kFastRcp<T>>(t, ct, sG, sD, sB, lane, sync);
      } else {
        dhs_eliminate<T, uint16_t, TPC, Sync, kFastRcp<T>>(t, sG, sD, sB, lane, sync);
        dhs_substitute<T, uint16_t, TPC, Sync, kFastRcp<T>>(t, sG, sD, sB, lane, sync);
      }
      for (int i = lane; i < K; i += TPC) sV[i] = sV[i] + sB[i];
      cell_sync<T, TPC>(group);
    }
    for (int i = lane; i < K; i += TPC) A.v[base + i] = sV[i];
    if (lane == 0) {
      A.m[cell] = m;
      A.h[cell] = h;
      A.n[cell] = nn;
      A.below[cell] = (uint8_t)below;
      A.spike_count[cell] = count;
      A.spike_bits[cell] = bits;
    }
    cell_sync<T, TPC>(group);
  }
}

// ring[(slot0 + s + delay[e]) % depth][t] += weight[e] for every connection e
// of target t whose source spiked at window step s.
template <typename T>
__global__ void net_enqueue_kernel(T* __restrict__ ring, int64_t depth, int64_t n_syn,
                                   int64_t slot0, const int64_t* __restrict__ post_ptr,
                                   int64_t n_post, const int64_t* __restrict__ post_col,
                                   const int64_t* __restrict__ pre,
                                   const int64_t* __restrict__ delay, const T* __restrict__ weight,
                                   const unsigned long long* __restrict__ spike_bits) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_post) return;
  const int64_t col = post_col ? post_col[p] : p;
  for (int64_t e = post_ptr[p]; e < post_ptr[p + 1]; ++e) {
    unsigned long long bits = spike_bits[pre[e]];
    while (bits) {
      const int s = __ffsll((long long)bits) - 1;
      bits &= bits - 1;
      const int64_t r = (slot0 + s + delay[e]) % depth;
      T* cell = ring + r * n_syn + col;
      *cell = *cell + weight[e];
    }
  }
}

template <typename T>
static NetArgsT<T> net_typed(const dgb_net_args* a) {
  NetArgsT<T> t;
  t.n_cells = a->n_cells;
  t.n_steps = a->n_steps;
  t.step0 = a->step0;
  t.depth = a->depth;
  t.slot0 = a->slot0;
  t.n_syn = a->n_syn;
  t.node_ptr = a->forest.node_ptr;
  t.plan_of = a->forest.plan_of;
  t.plan_node_ptr = a->forest.plan_node_ptr;
  t.plan_layer_off = a->forest.plan_layer_off;
  t.parent = a->forest.parent;
  t.order = a->forest.order;
  t.layer_ptr = a->forest.layer_ptr;
  t.child_ptr = a->forest.child_ptr;
  t.child_idx = a->forest.child_idx;
  t.plan_chain_off = a->forest.plan_chain_off;
  t.plan_clevel_off = a->forest.plan_clevel_off;
  t.chain_nodes = a->forest.chain_nodes;
  t.chain_ptr = a->forest.chain_ptr;
  t.chain_level = a->forest.chain_level;
  t.v = (T*)a->v;
  t.area = (const T*)a->area;
  t.cm_dt = (const T*)a->cm_dt;
  t.a_geom = (const T*)a->a_geom;
  t.gl = (const T*)a->gl;
  t.el = (const T*)a->el;
  t.m = (T*)a->m;
  t.h = (T*)a->h;
  t.n = (T*)a->n;
  t.gnabar = (T)a->gnabar;
  t.gkbar = (T)a->gkbar;
  t.ena = (T)a->ena;
  t.ek = (T)a->ek;
  t.q10 = (T)a->q10;
  t.dt = (T)a->dt_ms;
  t.thr = (T)a->spk_thr;
  t.syn_ptr = a->syn_ptr;
  t.node_syn_ptr = a->node_syn_ptr;
  t.syn_A = (T*)a->syn_A;
  t.syn_B = (T*)a->syn_B;
  t.syn_factor = (const T*)a->syn_factor;
  t.syn_decay_A = (const T*)a->syn_decay_A;
  t.syn_decay_B = (const T*)a->syn_decay_B;
  t.e_syn = (T)a->e_syn;
  t.ring = (T*)a->ring;
  t.bg_bits = (const unsigned long long*)a->bg_bits;
  t.bg_words = a->bg_words;
  t.bg_syn = a->bg_syn;
  t.bg_weight = (T)a->bg_weight;
  t.ve_field = (const T*)a->ve_field;
  t.ve_amp = (const T*)a->ve_amp;
  t.ve_delay = (const T*)a->ve_delay;
  t.ve_pw = (const T*)a->ve_pw;
  t.in_node = a->in_node;
  t.in_amp = (const T*)a->in_amp;
  t.in_delay = (const T*)a->in_delay;
  t.in_pw = (const T*)a->in_pw;
  t.t0_ms = a->t0_ms;
  t.dt_d = a->dt_ms;
  t.below = a->below;
  t.spike_bits = (unsigned long long*)a->spike_bits;
  t.spike_count = a->spike_count;
  t.cell_list = a->cell_list;
  t.n_list = a->n_list;
  return t;
}

template <typename T>
static int net_window_t(const dgb_net_args* a, cudaStream_t st) {
  const int kmax = a->cell_list ? a->list_max_k : a->forest.max_k;
  const int n_items = a->cell_list ? a->n_list : a->n_cells;
  if (kmax > 65534) {
    set_error("cells of more than 65,534 compartments are not supported (got %d)", kmax);
    return DGB_ERANGE;
  }
  const size_t per_cell = net_warp_smem<T>(kmax);
  const int tpc = a->threads_per_cell > 0 ? a->threads_per_cell : 128;
  // block: warps_per_block warps (at least one group), cells = threads / tpc,
  // halved while the cells' shared memory exceeds 227 KB
  int threads = 32 * (a->warps_per_block > 0 ? a->warps_per_block : 4);
  if (threads < tpc) threads = tpc;
  const int max_threads = tpc > 128 ? tpc : 128;  // the instantiation's launch bound
  if (threads > max_threads) threads = max_threads;
  while (threads > tpc && (size_t)(threads / tpc) * per_cell > 227 * 1024) threads >>= 1;
  const size_t smem = (size_t)(threads / tpc) * per_cell;
  if (smem > 227 * 1024) {
    set_error("cell of %d compartments too large for shared memory", kmax);
    return DGB_ERANGE;
  }
  auto kern = tpc == 512   ? net_window_kernel<T, 512>
              : tpc == 256 ? net_window_kernel<T, 256>
              : tpc == 128 ? net_window_kernel<T, 128>
              : tpc == 64  ? net_window_kernel<T, 64>
                           : net_window_kernel<T, 32>;
  DGB_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  int per_sm = 0;
  DGB_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  int blocks = device_sm_count() * per_sm;
  const int cpb = threads / tpc;
  const int need = (n_items + cpb - 1) / cpb;
  if (blocks > need) blocks = need;
  kern<<<blocks, threads, smem, st>>>(net_typed<T>(a), kmax);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_net_window(const dgb_net_args* a, void* stream) {
  clear_error();
  DGB_REQUIRE(a != nullptr, "args must be non-null");
  DGB_REQUIRE(a->dtype == DGB_F32 || a->dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(a->n_steps >= 0 && a->n_steps <= 64, "window length must be in [0, 64]");
  DGB_REQUIRE(a->depth >= 1 && a->slot0 >= 0 && a->slot0 < a->depth, "bad ring depth/slot");
  DGB_REQUIRE(a->n_cells >= 0, "n_cells must be >= 0");
  if (a->n_cells == 0) return DGB_OK;
  DGB_REQUIRE(a->forest.node_ptr && a->forest.plan_node_ptr && a->forest.plan_layer_off &&
                  a->forest.parent && a->forest.order && a->forest.layer_ptr &&
                  a->forest.child_ptr && a->forest.child_idx,
              "forest arrays must be non-null");
  DGB_REQUIRE(a->v && a->area && a->cm_dt && a->a_geom && a->gl && a->el && a->m && a->h && a->n,
              "per-node and soma arrays must be non-null");
  DGB_REQUIRE(a->syn_ptr && a->node_syn_ptr && a->syn_A && a->syn_B && a->syn_factor &&
                  a->syn_decay_A && a->syn_decay_B && a->ring,
              "synapse arrays and ring must be non-null");
  DGB_REQUIRE(a->below && a->spike_bits && a->spike_count, "spike outputs must be non-null");
  DGB_REQUIRE(a->forest.max_k >= 1, "cells must have at least one compartment");
  DGB_REQUIRE(!a->cell_list || (a->n_list >= 0 && a->list_max_k >= 1),
              "a cell list needs n_list >= 0 and list_max_k >= 1");
  if (a->cell_list && a->n_list == 0) return DGB_OK;
  DGB_REQUIRE(!a->ve_field || (a->ve_amp && a->ve_delay && a->ve_pw),
              "ve_field requires ve_amp, ve_delay and ve_pw");
  DGB_REQUIRE(!a->in_node || (a->in_amp && a->in_delay && a->in_pw),
              "in_node requires in_amp, in_delay and in_pw");
  DGB_REQUIRE(!a->forest.chain_nodes || (a->forest.chain_ptr && a->forest.chain_level &&
                                         a->forest.plan_chain_off && a->forest.plan_clevel_off),
              "the chain schedule needs chain_ptr, chain_level and their plan offsets");
  DGB_REQUIRE(a->warps_per_block == 0 || a->warps_per_block == 1 || a->warps_per_block == 2 ||
                  a->warps_per_block == 4 || a->warps_per_block == 8,
              "warps_per_block must be 0 (default), 1, 2, 4 or 8, got %d", a->warps_per_block);
  DGB_REQUIRE(a->threads_per_cell == 0 || a->threads_per_cell == 32 ||
                  a->threads_per_cell == 64 || a->threads_per_cell == 128 ||
                  a->threads_per_cell == 256 || a->threads_per_cell == 512,
              "threads_per_cell must be 0 (default 128), 32, 64, 128, 256 or 512, got %d",
              a->threads_per_cell);
  cudaStream_t st = as_stream(stream);
  if (a->dtype == DGB_F32) return net_window_t<float>(a, st);
  return net_window_t<double>(a, st);
}

extern "C" int dgb_net_enqueue(int dtype, void* ring, int64_t depth, int64_t n_syn, int64_t slot0,
                               const int64_t* post_ptr, int64_t n_post, const int64_t* post_col,
                               const int64_t* pre, const int64_t* delay_steps,
                               const void* weight, const uint64_t* spike_bits, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(depth >= 1 && slot0 >= 0 && n_post >= 0 && n_syn >= 0, "bad sizes");
  if (n_post == 0) return DGB_OK;
  DGB_REQUIRE(ring && post_ptr && pre && delay_steps && weight && spike_bits,
              "pointers must be non-null");
  const int th = 256;
  const unsigned blocks = (unsigned)((n_post + th - 1) / th);
  cudaStream_t st = as_stream(stream);
  const auto* bits = (const unsigned long long*)spike_bits;
  if (dtype == DGB_F32)
    net_enqueue_kernel<float><<<blocks, th, 0, st>>>((float*)ring, depth, n_syn, slot0, post_ptr,
                                                     n_post, post_col, pre, delay_steps,
                                                     (const float*)weight, bits);
  else
    net_enqueue_kernel<double><<<blocks, th, 0, st>>>((double*)ring, depth, n_syn, slot0, post_ptr,
                                                      n_post, post_col, pre, delay_steps,
                                                      (const double*)weight, bits);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}
