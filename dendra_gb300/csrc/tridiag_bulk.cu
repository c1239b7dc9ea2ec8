// Bulk-staged batched tridiagonal solve for sm_103a: the same chunked
// Thomas + PCR solve as tridiag_kernel (chunk_solve.cuh), with the bands
// brought into shared memory by bulk copies instead of per-lane loads.
//
// A CTA of four warps owns tiles of S consecutive systems (S = 4 * 32/P):
// the tile's slices of a, c, b and d are contiguous byte ranges, so one
// thread posts four cp.async.bulk copies per tile and the copy engine streams
// them into shared memory while the warps solve the previous tile (two
// stages, one mbarrier each).  Every lane then reads its CH consecutive rows
// from shared memory (a stride of CH words across lanes: conflict-free for
// odd CH), solves in registers, writes x back over its d rows and the warp
// stores its systems' x with coalesced 16-byte stores.
//
// Bulk copies need 16-byte aligned addresses and sizes: each band slice is
// widened down to the 16-byte boundary below its first element (those extra
// elements belong to the previous tile and are not used) and its last
// partial 16 bytes are loaded by plain loads.  Band pointers that are not
// 16-byte aligned, or tiles whose two stages do not fit kMaxSmem, take the
// register-direct kernel instead (tridiag.cu).
//
// Every mbarrier wait is bounded.  A wait that gives up sets the fault word
// (read by dgb_tridiag_status), lets thread 0 wait for the copies still in
// flight, and ends the CTA; the context stays usable.
#include <atomic>

#include "bulk.cuh"
#include "chunk_solve.cuh"

namespace dgb {

namespace tbulk {

constexpr int kWarps = 4;  // warps per CTA; 2 or 1 when four systems' stages do not fit
constexpr uint32_t kWaitLimit = 1u << 22;  // polls before a wait gives up
constexpr int64_t kMaxSmem = 110 * 1024;   // two stages; keeps >= 2 CTAs per SM
constexpr unsigned kFaultTimeout = 1;      // a stage wait gave up; its tiles were not solved
constexpr unsigned kFaultSuspect = 2;      // the drain gave up too: copies may be in flight

// fault bits of the bulk-staged solves on this device since the last status read
__device__ unsigned g_fault;
// polls per stage wait; lowered only by dgb_tridiag_set_wait_limit
std::atomic<uint32_t> g_wait_limit{kWaitLimit};

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
};
template <>
struct Vec16<double> {
  using type = double2;
};

// Shared-memory band region of one stage, in elements:
//   [E front gap][copied slice: up to E-1 widening elements + S systems][slack]
// The front gap keeps the read of row -1 (the absent a_0) inside the region;
// the slack keeps the reads of rows past K of the tile's last system inside
// it.  Rows outside a system are read unconditionally and replaced by
// identity rows, so every read must land in shared memory, never be used.
template <typename T>
__host__ __device__ inline int64_t band_cap(int64_t S, int64_t L, int64_t rows_per_system) {
  constexpr int64_t E = 16 / sizeof(T);
  const int64_t span = (S - 1) * L + (rows_per_system > L ? rows_per_system : L);
  return (E + E - 1 + span + E - 1) / E * E;
}

// Post the copies of systems [s0, s1) into one stage: bands a, c (L = K-1)
// then b, d (L = K), each landing E elements into its region.  Thread 0 arms
// the barrier and posts the bulk copies; threads 0..3 load the partial last
// 16 bytes of bands 0..3.
template <typename T>
__device__ __forceinline__ void stage_tile(const T* a, const T* b, const T* c, const T* d,
                                           int64_t K, int64_t s0, int64_t s1, T* stage,
                                           int64_t cap_ac, int64_t cap_bd, uint32_t bar,
                                           int tid) {
  constexpr int64_t E = 16 / sizeof(T);
  const T* src[4] = {a, c, b, d};
  const int64_t len[4] = {K - 1, K - 1, K, K};
  const int64_t off[4] = {E, cap_ac + E, 2 * cap_ac + E, 2 * cap_ac + cap_bd + E};
  if (tid == 0) {
    uint32_t bytes = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t lo16 = (s0 * len[q]) & ~(E - 1);
      const int64_t hi16 = (s1 * len[q]) & ~(E - 1);
      if (hi16 > lo16) bytes += (uint32_t)((hi16 - lo16) * (int64_t)sizeof(T));
    }
    bulk::bar_expect(bar, bytes);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t lo16 = (s0 * len[q]) & ~(E - 1);
      const int64_t hi16 = (s1 * len[q]) & ~(E - 1);
      if (hi16 > lo16)
        bulk::load(bulk::smem_addr(stage + off[q]), src[q] + lo16,
                   (uint32_t)((hi16 - lo16) * (int64_t)sizeof(T)), bar);
    }
  }
  if (tid < 4) {
    const T* s = tid == 0 ? a : tid == 1 ? c : tid == 2 ? b : d;
    const int64_t L = tid < 2 ? K - 1 : K;
    T* dst = stage + E + (tid == 0 ? 0 : tid == 1 ? cap_ac : tid == 2 ? 2 * cap_ac
                                                                      : 2 * cap_ac + cap_bd);
    const int64_t lo = s0 * L, hi = s1 * L;
    const int64_t lo16 = lo & ~(E - 1);
    int64_t e = hi & ~(E - 1);
    if (e < lo) e = lo;
    for (; e < hi; ++e) dst[e - lo16] = s[e];
  }
}

template <typename T, int CH, int P, int NW>
__global__ void __launch_bounds__(NW * 32)
    tridiag_bulk_kernel(int64_t B, int64_t K, const T* __restrict__ a, const T* __restrict__ b,
                        const T* __restrict__ c, const T* d, T* x, int64_t cap_ac,
                        int64_t cap_bd, uint32_t wait_limit) {
  constexpr int G = 32 / P;       // systems per warp
  constexpr int S = NW * G;       // systems per tile
  constexpr int E = 16 / sizeof(T);
  using V = typename Vec16<T>::type;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const int r = lane % P;
  const int g = lane / P;
  const int Ki = (int)K;  // K <= 32 * 32 on this path
  const int64_t stage_elems = 2 * cap_ac + 2 * cap_bd;
  T* const stages = reinterpret_cast<T*>(smem_raw);
  const uint32_t bar0 = bulk::smem_addr(&bars[0]);
  const uint32_t bar1 = bulk::smem_addr(&bars[1]);
  const int64_t n_tiles = (B + S - 1) / S;

  // rows of this lane inside a system: [r*CH, r*CH + n_in) have a diagonal,
  // [r*CH, r*CH + n_up) a super-diagonal; row 0 has no sub-diagonal
  const int row0 = r * CH;
  const int n_in = min(max(Ki - row0, 0), CH);
  const int n_up = min(max(Ki - 1 - row0, 0), CH);

  if (tid == 0) {
    bulk::bar_init(bar0, 1);
    bulk::bar_init(bar1, 1);
    bulk::bar_init_fence();
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int64_t tile = blockIdx.x + (int64_t)k * gridDim.x;
    if (tile < n_tiles)
      stage_tile(a, b, c, d, K, tile * S, min(B, tile * S + S), stages + k * stage_elems,
                 cap_ac, cap_bd, k ? bar1 : bar0, tid);
  }

  int k = 0;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++k) {
    const int s = k & 1;
    T* const st = stages + s * stage_elems;
    const uint32_t bar = s ? bar1 : bar0;
    const bool landed = bulk::bar_wait(bar, (k >> 1) & 1, wait_limit);
    // also publishes the plain tail loads of this stage
    if (__syncthreads_or(!landed)) {
      if (tid == 0) {
        unsigned bits = kFaultTimeout;
        // drain: this stage's copies, and the other stage's if it was posted
        if (!bulk::bar_wait(bar, (k >> 1) & 1, kWaitLimit)) bits |= kFaultSuspect;
        if (tile + gridDim.x < n_tiles &&
            !bulk::bar_wait(s ? bar0 : bar1, ((k + 1) >> 1) & 1, kWaitLimit))
          bits |= kFaultSuspect;
        atomicOr(&g_fault, bits);
      }
      return;
    }

    const int64_t t0 = tile * S;
    const int gs = warp * G + g;  // this group's system within the tile
    const bool live = t0 + gs < B;
    // widening of the tile's first element to 16 bytes, per band pair
    const int sh_ac = (int)((t0 * (K - 1)) & (E - 1));
    const int sh_bd = (int)((t0 * K) & (E - 1));
    const T* sa = st + E + sh_ac + gs * (Ki - 1) + row0;
    const T* sc = sa + cap_ac;
    T* const sb = st + 2 * cap_ac + E + sh_bd + gs * Ki + row0;
    T* const sd = sb + cap_bd;

    T ra[CH], rb[CH], rc[CH], rd[CH];
#pragma unroll
    for (int j = 0; j < CH; ++j) {
      // unconditional reads (inside the region by its gap and slack), then
      // identity rows outside the system
      const T av = sa[j - 1], bv = sb[j], cv = sc[j], dv = sd[j];
      const bool in = live && j < n_in;
      ra[j] = (in && (j > 0 || r > 0)) ? av : T(0);
      rc[j] = (live && j < n_up) ? cv : T(0);
      rb[j] = in ? bv : T(1);
      rd[j] = in ? dv : T(0);
    }
    chunk_solve<T, CH, P, kFastRcp<T>>(ra, rb, rc, rd, r);
#pragma unroll
    for (int j = 0; j < CH; ++j)
      if (live && j < n_in) sd[j] = rd[j];
    __syncwarp();

    // coalesced store of this warp's systems: n elements from x + e0; the
    // first `head` up to a 16-byte boundary, then 16-byte vectors, then the
    // rest (element e of x sits at e - lo16 after the region's gap)
    {
      const int64_t w0 = min(B, t0 + warp * G), w1 = min(B, t0 + warp * G + G);
      const int64_t e0 = w0 * K;
      const int n = (int)((w1 - w0) * K);
      T* xw = x + e0;
      const T* sw = st + 2 * cap_ac + cap_bd + E + (e0 - ((t0 * K) & ~(int64_t)(E - 1)));
      const int head = min(n, (int)((E - (e0 & (E - 1))) & (E - 1)));
      const int nv = (n - head) / E;
      if (lane < head) xw[lane] = sw[lane];
      for (int v = lane; v < nv; v += 32)
        *reinterpret_cast<V*>(xw + head + v * E) =
            *reinterpret_cast<const V*>(sw + head + v * E);
      for (int t = head + nv * E + lane; t < n; t += 32) xw[t] = sw[t];
    }

    // every warp is done with this stage before the next copies overwrite it
    bulk::fence_async_smem();
    __syncthreads();
    const int64_t next = tile + 2 * (int64_t)gridDim.x;
    if (next < n_tiles)
      stage_tile(a, b, c, d, K, next * S, min(B, next * S + S), st, cap_ac, cap_bd, bar, tid);
  }
}

// Resident CTAs per SM of `kern` with `smem` bytes of dynamic shared memory,
// cached per device as (smem << 8 | CTAs): the shared-memory opt-in and the
// occupancy query run once per device and size, not on every solve.
constexpr int kMaxDevices = 64;
template <typename K_>
static int resident_per_sm(K_ kern, int threads, int64_t smem, std::atomic<int64_t>* cache) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) dev = -1;
  if (dev >= 0) {
    const int64_t v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0 && (v >> 8) == smem) return (int)(v & 255);
  }
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem) !=
          cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, (size_t)smem) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 1;
  if (per_sm > 255) per_sm = 255;
  if (dev >= 0) cache[dev].store((smem << 8) | per_sm, std::memory_order_relaxed);
  return per_sm;
}

template <typename T, int CH, int P, int NW>
static int launch_nw(int64_t B, int64_t K, const T* a, const T* b, const T* c, const T* d, T* x,
                     cudaStream_t st) {
  constexpr int S = NW * (32 / P);
  const int64_t cap_ac = band_cap<T>(S, K - 1, (int64_t)P * CH),
                cap_bd = band_cap<T>(S, K, (int64_t)P * CH);
  const int64_t smem = 2 * (2 * cap_ac + 2 * cap_bd) * (int64_t)sizeof(T);
  if (smem > kMaxSmem) return 1;
  auto kern = tridiag_bulk_kernel<T, CH, P, NW>;
  static std::atomic<int64_t> cache[kMaxDevices];
  const int per_sm = resident_per_sm(kern, NW * 32, smem, cache);
  if (per_sm < 0) {
    set_error("cudaFuncSetAttribute(tridiag_bulk_kernel, %lld bytes of shared memory) failed: %s",
              (long long)smem, cudaGetErrorString(cudaGetLastError()));
    return DGB_ECUDA;
  }
  const int64_t n_tiles = (B + S - 1) / S;
  const int64_t cap = (int64_t)device_sm_count() * per_sm;
  const int blocks = (int)(n_tiles < cap ? n_tiles : cap);
  kern<<<blocks, NW * 32, (size_t)smem, st>>>(B, K, a, b, c, d, x, cap_ac, cap_bd,
                                             g_wait_limit.load());
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

// Four warps per CTA; long systems at 32 lanes whose four-system stages do
// not fit fall back to two-warp, then one-warp CTAs (fewer systems per tile).
template <typename T, int CH, int P>
static int launch(int64_t B, int64_t K, const T* a, const T* b, const T* c, const T* d, T* x,
                  cudaStream_t st) {
  int rc = launch_nw<T, CH, P, kWarps>(B, K, a, b, c, d, x, st);
  if constexpr (P == 32 && CH >= 13) {
    if (rc == 1) rc = launch_nw<T, CH, P, 2>(B, K, a, b, c, d, x, st);
    if (rc == 1) rc = launch_nw<T, CH, P, 1>(B, K, a, b, c, d, x, st);
  }
  return rc;
}

template <typename T, int P>
static int launch_p(int ch, int64_t B, int64_t K, const T* a, const T* b, const T* c,
                    const T* d, T* x, cudaStream_t st) {
  switch (ch) {
#define DGB_CASE(CHV) \
  case CHV:           \
    return launch<T, CHV, P>(B, K, a, b, c, d, x, st);
    DGB_CASE(1) DGB_CASE(3) DGB_CASE(5) DGB_CASE(7) DGB_CASE(9) DGB_CASE(11)
    DGB_CASE(13) DGB_CASE(15) DGB_CASE(17) DGB_CASE(21) DGB_CASE(25) DGB_CASE(33)
#undef DGB_CASE
    default:
      return 1;
  }
}

template <typename T>
static int dispatch(int P, int ch, int64_t B, int64_t K, const T* a, const T* b, const T* c,
                    const T* d, T* x, cudaStream_t st) {
  // every band base 16-byte aligned (a and c are unused when K == 1)
  auto al = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
  if (!al(b) || !al(d) || !al(x) || (K > 1 && (!al(a) || !al(c)))) return 1;
  switch (P) {
    case 4: return launch_p<T, 4>(ch, B, K, a, b, c, d, x, st);
    case 8: return launch_p<T, 8>(ch, B, K, a, b, c, d, x, st);
    case 16: return launch_p<T, 16>(ch, B, K, a, b, c, d, x, st);
    case 32: return launch_p<T, 32>(ch, B, K, a, b, c, d, x, st);
    default: return 1;
  }
}

}  // namespace tbulk

int tridiag_bulk(int P, int ch, int64_t B, int64_t K, const float* a, const float* b,
                 const float* c, const float* d, float* x, cudaStream_t st) {
  return tbulk::dispatch<float>(P, ch, B, K, a, b, c, d, x, st);
}
int tridiag_bulk(int P, int ch, int64_t B, int64_t K, const double* a, const double* b,
                 const double* c, const double* d, double* x, cudaStream_t st) {
  return tbulk::dispatch<double>(P, ch, B, K, a, b, c, d, x, st);
}

}  // namespace dgb

extern "C" int dgb_tridiag_status(void* stream) {
  dgb::clear_error();
  DGB_CUDA_CHECK(cudaStreamSynchronize(dgb::as_stream(stream)));
  unsigned h = 0, zero = 0;
  DGB_CUDA_CHECK(cudaMemcpyFromSymbol(&h, dgb::tbulk::g_fault, sizeof(h)));
  if (!h) return DGB_OK;
  DGB_CUDA_CHECK(cudaMemcpyToSymbol(dgb::tbulk::g_fault, &zero, sizeof(zero)));
  if (h & dgb::tbulk::kFaultSuspect) {
    dgb::set_error("a tridiagonal stage wait gave up and its drain did not finish (fault bits "
                   "%u): copies may still be outstanding, treat this CUDA context as unusable",
                   h);
    return DGB_ETIMEOUT;
  }
  dgb::set_error("a tridiagonal stage wait gave up (fault bits %u); the affected systems were "
                 "not solved, the context is still usable", h);
  return DGB_ETIMEOUT;
}

extern "C" int dgb_tridiag_set_wait_limit(int64_t polls) {
  dgb::clear_error();
  const int64_t full = (int64_t)dgb::tbulk::kWaitLimit;
  dgb::tbulk::g_wait_limit.store((uint32_t)(polls < 0 ? full : (polls > full ? full : polls)));
  return DGB_OK;
}
