// Event transport for spiking networks on sm_103a: spike detection, bit
// packing, delayed delivery.  Deterministic everywhere: every output value is
// produced by exactly one thread, summing its inputs in a fixed order, so no
// floating-point atomics are used (the reference's CUDA/Triton delivery
// kernels use atomicAdd, netcon_bitpack_kernel.cu:91,124).
//
//   dgb_detect_spikes        threshold_transition / update_active
//                            (networks/spiking.py:7-73): rising edge v >= thr
//   dgb_pack_source_spikes   pack_source_spikes (netcon_bitpack_kernel.cu:20-57)
//   dgb_build_delivery       build_delivery (netcon_bitpack_kernel.cu:59-93)
//   dgb_ring_enqueue         the enqueue of dense_fixed_delay_transition
//                            (networks/_event_delivery.py:61-199)
#include "common.cuh"

namespace dgb {

constexpr int kBitsPerWord = 63;

// spikes[s] = (v[comp[s]] >= thr) && below[s];  below[s] = !(v >= thr)
template <typename T>
__global__ void detect_kernel(const T* __restrict__ v, const int64_t* __restrict__ comp,
                              int64_t n, T thr, uint8_t* __restrict__ below,
                              uint8_t* __restrict__ spikes) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const bool above = v[comp ? comp[s] : s] >= thr;
  spikes[s] = (above && below[s]) ? 1 : 0;
  below[s] = above ? 0 : 1;
}

// One warp per 63-source word: two ballots, no atomics.
__global__ void pack_kernel(const uint8_t* __restrict__ src, int64_t n_source,
                            unsigned long long* __restrict__ hist, int64_t n_words,
                            const int64_t* __restrict__ step_ptr) {
  const int64_t word = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (word >= n_words) return;
  const int64_t s0 = word * kBitsPerWord + lane;
  const int64_t s1 = s0 + 32;
  const bool b0 = s0 < n_source && src[s0] != 0;
  const bool b1 = lane < kBitsPerWord - 32 && s1 < n_source && src[s1] != 0;
  const unsigned lo = __ballot_sync(0xffffffffu, b0);
  const unsigned hi = __ballot_sync(0xffffffffu, b1) & 0x7fffffffu;
  if (lane == 0) hist[step_ptr[0] * n_words + word] = (unsigned long long)lo | ((unsigned long long)hi << 32);
}

// Connections sorted by target (CSR post_ptr); thread p sums its targets'
// delayed events in connection order and adds the sum to out[p].  delay ==
// nullptr: every connection has the delay uniform_delay.
template <typename T>
__global__ void deliver_kernel(const unsigned long long* __restrict__ hist,
                               const int64_t* __restrict__ step_ptr,
                               const int64_t* __restrict__ delay, int64_t uniform_delay,
                               const int64_t* __restrict__ word_idx,
                               const int64_t* __restrict__ bit_mask,
                               const int64_t* __restrict__ post_ptr, int64_t n_post,
                               const T* __restrict__ weight, T* __restrict__ out,
                               int64_t max_delay, int64_t n_words) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_post) return;
  const int64_t now = step_ptr[0];
  // sequential adds in connection order: the result of adding each event to
  // out[p] one after another, like a CPU scatter-add over sorted connections
  T acc = out[p];
  bool any = false;
  for (int64_t e = post_ptr[p]; e < post_ptr[p + 1]; ++e) {
    int64_t row = now - (delay ? delay[e] : uniform_delay);
    if (row < 0) row += max_delay;
    const unsigned long long w = hist[row * n_words + word_idx[e]];
    if (w & (unsigned long long)bit_mask[e]) {
      acc = acc + weight[e];
      any = true;
    }
  }
  if (any) out[p] = acc;
}

// ring[(slot + delay[e]) % depth][p] += weight[e] * gate[pre[e]] for the
// connections e of target p, in connection order (CSR by target).
template <typename T>
__global__ void enqueue_kernel(T* __restrict__ ring, int64_t depth, int64_t width,
                               const int64_t* __restrict__ slot_ptr,
                               const int64_t* __restrict__ post_ptr, int64_t n_post,
                               const int64_t* __restrict__ post_col,
                               const int64_t* __restrict__ pre, const uint8_t* __restrict__ gate,
                               const int64_t* __restrict__ delay, const T* __restrict__ weight) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_post) return;
  const int64_t slot = slot_ptr[0];
  const int64_t col = post_col ? post_col[p] : p;
  for (int64_t e = post_ptr[p]; e < post_ptr[p + 1]; ++e) {
    if (!gate[pre[e]]) continue;
    int64_t row = slot + delay[e];
    row %= depth;
    T* cell = ring + row * width + col;
    *cell = *cell + weight[e];
  }
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_detect_spikes(int dtype, const void* v, const int64_t* comp, int64_t n,
                                 double thr, uint8_t* below, uint8_t* spikes, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n >= 0, "n must be >= 0");
  if (n == 0) return DGB_OK;
  DGB_REQUIRE(v && below && spikes, "v, below and spikes must be non-null");
  const int th = 256;
  const unsigned blocks = (unsigned)((n + th - 1) / th);
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32)
    detect_kernel<float><<<blocks, th, 0, st>>>((const float*)v, comp, n, (float)thr, below,
                                                spikes);
  else
    detect_kernel<double><<<blocks, th, 0, st>>>((const double*)v, comp, n, thr, below, spikes);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_pack_source_spikes(const uint8_t* source_spikes, int64_t n_source,
                                      int64_t* packed_history, int64_t n_words,
                                      const int64_t* current_time_step, void* stream) {
  clear_error();
  DGB_REQUIRE(n_source >= 0 && n_words >= 0, "sizes must be >= 0");
  DGB_REQUIRE(n_words * kBitsPerWord >= n_source,
              "n_words (%lld) too small for %lld sources (63 per word)", (long long)n_words,
              (long long)n_source);
  if (n_words == 0) return DGB_OK;
  DGB_REQUIRE(packed_history && current_time_step && (source_spikes || n_source == 0),
              "pointers must be non-null");
  const int wpb = 8;
  const unsigned blocks = (unsigned)((n_words + wpb - 1) / wpb);
  pack_kernel<<<blocks, wpb * 32, 0, as_stream(stream)>>>(
      source_spikes, n_source, (unsigned long long*)packed_history, n_words, current_time_step);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_build_delivery(int dtype, const int64_t* packed_history,
                                  const int64_t* current_time_step, const int64_t* delay_steps,
                                  const int64_t* conn_word_idx, const int64_t* conn_bit_mask,
                                  const int64_t* post_ptr, int64_t n_post, const void* weight,
                                  void* delivery_out, int64_t n_conn, int64_t max_delay_steps,
                                  int64_t n_words, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n_post >= 0 && n_conn >= 0, "sizes must be >= 0");
  DGB_REQUIRE(max_delay_steps >= 1, "max_delay_steps must be >= 1");
  if (n_post == 0) return DGB_OK;
  DGB_REQUIRE(packed_history && current_time_step && post_ptr && delivery_out,
              "pointers must be non-null");
  DGB_REQUIRE(n_conn == 0 || (delay_steps && conn_word_idx && conn_bit_mask && weight),
              "connection arrays must be non-null");
  const int th = 256;
  const unsigned blocks = (unsigned)((n_post + th - 1) / th);
  cudaStream_t st = as_stream(stream);
  const auto* h = (const unsigned long long*)packed_history;
  if (dtype == DGB_F32)
    deliver_kernel<float><<<blocks, th, 0, st>>>(h, current_time_step, delay_steps, 0,
                                                 conn_word_idx, conn_bit_mask, post_ptr, n_post,
                                                 (const float*)weight, (float*)delivery_out,
                                                 max_delay_steps, n_words);
  else
    deliver_kernel<double><<<blocks, th, 0, st>>>(h, current_time_step, delay_steps, 0,
                                                  conn_word_idx, conn_bit_mask, post_ptr, n_post,
                                                  (const double*)weight, (double*)delivery_out,
                                                  max_delay_steps, n_words);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_build_delivery_uniform(int dtype, const int64_t* packed_history,
                                          const int64_t* current_time_step, int64_t delay_step,
                                          const int64_t* conn_word_idx,
                                          const int64_t* conn_bit_mask, const int64_t* post_ptr,
                                          int64_t n_post, const void* weight, void* delivery_out,
                                          int64_t n_conn, int64_t max_delay_steps,
                                          int64_t n_words, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(n_post >= 0 && n_conn >= 0, "sizes must be >= 0");
  DGB_REQUIRE(max_delay_steps >= 1, "max_delay_steps must be >= 1");
  DGB_REQUIRE(delay_step >= 0 && delay_step < max_delay_steps,
              "delay_step must be in [0, max_delay_steps)");
  if (n_post == 0) return DGB_OK;
  DGB_REQUIRE(packed_history && current_time_step && post_ptr && delivery_out,
              "pointers must be non-null");
  DGB_REQUIRE(n_conn == 0 || (conn_word_idx && conn_bit_mask && weight),
              "connection arrays must be non-null");
  const int th = 256;
  const unsigned blocks = (unsigned)((n_post + th - 1) / th);
  cudaStream_t st = as_stream(stream);
  const auto* h = (const unsigned long long*)packed_history;
  if (dtype == DGB_F32)
    deliver_kernel<float><<<blocks, th, 0, st>>>(h, current_time_step, nullptr, delay_step,
                                                 conn_word_idx, conn_bit_mask, post_ptr, n_post,
                                                 (const float*)weight, (float*)delivery_out,
                                                 max_delay_steps, n_words);
  else
    deliver_kernel<double><<<blocks, th, 0, st>>>(h, current_time_step, nullptr, delay_step,
                                                  conn_word_idx, conn_bit_mask, post_ptr, n_post,
                                                  (const double*)weight, (double*)delivery_out,
                                                  max_delay_steps, n_words);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}

extern "C" int dgb_ring_enqueue(int dtype, void* ring, int64_t depth, int64_t width,
                                const int64_t* slot, const int64_t* post_ptr, int64_t n_post,
                                const int64_t* post_col, const int64_t* pre, const uint8_t* gate,
                                const int64_t* delay_steps, const void* weight, void* stream) {
  clear_error();
  DGB_REQUIRE(dtype == DGB_F32 || dtype == DGB_F64, "dtype must be DGB_F32 or DGB_F64");
  DGB_REQUIRE(depth >= 1 && width >= 0 && n_post >= 0, "bad ring sizes");
  if (n_post == 0) return DGB_OK;
  DGB_REQUIRE(ring && slot && post_ptr && pre && gate && delay_steps && weight,
              "pointers must be non-null");
  const int th = 256;
  const unsigned blocks = (unsigned)((n_post + th - 1) / th);
  cudaStream_t st = as_stream(stream);
  if (dtype == DGB_F32)
    enqueue_kernel<float><<<blocks, th, 0, st>>>((float*)ring, depth, width, slot, post_ptr, n_post,
                                                 post_col, pre, gate, delay_steps,
                                                 (const float*)weight);
  else
    enqueue_kernel<double><<<blocks, th, 0, st>>>((double*)ring, depth, width, slot, post_ptr,
                                                  n_post, post_col, pre, gate, delay_steps,
                                                  (const double*)weight);
  DGB_LAUNCH_CHECK();
  return DGB_OK;
}
