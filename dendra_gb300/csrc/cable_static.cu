// Allocation-free variant of the unfused cable step (dgb_cable_step_static).
//
// Some callers cannot allocate device memory on their call path: a host that
// preallocates all GPU memory at start-up and forbids later allocations (a
// real-time or embedded controller), a plugin invoked while another runtime
// owns the CUDA allocator, or a foreign-language caller that is handed
// preallocated device buffers but has no CUDA allocation binding.  For them
// this entry point keeps the step's scratch (the four tridiagonal bands that
// pass between the assembly and the solve kernels) in a fixed array compiled
// into the library, so a call allocates nothing.  The caller still passes all
// inputs and outputs (state, workspace, comp_cable) through dgb_cable_args.
#include <mutex>

#include "cable_decl.cuh"

namespace dgb {

// Scratch bands lower/main/upper/rhs for up to kStaticBandBytes in total.
// Every GPU that loads the library holds this array until the process exits.
constexpr size_t kStaticBandBytes = size_t(4) << 20;  // 4 MiB
static __device__ __align__(256) unsigned char g_static_bands[kStaticBandBytes];

constexpr int kMaxDevices = 64;
struct BandAddr {
  void* ctx;  // context the address belongs to
  void* ptr;  // device address of g_static_bands in that context
};
static BandAddr g_band[kMaxDevices] = {};
static std::mutex g_band_mutex;

// The current context of the calling thread (the device's primary context
// for runtime-API callers; NULL before the runtime has bound one), through the
// driver entry point of cuCtxGetCurrent.
static int current_context(void** ctx) {
  using GetCurrent = int (*)(void**);
  static GetCurrent fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<GetCurrent>(p);
  });
  DGB_REQUIRE(fn != nullptr, "cuCtxGetCurrent is not available from the driver");
  *ctx = nullptr;
  DGB_REQUIRE(fn(ctx) == 0, "cuCtxGetCurrent failed");
  return DGB_OK;
}

// Device address of g_static_bands on the current device.  In host code the
// symbol is only a host stand-in; kernels must be given this address.  It is
// looked up with the device current on the first call and again whenever the
// device's context has changed since (cudaDeviceReset destroys the primary
// context and the library's module with it, so the old address is stale).
static int static_bands(void** out) {
  int dev = 0;
  DGB_CUDA_CHECK(cudaGetDevice(&dev));
  DGB_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d beyond %d", dev, kMaxDevices);
  void* ctx = nullptr;
  int rc = current_context(&ctx);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_band_mutex);
  if (g_band[dev].ptr == nullptr || ctx == nullptr || g_band[dev].ctx != ctx) {
    void* ptr = nullptr;
    // also binds the device's primary context if none is current yet
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_bands);
    if (e != cudaSuccess || ptr == nullptr) {
      set_error("cudaGetSymbolAddress(static cable bands) failed on device %d: %s", dev,
                cudaGetErrorString(e));
      return DGB_ECUDA;
    }
    rc = current_context(&ctx);
    if (rc) return rc;
    DGB_REQUIRE(ctx != nullptr, "no current CUDA context on device %d", dev);
    g_band[dev] = BandAddr{ctx, ptr};
  }
  *out = g_band[dev].ptr;
  return DGB_OK;
}

}  // namespace dgb

using namespace dgb;

extern "C" int dgb_cable_step_static(const dgb_cable_args* args, int32_t step, void* stream) {
  clear_error();
  int rc = validate_cable_args(args);
  if (rc) return rc;
  DGB_REQUIRE(args->comp_cable != nullptr,
              "comp_cable (cable index per compartment, int32[n_comp]) is required");
  if (args->n_comp == 0 || args->n_cables == 0) return DGB_OK;
  const int64_t kmax = args->max_k;
  DGB_REQUIRE(kmax >= 1 && kmax <= 32 * kSolveUpdateMaxCH,
              "max compartments per cable (max_k) must be in [1, %d], got %lld",
              32 * kSolveUpdateMaxCH, (long long)kmax);
  const size_t elem = args->dtype == DGB_F64 ? sizeof(double) : sizeof(float);
  const size_t need = (size_t)4 * (size_t)args->n_comp * elem;
  if (need > kStaticBandBytes) {
    set_error("dgb_cable_step_static: %lld compartments need %zu bytes of band scratch; the "
              "static scratch holds %zu bytes (at most %zu compartments in this dtype)",
              (long long)args->n_comp, need, kStaticBandBytes, kStaticBandBytes / (4 * elem));
    return DGB_ERANGE;
  }
  void* base = nullptr;
  rc = static_bands(&base);
  if (rc) return rc;
  // The assembly kernel writes every band entry of the n_comp compartments
  // before the solve reads it, so nothing has to be cleared between calls.
  unsigned char* b = static_cast<unsigned char*>(base);
  const size_t band = (size_t)args->n_comp * elem;
  void* lower = b;
  void* mainv = b + band;
  void* upper = b + 2 * band;
  void* rhs = b + 3 * band;
  cudaStream_t st = as_stream(stream);
  if (args->dtype == DGB_F32) {
    rc = cable_assemble_t<float>(args, step, lower, mainv, upper, rhs, st);
    if (rc) return rc;
    return cable_solve_update_t<float>(args, lower, mainv, upper, rhs, st);
  }
  rc = cable_assemble_t<double>(args, step, lower, mainv, upper, rhs, st);
  if (rc) return rc;
  return cable_solve_update_t<double>(args, lower, mainv, upper, rhs, st);
}
