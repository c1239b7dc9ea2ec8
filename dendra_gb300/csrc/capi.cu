// Library-wide C-ABI helpers: version, last error, device properties.
#include <stdarg.h>

#include <atomic>

#include "common.cuh"

namespace dgb {

static thread_local char g_last_error[512] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

void clear_error() { g_last_error[0] = 0; }

// SM count of the current device, cached per device (launchers ask on every
// call; the attribute query costs host time on the launch path).
int device_sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev >= 0 && dev < 64 && (n = cached[dev].load(std::memory_order_relaxed)) > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  if (n < 1) n = 1;
  if (dev >= 0 && dev < 64) cached[dev].store(n, std::memory_order_relaxed);
  return n;
}

}  // namespace dgb

extern "C" const char* dgb_version(void) { return "dendra_gb300 0.1.0 (sm_103a)"; }

extern "C" const char* dgb_last_error(void) { return dgb::g_last_error; }

// Size of dgb_cable_args as compiled, so bindings can check their mirror.
extern "C" size_t dgb_cable_args_size(void) { return sizeof(dgb_cable_args); }

// Size of dgb_net_args as compiled, for foreign mirrors of the struct.
extern "C" size_t dgb_net_args_size(void) { return sizeof(dgb_net_args); }

// Size of dgb_cable_adjoint_args as compiled, for foreign mirrors of the struct.
extern "C" size_t dgb_cable_adjoint_args_size(void) { return sizeof(dgb_cable_adjoint_args); }
