// Unbranched HH cable kernels: float64 plain per-step kernels (assembly, ragged solve + update).
#define DGB_CASE_F32(CHV)
#include "cable_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE_PLAIN(double)
}
