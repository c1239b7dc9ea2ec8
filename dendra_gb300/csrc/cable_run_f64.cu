// Unbranched HH cable kernels: float64 persistent run.
#define DGB_CASE_F32(CHV)
#include "cable_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE_RUN(double, false, false)
}
