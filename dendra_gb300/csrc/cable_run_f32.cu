// Unbranched HH cable kernels: float32 persistent run, exact arithmetic.
#define DGB_CASE_F32(CHV) DGB_CASE(CHV)
#include "cable_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE_RUN(float, false, false)
}
