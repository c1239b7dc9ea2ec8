// float64 instantiation of the unbranched HH cable kernels (chunk sizes
// 1, 2, 4, 8, 16 only).
#define DGB_CASE_F32(CHV)
#include "cable_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE(double)
}
