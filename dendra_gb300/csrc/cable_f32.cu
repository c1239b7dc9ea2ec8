// float32 instantiation of the unbranched HH cable kernels.
#define DGB_CASE_F32(CHV) DGB_CASE(CHV)
#include "cable_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE(float)
}
