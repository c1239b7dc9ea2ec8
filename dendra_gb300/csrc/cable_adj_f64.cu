// float64 instantiation of the cable adjoint kernel.
#include "cable_adjoint_impl.cuh"
namespace dgb {
DGB_INSTANTIATE_CABLE_ADJOINT(double)
}
