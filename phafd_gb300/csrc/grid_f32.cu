// Single-precision instantiation of the grid kernels.
#include "plane_impl.cuh"
namespace phafd {
template struct GridOps<float>;
}
