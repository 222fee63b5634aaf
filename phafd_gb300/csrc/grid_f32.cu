// Single-precision instantiation of the grid kernels.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template struct GridOps<float>;
}
