// Single-precision instantiation of the grid kernels.
#include "grid_impl.cuh"
namespace phafd {
template struct GridOps<float>;
}
