// Explicit instantiation of a subset of the grid operations (the fused z pass of the step) for FP64,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<double>::zfused(const Geom&, const cpx<double>*, cpx<double>*, cpx<double>*, cpx<double>*, const cpx<double>*,
                                  const cpx<double>*, const UpdateArgs<double>&, int, int, cudaStream_t);
}
