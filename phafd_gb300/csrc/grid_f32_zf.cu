// Explicit instantiation of a subset of the grid operations (the fused z pass of the step) for FP32,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<float>::zfused(const Geom&, const cpx<float>*, cpx<float>*, cpx<float>*, cpx<float>*, const cpx<float>*,
                                  const cpx<float>*, const UpdateArgs<float>&, int, int, cudaStream_t);
}
