// Explicit instantiation of a subset of the grid operations (z passes of the set-up, gradient and Hermitian-plane paths) for FP32,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<float>::zpass(const Geom&, int, const cpx<float>*, cpx<float>*, cpx<float>*, const cpx<float>*,
                                 const UpdateArgs<float>*, cudaStream_t);
template int GridOps<float>::zfwd_planes(const Geom&, const cpx<float>*, cpx<float>*, const cpx<float>*, cudaStream_t);
template int GridOps<float>::zpass_planes(const Geom&, cpx<float>*, cpx<float>*, const cpx<float>*, const UpdateArgs<float>&,
                                        cudaStream_t);
}
