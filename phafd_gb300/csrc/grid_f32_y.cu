// Explicit instantiation of a subset of the grid operations (y passes and the plane-fused x/y passes) for FP32,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<float>::ypass(const Geom&, int, const cpx<float>*, cpx<float>*, cpx<float>*, const cpx<float>*,
                                 cudaStream_t);
template int GridOps<float>::yinv2(const Geom&, const cpx<float>*, cpx<float>*, cpx<float>*, const cpx<float>*, cpx<float>*,
                                 const cpx<float>*, cudaStream_t);
template int GridOps<float>::xy_fwd(const Geom&, const float*, const float*, cpx<float>*, const cpx<float>*, const cpx<float>*,
                                  const FHArgs&, cudaStream_t);
template int GridOps<float>::yx_inv(const Geom&, const cpx<float>*, float*, float, bool, float*, float, const cpx<float>*,
                                  const cpx<float>*, const NanArgs&, cudaStream_t);
}
