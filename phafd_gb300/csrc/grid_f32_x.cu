// Explicit instantiation of a subset of the grid operations (x passes) for FP32,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<float>::xr2c(const Geom&, const float*, const float*, cpx<float>*, const cpx<float>*, const FHArgs&,
                                cudaStream_t);
template int GridOps<float>::xc2r(const Geom&, const cpx<float>*, float*, float, bool, float*, float, const cpx<float>*, const NanArgs&,
                                cudaStream_t);
template int GridOps<float>::xc2r3(const Geom&, const cpx<float>*, float*, float*, const cpx<float>*, float*, const cpx<float>*, float*,
                                 float, float, const cpx<float>*, const NanArgs&, const NanArgs&, const uint32_t*, const int*,
                                 int*, cudaStream_t);
}
