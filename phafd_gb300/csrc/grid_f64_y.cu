// Explicit instantiation of a subset of the grid operations (y passes and the plane-fused x/y passes) for FP64,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<double>::ypass(const Geom&, int, const cpx<double>*, cpx<double>*, cpx<double>*, const cpx<double>*,
                                 cudaStream_t);
template int GridOps<double>::yinv2(const Geom&, const cpx<double>*, cpx<double>*, cpx<double>*, const cpx<double>*, cpx<double>*,
                                 const cpx<double>*, cudaStream_t);
template int GridOps<double>::xy_fwd(const Geom&, const double*, const double*, cpx<double>*, const cpx<double>*, const cpx<double>*,
                                  const FHArgs&, cudaStream_t);
template int GridOps<double>::yx_inv(const Geom&, const cpx<double>*, double*, double, bool, double*, double, const cpx<double>*,
                                  const cpx<double>*, const NanArgs&, cudaStream_t);
}
