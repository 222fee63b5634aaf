// Explicit instantiation of a subset of the grid operations (x passes) for FP64,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<double>::xr2c(const Geom&, const double*, const double*, cpx<double>*, const cpx<double>*, const FHArgs&,
                                cudaStream_t);
template int GridOps<double>::xc2r(const Geom&, const cpx<double>*, double*, double, bool, double*, double, const cpx<double>*, const NanArgs&,
                                cudaStream_t);
template int GridOps<double>::xc2r3(const Geom&, const cpx<double>*, double*, double*, const cpx<double>*, double*, const cpx<double>*, double*,
                                 double, double, const cpx<double>*, const NanArgs&, const NanArgs&, const uint32_t*, const int*,
                                 int*, cudaStream_t);
}
