// Explicit instantiation of a subset of the grid operations (z passes of the set-up, gradient and Hermitian-plane paths) for FP64,
// one of the grid translation units that compile in parallel.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template int GridOps<double>::zpass(const Geom&, int, const cpx<double>*, cpx<double>*, cpx<double>*, const cpx<double>*,
                                 const UpdateArgs<double>*, cudaStream_t);
template int GridOps<double>::zfwd_planes(const Geom&, const cpx<double>*, cpx<double>*, const cpx<double>*, cudaStream_t);
template int GridOps<double>::zpass_planes(const Geom&, cpx<double>*, cpx<double>*, const cpx<double>*, const UpdateArgs<double>&,
                                        cudaStream_t);

bool fft_size_supported(int n) {
  switch (n) {
    case 16: case 32: case 64: case 96: case 128: case 160: case 256: case 512: return true;
  }
  return false;
}
}
