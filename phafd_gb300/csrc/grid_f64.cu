// Double-precision instantiation of the grid kernels.
#include "plane_impl.cuh"
#include "reg256.cuh"
namespace phafd {
template struct GridOps<double>;
bool fft_size_supported(int n) {
  switch (n) {
    case 16: case 32: case 64: case 96: case 128: case 160: case 256: case 512: return true;
  }
  return false;
}
}
