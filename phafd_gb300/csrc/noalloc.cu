// Allocation-free spectral gradient.
//
// Some callers of this library cannot allocate device memory at the point
// where they need the gradient: a host code that hands the library a slice
// of its own memory pool and forbids cudaMalloc / cudaFree inside a time
// step (allocation there synchronises the device and fragments the pool),
// or an embedding framework that owns the device heap itself.  For them,
// phafd_gradphi_noalloc computes grad phi of a device-resident phi without
// allocating anything: the caller passes phi and the three outputs, and the
// three spectral scratch arrays the transform needs live in a file-scope
// device array of fixed size, compiled into the library.
//
// Limits and sharing rules
//   * every axis of the grid is 16, 32 or 64 points (at most 64^3 nodes);
//     larger or other sizes return PHAFD_ERR_UNSUPPORTED and do nothing;
//   * the scratch array (3 x 33 x 64 x 64 complex doubles, 6.5 MB) and the
//     twiddle tables of the three lengths exist on every GPU that loads the
//     library, until exit;
//   * every call shares that one scratch array: calls whose work overlaps on
//     the GPU (different streams, or different host threads on one device)
//     race and corrupt each other's results.  Calls ordered on one stream
//     need no synchronisation between them;
//   * the first call on a device resolves the device addresses of the arrays
//     (cudaGetSymbolAddress) with that device current and fills the twiddle
//     tables with a synchronous copy; later calls only enqueue kernels.  Make
//     that first call before any stream capture on the device.
#include <cmath>
#include <mutex>

#include "internal.h"

namespace {

constexpr int kNoAllocMaxN = 64;
constexpr size_t kNoAllocModes = (size_t)(kNoAllocMaxN / 2 + 1) * kNoAllocMaxN * kNoAllocMaxN;
constexpr int kMaxDevices = 64;

// three spectra: phi_hat, then the z / y inverse intermediates
static __device__ __align__(256) cpx<double> g_noalloc_scratch[3 * kNoAllocModes];
// W_N^m for N = 16, 32, 64, forward then inverse: written once per device
constexpr int kTwiddleEntries = 2 * (16 + 32 + 64);
static __device__ __align__(256) cpx<double> g_noalloc_twiddle[kTwiddleEntries];

// offset of the table of length n (16, 32 or 64) and direction dir (0 forward, 1 inverse)
int twiddle_offset(int n, int dir) {
  const int base = n == 16 ? 0 : (n == 32 ? 2 * 16 : 2 * (16 + 32));
  return base + dir * n;
}

struct DeviceSlot {
  bool ready = false;
  cpx<double>* scratch = nullptr;
  cpx<double>* twiddle = nullptr;
};
static DeviceSlot g_slots[kMaxDevices];
static std::mutex g_slots_mu;

bool size_ok(int n) { return n == 16 || n == 32 || n == 64; }

}  // namespace

extern "C" int phafd_gradphi_noalloc(const double* phi, double* gradx, double* grady, double* gradz, int nx, int ny,
                                     int nz, const double* period, void* stream) {
  using namespace phafd;
  if (!phi || !gradx || !grady || !gradz || !period) return PHAFD_ERR_INVALID;
  if (!size_ok(nx) || !size_ok(ny) || !size_ok(nz)) return PHAFD_ERR_UNSUPPORTED;
  for (int d = 0; d < 3; ++d)
    if (!(period[d] > 0)) return PHAFD_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PHAFD_ERR_CUDA;
  DeviceSlot slot;
  {
    std::lock_guard<std::mutex> lock(g_slots_mu);
    DeviceSlot& s = g_slots[dev];
    if (!s.ready) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return PHAFD_ERR_CUDA;
      s.scratch = reinterpret_cast<cpx<double>*>(p);
      if (cudaGetSymbolAddress(&p, g_noalloc_twiddle) != cudaSuccess) return PHAFD_ERR_CUDA;
      s.twiddle = reinterpret_cast<cpx<double>*>(p);
      // W_N^m = exp(-+ 2 pi i m / N) for every supported length, once
      double tw[2 * kTwiddleEntries];
      for (int n : {16, 32, 64})
        for (int dir = 0; dir < 2; ++dir)
          for (int m = 0; m < n; ++m) {
            const long double ang = 2.0L * 3.141592653589793238462643383279502884L * m / n;
            const int k = 2 * (twiddle_offset(n, dir) + m);
            tw[k] = (double)std::cos(ang);
            tw[k + 1] = (dir == 0 ? -1.0 : 1.0) * (double)std::sin(ang);
          }
      if (cudaMemcpy(s.twiddle, tw, sizeof(tw), cudaMemcpyHostToDevice) != cudaSuccess) return PHAFD_ERR_CUDA;
      s.ready = true;
    }
    slot = s;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  const int ns[3] = {nx, ny, nz};
  auto twp = [&](int axis, int dir) { return slot.twiddle + twiddle_offset(ns[axis], dir); };

  Geom g{};
  g.nx = nx; g.ny = ny; g.nz = nz; g.nxh = nx / 2 + 1;
  // dq per axis with the same truncated pi as the context's gradient
  for (int d = 0; d < 3; ++d) g.kq[d] = 2 * 3.141592 / period[d];
  cpx<double>* S0 = slot.scratch;
  cpx<double>* S1 = slot.scratch + kNoAllocModes;
  cpx<double>* S2 = slot.scratch + 2 * kNoAllocModes;
  const double inv_n = 1.0 / ((double)nx * ny * nz);
  FHArgs none{0.0, 0.0, nullptr, 0, nullptr};
  NanArgs nonan{0, nullptr, nullptr};
  // phi_hat = r2c(phi) into S0
  if (GridOps<double>::xr2c(g, phi, nullptr, S0, twp(0, 0), none, st)) return PHAFD_ERR_CUDA;
  if (GridOps<double>::ypass(g, -1, S0, S0, nullptr, twp(1, 0), st)) return PHAFD_ERR_CUDA;
  if (GridOps<double>::zpass(g, -1, S0, S0, nullptr, twp(2, 0), nullptr, st)) return PHAFD_ERR_CUDA;
  // z ifft of phi_hat (S1) and of i qz phi_hat (S2)
  if (GridOps<double>::zpass(g, +1, S0, S1, S2, twp(2, 1), nullptr, st)) return PHAFD_ERR_CUDA;
  // y ifft: S1 -> S1 (plain) and S0 (i qy); S2 -> S2
  if (GridOps<double>::ypass(g, +1, S1, S1, S0, twp(1, 1), st)) return PHAFD_ERR_CUDA;
  if (GridOps<double>::ypass(g, +1, S2, S2, nullptr, twp(1, 1), st)) return PHAFD_ERR_CUDA;
  // x c2r with the 1/N normalisation
  if (GridOps<double>::xc2r(g, S1, gradx, inv_n, true, nullptr, inv_n, twp(0, 1), nonan, st)) return PHAFD_ERR_CUDA;
  if (GridOps<double>::xc2r(g, S0, grady, inv_n, false, nullptr, inv_n, twp(0, 1), nonan, st)) return PHAFD_ERR_CUDA;
  if (GridOps<double>::xc2r(g, S2, gradz, inv_n, false, nullptr, inv_n, twp(0, 1), nonan, st)) return PHAFD_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? PHAFD_OK : PHAFD_ERR_CUDA;
}
