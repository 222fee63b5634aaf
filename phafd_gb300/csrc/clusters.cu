// compute grid/cluster on the device (compute_grid_clusters.cpp:66-229).
//
// The reference labels every node past the threshold with
// id = z + (y Nx + x) Ny (compute_grid_clusters.cpp:72-94) and sweeps until
// each labelled node carries the smallest id of its 6-connected, periodic
// component (:103-196).  Here the components come from a lock-free
// union-find over node indices (hooks always attach the larger root to the
// smaller, so parents never exceed their children; finds halve paths), then
// each component's smallest id is gathered at its root with atomicMin and
// broadcast back: the same labels, in a fixed number of passes instead of a
// diameter-long sweep.  Every loop carries an iteration cap that sets the
// error flag instead of spinning on.
#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>

#include "internal.h"

namespace phafd {
namespace {

constexpr int T = 256;

// root of v (parents are never larger than their children); path halving
// (benign races: any ancestor is a valid parent)
__device__ int cl_find(int* p, int v, long long cap, int* err) {
  int x = v;
  for (long long it = 0;; ++it) {
    const int px = p[x];
    if (px == x) return x;
    const int ppx = p[px];
    if (ppx != px) p[x] = ppx;
    x = ppx;
    if (it > cap) {
      atomicExch(err, 1);
      return x;
    }
  }
}

// root of v without writing: in the flatten pass each thread stores only its
// own node's root, and a halving write from another thread could otherwise
// put an older ancestor back over it
__device__ int cl_root(const int* p, int v, long long cap, int* err) {
  for (long long it = 0;; ++it) {
    const int pv = p[v];
    if (pv == v) return v;
    v = pv;
    if (it > cap) {
      atomicExch(err, 1);
      return v;
    }
  }
}

__device__ void cl_hook(int* p, int a, int b, long long cap, int* err) {
  int ra = cl_find(p, a, cap, err), rb = cl_find(p, b, cap, err);
  for (long long it = 0; ra != rb; ++it) {
    if (it > cap) {
      atomicExch(err, 1);
      return;
    }
    if (ra < rb) {
      const int old = atomicCAS(&p[rb], rb, ra);
      if (old == rb) return;
      rb = cl_find(p, old, cap, err);  // rb was linked meanwhile: continue from its new root
    } else {
      const int old = atomicCAS(&p[ra], ra, rb);
      if (old == ra) return;
      ra = cl_find(p, old, cap, err);
    }
  }
}

template <typename F>
__global__ void k_cl_init(const F* __restrict__ phi, double thr, int greater, int* __restrict__ p, long long n) {
  for (long long i = blockIdx.x * (long long)T + threadIdx.x; i < n; i += (long long)gridDim.x * T) {
    const double v = (double)phi[i];
    p[i] = (greater ? v > thr : v < thr) ? (int)i : -1;
  }
}

__global__ void k_cl_hook(int* p, int nx, int ny, int nz, long long cap, int* err) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)T + threadIdx.x; i < n; i += (long long)gridDim.x * T) {
    if (p[i] < 0) continue;
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long long)nx * ny));
    const long long nb[3] = {i - x + (x + 1) % nx, ((long long)z * ny + (y + 1) % ny) * nx + x,
                             ((long long)((z + 1) % nz) * ny + y) * nx + x};
    for (int d = 0; d < 3; ++d)
      if (nb[d] != i && p[nb[d]] >= 0) cl_hook(p, (int)i, (int)nb[d], cap, err);
  }
}

// flatten to roots; each root collects the smallest reference id of its component
__global__ void k_cl_roots(int* p, int* minid, int nx, int ny, long long n, long long cap, int* err,
                           int* count) {
  for (long long i = blockIdx.x * (long long)T + threadIdx.x; i < n; i += (long long)gridDim.x * T) {
    if (p[i] < 0) continue;
    const int r = cl_root(p, (int)i, cap, err);
    p[i] = r;
    if (r == (int)i) atomicAdd(count, 1);
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long long)nx * ny));
    atomicMin(&minid[r], z + (y * nx + x) * ny);  // compute_grid_clusters.cpp:76
  }
}

__global__ void k_cl_label(const int* __restrict__ p, const int* __restrict__ minid, int* __restrict__ labels,
                           long long n) {
  for (long long i = blockIdx.x * (long long)T + threadIdx.x; i < n; i += (long long)gridDim.x * T)
    labels[i] = p[i] < 0 ? -1 : minid[p[i]];
}

}  // namespace

template <typename F>
int grid_clusters(const F* phi, int nx, int ny, int nz, double threshold, int greater, int* labels, int* nclusters,
                  cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  if (n <= 0 || n > INT_MAX) return -1;
  int *p = nullptr, *minid = nullptr, *flags = nullptr;
  if (cudaMalloc(&p, n * sizeof(int)) != cudaSuccess) return -7;
  if (cudaMalloc(&minid, n * sizeof(int)) != cudaSuccess) {
    cudaFree(p);
    return -7;
  }
  if (cudaMalloc(&flags, 2 * sizeof(int)) != cudaSuccess) {
    cudaFree(p);
    cudaFree(minid);
    return -7;
  }
  const unsigned grid = (unsigned)((n + T - 1) / T < 65535 * 16 ? (n + T - 1) / T : 65535 * 16);
  int rc = 0;
  cudaMemsetAsync(flags, 0, 2 * sizeof(int), st);
  cudaMemsetAsync(minid, 0x7f, n * sizeof(int), st);
  k_cl_init<F><<<grid, T, 0, st>>>(phi, threshold, greater, p, n);
  k_cl_hook<<<grid, T, 0, st>>>(p, nx, ny, nz, n, flags);
  k_cl_roots<<<grid, T, 0, st>>>(p, minid, nx, ny, n, n, flags, flags + 1);
  k_cl_label<<<grid, T, 0, st>>>(p, minid, labels, n);
  int h[2] = {0, 0};
  if (cudaMemcpyAsync(h, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    rc = -2;
  else if (h[0])
    rc = -8;  // an iteration cap was reached
  if (nclusters) *nclusters = h[1];
  cudaFree(p);
  cudaFree(minid);
  cudaFree(flags);
  return rc;
}

template int grid_clusters<float>(const float*, int, int, int, double, int, int*, int*, cudaStream_t);
template int grid_clusters<double>(const double*, int, int, int, double, int, int*, int*, cudaStream_t);

}  // namespace phafd
