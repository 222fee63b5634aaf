// Internal declarations shared by the translation units of libphafd_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "common.cuh"
#include "../../include/phafd_gpu.h"

namespace phafd {

struct Geom {
  int nx, ny, nz, nxh;
  double kq[3];  // 2*3.141592/L per physical axis (domain.cpp:206-208)
  int generic256;  // 256-point axes take the shared-memory tile transforms, not the register-resident ones
  int xc2r_tma = 1;  // FP32 merged x c2r on 256-point rows fed by tensor-map loads (persistent grid)
  int xr2c_tma = 1;  // FP32 x r2c on 256-point rows fed by tensor-map loads (persistent grid)
};

struct FHArgs {
  double tv;   // temp / volFH
  double chi;
  unsigned long long* counters;  // [0] phi <= 0 reflections, [1] phi >= 1 reflections
  int enabled;                   // 0: mu = deposit only (no fix grid/floryhuggins)
  void* mu_out;                  // optional: materialised chempot (T*)
  // FP32 contexts with a reference concentration c (centered != 0): the r2c
  // of phi transforms phi - c; the Flory-Huggins part of mu is evaluated as
  // f(p) - f(c) (its rounding then scales with p - c, not with f(p)), and
  // fconst = tv f(c) is added back only where mu is materialised.
  double c, inv_c, fconst;
  int centered;
  int* status = nullptr;  // device status word a pass with bounded waits flags with ST_TIMEOUT (null: no such pass)
  // bit per 32-byte sector of the deposit holding a node of the current grid
  // lists (the only nodes the pair stage deposits on); a pass may read the
  // deposit only where the bit is set (null: everywhere)
  const uint32_t* dep_mask = nullptr;
};

struct NanArgs {
  int check;
  long long* nan_step;
  const long long* d_step;
  double offset;  // added to the phi output of a c2r (the reference concentration taken out of its k = 0 mode)
};

template <typename T>
struct UpdateArgs {
  const cpx<T>* phi_old;
  const cpx<T>* mu_hat;
  cpx<T>* phi_new;
  const double2* uref;
  T mobility, tvg, dt, norm, cpref, rpref, sqrtdt, phi_scale, store_scale;
  T qx, qy, qz;
  int noise;
  uint32_t seed;
  const long long* d_step;
  int Ny, Nz, Nxh;
  // nsub > 1: nsub linearised substeps with the nonlinear part of mu frozen
  // (the base propagator of the learned macro step); f2 = dmu/dphi at the mean
  int nsub;
  T f2;
  // subtracted from the k = 0 mode in the transform that follows the update
  // (not in the stored spectrum); the c2r adds it back to phi
  T phi_off;
};

// compute grid/cluster: labels (device, nx*ny*nz) of the periodic
// 6-connected components of phi > threshold (greater) or < threshold, each
// the smallest z + (y Nx + x) Ny of its component, -1 elsewhere (clusters.cu)
template <typename F>
int grid_clusters(const F* phi, int nx, int ny, int nz, double threshold, int greater, int* labels, int* nclusters,
                  cudaStream_t st);

template <typename T>
struct GridOps {
  static int xr2c(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* tw, const FHArgs& fh,
                  cudaStream_t st);
  static int xc2r(const Geom& g, const cpx<T>* in, T* out0, T s0, bool mul0, T* out1, T s1, const cpx<T>* tw,
                  const NanArgs& nan, cudaStream_t st);
  static int ypass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
                   cudaStream_t st);
  // the inverse chain's three x c2r (phi + dphi/dx from C, dphi/dy from D,
  // dphi/dz from E) and two inverse y passes (A -> C, D; B -> E) as one
  // launch each (-3: not available for this length)
  // (gmask: node bitset; unless gmask is null or *gmask_off is set, the three
  // gradients are stored at set bits only; status: device status word that a
  // pass with bounded waits flags with ST_TIMEOUT)
  static int xc2r3(const Geom& g, const cpx<T>* C, T* phi, T* gx, const cpx<T>* D, T* gy, const cpx<T>* E, T* gz,
                   T sp, T sg, const cpx<T>* tw, const NanArgs& nan, const NanArgs& nonan, const uint32_t* gmask,
                   const int* gmask_off, int* status, cudaStream_t st);
  static int yinv2(const Geom& g, const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E,
                   const cpx<T>* tw, cudaStream_t st);
  static int zpass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
                   const UpdateArgs<T>* u, cudaStream_t st);
  // forward z FFT of mu + update + z inverse FFT (bulk kx); plane tiles store mu_hat only
  // (bulk_only: kx in [1, Nx/2) only; the planes then take zfwd_planes + zpass_planes)
  static int zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1,
                    const cpx<T>* twf, const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only,
                    cudaStream_t st);
  // forward z FFT of the kx = 0 and kx = Nx/2 planes of mu into mu_hat
  static int zfwd_planes(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, const cpx<T>* tw, cudaStream_t st);
  // plane-fused x r2c + y fft (returns -3 when the plane path does not apply)
  static int xy_fwd(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* twx, const cpx<T>* twy,
                    const FHArgs& fh, cudaStream_t st);
  // plane-fused y ifft (optionally times i qy) + x c2r to out0 (plain) and out1 (i qx)
  static int yx_inv(const Geom& g, const cpx<T>* in, T* out0, T s0, bool ymul, T* out1, T s1, const cpx<T>* twy,
                    const cpx<T>* twx, const NanArgs& nan, cudaStream_t st);
  // update + z inverse FFT of the kx = 0 and kx = Nx/2 planes (reads mu_hat)
  static int zpass_planes(const Geom& g, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw, const UpdateArgs<T>& u,
                          cudaStream_t st);
};

bool fft_size_supported(int n);

}  // namespace phafd
