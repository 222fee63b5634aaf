// Register-resident transforms of length 256 = 16 x 16.
//
// A length-256 Stockham FFT is two radix-16 stages.  Butterfly j (0..15) of
// stage 1 reads elements j + 16 r and writes 16 j + r; butterfly j of stage 2
// reads j + 16 r, multiplies by W_256^(j r) and writes j + 16 r.  So a thread
// that owns butterfly j of one line loads its 16 inputs straight from HBM,
// does the first DFT-16 in registers, exchanges once through shared memory,
// does the twiddles and the second DFT-16, and stores its 16 outputs straight
// to HBM: one shared-memory round trip per element instead of three in the
// generic tile kernels (fft.cuh).
//
// Column passes (z): 16 columns x 16 butterflies = 256 threads per CTA, a
// warp = 16 consecutive columns x 2 butterflies, so every load and store of
// a warp touches two 128-byte row segments.  The exchange buffer is
// element-major [e][column], conflict-free for both stage directions.
#pragma once
#include "grid_impl.cuh"

namespace phafd {
namespace r256 {

constexpr int N = 256, W = 16;  // columns per CTA

template <typename T, int S>
PHAFD_D void twiddle16(cpx<T>* v, int j, const cpx<T>* __restrict__ tw) {
#pragma unroll
  for (int r = 1; r < 16; ++r) v[r] = v[r] * tw[j * r];
}

// exchange buffer: element e of column c at buf[e * W + c]
template <typename T>
PHAFD_D void put16(cpx<T>* buf, const cpx<T>* v, int j, int c) {
#pragma unroll
  for (int r = 0; r < 16; ++r) buf[(16 * j + r) * W + c] = v[r];
}
template <typename T>
PHAFD_D void get16(const cpx<T>* buf, cpx<T>* v, int j, int c) {
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = buf[(j + 16 * r) * W + c];
}

// z fft of mu + Model-B update + z ifft of phi_hat' and i qz phi_hat', for
// Nz = 256.  Same contract as k_zfused (grid_impl.cuh).
template <typename T>
__global__ void __launch_bounds__(256)
k_zfused256(const cpx<T>* __restrict__ muin, cpx<T>* __restrict__ muhat, cpx<T>* __restrict__ out0,
            cpx<T>* __restrict__ out1, T dq, const cpx<T>* __restrict__ twf, const cpx<T>* __restrict__ twi, int Ny,
            UpdateArgs<T> u, int store_mu, int kx0) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* bufA = reinterpret_cast<cpx<T>*>(smraw);  // N x W
  cpx<T>* bufB = bufA + N * W;                        // N x W (phi_hat staging, then second ifft)
  const int c = threadIdx.x & 15;
  const int j = threadIdx.x >> 4;
  const int kx = (int)blockIdx.y + kx0;
  const int ky = blockIdx.x * W + c;
  const bool plane = (kx == 0 || kx == u.Nxh - 1);
  const bool live = ky < Ny;
  const size_t col = (size_t)kx * N * Ny + (live ? ky : 0);
  // phi_hat tile -> bufB asynchronously (needed after the forward FFT)
  if (!plane && live) {
#pragma unroll
    for (int r = 0; r < 16; ++r) cp_async_elem(&bufB[(j + 16 * r) * W + c], &u.phi_old[col + (size_t)(j + 16 * r) * Ny]);
  }
  cp_async_commit();
  cpx<T> v[16];
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = live ? muin[col + (size_t)(j + 16 * r) * Ny] : mk<T>(0, 0);
  // forward z FFT
  fft::dft16<-1>(v);
  put16(bufA, v, j, c);
  __syncthreads();
  get16(bufA, v, j, c);
  twiddle16<T, -1>(v, j, twf);
  fft::dft16<-1>(v);  // v[r] = mu_hat at kz = j + 16 r
  if (plane || store_mu) {
    if (live) {
#pragma unroll
      for (int r = 0; r < 16; ++r) muhat[col + (size_t)(j + 16 * r) * Ny] = v[r];
    }
  }
  if (plane) return;  // uniform per CTA; k_zpass<planes_only> finishes these modes
  cp_async_wait<0>();
  __syncthreads();  // phi_hat landed; everyone done reading bufA
  cpx<T> d[16];
  uint32_t words[4] = {0, 0, 0, 0};
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const int kz = j + 16 * r;  // bit 4 of kz is r & 1: modes r and r+1 share one Philox call
    if (u.noise == PHAFD_NOISE_PHILOX && (r & 1) == 0)
      field_noise_words(kx, ky, kz, Ny, N, (uint32_t)(*u.d_step), u.seed, words);
    cpx<T> nv = mk<T>(0, 0);
    if (live) {
      const cpx<T> ph = scale(bufB[kz * W + c], u.phi_scale);
      nv = update_value(u, kx, ky, kz, ph, v[r], false, words);
      u.phi_new[col + (size_t)kz * Ny] = scale(nv, u.store_scale);
    }
    v[r] = nv;
    d[r] = deriv(nv, dq, wrap_index(kz, N));
  }
  __syncthreads();  // every thread has read its phi_hat from bufB
  // inverse z FFT of both
  fft::dft16<+1>(v);
  fft::dft16<+1>(d);
  put16(bufA, v, j, c);
  put16(bufB, d, j, c);
  __syncthreads();
  get16(bufA, v, j, c);
  get16(bufB, d, j, c);
  twiddle16<T, +1>(v, j, twi);
  twiddle16<T, +1>(d, j, twi);
  fft::dft16<+1>(v);
  fft::dft16<+1>(d);
  if (live) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      out0[col + (size_t)(j + 16 * r) * Ny] = v[r];
      out1[col + (size_t)(j + 16 * r) * Ny] = d[r];
    }
  }
}

template <typename T>
int zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1, const cpx<T>* twf,
           const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only, cudaStream_t st) {
  const size_t sm = (size_t)2 * N * W * sizeof(cpx<T>);
  auto k = k_zfused256<T>;
  if (set_smem(k, sm)) return -1;
  const int kx0 = bulk_only ? 1 : 0;
  if (g.nxh - 2 * kx0 <= 0) return 0;
  dim3 grid((g.ny + W - 1) / W, g.nxh - 2 * kx0);
  launch_grid(k, grid, dim3(256), sm, st, muin, muhat, out0, out1, (T)g.kq[2], twf, twi, g.ny, u, store_mu, kx0);
  return 0;
}

}  // namespace r256
}  // namespace phafd
