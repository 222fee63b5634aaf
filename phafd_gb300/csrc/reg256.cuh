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
// FP32: at most 80 registers so three CTAs (24 warps) share an SM
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1)
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

// Row passes (y): lines contiguous, in[line * 256 + e].  The 16 butterflies
// of a line are 16 consecutive lanes (a warp = two lines), so every load and
// store of a warp touches two contiguous 16-element segments, and the
// exchange between the two radix-16 stages stays inside the warp
// (__syncwarp, no CTA barrier).  Exchange buffer of a line: element e at
// e + e / 16 (stride 17 between the butterflies' writes: conflict-free).
constexpr int RS = N + N / 16;

template <typename T>
PHAFD_D void rput16(cpx<T>* rb, const cpx<T>* v, int j) {
#pragma unroll
  for (int r = 0; r < 16; ++r) rb[17 * j + r] = v[r];  // element 16 j + r
}
template <typename T>
PHAFD_D void rget16(const cpx<T>* rb, cpx<T>* v, int j) {
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = rb[j + 17 * r];  // element j + 16 r
}

// v[r] = element j + 16 r of the line in, of its transform (sign S) out
template <typename T, int S>
PHAFD_D void row256(cpx<T>* v, cpx<T>* rb, int j, const cpx<T>* __restrict__ tw) {
  fft::dft16<S>(v);
  rput16(rb, v, j);
  __syncwarp();
  rget16(rb, v, j);
  twiddle16<T, S>(v, j, tw);
  fft::dft16<S>(v);
}

// 16 lines from line 16 bx: out0 = FFT_S(in), out1 = FFT_S(i dq m(e) in)
// (NOUT == 2, which reads `in` again after storing out0: not in place)
template <typename T, int S, int NOUT>
PHAFD_D void yrow_tile(long long bx, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, T dq,
                       const cpx<T>* __restrict__ tw, long long nlines, unsigned char* smraw) {
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4;
  cpx<T>* rb = reinterpret_cast<cpx<T>*>(smraw) + c * RS;
  const long long line = bx * W + c;
  const bool live = line < nlines;
  const cpx<T>* src = in + (live ? line : 0) * N;
  cpx<T> v[16];
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = live ? src[j + 16 * r] : mk<T>(0, 0);
  row256<T, S>(v, rb, j, tw);
  if (live) {
#pragma unroll
    for (int r = 0; r < 16; ++r) out0[line * N + j + 16 * r] = v[r];
  }
  if constexpr (NOUT == 2) {
    __syncwarp();  // the exchange buffer is read before it is rewritten
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int e = j + 16 * r;
      v[r] = live ? deriv(src[e], dq, wrap_index(e, N)) : mk<T>(0, 0);
    }
    row256<T, S>(v, rb, j, tw);
    if (live) {
#pragma unroll
      for (int r = 0; r < 16; ++r) out1[line * N + j + 16 * r] = v[r];
    }
  }
}

template <typename T, int S, int NOUT>
__global__ void __launch_bounds__(256)
k_yrow256(const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, T dq, const cpx<T>* __restrict__ tw, long long nlines) {
  extern __shared__ __align__(16) unsigned char smraw[];
  yrow_tile<T, S, NOUT>(blockIdx.x, in, out0, out1, dq, tw, nlines, smraw);
}

// the two inverse y passes of the inverse chain: A -> (C, D = i qy) in CTAs
// [0, nb), B -> E in [nb, 2 nb)
template <typename T>
__global__ void __launch_bounds__(256)
k_yinv2row256(const cpx<T>* __restrict__ A, cpx<T>* __restrict__ C, cpx<T>* __restrict__ D,
              const cpx<T>* __restrict__ B, cpx<T>* __restrict__ E, T dq, const cpx<T>* __restrict__ tw,
              long long nlines, long long nb) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const long long bx = blockIdx.x;
  if (bx < nb) yrow_tile<T, +1, 2>(bx, A, C, D, dq, tw, nlines, smraw);
  else yrow_tile<T, +1, 1>(bx - nb, B, E, nullptr, dq, tw, nlines, smraw);
}

template <typename T>
int ypass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
          cudaStream_t st) {
  const long long nlines = (long long)g.nxh * g.nz;
  const size_t sm = (size_t)W * RS * sizeof(cpx<T>);
  const unsigned nb = (unsigned)((nlines + W - 1) / W);
  const T dq = (T)g.kq[1];
  if (out1 && (in == out0 || in == out1)) return -1;
#define YROW(S, NO)                                                                                  \
  {                                                                                                  \
    auto k = k_yrow256<T, S, NO>;                                                                    \
    if (set_smem(k, sm)) return -1;                                                                  \
    launch_grid(k, dim3(nb), dim3(256), sm, st, in, out0, out1, dq, tw, nlines);                     \
    return 0;                                                                                        \
  }
  if (sign < 0) {
    if (out1) YROW(-1, 2) else YROW(-1, 1)
  } else {
    if (out1) YROW(+1, 2) else YROW(+1, 1)
  }
#undef YROW
}

template <typename T>
int yinv2(const Geom& g, const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E, const cpx<T>* tw,
          cudaStream_t st) {
  const long long nlines = (long long)g.nxh * g.nz;
  const size_t sm = (size_t)W * RS * sizeof(cpx<T>);
  const long long nb = (nlines + W - 1) / W;
  auto k = k_yinv2row256<T>;
  if (set_smem(k, sm)) return -1;
  launch_grid(k, dim3((unsigned)(2 * nb)), dim3(256), sm, st, A, C, D, B, E, (T)g.kq[1], tw, nlines, nb);
  return 0;
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
