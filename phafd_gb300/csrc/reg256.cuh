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
#include "tma.cuh"

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
// FP32: at most 80 registers so three CTAs (24 warps) share an SM.
// NOISE and MACRO fix the noise mode and whether the update is a macro step
// (nsub > 1) at compile time, so the update inlined for the 16 modes of a
// thread carries no branches or code for the other cases.
// NYC: Ny known at compile time (256: every strided address is a constant
// offset from the column's base), 0: run time.
template <typename T, int NOISE, bool MACRO, int NYC>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1)
k_zfused256(const cpx<T>* __restrict__ muin, cpx<T>* __restrict__ muhat, cpx<T>* __restrict__ out0,
            cpx<T>* __restrict__ out1, T dq, const cpx<T>* __restrict__ twf, const cpx<T>* __restrict__ twi, int Ny_rt,
            UpdateArgs<T> u, int store_mu, int kx0) {
  u.noise = NOISE;
  if (!MACRO) u.nsub = 1;
  const int Ny = NYC > 0 ? NYC : Ny_rt;
  if (NYC > 0) u.Ny = NYC;
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
      nv = update_value<T, true>(u, kx, ky, kz, ph, v[r], false, words);  // bulk kx >= 1: q^2 > 0
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

// x c2r of 256-point rows.  A CTA takes 16 complex lines: LP = 16 / NOUT row
// pairs (rows y0 .. y0 + 2 LP of plane z) times NOUT outputs (output 1 of
// the spectrum times i dq kx).  Line c = q LP + l packs rows 2l (real part)
// and 2l + 1 (imaginary part) of output q.  The half spectrum is read with
// the lanes over y (two rows' values, 16 contiguous bytes per lane) and
// written Hermitian-completed into the line buffers (element e at
// e + e / 16, lines RX apart, RX odd: conflict-free in both directions);
// each line's 16 lanes then run the 256-point inverse in registers and store
// their rows directly, 16 consecutive nodes per lane group.  Stores of an
// output with a mask go only to the 32-byte sectors whose bit is set.
constexpr int RX = N + N / 16 + 1;

// x c2r of one line, second part: element j + 16 r of the line's transform
// v holds nodes x = j + 16 r of rows y0 (real part) and y0 + 1 (imaginary
// part) of plane z; they are stored scaled by sc.  PHI: the phi output,
// which also gets nan.offset, runs the step's NaN check and is stored
// everywhere; otherwise a gradient, stored only to the 32-byte sectors set in
// msk unless msk is null.
template <typename T, bool PHI>
PHAFD_D void xc2r_store256(const cpx<T>* v, int j, int y0, int z, T* __restrict__ out, T sc, int Ny,
                           const NanArgs& nan, const uint32_t* msk) {
  constexpr int G = 32 / (int)sizeof(T);  // nodes per 32-byte sector
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int y = y0 + h;
    if (y >= Ny) continue;
    const size_t row = ((size_t)z * Ny + y) * N;
    if (PHI || !msk) {
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const T val = (h == 0 ? v[r].x : v[r].y) * sc;
        out[row + j + 16 * r] = PHI ? val + (T)nan.offset : val;
      }
    } else {
      // the row's sectors are N / G consecutive bits starting at a word boundary
      const uint32_t m0 = msk[(row / G) >> 5];
      const uint32_t m1 = N / G > 32 ? msk[((row / G) >> 5) + 1] : 0u;
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int x = j + 16 * r;
        const int sec = x / G;
        const uint32_t bit = sec < 32 ? (m0 >> sec) & 1u : (m1 >> (sec & 31)) & 1u;
        if (bit) out[row + x] = (h == 0 ? v[r].x : v[r].y) * sc;
      }
    }
    // integrate.cpp:190: the step's NaN check reads phi at node (0, 0, 0)
    if (PHI && nan.check && z == 0 && y == 0 && j == 0 && isnan(v[0].x * sc))
      atomicCAS(reinterpret_cast<unsigned long long*>(nan.nan_step), (unsigned long long)-1LL,
                (unsigned long long)(*nan.d_step));
  }
}

template <typename T, int NOUT>
PHAFD_D void xc2r_tile256(int bx, int z, const cpx<T>* __restrict__ in, T* __restrict__ out0,
                          T* __restrict__ out1, T s0, T s1, T dq, const cpx<T>* __restrict__ tw, int Ny, int Nz,
                          const NanArgs& nan, const uint32_t* mask0, const uint32_t* mask1, unsigned char* smraw) {
  constexpr int LP = W / NOUT;
  cpx<T>* zs = reinterpret_cast<cpx<T>*>(smraw);
  const int y0 = bx * 2 * LP;
  TILE_LOOP(idx, (N / 2 + 1) * LP, 256) {  // unrolled: every load of a thread in flight at once
    const int l = idx % LP, k = idx / LP;
    const int y = y0 + 2 * l;
    const size_t o = ((size_t)k * Nz + z) * Ny + y;
    cpx<T> A = mk<T>(0, 0), B = mk<T>(0, 0);
    if constexpr (sizeof(T) == 4) {
      if (y + 1 < Ny && (Ny & 1) == 0) {  // o even: one 16-byte load of the pair
        const float4 ab = *reinterpret_cast<const float4*>(&in[o]);
        A = mk<T>(ab.x, ab.y);
        B = mk<T>(ab.z, ab.w);
      } else {
        if (y < Ny) A = in[o];
        if (y + 1 < Ny) B = in[o + 1];
      }
    } else {
      if (y < Ny) A = in[o];
      if (y + 1 < Ny) B = in[o + 1];
    }
#pragma unroll
    for (int q = 0; q < NOUT; ++q) {
      cpx<T> a = A, b = B;
      if (q == 1) { a = deriv(a, dq, k); b = deriv(b, dq, k); }
      if (k == 0 || k == N / 2) { a.y = (T)0; b.y = (T)0; }
      cpx<T>* line = zs + (q * LP + l) * RX;
      line[k + (k >> 4)] = mk<T>(a.x - b.y, a.y + b.x);
      if (k > 0 && k < N / 2) line[(N - k) + ((N - k) >> 4)] = mk<T>(a.x + b.y, b.x - a.y);
    }
  }
  __syncthreads();
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4;
  const int q = c / LP, l = c % LP;
  cpx<T>* rb = zs + c * RX;
  cpx<T> v[16];
#pragma unroll
  for (int r = 0; r < 16; ++r) v[r] = rb[j + 17 * r];  // element j + 16 r
  __syncwarp();
  row256<T, +1>(v, rb, j, tw);
  if (NOUT == 2 && q == 0) xc2r_store256<T, true>(v, j, y0 + 2 * l, z, out0, s0, Ny, nan, nullptr);
  else xc2r_store256<T, false>(v, j, y0 + 2 * l, z, q == 0 ? out0 : out1, q == 0 ? s0 : s1, Ny, nan,
                               q == 0 ? mask0 : mask1);
}

// x r2c of 256-point rows, optionally fused with mu = deposit + FH(phi)
// (PRO == 1; PRO == 2 with the Flory-Huggins part taken relative to f(c),
// FP32).  A CTA takes rows y0 .. y0 + 32 of plane z: 16-byte
// asynchronous copies of the rows (phi, and the deposit) to shared memory,
// then line c (rows 2c, 2c + 1 as real and imaginary parts) is formed by its
// 16 lanes, transformed in registers and written back to its line buffer;
// the Hermitian split of every line's spectrum goes out with the lanes over
// y, two rows' modes (16 contiguous bytes) per lane.
template <typename T, int PRO>
__global__ void __launch_bounds__(256)
k_xr2c256(const T* __restrict__ in0, const T* __restrict__ dep, cpx<T>* __restrict__ out,
          const cpx<T>* __restrict__ tw, int Ny, int Nz, FHArgs fh) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int ROWS = 2 * W;
  T* sphi = reinterpret_cast<T*>(smraw);  // [ROWS][N]
  T* sdep = sphi + ROWS * N;              // [ROWS][N] (PRO >= 1)
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * ROWS;
  constexpr int PER = 16 / (int)sizeof(T);  // reals per 16-byte copy
  for (int i = threadIdx.x; i < ROWS * N / PER; i += 256) {
    const int row = i / (N / PER), x = (i % (N / PER)) * PER;
    const int y = y0 + row;
    if (y < Ny) {
      const size_t o = ((size_t)z * Ny + y) * N + x;
      cp_async16(sphi + row * N + x, in0 + o);
      if constexpr (PRO >= 1) cp_async16(sdep + row * N + x, dep + o);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4;
  cpx<T> v[16];
  unsigned long long nless = 0, ngreat = 0;
#pragma unroll
  for (int r = 0; r < 16; ++r) {
    const int x = j + 16 * r;
    T pr[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int row = 2 * c + h;
      T p = (T)0;
      if (y0 + row < Ny) {
        p = sphi[row * N + x];
        if constexpr (PRO >= 1) {  // PRO 2: the Flory-Huggins part relative to f(c)
          T keep;
          p = fh_node_t<T, PRO == 2>(p, sdep[row * N + x], fh, nless, ngreat, &keep);
          if (fh.mu_out) reinterpret_cast<T*>(fh.mu_out)[((size_t)z * Ny + y0 + row) * N + x] = keep;
        } else {
          if (fh.centered) p -= (T)fh.c;  // transform phi - c
        }
      }
      pr[h] = p;
    }
    v[r] = mk<T>(pr[0], pr[1]);
  }
  if constexpr (PRO >= 1) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      nless += __shfl_down_sync(0xffffffffu, nless, off);
      ngreat += __shfl_down_sync(0xffffffffu, ngreat, off);
    }
    if ((threadIdx.x & 31) == 0 && (nless | ngreat)) {
      if (nless) atomicAdd(fh.counters + 0, nless);
      if (ngreat) atomicAdd(fh.counters + 1, ngreat);
    }
  }
  __syncthreads();  // the row tiles are read: their memory becomes the line buffers
  cpx<T>* zs = reinterpret_cast<cpx<T>*>(smraw);
  cpx<T>* rb = zs + c * RX;
  row256<T, -1>(v, rb, j, tw);
  __syncwarp();
#pragma unroll
  for (int r = 0; r < 16; ++r) rb[j + 17 * r] = v[r];  // mode j + 16 r
  __syncthreads();
  for (int idx = threadIdx.x; idx < (N / 2 + 1) * W; idx += 256) {
    const int l = idx % W, k = idx / W;
    const cpx<T>* line = zs + l * RX;
    const int km = (N - k) % N;
    const cpx<T> zk = line[k + (k >> 4)];
    const cpx<T> zm = conjg(line[km + (km >> 4)]);
    const cpx<T> a = scale(zk + zm, (T)0.5);
    const cpx<T> d = zk - zm;
    const cpx<T> b = mk<T>((T)0.5 * d.y, (T)-0.5 * d.x);
    const int y = y0 + 2 * l;
    const size_t o = ((size_t)k * Nz + z) * Ny + y;
    if constexpr (sizeof(T) == 4) {
      if (y + 1 < Ny && (Ny & 1) == 0) {  // o even: a 16-byte aligned pair
        *reinterpret_cast<float4*>(&out[o]) = make_float4(a.x, a.y, b.x, b.y);
        continue;
      }
    }
    if (y < Ny) out[o] = a;
    if (y + 1 < Ny) out[o + 1] = b;
  }
}

// The same x r2c fed by the tensor memory accelerator (FP32, Ny a multiple
// of XR_ROWS): a persistent grid whose CTAs walk tiles of XR_ROWS rows (rows
// y0 .. y0 + XR_ROWS of plane z, numbered plane by plane) with the grid's
// stride.  A tile's rows of phi arrive as one box; the deposit, zero except on
// the nodes of the grid lists, is read straight from global memory in the
// 32-byte sectors its support mask sets (fh.dep_mask; every sector when the
// mask is null), so the mostly-zero array costs no full read and no shared
// memory.  Line c (rows 2c, 2c + 1) is formed by its 16 lanes; after the
// first DFT-16 the box is dead and its memory serves as the lines' exchange
// buffer; once every line has read its exchange back, thread 0 queues the
// box of the CTA's next tile, which lands while the CTA finishes the
// transform and writes the current tile.  The Hermitian split needs mode
// N - k next to mode k: it lives in lane (16 - j) % 16 of the same line, at
// register 15 - r (lane 0: its own register (16 - r) % 16), so one shuffle
// per mode brings it and each lane writes its modes k = j + 16 r (r < 8, and
// k = N/2 at lane 0) directly, 16 bytes (rows 2c, 2c + 1) per mode.
// Lines per CTA: 8 (128 threads, 16-row tiles).  The tiles per SM then come
// in finer steps than with 16 lines, so the last round over them leaves
// fewer SMs idle (2048 32-row tiles at 256^3 are 13.5 per SM).
constexpr int XR_LINES = 8;
constexpr int XR_THREADS = 16 * XR_LINES;
constexpr int XR_ROWS = 2 * XR_LINES;         // rows per tile
constexpr int XR_BOX = XR_ROWS * N * 4;       // bytes of one tile's box
constexpr int XR_BUF = XR_LINES * RX * 8;     // the lines' exchange buffer (covers the box)
static_assert(XR_BOX <= XR_BUF, "the box fits in the exchange buffer");
constexpr size_t XR_SMEM = (size_t)XR_BUF + 1024 + 16;  // + alignment slack + the mbarrier

template <int PRO, int MINB>
__global__ void __launch_bounds__(XR_THREADS, MINB)
k_xr2c256t(const __grid_constant__ CUtensorMap mphi, const float* __restrict__ dep, cpx<float>* __restrict__ out,
           const cpx<float>* __restrict__ tw, int Ny, int Nz, FHArgs fh, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smraw[];  // aligned to 1024 below
  unsigned char* buf = smraw + ((1024u - (tc::smem_u32(smraw) & 1023u)) & 1023u);
  const float* sphi = reinterpret_cast<const float*>(buf);
  uint64_t* bar = reinterpret_cast<uint64_t*>(buf + XR_BUF);
  const int tpp = Ny / XR_ROWS;  // tiles per plane
  const int ntiles = tpp * Nz;
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4;
  const uint32_t* __restrict__ dmask = fh.dep_mask;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int t) {  // thread 0: the box of tile t
    tc::fence_async_smem();
    tma::arrive_expect(bar, (uint32_t)XR_BOX);
    tma::load2d(buf, &mphi, 0, (t / tpp) * Ny + (t % tpp) * XR_ROWS, bar);
  };
  int t = blockIdx.x;
  if (threadIdx.x == 0 && t < ntiles) issue(t);
  uint32_t phase = 0;
  bool failed = false;
  unsigned nless = 0, ngreat = 0;
  const FHf fhf = fh_floats(fh);
  float* __restrict__ mu_out = reinterpret_cast<float*>(fh.mu_out);
  const float cshift = (float)fh.c;
  const bool center_fft = fh.centered != 0;
  const int src = (threadIdx.x & 16) | ((16 - j) & 15);  // the lane holding mode N - k
  for (; t < ntiles; t += gridDim.x, phase ^= 1u) {
    const int z = t / tpp, y0 = (t % tpp) * XR_ROWS;
    const size_t row0 = (size_t)z * Ny + y0 + 2 * c;  // the line's first row
    // the deposit of the line's two rows where its support mask is set (one
    // mask word per 256-node row), loaded while the box is in flight
    float dd[2][16];
    if constexpr (PRO >= 1) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint32_t m = dmask ? dmask[row0 + h] >> (j >> 3) : 0xffffffffu;
        const float* drow = dep + (row0 + h) * N + j;
#pragma unroll
        for (int r = 0; r < 16; ++r) dd[h][r] = (m >> (2 * r)) & 1u ? drow[16 * r] : 0.f;
      }
    }
    const bool got = tc::mbar_wait(bar, phase);
    cpx<float> v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      const int x = j + 16 * r;
      float pr[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float p = sphi[(2 * c + h) * N + x];
        if constexpr (PRO >= 1) {  // PRO 2: the Flory-Huggins part relative to f(c)
          float keep;
          p = fh_node_f<PRO == 2>(p, dd[h][r], fhf, nless, ngreat, &keep);
          if (mu_out) mu_out[(row0 + h) * N + x] = keep;
        } else {
          if (center_fft) p -= cshift;  // transform phi - c
        }
        pr[h] = p;
      }
      v[r] = mk<float>(pr[0], pr[1]);
    }
    fft::dft16<-1>(v);
    if (__syncthreads_or(!got)) {  // every line has read the box
      failed = true;
      break;
    }
    cpx<float>* rb = reinterpret_cast<cpx<float>*>(buf) + c * RX;
    rput16(rb, v, j);
    __syncwarp();
    rget16(rb, v, j);
    __syncthreads();  // the box's memory is free for the next tile
    if (threadIdx.x == 0 && t + (int)gridDim.x < ntiles) issue(t + (int)gridDim.x);
    twiddle16<float, -1>(v, j, tw);
    fft::dft16<-1>(v);  // v[r] = mode j + 16 r of line c
    const int y = y0 + 2 * c;
#pragma unroll
    for (int r = 0; r <= 8; ++r) {
      // mode N - k of k = j + 16 r: lane src's register 15 - r, or (lane 0) own register (16 - r) % 16
      cpx<float> zm;
      if (r < 8) {
        zm.x = __shfl_sync(0xffffffffu, v[15 - r].x, src);
        zm.y = __shfl_sync(0xffffffffu, v[15 - r].y, src);
        if (j == 0) zm = v[(16 - r) & 15];
      } else {
        if (j != 0) continue;
        zm = v[8];
      }
      zm = conjg(zm);
      const cpx<float> zk = v[r];
      const cpx<float> a = scale(zk + zm, 0.5f);
      const cpx<float> d = zk - zm;
      const cpx<float> b = mk<float>(0.5f * d.y, -0.5f * d.x);
      const int k = j + 16 * r;
      *reinterpret_cast<float4*>(&out[((size_t)k * Nz + z) * Ny + y]) = make_float4(a.x, a.y, b.x, b.y);
    }
  }
  if constexpr (PRO >= 1) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      nless += __shfl_down_sync(0xffffffffu, nless, off);
      ngreat += __shfl_down_sync(0xffffffffu, ngreat, off);
    }
    if ((threadIdx.x & 31) == 0 && (nless | ngreat)) {
      if (nless) atomicAdd(fh.counters + 0, (unsigned long long)nless);
      if (ngreat) atomicAdd(fh.counters + 1, (unsigned long long)ngreat);
    }
  }
  if (failed && threadIdx.x == 0) {
    atomicOr(status, ST_TIMEOUT);
    tc::mbar_wait(bar, phase);  // give the late load time to land before the CTA's shared memory is released
  }
}

// launch of k_xr2c256t: -3 when it does not apply (tensor maps unavailable)
inline int xr2c_tma(const Geom& g, const float* in, const float* dep, cpx<float>* out, const cpx<float>* tw,
                    const FHArgs& fh, int* status, cudaStream_t st) {
  constexpr int MINB = 4 * 256 / XR_THREADS;  // 64 registers a thread
  CUtensorMap mphi;
  if (!tma::map2d_f32(&mphi, in, N, (uint64_t)g.ny * g.nz, N, XR_ROWS)) return -3;
  const int pro = !dep ? 0 : (fh.centered && fh.enabled) ? 2 : 1;
  void (*k)(const CUtensorMap, const float*, cpx<float>*, const cpx<float>*, int, int, FHArgs, int*) =
      pro == 0 ? k_xr2c256t<0, MINB> : pro == 1 ? k_xr2c256t<1, MINB> : k_xr2c256t<2, MINB>;
  if (set_smem(k, XR_SMEM)) return -1;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  static std::mutex mu;
  static std::map<std::pair<int, int>, int> resident;  // (device, pro) -> CTAs the device holds at once
  int slots = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = resident.find({dev, pro});
    if (it == resident.end()) {
      int sms = 0, per_sm = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, XR_THREADS, XR_SMEM) != cudaSuccess || per_sm < 1)
        return -1;
      it = resident.emplace(std::make_pair(dev, pro), sms * per_sm).first;
    }
    slots = it->second;
  }
  const long long ntiles = (long long)(g.ny / XR_ROWS) * g.nz;
  const int grid = (int)(ntiles < (long long)slots ? ntiles : (long long)slots);
  k<<<grid, XR_THREADS, XR_SMEM, st>>>(mphi, dep, out, tw, g.ny, g.nz, fh, status);
  return 0;
}

template <typename T>
int xr2c(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* tw, const FHArgs& fh,
         cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (g.xr2c_tma && g.ny % XR_ROWS == 0 && fh.status) {
      const int rc = xr2c_tma(g, in, dep, out, tw, fh, fh.status, st);
      if (rc != -3) return rc;
    }
  }
  const size_t tiles = (size_t)2 * W * N * sizeof(T) * (dep ? 2 : 1);
  const size_t lines = (size_t)W * RX * sizeof(cpx<T>);
  const size_t sm = tiles > lines ? tiles : lines;
  dim3 grid((g.ny + 2 * W - 1) / (2 * W), g.nz);
  if (dep && fh.centered && fh.enabled && sizeof(T) == 4) {
    auto k = k_xr2c256<T, 2>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, grid, dim3(256), sm, st, in, dep, out, tw, g.ny, g.nz, fh);
  } else if (dep) {
    auto k = k_xr2c256<T, 1>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, grid, dim3(256), sm, st, in, dep, out, tw, g.ny, g.nz, fh);
  } else {
    auto k = k_xr2c256<T, 0>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, grid, dim3(256), sm, st, in, dep, out, tw, g.ny, g.nz, fh);
  }
  return 0;
}

// the inverse chain's three x c2r in one launch: C -> (phi, dphi/dx) in CTAs
// [0, nb0), D -> dphi/dy in [nb0, nb0 + nb1), E -> dphi/dz after
template <typename T>
__global__ void __launch_bounds__(256)
k_xc2r3_256(const cpx<T>* __restrict__ C, T* __restrict__ phi, T* __restrict__ gx, const cpx<T>* __restrict__ D,
            T* __restrict__ gy, const cpx<T>* __restrict__ E, T* __restrict__ gz, T sp, T sg, T dq,
            const cpx<T>* __restrict__ tw, int Ny, int Nz, NanArgs nan, NanArgs nonan, int nb0, int nb1,
            const uint32_t* __restrict__ mask, const int* __restrict__ mask_off) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int bx = blockIdx.x, z = blockIdx.y;
  const uint32_t* gm = mask && !*mask_off ? mask : nullptr;
  if (bx < nb0)
    xc2r_tile256<T, 2>(bx, z, C, phi, gx, sp, sg, dq, tw, Ny, Nz, nan, nullptr, gm, smraw);
  else if (bx < nb0 + nb1)
    xc2r_tile256<T, 1>(bx - nb0, z, D, gy, nullptr, sg, sg, dq, tw, Ny, Nz, nonan, gm, nullptr, smraw);
  else
    xc2r_tile256<T, 1>(bx - nb0 - nb1, z, E, gz, nullptr, sg, sg, dq, tw, Ny, Nz, nonan, gm, nullptr, smraw);
}

// The same three x c2r fed by the tensor memory accelerator (FP32, Ny a
// multiple of 32): a persistent grid whose CTAs walk the tiles of
// k_xc2r3_256, numbered plane by plane (per plane z: nb0 tiles of C, nb1
// of D, nb1 of E), with the grid's stride.  A tile's half-spectrum block
// (kx = 0..128 by the tile's row pairs) arrives as one or two tensor-map
// boxes of 129 rows x 128 bytes in a 1024-byte-aligned buffer, 128-byte
// swizzled (16-byte chunk c of row k at chunk c ^ (k & 7)), so the 16 lanes
// of a line, which read one pair column at 16 different kx, hit different
// banks.  Each thread reads its line's 16 elements straight from the block
// and Hermitian-completes them on the fly.  After the first DFT-16 the
// block is dead and the same buffer serves as the lines' exchange buffer;
// once every line has read its exchange back, thread 0 queues the loads of
// the CTA's next tile into the buffer, which land while the CTA finishes the
// transform and the stores of the current tile.  A load that does not land
// within the wait limit sets ST_TIMEOUT and ends the CTA.
constexpr int XT_BOX = (N / 2 + 1) * 128;  // bytes of one 129 x 128-byte box
constexpr int XT_HALF = 17 * 1024;         // second box of a one-output tile, 1024-byte aligned
constexpr int XT_BUF = W * RX * 8;         // the FP32 exchange buffer of 16 lines
static_assert(XT_HALF + XT_BOX <= XT_BUF, "both boxes of a tile fit in the exchange buffer");
constexpr size_t XT_SMEM = XT_BUF + 1024 + 16;  // + alignment slack + the mbarrier

struct XTile {
  int kind, z, y0;  // kind 0: C (phi and dphi/dx, 8 row pairs), 1: D (dphi/dy), 2: E (dphi/dz) (16 pairs)
};
PHAFD_D XTile xt_tile(int t, int nb0, int nb1) {
  const int tp = nb0 + 2 * nb1;
  XTile x;
  x.z = t / tp;
  int b = t - x.z * tp;
  if (b < nb0) {
    x.kind = 0;
    x.y0 = b * W;
  } else if ((b -= nb0) < nb1) {
    x.kind = 1;
    x.y0 = b * 2 * W;
  } else {
    x.kind = 2;
    x.y0 = (b - nb1) * 2 * W;
  }
  return x;
}

// thread 0: the loads of tile x's block into buf, completing on bar
PHAFD_D void xt_issue(const XTile& x, const CUtensorMap* mC, const CUtensorMap* mD, const CUtensorMap* mE,
                      unsigned char* buf, uint64_t* bar) {
  const CUtensorMap* m = x.kind == 0 ? mC : x.kind == 1 ? mD : mE;
  tc::fence_async_smem();  // the buffer's earlier generic-proxy accesses come before the loads' writes
  tma::arrive_expect(bar, (x.kind == 0 ? 1u : 2u) * (uint32_t)XT_BOX);
  tma::load3d(buf, m, 2 * x.y0, x.z, 0, bar);
  if (x.kind != 0) tma::load3d(buf + XT_HALF, m, 2 * x.y0 + 32, x.z, 0, bar);
}

// (MINB: CTAs per SM the register allocation is fitted to)
template <int MINB>
__global__ void __launch_bounds__(256, MINB)
k_xc2r3t_256(const __grid_constant__ CUtensorMap mC, const __grid_constant__ CUtensorMap mD,
             const __grid_constant__ CUtensorMap mE, float* __restrict__ phi, float* __restrict__ gx,
             float* __restrict__ gy, float* __restrict__ gz, float sp, float sg, float dq,
             const cpx<float>* __restrict__ tw, int Ny, int Nz, NanArgs nan, const uint32_t* __restrict__ mask,
             const int* __restrict__ mask_off, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smraw[];  // aligned to 1024 below
  unsigned char* buf = smraw + ((1024u - (tc::smem_u32(smraw) & 1023u)) & 1023u);
  uint64_t* bar = reinterpret_cast<uint64_t*>(buf + XT_BUF);
  const int nb0 = Ny / W, nb1 = Ny / (2 * W);
  const int ntiles = (nb0 + 2 * nb1) * Nz;
  const uint32_t* gm = mask && !*mask_off ? mask : nullptr;
  const int j = threadIdx.x & 15, c = threadIdx.x >> 4;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  int t = blockIdx.x;
  if (threadIdx.x == 0 && t < ntiles) xt_issue(xt_tile(t, nb0, nb1), &mC, &mD, &mE, buf, bar);
  uint32_t phase = 0;
  bool failed = false;
  for (; t < ntiles; t += gridDim.x, phase ^= 1u) {
    const XTile x = xt_tile(t, nb0, nb1);
    const bool got = tc::mbar_wait(bar, phase);
    // line c: output q of row pair l (kind 0: q = c / 8, l = c % 8; else q = 0, l = c)
    const int q = x.kind == 0 ? c >> 3 : 0;
    const int l = x.kind == 0 ? c & 7 : c;
    const unsigned char* box = buf + (l >= 8 ? XT_HALF : 0);
    const int ch = l & 7;
    cpx<float> v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {  // element e = j + 16 r of the line: mode k = e (e < 128) or N - e
      const int e = j + 16 * r;
      const int k = r < 8 ? e : N - e;
      const float4 p = *reinterpret_cast<const float4*>(box + k * 128 + ((ch ^ (k & 7)) << 4));
      cpx<float> a = mk<float>(p.x, p.y), b = mk<float>(p.z, p.w);
      if (q == 1) {
        a = deriv(a, dq, k);
        b = deriv(b, dq, k);
      }
      if ((r == 0 || r == 8) && j == 0) {  // k = 0 (r = 0) or N / 2 (r = 8): only at lane 0
        a.y = 0.f;
        b.y = 0.f;
      }
      v[r] = r < 8 ? mk<float>(a.x - b.y, a.y + b.x) : mk<float>(a.x + b.y, b.x - a.y);
    }
    fft::dft16<+1>(v);
    if (__syncthreads_or(!got)) {  // every line has read the block
      failed = true;
      break;
    }
    cpx<float>* rb = reinterpret_cast<cpx<float>*>(buf) + c * RX;
    rput16(rb, v, j);
    __syncwarp();
    rget16(rb, v, j);
    __syncthreads();  // the buffer is free for the next block
    if (threadIdx.x == 0 && t + (int)gridDim.x < ntiles)
      xt_issue(xt_tile(t + (int)gridDim.x, nb0, nb1), &mC, &mD, &mE, buf, bar);
    twiddle16<float, +1>(v, j, tw);
    fft::dft16<+1>(v);
    if (x.kind == 0 && q == 0) xc2r_store256<float, true>(v, j, x.y0 + 2 * l, x.z, phi, sp, Ny, nan, nullptr);
    else xc2r_store256<float, false>(v, j, x.y0 + 2 * l, x.z, x.kind == 0 ? gx : x.kind == 1 ? gy : gz, sg, Ny, nan, gm);
  }
  if (failed && threadIdx.x == 0) {
    atomicOr(status, ST_TIMEOUT);
    tc::mbar_wait(bar, phase);  // give the late loads time to land before the CTA's shared memory is released
  }
}

// launch of k_xc2r3t_256: -3 when it does not apply (tensor maps unavailable)
inline int xc2r3_tma(const Geom& g, const cpx<float>* C, float* phi, float* gx, const cpx<float>* D, float* gy,
                     const cpx<float>* E, float* gz, float sp, float sg, const cpx<float>* tw, const NanArgs& nan,
                     const uint32_t* gmask, const int* gmask_off, int* status, cudaStream_t st) {
  CUtensorMap m[3];
  const cpx<float>* src[3] = {C, D, E};
  for (int i = 0; i < 3; ++i)
    if (!tma::map3d_f32(&m[i], src[i], 2 * (uint64_t)g.ny, (uint64_t)g.nz, (uint64_t)g.nxh, 32, 1, N / 2 + 1,
                        CU_TENSOR_MAP_SWIZZLE_128B))
      return -3;
  auto k = k_xc2r3t_256<5>;
  if (set_smem(k, XT_SMEM)) return -1;
  // resident CTAs of the device, found once per device (outside graph capture: the first launch is eager)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  static std::mutex mu;
  static std::map<int, int> resident;
  int slots = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = resident.find(dev);
    if (it == resident.end()) {
      int sms = 0, per_sm = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, XT_SMEM) != cudaSuccess || per_sm < 1)
        return -1;
      it = resident.emplace(dev, sms * per_sm).first;
    }
    slots = it->second;
  }
  const long long ntiles = (long long)(g.ny / W + 2 * (g.ny / (2 * W))) * g.nz;
  const int grid = (int)(ntiles < (long long)slots ? ntiles : (long long)slots);
  k<<<grid, 256, XT_SMEM, st>>>(m[0], m[1], m[2], phi, gx, gy, gz, sp, sg, (float)g.kq[0], tw, g.ny, g.nz, nan, gmask,
                                gmask_off, status);
  return 0;
}

template <typename T>
int xc2r3(const Geom& g, const cpx<T>* C, T* phi, T* gx, const cpx<T>* D, T* gy, const cpx<T>* E, T* gz, T sp,
          T sg, const cpx<T>* tw, const NanArgs& nan, const NanArgs& nonan, const uint32_t* gmask,
          const int* gmask_off, int* status, cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    if (g.xc2r_tma && g.ny % (2 * W) == 0 && status) {
      const int rc = xc2r3_tma(g, C, phi, gx, D, gy, E, gz, sp, sg, tw, nan, gmask, gmask_off, status, st);
      if (rc != -3) return rc;
    }
  }
  const size_t sm = (size_t)W * RX * sizeof(cpx<T>);
  const int nb0 = (g.ny + W - 1) / W, nb1 = (g.ny + 2 * W - 1) / (2 * W);
  auto k = k_xc2r3_256<T>;
  if (set_smem(k, sm)) return -1;
  launch_grid(k, dim3(nb0 + 2 * nb1, g.nz), dim3(256), sm, st, C, phi, gx, D, gy, E, gz, sp, sg, (T)g.kq[0], tw,
              g.ny, g.nz, nan, nonan, nb0, nb1, gmask, gmask_off);
  return 0;
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

template <typename T, int NOISE, bool MACRO>
int zfused_launch(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1, const cpx<T>* twf,
                  const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int kx0, cudaStream_t st) {
  const size_t sm = (size_t)2 * N * W * sizeof(cpx<T>);
  auto k = g.ny == N ? k_zfused256<T, NOISE, MACRO, N> : k_zfused256<T, NOISE, MACRO, 0>;
  if (set_smem(k, sm)) return -1;
  dim3 grid((g.ny + W - 1) / W, g.nxh - 2 * kx0);
  launch_grid(k, grid, dim3(256), sm, st, muin, muhat, out0, out1, (T)g.kq[2], twf, twi, g.ny, u, store_mu, kx0);
  return 0;
}

template <typename T>
int zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1, const cpx<T>* twf,
           const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only, cudaStream_t st) {
  const int kx0 = bulk_only ? 1 : 0;
  if (g.nxh - 2 * kx0 <= 0) return 0;
  const bool macro = u.nsub > 1;
#define ZF(NZ, M) zfused_launch<T, NZ, M>(g, muin, muhat, out0, out1, twf, twi, u, store_mu, kx0, st)
  switch (u.noise) {
    case PHAFD_NOISE_OFF: return macro ? ZF(PHAFD_NOISE_OFF, true) : ZF(PHAFD_NOISE_OFF, false);
    case PHAFD_NOISE_REFERENCE: return macro ? ZF(PHAFD_NOISE_REFERENCE, true) : ZF(PHAFD_NOISE_REFERENCE, false);
    default: return macro ? ZF(PHAFD_NOISE_PHILOX, true) : ZF(PHAFD_NOISE_PHILOX, false);
  }
#undef ZF
}

}  // namespace r256
}  // namespace phafd
