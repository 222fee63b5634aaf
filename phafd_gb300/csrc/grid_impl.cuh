// Grid-side kernels of the particle-field step, templated on the arithmetic
// type T (float or double).  The grid_{f32,f64}_{x,y,z}.cu translation units
// instantiate the GridOps members of one type and one axis family each.
//
// Layouts (all in HBM, resident for the whole run)
//   real field   R[z][y][x]                       x fastest
//   spectrum     C[kx][kz][ky], kx in [0, Nx/2]    ky fastest
//   after x pass C[kx][z][y]; after y pass C[kx][z][ky]
//
// A 3D r2c is three passes (x rows -> y lines -> z columns); a c2r runs them
// backwards.  Every pass moves one tile HBM -> shared memory -> HBM with the
// pointwise stages of the step fused into its load or store:
//   x-forward : Flory-Huggins mu + bead deposit (fixgrid_floryhuggins.cpp:71-83)
//   z pass    : Model-B update with the Hermitian planes and the real points
//               (conjugate.cpp:163-327, conjugate_volfrac.cpp:89-144)
//   y / z / x : the spectral derivative i*dq*m (fixgrid_conjugate.cpp:80-105)
//   x-inverse : the 1/N of the gradient and the NaN check of phi(0,0,0)
#pragma once
#include <map>
#include <mutex>
#include <utility>

#include "fft.cuh"
#include "internal.h"

namespace phafd {

// Loop over the TOTAL elements of a tile with NT threads: a fixed trip count
// the compiler unrolls, so all global loads of a thread are in flight at once.
#define TILE_LOOP(idx, TOTAL, NT)                                                           \
  _Pragma("unroll") for (int it_##idx = 0; it_##idx < ((TOTAL) + (NT)-1) / (NT); ++it_##idx) \
    if (const int idx = (int)threadIdx.x + it_##idx * (NT); ((TOTAL) % (NT)) == 0 || idx < (TOTAL))

// Flory-Huggins part of mu at phi = p (fixgrid_floryhuggins.cpp:81-82),
// tv (ln(p / (1 - p)) + chi (1 - 2 p)).  FP64: the reference's expression.
// FP32 with a reference concentration c: tv (f(p) - f(c)) written as
// log1p((p - c) / (c (1 - p))) - 2 chi (p - c), whose rounding is relative to
// the deviation p - c (the constant tv f(c) only moves the k = 0 mode of mu,
// which the update multiplies by q^2 = 0).  FP32 without c: the difference of
// two hardware logarithms.
// (CENTER: the centered FP32 form; a compile-time choice, so the plain
// kernels carry no code or registers for it)
template <bool CENTER>
PHAFD_D double fh_part(double p, const FHArgs& fh) { return fh.tv * (log(p / (1.0 - p)) + fh.chi * (1.0 - 2.0 * p)); }
template <bool CENTER>
PHAFD_D float fh_part(float p, const FHArgs& fh) {
  if constexpr (CENTER) {
    const float d = p - (float)fh.c;
    return (float)fh.tv * (log1pf(__fdividef(d * (float)fh.inv_c, 1.0f - p)) - 2.0f * (float)fh.chi * d);
  }
  return (float)fh.tv * ((__logf(p) - __logf(1.0f - p)) + (float)fh.chi * (1.0f - 2.0f * p));
}

// mu at one node from phi = p and the bead deposit dd: the reflections of
// fixgrid_floryhuggins.cpp:72-80 (counted), then deposit + FH part.  Returns
// the value the r2c transforms; *keep is the materialised chempot.
template <typename T, bool CENTER>
PHAFD_D T fh_node_t(T p, T dd, const FHArgs& fh, unsigned long long& nless, unsigned long long& ngreat, T* keep) {
  if (!fh.enabled) {
    *keep = dd;
    return dd;
  }
  if (p <= (T)0) { p = -p; nless++; }
  else if (p >= (T)1) { p = (T)1 - (p - (T)1); ngreat++; }
  const T m = dd + fh_part<CENTER>(p, fh);
  *keep = CENTER ? m + (T)fh.fconst : m;
  return m;
}
// The FP32 constants of the Flory-Huggins node, converted once per thread
// (the same roundings as fh_node_t's casts, so the same results): for the
// persistent x pass, whose loop over tiles would otherwise convert them per
// node.
struct FHf {
  float tv, chi, c, inv_c, fconst;
  bool enabled;
};
PHAFD_D FHf fh_floats(const FHArgs& fh) {
  return FHf{(float)fh.tv, (float)fh.chi, (float)fh.c, (float)fh.inv_c, (float)fh.fconst, fh.enabled != 0};
}
template <bool CENTER>
PHAFD_D float fh_node_f(float p, float dd, const FHf& f, unsigned& nless, unsigned& ngreat, float* keep) {
  if (!f.enabled) {
    *keep = dd;
    return dd;
  }
  if (p <= 0.0f) { p = -p; nless++; }
  else if (p >= 1.0f) { p = 1.0f - (p - 1.0f); ngreat++; }
  float part;
  if constexpr (CENTER) {
    const float d = p - f.c;
    part = f.tv * (log1pf(__fdividef(d * f.inv_c, 1.0f - p)) - 2.0f * f.chi * d);
  } else {
    part = f.tv * ((__logf(p) - __logf(1.0f - p)) + f.chi * (1.0f - 2.0f * p));
  }
  const float m = dd + part;
  *keep = CENTER ? m + f.fconst : m;
  return m;
}

// the same with the form chosen at run time (the generic and plane kernels)
template <typename T>
PHAFD_D T fh_node(T p, T dd, const FHArgs& fh, unsigned long long& nless, unsigned long long& ngreat, T* keep) {
  return (sizeof(T) == 4 && fh.centered) ? fh_node_t<T, true>(p, dd, fh, nless, ngreat, keep)
                                         : fh_node_t<T, false>(p, dd, fh, nless, ngreat, keep);
}

template <typename T>
PHAFD_D cpx<T> deriv(cpx<T> a, T dq, int m) {
  // fixgrid_conjugate.cpp:101-103: phi_hat * (0, dq) * m
  const T mm = (T)m;
  return mk<T>(-(a.y * dq) * mm, (a.x * dq) * mm);
}

// number of lines a CTA transforms for axis length N, so that N*NL/16 = 256
template <int N>
__host__ __device__ constexpr int lines_for() {
  int t = 4096 / N, p = 1;
  while (p * 2 <= t) p *= 2;
  return p > 32 ? 32 : (p < 4 ? 4 : p);
}

// -------------------------------------------------------------------- x r2c
template <typename T, int N, int LB, int PRO>
__global__ void __launch_bounds__(N * LB / 16)
k_xr2c(const T* __restrict__ in0, const T* __restrict__ dep, cpx<T>* __restrict__ out,
       const cpx<T>* __restrict__ tw, int Ny, int Nz, FHArgs fh) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* s = reinterpret_cast<cpx<T>*>(smraw);
  constexpr int NT = N * LB / 16, STR = LB + 1;
  cpx<T>* sd = s + (size_t)N * STR;  // deposit rows, same layout (PRO == 1)
  const int z = blockIdx.y;
  const int y0 = blockIdx.x * 2 * LB;
  unsigned long long nless = 0, ngreat = 0;
  // rows 2l and 2l+1 of the tile land as the real and imaginary parts of line l
  TILE_LOOP(idx, LB * N, NT) {
    const int l = idx / N, x = idx % N;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int y = y0 + 2 * l + h;
      T* dst = reinterpret_cast<T*>(&s[x * STR + l]) + h;
      T* dstd = reinterpret_cast<T*>(&sd[x * STR + l]) + h;
      if (y < Ny) {
        const size_t o = ((size_t)z * Ny + y) * N + x;
        cp_async_real(dst, in0 + o);
        if constexpr (PRO == 1) cp_async_real(dstd, dep + o);
      } else {
        *dst = (T)0;
        if constexpr (PRO == 1) *dstd = (T)0;
      }
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if constexpr (PRO == 1) {
    TILE_LOOP(idx, LB * N, NT) {
      const int l = idx / N, x = idx % N;
      T* v = reinterpret_cast<T*>(&s[x * STR + l]);
      const T* dd = reinterpret_cast<const T*>(&sd[x * STR + l]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int y = y0 + 2 * l + h;
        if (y < Ny) {
          T keep;
          v[h] = fh_node(v[h], dd[h], fh, nless, ngreat, &keep);
          if (fh.mu_out) reinterpret_cast<T*>(fh.mu_out)[((size_t)z * Ny + y) * N + x] = keep;
        }
      }
    }
  } else {
    if (fh.centered) {  // transform phi - c
      TILE_LOOP(idx, LB * N, NT) {
        const int l = idx / N, x = idx % N;
        T* v = reinterpret_cast<T*>(&s[x * STR + l]);
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (y0 + 2 * l + h < Ny) v[h] -= (T)fh.c;
      }
    }
  }
  if constexpr (PRO == 1) {
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
  __syncthreads();
  fft::run<T, N, LB, -1>(s, tw);
  TILE_LOOP(idx, LB * (N / 2 + 1), NT) {
    const int l = idx % LB, k = idx / LB;
    const cpx<T> zk = s[k * STR + l];
    const cpx<T> zm = conjg(s[((N - k) % N) * STR + l]);
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

// -------------------------------------------------------------------- x c2r
// out0 = c2r(m0 * in) * s0 with m0 = i dqx kx if MUL0 else 1
// out1 = c2r(i dqx kx * in) * s1          (NOUT == 2)
// one tile (rows y0 .. y0 + 2 LB of plane z); bx is the tile's index along y;
// mask0 / mask1 limit the stores of output 0 / 1 (null: all) to the 32-byte
// sectors whose bit is set: bit g covers nodes [g G, g G + G), G = 32 / sizeof(T),
// so a store never fills part of a sector.  The tile's mask words are staged
// in shared memory behind the FFT lines (xc2r_mask_words of them).
template <typename T, int N, int LB>
constexpr int xc2r_mask_words() { return (2 * LB * N) / ((32 / (int)sizeof(T)) * 32) + 2; }

template <typename T, int N, int LB, bool MUL0, int NOUT>
PHAFD_D void xc2r_tile(int bx, int z, const cpx<T>* __restrict__ in, T* __restrict__ out0, T* __restrict__ out1,
                       T s0, T s1, T dq, const cpx<T>* __restrict__ tw, int Ny, int Nz, const NanArgs& nan,
                       unsigned char* smraw, const uint32_t* mask0 = nullptr, const uint32_t* mask1 = nullptr) {
  cpx<T>* s = reinterpret_cast<cpx<T>*>(smraw);
  constexpr int NL = LB * NOUT;
  constexpr int NT = N * NL / 16, STR = NL + 1;
  constexpr int G = 32 / (int)sizeof(T);
  const int y0 = bx * 2 * LB;
  uint32_t* mw = reinterpret_cast<uint32_t*>(s + (size_t)N * STR);
  const size_t row0 = ((size_t)z * Ny + y0) * N;
  const size_t w0 = (row0 / G) >> 5;
  if (mask0 || mask1) {
    const int rows = Ny - y0 < 2 * LB ? Ny - y0 : 2 * LB;
    const int nw = (int)((((row0 + (size_t)rows * N - 1) / G) >> 5) - w0 + 1);
    const uint32_t* m = mask0 ? mask0 : mask1;
    for (int i = threadIdx.x; i < nw; i += NT) mw[i] = m[w0 + i];
  }
  TILE_LOOP(idx, LB * (N / 2 + 1), NT) {
    const int l = idx % LB, k = idx / LB;
    const int y = y0 + 2 * l;
    const size_t o = ((size_t)k * Nz + z) * Ny + y;
    cpx<T> A = mk<T>(0, 0), B = mk<T>(0, 0);
    if (y < Ny) A = in[o];
    if (y + 1 < Ny) B = in[o + 1];
#pragma unroll
    for (int q = 0; q < NOUT; ++q) {
      cpx<T> a = A, b = B;
      if (q == 1 || MUL0) { a = deriv(a, dq, k); b = deriv(b, dq, k); }
      if (k == 0 || k == N / 2) { a.y = (T)0; b.y = (T)0; }
      s[k * STR + q * LB + l] = mk<T>(a.x - b.y, a.y + b.x);
      if (k > 0 && k < N / 2) s[(N - k) * STR + q * LB + l] = mk<T>(a.x + b.y, b.x - a.y);
    }
  }
  __syncthreads();
  fft::run<T, N, NL, +1>(s, tw);
  TILE_LOOP(idx, LB * N, NT) {
    const int x = idx % N, l = idx / N;
#pragma unroll
    for (int q = 0; q < NOUT; ++q) {
      const cpx<T> v = s[x * STR + q * LB + l];
      T* out = q == 0 ? out0 : out1;
      const T sc = q == 0 ? s0 : s1;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int y = y0 + 2 * l + h;
        if (y < Ny) {
          const T val = (h == 0 ? v.x : v.y) * sc + (q == 0 ? (T)nan.offset : (T)0);
          const size_t node = ((size_t)z * Ny + y) * N + x;
          const size_t sec = node / G;
          if (!(q == 0 ? mask0 : mask1) || ((mw[(sec >> 5) - w0] >> (sec & 31)) & 1u)) out[node] = val;
          if (q == 0 && nan.check && z == 0 && y == 0 && x == 0 && isnan(val))
            atomicCAS(reinterpret_cast<unsigned long long*>(nan.nan_step), (unsigned long long)-1LL,
                      (unsigned long long)(*nan.d_step));
        }
      }
    }
  }
}

template <typename T, int N, int LB, bool MUL0, int NOUT>
__global__ void __launch_bounds__(N * LB * NOUT / 16)
k_xc2r(const cpx<T>* __restrict__ in, T* __restrict__ out0, T* __restrict__ out1, T s0, T s1, T dq,
       const cpx<T>* __restrict__ tw, int Ny, int Nz, NanArgs nan) {
  extern __shared__ __align__(16) unsigned char smraw[];
  xc2r_tile<T, N, LB, MUL0, NOUT>(blockIdx.x, blockIdx.y, in, out0, out1, s0, s1, dq, tw, Ny, Nz, nan, smraw);
}

// the three x c2r of the inverse chain in one launch: C -> (phi, dphi/dx)
// with 2 LB2 rows per tile, D -> dphi/dy and E -> dphi/dz with 2 LB1 rows
// per tile (LB1 = 2 LB2: same threads and shared memory per tile)
template <typename T, int N, int LB2>
__global__ void __launch_bounds__(N * LB2 * 2 / 16)
k_xc2r3(const cpx<T>* __restrict__ C, T* __restrict__ phi, T* __restrict__ gx, const cpx<T>* __restrict__ D,
        T* __restrict__ gy, const cpx<T>* __restrict__ E, T* __restrict__ gz, T sp, T sg, T dq,
        const cpx<T>* __restrict__ tw, int Ny, int Nz, NanArgs nan, NanArgs nonan, int nb0, int nb1,
        const uint32_t* __restrict__ mask, const int* __restrict__ mask_off) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int bx = blockIdx.x, z = blockIdx.y;
  const uint32_t* gmask = mask && !*mask_off ? mask : nullptr;
  if (bx < nb0)
    xc2r_tile<T, N, LB2, false, 2>(bx, z, C, phi, gx, sp, sg, dq, tw, Ny, Nz, nan, smraw, nullptr, gmask);
  else if (bx < nb0 + nb1)
    xc2r_tile<T, N, 2 * LB2, false, 1>(bx - nb0, z, D, gy, nullptr, sg, sg, dq, tw, Ny, Nz, nonan, smraw, gmask);
  else
    xc2r_tile<T, N, 2 * LB2, false, 1>(bx - nb0 - nb1, z, E, gz, nullptr, sg, sg, dq, tw, Ny, Nz, nonan, smraw,
                                       gmask);
}

// -------------------------------------------------------------------- y pass
// lines contiguous: in[line * N + e]; out0 = FFT_S(in), out1 = FFT_S(i dq m(e) in)
template <typename T, int N, int LB, int S, int NOUT>
PHAFD_D void ypass_tile(long long bx, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, T dq,
                        const cpx<T>* __restrict__ tw, long long nlines, unsigned char* smraw) {
  cpx<T>* s = reinterpret_cast<cpx<T>*>(smraw);
  constexpr int NL = LB * NOUT;
  constexpr int NT = N * NL / 16, STR = NL + 1;
  const long long line0 = bx * LB;
  TILE_LOOP(idx, LB * N, NT) {
    const int l = idx / N, e = idx % N;
    cpx<T> v = mk<T>(0, 0);
    if (line0 + l < nlines) v = in[(line0 + l) * N + e];
    s[e * STR + l] = v;
    if constexpr (NOUT == 2) s[e * STR + LB + l] = deriv(v, dq, wrap_index(e, N));
  }
  __syncthreads();
  fft::run<T, N, NL, S>(s, tw);
  TILE_LOOP(idx, LB * N, NT) {
    const int l = idx / N, e = idx % N;
    if (line0 + l < nlines) {
      out0[(line0 + l) * N + e] = s[e * STR + l];
      if constexpr (NOUT == 2) out1[(line0 + l) * N + e] = s[e * STR + LB + l];
    }
  }
}

template <typename T, int N, int LB, int S, int NOUT>
__global__ void __launch_bounds__(N * LB * NOUT / 16)
k_ypass(const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, T dq, const cpx<T>* __restrict__ tw, long long nlines) {
  extern __shared__ __align__(16) unsigned char smraw[];
  ypass_tile<T, N, LB, S, NOUT>(blockIdx.x, in, out0, out1, dq, tw, nlines, smraw);
}

// the two inverse y passes of the inverse chain in one launch: A -> (C, D = i qy)
// with LB2 lines per tile, B -> E with 2 LB2 lines per tile
template <typename T, int N, int LB2>
__global__ void __launch_bounds__(N * LB2 * 2 / 16)
k_ypass_inv2(const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E, T dq,
             const cpx<T>* __restrict__ tw, long long nlines, long long nb0) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const long long bx = blockIdx.x;
  if (bx < nb0) ypass_tile<T, N, LB2, +1, 2>(bx, A, C, D, dq, tw, nlines, smraw);
  else ypass_tile<T, N, 2 * LB2, +1, 1>(bx - nb0, B, E, nullptr, dq, tw, nlines, smraw);
}

// -------------------------------------------------------------------- update
// One mode of ConjugateVolFrac::complex_update / real_update / origin_update
// (conjugate_volfrac.cpp:89-144) with the Hermitian bookkeeping of
// Conjugate::update for one rank (conjugate.cpp:163-327).  (kx, ky, kz) are
// this project's indices: the reference's (i, j, k) = (ky, kz, kx).
// Model-B update of one mode from its old spectrum value ph (unnormalised)
// and mu_hat value mu; (cy, cz) is the canonical mode that owns the noise.
// (QPOS: the caller guarantees q^2 > 0, so the FP32 path may take |q| as
// q^2 rsqrt(q^2): a few ulps, on the noise amplitude only)
template <typename T, bool QPOS = false>
PHAFD_D cpx<T> update_value(const UpdateArgs<T>& u, int kx, int cy, int cz, cpx<T> ph, cpx<T> mu, bool real,
                            const uint32_t* words = nullptr) {
  const int Ny = u.Ny, Nz = u.Nz;
  const T qx = u.qx * (T)kx;
  const T qy = u.qy * (T)wrap_index(cy, Ny);
  const T qz = u.qz * (T)wrap_index(cz, Nz);
  const T q2 = qx * qx + qz * qz + qy * qy;  // reference order: qx^2 + q(kz)^2 + q(ky)^2
  const T pre = u.mobility * q2 * u.dt;
  const T g = u.tvg * q2;
  cpx<T> r;
  T namp = (T)1;
  if (u.nsub > 1) {
    // a = 1 - pre (f2 + g) per substep: phi' = a^K phi - S_K pre (mu - f2 phi),
    // S_K = sum_{s<K} a^s; the noise of K substeps has variance sum a^(2s)
    const T a = (T)1 - pre * (u.f2 + g);
    T ak = (T)1, sk = (T)0, s2 = (T)0;
    for (int k = 0; k < u.nsub; ++k) {
      sk += ak;
      s2 += ak * ak;
      ak *= a;
    }
    const cpx<T> src = mk<T>(mu.x - u.f2 * ph.x, mu.y - u.f2 * ph.y);
    r = mk<T>((ak * ph.x - sk * pre * src.x) * u.norm, (ak * ph.y - sk * pre * src.y) * u.norm);
    namp = sqrt(s2);
  } else {
    const cpx<T> inner = mk<T>(mu.x + g * ph.x, mu.y + g * ph.y);
    r = mk<T>((ph.x - pre * inner.x) * u.norm, (ph.y - pre * inner.y) * u.norm);
  }
  T u0 = 0, u1 = 0;
  if (u.noise == PHAFD_NOISE_REFERENCE) {
    const double2 w = u.uref[((size_t)kx * Nz + cz) * Ny + cy];
    u0 = (T)w.x; u1 = (T)w.y;
  } else if (u.noise == PHAFD_NOISE_PHILOX) {
    uint32_t c[4];
    if (words) { c[0] = words[0]; c[1] = words[1]; c[2] = words[2]; c[3] = words[3]; }
    else field_noise_words(kx, cy, cz, Ny, Nz, (uint32_t)(*u.d_step), u.seed, c);
    field_noise_pair(c, cz, u0, u1);
  }
  T sq;
  if constexpr (QPOS && sizeof(T) == 4) sq = q2 * rsqrtf(q2);
  else sq = sqrt(q2);
  if (real) {
    r.x += u.rpref * sq * u.sqrtdt * u0 * namp;
  } else {
    const T a = u.cpref * sq * u.sqrtdt * namp;
    r.x += a * u0;
    r.y += a * u1;
  }
  return r;
}

template <typename T>
PHAFD_D cpx<T> update_mode(const UpdateArgs<T>& u, int kx, int ky, int kz, size_t o) {
  const int Ny = u.Ny, Nz = u.Nz, Nxh = u.Nxh;
  const bool plane = (kx == 0 || kx == Nxh - 1);
  int cy = ky, cz = kz;  // canonical mode whose update this element takes
  bool mirror = false, real = false, origin = false;
  if (plane) {
    const bool ry = (ky == 0 || ky == Ny / 2), rz = (kz == 0 || kz == Nz / 2);
    if (ry && rz) {
      real = true;
      origin = (kx == 0 && ky == 0 && kz == 0);
    } else {
      const bool canon = (kz >= 1 && kz < Nz / 2) || (kz == 0 && ky >= 1 && ky < Ny / 2) ||
                         (kz == Nz / 2 && ky > Ny / 2);
      if (!canon) {
        mirror = true;
        cy = (Ny - ky) % Ny;
        cz = (Nz - kz) % Nz;
      }
    }
  }
  const size_t oc = mirror ? ((size_t)kx * Nz + cz) * Ny + cy : o;
  cpx<T> ph = u.phi_old[oc];
  ph = scale(ph, u.phi_scale);
  if (origin) return scale(ph, u.norm);
  const cpx<T> r = update_value(u, kx, cy, cz, ph, u.mu_hat[oc], real);
  return mirror ? conjg(r) : r;
}

// -------------------------------------------------------------------- z pass
// tile = (kx, ky in [c0, c0+LB)), transform along kz with stride Ny.
// UPD: the loaded element is replaced by its Model-B update, stored to
// u.phi_new, then transformed.
template <typename T, int N, int LB, int S, int NOUT, bool UPD>
__global__ void __launch_bounds__(N * LB * NOUT / 16)
k_zpass(const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, T dq, const cpx<T>* __restrict__ tw, int Ny,
        UpdateArgs<T> u, int planes_only) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* s = reinterpret_cast<cpx<T>*>(smraw);
  constexpr int NL = LB * NOUT;
  constexpr int NT = N * NL / 16, STR = NL + 1;
  const int kx = planes_only ? (blockIdx.y == 0 ? 0 : u.Nxh - 1) : (int)blockIdx.y;
  const int c0 = blockIdx.x * LB;
  TILE_LOOP(idx, LB * N, NT) {
    const int c = idx % LB, e = idx / LB;
    const int ky = c0 + c;
    cpx<T> v = mk<T>(0, 0);
    if (ky < Ny) {
      const size_t o = ((size_t)kx * N + e) * Ny + ky;
      if constexpr (UPD) {
        v = update_mode(u, kx, ky, e, o);
        u.phi_new[o] = scale(v, u.store_scale);
        if (kx == 0 && ky == 0 && e == 0) v.x -= u.phi_off;
      } else {
        v = in[o];
      }
    }
    s[e * STR + c] = v;
    if constexpr (NOUT == 2) s[e * STR + LB + c] = deriv(v, dq, wrap_index(e, N));
  }
  __syncthreads();
  fft::run<T, N, NL, S>(s, tw);
  TILE_LOOP(idx, LB * N, NT) {
    const int c = idx % LB, e = idx / LB;
    const int ky = c0 + c;
    if (ky < Ny) {
      const size_t o = ((size_t)kx * N + e) * Ny + ky;
      out0[o] = s[e * STR + c];
      if constexpr (NOUT == 2) out1[o] = s[e * STR + LB + c];
    }
  }
}

// ------------------------------------------------------- z fft + update + z ifft
// One tile (kx, ky in [c0, c0+LB)) of the spectrum after the x and y passes
// of mu: forward z FFT -> mu_hat in shared memory; Model-B update against
// phi_hat (global) for the bulk modes (1 <= kx < Nx/2), phi_hat' stored;
// z inverse FFT of phi_hat' and of i qz phi_hat' -> out0, out1.  Tiles of the
// kx = 0 and kx = Nx/2 planes, whose modes pair with mirror modes in other
// tiles, only store mu_hat; k_zpass<planes_only> finishes them.  With
// kx0 = 1 the grid covers the bulk planes only and the Hermitian planes are
// transformed by k_zpass<planes_only> on a parallel branch.
// NOISE and MACRO fix the noise mode and the macro-step flag at compile time
// (no branches or code for the other cases in the update).
template <typename T, int N, int LB, int NOISE, bool MACRO>
__global__ void __launch_bounds__(N * LB * 2 / 16)
k_zfused(const cpx<T>* __restrict__ muin, cpx<T>* __restrict__ muhat, cpx<T>* __restrict__ out0,
         cpx<T>* __restrict__ out1, T dq, const cpx<T>* __restrict__ twf, const cpx<T>* __restrict__ twi, int Ny,
         UpdateArgs<T> u, int store_mu, int kx0) {
  u.noise = NOISE;
  if (!MACRO) u.nsub = 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  cpx<T>* s = reinterpret_cast<cpx<T>*>(smraw);
  constexpr int NL = 2 * LB;
  constexpr int NT = N * NL / 16, STR = NL + 1;
  const int kx = (int)blockIdx.y + kx0;
  const int c0 = blockIdx.x * LB;
  const bool plane = (kx == 0 || kx == u.Nxh - 1);
  cpx<T>* sph = s + (size_t)N * STR;  // phi_hat tile, [kz][c]
  // two async groups: mu (needed first) and phi_hat (needed after the forward FFT)
  TILE_LOOP(idx, LB * N, NT) {
    const int c = idx % LB, e = idx / LB;
    const int ky = c0 + c;
    if (ky < Ny) cp_async_elem(&s[e * STR + c], &muin[((size_t)kx * N + e) * Ny + ky]);
    else s[e * STR + c] = mk<T>(0, 0);
  }
  cp_async_commit();
  if (!plane) {
    TILE_LOOP(idx, LB * N, NT) {
      const int c = idx % LB, e = idx / LB;
      const int ky = c0 + c;
      if (ky < Ny) cp_async_elem(&sph[e * LB + c], &u.phi_old[((size_t)kx * N + e) * Ny + ky]);
    }
  }
  cp_async_commit();
  cp_async_wait<1>();
  __syncthreads();
  fft::run_sub<T, N, LB, -1, NT, STR>(s, twf);
  if (plane || store_mu) {
    TILE_LOOP(idx, LB * N, NT) {
      const int c = idx % LB, e = idx / LB;
      const int ky = c0 + c;
      if (ky < Ny) muhat[((size_t)kx * N + e) * Ny + ky] = s[e * STR + c];
    }
  }
  if (plane) return;  // uniform per CTA
  cp_async_wait<0>();
  __syncthreads();
  TILE_LOOP(idx, LB * N, NT) {
    const int c = idx % LB, e = idx / LB;
    const int ky = c0 + c;
    cpx<T> v = mk<T>(0, 0);
    if (ky < Ny) {
      const size_t o = ((size_t)kx * N + e) * Ny + ky;
      const cpx<T> ph = scale(sph[e * LB + c], u.phi_scale);
      v = update_value(u, kx, ky, e, ph, s[e * STR + c], false);
      u.phi_new[o] = scale(v, u.store_scale);
    }
    s[e * STR + c] = v;
    s[e * STR + LB + c] = deriv(v, dq, wrap_index(e, N));
  }
  __syncthreads();
  fft::run<T, N, NL, +1>(s, twi);
  TILE_LOOP(idx, LB * N, NT) {
    const int c = idx % LB, e = idx / LB;
    const int ky = c0 + c;
    if (ky < Ny) {
      const size_t o = ((size_t)kx * N + e) * Ny + ky;
      out0[o] = s[e * STR + c];
      out1[o] = s[e * STR + LB + c];
    }
  }
}

// -------------------------------------------------------------------- launchers
// kernel launch (programmatic dependent launch between the passes was
// measured 9% slower per step on GB300 and is not used)
template <typename... KArgs, typename... Args>
static void launch_grid(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  k<<<grid, block, smem, st>>>(args...);
}

// Opt a kernel into more than 48 KB of dynamic shared memory; done once per
// (device, kernel) so that graph capture never sees the attribute call.  The
// attribute belongs to the device that is current when it is set, so a
// process with contexts on two GPUs sets it on each.
template <typename Kern>
static int set_smem(Kern k, size_t bytes) {
  if (bytes <= 48 * 1024) return 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> done;
  std::lock_guard<std::mutex> lock(mu);
  size_t& d = done[std::make_pair(dev, reinterpret_cast<const void*>(k))];
  if (bytes > d) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return -1;
    d = bytes;
  }
  return 0;
}

template <typename T, int N>
struct Axis {
  static constexpr int NLT = lines_for<N>();

  static int xr2c(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* tw, const FHArgs& fh,
                  cudaStream_t st) {
    constexpr int LB = NLT;
    const size_t sm = (size_t)N * (LB + 1) * sizeof(cpx<T>) * (dep ? 2 : 1);
    dim3 grid((g.ny + 2 * LB - 1) / (2 * LB), g.nz);
    if (dep) {
      auto k = k_xr2c<T, N, LB, 1>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3(grid), dim3(N * LB / 16), sm, st, in, dep, out, tw, g.ny, g.nz, fh);
    } else {
      auto k = k_xr2c<T, N, LB, 0>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3(grid), dim3(N * LB / 16), sm, st, in, dep, out, tw, g.ny, g.nz, fh);
    }
    return 0;
  }

  static int xc2r(const Geom& g, const cpx<T>* in, T* out0, T s0, bool mul0, T* out1, T s1, const cpx<T>* tw,
                  const NanArgs& nan, cudaStream_t st) {
    const T dq = (T)g.kq[0];
    if (out1) {
      constexpr int LB = NLT / 2 >= 1 ? NLT / 2 : 1;
      const size_t sm = (size_t)N * (2 * LB + 1) * sizeof(cpx<T>);
      dim3 grid((g.ny + 2 * LB - 1) / (2 * LB), g.nz);
      if (mul0) return -1;
      auto k = k_xc2r<T, N, LB, false, 2>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3(grid), dim3(N * LB * 2 / 16), sm, st, in, out0, out1, s0, s1, dq, tw, g.ny, g.nz, nan);
    } else {
      constexpr int LB = NLT;
      const size_t sm = (size_t)N * (LB + 1) * sizeof(cpx<T>);
      dim3 grid((g.ny + 2 * LB - 1) / (2 * LB), g.nz);
      if (mul0) {
        auto k = k_xc2r<T, N, LB, true, 1>;
        if (set_smem(k, sm)) return -1;
        launch_grid(k, dim3(grid), dim3(N * LB / 16), sm, st, in, out0, out1, s0, s1, dq, tw, g.ny, g.nz, nan);
      } else {
        auto k = k_xc2r<T, N, LB, false, 1>;
        if (set_smem(k, sm)) return -1;
        launch_grid(k, dim3(grid), dim3(N * LB / 16), sm, st, in, out0, out1, s0, s1, dq, tw, g.ny, g.nz, nan);
      }
    }
    return 0;
  }

  template <int S>
  static int ypass(const Geom& g, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw, cudaStream_t st) {
    const long long nlines = (long long)g.nxh * g.nz;
    const T dq = (T)g.kq[1];
    if (out1) {
      constexpr int LB = NLT / 2 >= 1 ? NLT / 2 : 1;
      const size_t sm = (size_t)N * (2 * LB + 1) * sizeof(cpx<T>);
      auto k = k_ypass<T, N, LB, S, 2>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3((unsigned)((nlines + LB - 1) / LB)), dim3(N * LB * 2 / 16), sm, st, in, out0, out1, dq, tw, nlines);
    } else {
      constexpr int LB = NLT;
      const size_t sm = (size_t)N * (LB + 1) * sizeof(cpx<T>);
      auto k = k_ypass<T, N, LB, S, 1>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3((unsigned)((nlines + LB - 1) / LB)), dim3(N * LB / 16), sm, st, in, out0, out1, dq, tw, nlines);
    }
    return 0;
  }

  static int xc2r3(const Geom& g, const cpx<T>* C, T* phi, T* gx, const cpx<T>* D, T* gy, const cpx<T>* E, T* gz,
                   T sp, T sg, const cpx<T>* tw, const NanArgs& nan, const NanArgs& nonan, const uint32_t* gmask,
                   const int* gmask_off, cudaStream_t st) {
    constexpr int LB2 = NLT / 2 >= 1 ? NLT / 2 : 1;
    if (2 * LB2 != NLT) return -3;
    const size_t sm = (size_t)N * (2 * LB2 + 1) * sizeof(cpx<T>) + 4 * (size_t)xc2r_mask_words<T, N, 2 * LB2>();
    const int nb0 = (g.ny + 2 * LB2 - 1) / (2 * LB2), nb1 = (g.ny + 4 * LB2 - 1) / (4 * LB2);
    auto k = k_xc2r3<T, N, LB2>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, dim3(nb0 + 2 * nb1, g.nz), dim3(N * LB2 * 2 / 16), sm, st, C, phi, gx, D, gy, E, gz, sp, sg,
                (T)g.kq[0], tw, g.ny, g.nz, nan, nonan, nb0, nb1, gmask, gmask_off);
    return 0;
  }

  static int yinv2(const Geom& g, const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E,
                   const cpx<T>* tw, cudaStream_t st) {
    constexpr int LB2 = NLT / 2 >= 1 ? NLT / 2 : 1;
    if (2 * LB2 != NLT) return -3;
    const long long nlines = (long long)g.nxh * g.nz;
    const size_t sm = (size_t)N * (2 * LB2 + 1) * sizeof(cpx<T>);
    const long long nb0 = (nlines + LB2 - 1) / LB2, nb1 = (nlines + 2 * LB2 - 1) / (2 * LB2);
    auto k = k_ypass_inv2<T, N, LB2>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, dim3((unsigned)(nb0 + nb1)), dim3(N * LB2 * 2 / 16), sm, st, A, C, D, B, E, (T)g.kq[1], tw,
                nlines, nb0);
    return 0;
  }

  template <int S, bool UPD>
  static int zpass(const Geom& g, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
                   const UpdateArgs<T>& u, cudaStream_t st, int planes_only = 0) {
    const T dq = (T)g.kq[2];
    if (planes_only && u.Nxh != g.nxh) return -1;  // kx of the second plane comes from u.Nxh
    const unsigned gy = planes_only ? 2u : (unsigned)g.nxh;
    if (out1) {
      constexpr int LB = NLT / 2 >= 1 ? NLT / 2 : 1;
      const size_t sm = (size_t)N * (2 * LB + 1) * sizeof(cpx<T>);
      dim3 grid((g.ny + LB - 1) / LB, gy);
      auto k = k_zpass<T, N, LB, S, 2, UPD>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3(grid), dim3(N * LB * 2 / 16), sm, st, in, out0, out1, dq, tw, g.ny, u, planes_only);
    } else {
      constexpr int LB = NLT;
      const size_t sm = (size_t)N * (LB + 1) * sizeof(cpx<T>);
      dim3 grid((g.ny + LB - 1) / LB, gy);
      auto k = k_zpass<T, N, LB, S, 1, UPD>;
      if (set_smem(k, sm)) return -1;
      launch_grid(k, dim3(grid), dim3(N * LB / 16), sm, st, in, out0, out1, dq, tw, g.ny, u, planes_only);
    }
    return 0;
  }

  static int zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1,
                    const cpx<T>* twf, const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only,
                    cudaStream_t st) {
    // columns per tile: for N >= 512 a full NLT (64-byte row segments of the
    // strided z columns instead of 32-byte ones)
    constexpr int LB = N >= 512 ? NLT : (NLT / 2 >= 1 ? NLT / 2 : 1);
    const size_t sm = (size_t)N * (3 * LB + 1) * sizeof(cpx<T>);
    const int kx0 = bulk_only ? 1 : 0;
    if (g.nxh - 2 * kx0 <= 0) return 0;
    dim3 grid((g.ny + LB - 1) / LB, g.nxh - 2 * kx0);
    const bool macro = u.nsub > 1;
#define ZF(NZ, M) zfused_go<LB, NZ, M>(grid, sm, muin, muhat, out0, out1, (T)g.kq[2], twf, twi, g.ny, u, store_mu, kx0, st)
    switch (u.noise) {
      case PHAFD_NOISE_OFF: return macro ? ZF(PHAFD_NOISE_OFF, true) : ZF(PHAFD_NOISE_OFF, false);
      case PHAFD_NOISE_REFERENCE: return macro ? ZF(PHAFD_NOISE_REFERENCE, true) : ZF(PHAFD_NOISE_REFERENCE, false);
      default: return macro ? ZF(PHAFD_NOISE_PHILOX, true) : ZF(PHAFD_NOISE_PHILOX, false);
    }
#undef ZF
  }
  template <int LB, int NOISE, bool MACRO>
  static int zfused_go(dim3 grid, size_t sm, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1, T dq,
                       const cpx<T>* twf, const cpx<T>* twi, int ny, const UpdateArgs<T>& u, int store_mu, int kx0,
                       cudaStream_t st) {
    auto k = k_zfused<T, N, LB, NOISE, MACRO>;
    if (set_smem(k, sm)) return -1;
    launch_grid(k, dim3(grid), dim3(N * LB * 2 / 16), sm, st, muin, muhat, out0, out1, dq, twf, twi, ny, u, store_mu,
                kx0);
    return 0;
  }
};

#define PHAFD_FOR_SIZES(M) M(16) M(32) M(64) M(96) M(128) M(160) M(256) M(512)

namespace r256 {
template <typename T>
int xr2c(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* tw, const FHArgs& fh,
         cudaStream_t st);
template <typename T>
int xc2r3(const Geom& g, const cpx<T>* C, T* phi, T* gx, const cpx<T>* D, T* gy, const cpx<T>* E, T* gz, T sp,
          T sg, const cpx<T>* tw, const NanArgs& nan, const NanArgs& nonan, const uint32_t* gmask,
          const int* gmask_off, int* status, cudaStream_t st);
template <typename T>
int ypass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw, cudaStream_t st);
template <typename T>
int yinv2(const Geom& g, const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E, const cpx<T>* tw,
          cudaStream_t st);
template <typename T>
int zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1, const cpx<T>* twf,
           const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only, cudaStream_t st);
}

template <typename T>
int GridOps<T>::xr2c(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* tw, const FHArgs& fh,
                     cudaStream_t st) {
  if (g.nx == 256 && !g.generic256) return r256::xr2c<T>(g, in, dep, out, tw, fh, st);
  switch (g.nx) {
#define CASE(n) case n: return Axis<T, n>::xr2c(g, in, dep, out, tw, fh, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

template <typename T>
int GridOps<T>::xc2r(const Geom& g, const cpx<T>* in, T* out0, T s0, bool mul0, T* out1, T s1, const cpx<T>* tw,
                     const NanArgs& nan, cudaStream_t st) {
  switch (g.nx) {
#define CASE(n) case n: return Axis<T, n>::xc2r(g, in, out0, s0, mul0, out1, s1, tw, nan, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}


template <typename T>
int GridOps<T>::xc2r3(const Geom& g, const cpx<T>* C, T* phi, T* gx, const cpx<T>* D, T* gy, const cpx<T>* E,
                      T* gz, T sp, T sg, const cpx<T>* tw, const NanArgs& nan, const NanArgs& nonan,
                      const uint32_t* gmask, const int* gmask_off, int* status, cudaStream_t st) {
  if (g.nx == 256 && !g.generic256)
    return r256::xc2r3<T>(g, C, phi, gx, D, gy, E, gz, sp, sg, tw, nan, nonan, gmask, gmask_off, status, st);
  switch (g.nx) {
#define CASE(n) \
  case n: return Axis<T, n>::xc2r3(g, C, phi, gx, D, gy, E, gz, sp, sg, tw, nan, nonan, gmask, gmask_off, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}


template <typename T>
int GridOps<T>::yinv2(const Geom& g, const cpx<T>* A, cpx<T>* C, cpx<T>* D, const cpx<T>* B, cpx<T>* E,
                      const cpx<T>* tw, cudaStream_t st) {
  if (g.ny == 256 && !g.generic256) return r256::yinv2<T>(g, A, C, D, B, E, tw, st);
  switch (g.ny) {
#define CASE(n) case n: return Axis<T, n>::yinv2(g, A, C, D, B, E, tw, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

template <typename T>
int GridOps<T>::ypass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
                      cudaStream_t st) {
  if (g.ny == 256 && !g.generic256) return r256::ypass<T>(g, sign, in, out0, out1, tw, st);
  switch (g.ny) {
#define CASE(n)                                                                   \
  case n:                                                                         \
    return sign < 0 ? Axis<T, n>::template ypass<-1>(g, in, out0, out1, tw, st)   \
                    : Axis<T, n>::template ypass<+1>(g, in, out0, out1, tw, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}


template <typename T>
int GridOps<T>::zfused(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, cpx<T>* out0, cpx<T>* out1,
                       const cpx<T>* twf, const cpx<T>* twi, const UpdateArgs<T>& u, int store_mu, int bulk_only,
                       cudaStream_t st) {
  if (g.nz == 256 && !g.generic256) return r256::zfused<T>(g, muin, muhat, out0, out1, twf, twi, u, store_mu, bulk_only, st);
  switch (g.nz) {
#define CASE(n) case n: return Axis<T, n>::zfused(g, muin, muhat, out0, out1, twf, twi, u, store_mu, bulk_only, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

template <typename T>
int GridOps<T>::zpass_planes(const Geom& g, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw, const UpdateArgs<T>& u,
                             cudaStream_t st) {
  switch (g.nz) {
#define CASE(n) case n: return Axis<T, n>::template zpass<+1, true>(g, nullptr, out0, out1, tw, u, st, 1);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

template <typename T>
int GridOps<T>::zfwd_planes(const Geom& g, const cpx<T>* muin, cpx<T>* muhat, const cpx<T>* tw, cudaStream_t st) {
  UpdateArgs<T> none{};
  none.Ny = g.ny; none.Nz = g.nz; none.Nxh = g.nxh;  // the plane kernel takes kx = Nx/2 from Nxh
  switch (g.nz) {
#define CASE(n) case n: return Axis<T, n>::template zpass<-1, false>(g, muin, muhat, nullptr, tw, none, st, 1);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

template <typename T>
int GridOps<T>::zpass(const Geom& g, int sign, const cpx<T>* in, cpx<T>* out0, cpx<T>* out1, const cpx<T>* tw,
                      const UpdateArgs<T>* u, cudaStream_t st) {
  UpdateArgs<T> dummy{};
  switch (g.nz) {
#define CASE(n)                                                                                   \
  case n:                                                                                         \
    if (u) return Axis<T, n>::template zpass<+1, true>(g, in, out0, out1, tw, *u, st);            \
    return sign < 0 ? Axis<T, n>::template zpass<-1, false>(g, in, out0, out1, tw, dummy, st)     \
                    : Axis<T, n>::template zpass<+1, false>(g, in, out0, out1, tw, dummy, st);
    PHAFD_FOR_SIZES(CASE)
#undef CASE
  }
  return -2;
}

}  // namespace phafd
