// Shared-memory batched FFT core.
//
// A CTA transforms NL lines of length N held in shared memory in an
// element-major, line-minor layout: element e of line l lives at
// s[e * (NL + 1) + l].  The +1 pad keeps a warp's 8- or 16-byte accesses on
// distinct banks for both the loads from global memory and the butterflies.
//
// The transform is a mixed-radix Stockham autosort (no bit reversal): for
// stage radices R_1 R_2 ... (16, then 8/4/2, then 3 or 5) with NS the product
// of the radices already applied, butterfly j of a line reads elements
// j + r*N/R, multiplies by W_{NS*R}^{(j mod NS) r}, takes a length-R DFT in
// registers and writes elements (j/NS)*NS*R + (j mod NS) + r*NS.
//
// The CTA runs N*NL/16 threads, so each thread owns 16 complex values per
// stage (one radix-16 butterfly, two radix-8 ones, ...).  All reads of a
// stage complete before a barrier and all writes follow it, so the transform
// is in place.  Twiddles W_N^m come from a table built on the host in double
// precision (std::cos / std::sin), read through the read-only cache.
#pragma once
#include "common.cuh"

namespace fft {

__host__ __device__ constexpr int pick(int m) {
  return (m % 16 == 0) ? 16 : (m % 8 == 0) ? 8 : (m % 4 == 0) ? 4 : (m % 2 == 0) ? 2 : (m % 3 == 0) ? 3 : (m % 5 == 0) ? 5 : 1;
}
__host__ __device__ constexpr bool supported(int n) {
  int m = n;
  while (m > 1) {
    int r = pick(m);
    if (r == 1) return false;
    m /= r;
  }
  return n % 16 == 0;
}

// ---- length-R DFTs in registers; S = -1 forward, +1 backward
template <int S, typename T>
PHAFD_D void dft2(cpx<T>& a, cpx<T>& b) {
  cpx<T> t = a;
  a = t + b;
  b = t - b;
}

template <int S, typename T>
PHAFD_D void dft4(cpx<T>* v) {
  cpx<T> t0 = v[0] + v[2], t1 = v[0] - v[2];
  cpx<T> t2 = v[1] + v[3], t3 = mul_i<S>(v[1] - v[3]);
  v[0] = t0 + t2;
  v[2] = t0 - t2;
  v[1] = t1 + t3;
  v[3] = t1 - t3;
}

template <int S, typename T>
PHAFD_D void dft8(cpx<T>* v) {
  const T c = (T)0.70710678118654752440;
  cpx<T> e[4] = {v[0], v[2], v[4], v[6]};
  cpx<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<S>(e);
  dft4<S>(o);
  // W8^k = exp(S i pi k / 4)
  cpx<T> w1 = mk<T>(c * (o[1].x - S * o[1].y), c * (o[1].y + S * o[1].x));   // (1 + S i) c
  cpx<T> w2 = mul_i<S>(o[2]);
  cpx<T> w3 = mk<T>(c * (-o[3].x - S * o[3].y), c * (-o[3].y + S * o[3].x)); // (-1 + S i) c
  v[0] = e[0] + o[0]; v[4] = e[0] - o[0];
  v[1] = e[1] + w1;   v[5] = e[1] - w1;
  v[2] = e[2] + w2;   v[6] = e[2] - w2;
  v[3] = e[3] + w3;   v[7] = e[3] - w3;
}

template <int S, typename T>
PHAFD_D void dft16(cpx<T>* v) {
  const T c1 = (T)0.92387953251128675613, s1 = (T)0.38268343236508977173;
  const T c2 = (T)0.70710678118654752440;
  cpx<T> e[8], o[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) { e[k] = v[2 * k]; o[k] = v[2 * k + 1]; }
  dft8<S>(e);
  dft8<S>(o);
  // W16^k = (cos(pi k/8), S sin(pi k/8))
  const cpx<T> w[8] = {mk<T>(1, 0), mk<T>(c1, S * s1), mk<T>(c2, S * c2), mk<T>(s1, S * c1),
                       mk<T>(0, (T)S), mk<T>(-s1, S * c1), mk<T>(-c2, S * c2), mk<T>(-c1, S * s1)};
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    cpx<T> t = (k == 0) ? o[0] : o[k] * w[k];
    v[k] = e[k] + t;
    v[k + 8] = e[k] - t;
  }
}

template <int S, typename T>
PHAFD_D void dft3(cpx<T>* v) {
  const T h = (T)0.86602540378443864676;  // sin(2 pi / 3)
  cpx<T> t = v[1] + v[2], d = v[1] - v[2];
  cpx<T> m = v[0] - scale(t, (T)0.5);
  cpx<T> r = mul_i<S>(scale(d, h));
  v[0] = v[0] + t;
  v[1] = m + r;
  v[2] = m - r;
}

template <int S, typename T>
PHAFD_D void dft5(cpx<T>* v) {
  const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
  const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
  cpx<T> t1 = v[1] + v[4], t2 = v[2] + v[3], d1 = v[1] - v[4], d2 = v[2] - v[3];
  cpx<T> m1 = v[0] + scale(t1, c1) + scale(t2, c2);
  cpx<T> m2 = v[0] + scale(t1, c2) + scale(t2, c1);
  cpx<T> n1 = mul_i<S>(scale(d1, s1) + scale(d2, s2));
  cpx<T> n2 = mul_i<S>(scale(d1, s2) - scale(d2, s1));
  v[0] = v[0] + t1 + t2;
  v[1] = m1 + n1;
  v[4] = m1 - n1;
  v[2] = m2 + n2;
  v[3] = m2 - n2;
}

template <int R, int S, typename T>
PHAFD_D void dft(cpx<T>* v) {
  if constexpr (R == 2) dft2<S>(v[0], v[1]);
  else if constexpr (R == 4) dft4<S>(v);
  else if constexpr (R == 8) dft8<S>(v);
  else if constexpr (R == 16) dft16<S>(v);
  else if constexpr (R == 3) dft3<S>(v);
  else if constexpr (R == 5) dft5<S>(v);
}

// One Stockham stage, then recurse on the rest.  tw = W_N^m table for sign S.
// Transforms lines [0, NL) of a buffer with row stride STR using NT threads.
template <typename T, int N, int NL, int S, int NS, int NT, int STR>
PHAFD_D void stages(cpx<T>* s, const cpx<T>* __restrict__ tw) {
  if constexpr (NS < N) {
    constexpr int R = pick(N / NS);
    constexpr int NB = N / R;                   // butterflies per line
    constexpr int TOT = NB * NL;                // butterflies in the CTA
    constexpr int PER = (TOT + NT - 1) / NT;    // butterflies per thread
    constexpr int TWS = N / (NS * R);
    cpx<T> v[PER][R];
    const int tid = threadIdx.x;
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = tid + p * NT;
      if (TOT % NT == 0 || b < TOT) {
        const int l = b % NL, j = b / NL;
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][r] = s[(j + r * NB) * STR + l];
      }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = tid + p * NT;
      if (TOT % NT == 0 || b < TOT) {
        const int l = b % NL, j = b / NL;
        const int k = j % NS;
        if constexpr (NS > 1) {
#pragma unroll
          for (int r = 1; r < R; ++r) v[p][r] = v[p][r] * tw[k * r * TWS];
        }
        dft<R, S>(v[p]);
        const int idxD = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) s[(idxD + r * NS) * STR + l] = v[p][r];
      }
    }
    __syncthreads();
    stages<T, N, NL, S, NS * R, NT, STR>(s, tw);
  }
}

// Transform all NL lines in s (layout above) with N*NL/16 threads.  Caller syncs before.
template <typename T, int N, int NL, int S>
PHAFD_D void run(cpx<T>* s, const cpx<T>* __restrict__ tw) {
  stages<T, N, NL, S, 1, N * NL / 16, NL + 1>(s, tw);
}

// Transform lines [0, NL) of a buffer with row stride STR using NT threads.
template <typename T, int N, int NL, int S, int NT, int STR>
PHAFD_D void run_sub(cpx<T>* s, const cpx<T>* __restrict__ tw) {
  stages<T, N, NL, S, 1, NT, STR>(s, tw);
}

template <int N, int NL>
__host__ __device__ constexpr int threads() { return N * NL / 16; }

}  // namespace fft
