// Device-side helpers shared by the grid and bead kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define PHAFD_HD __host__ __device__ __forceinline__
#define PHAFD_D __device__ __forceinline__

template <typename T>
struct alignas(2 * sizeof(T)) cpx {
  T x, y;
};

template <typename T> PHAFD_HD cpx<T> mk(T a, T b) { cpx<T> r; r.x = a; r.y = b; return r; }
template <typename T> PHAFD_HD cpx<T> operator+(cpx<T> a, cpx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> PHAFD_HD cpx<T> operator-(cpx<T> a, cpx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> PHAFD_HD cpx<T> operator*(cpx<T> a, cpx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T> PHAFD_HD cpx<T> scale(cpx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> PHAFD_HD cpx<T> conjg(cpx<T> a) { return mk<T>(a.x, -a.y); }
// multiply by +i (S=+1) or -i (S=-1)
template <int S, typename T> PHAFD_HD cpx<T> mul_i(cpx<T> a) {
  return S > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11).  Identical bits to the oracle's host version.
PHAFD_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}
PHAFD_HD double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Field noise of the canonical mode (kx, ky, kz) at `step`: the oracle's
// philox_u.  One Philox4x32-10 call serves the mode pair (kz, kz ^ 16):
// words (c0, c1) for the mode with bit 4 of kz clear, (c2, c3) for the other;
// each word gives a 24-bit uniform in [-0.5, 0.5), exact in float and double.
PHAFD_D void field_noise_words(int kx, int ky, int kz, int Ny, int Nz, uint32_t step, uint32_t seed, uint32_t c[4]) {
  const uint64_t idx = ((uint64_t)kx * Nz + (kz & ~16)) * Ny + ky;
  c[0] = (uint32_t)idx; c[1] = (uint32_t)(idx >> 32); c[2] = step; c[3] = 0x46494c44u;
  philox4x32_10(c, seed, 0x434f4e4au);
}
template <typename T>
PHAFD_D T noise_u24(uint32_t w) {
  return (T)(w >> 8) * (T)5.9604644775390625e-8 - (T)0.5;
}
// the two uniforms of mode kz from the words of its pair
template <typename T>
PHAFD_D void field_noise_pair(const uint32_t c[4], int kz, T& u0, T& u1) {
  const int s = (kz >> 4) & 1;
  u0 = noise_u24<T>(c[2 * s]);
  u1 = noise_u24<T>(c[2 * s + 1]);
}

// Three standard normals for bead `bead`, half-step `half` of `step`
// (Box-Muller on Philox words): the oracle's oracle_bead_gauss.  The float
// version uses the top 24 bits of the same uniforms.
PHAFD_D void bead_gauss(uint32_t seed, uint64_t step, int half, int bead, double xi[3]) {
  double g[4];
#pragma unroll
  for (int call = 0; call < 2; ++call) {
    uint32_t c[4] = {(uint32_t)bead, (uint32_t)step, (uint32_t)(step >> 32) * 2u + (uint32_t)half,
                     0x4245414Du + (uint32_t)call};
    philox4x32_10(c, seed, 0x53454d49u);
    const double u1 = u53(c[0], c[1]), u2 = u53(c[2], c[3]);
    const double r = sqrt(-2.0 * log(1.0 - u1));
    double s, co;
    sincos(6.283185307179586 * u2, &s, &co);
    g[2 * call] = r * co;
    g[2 * call + 1] = r * s;
  }
  xi[0] = g[0]; xi[1] = g[1]; xi[2] = g[2];
}
PHAFD_D void bead_gauss(uint32_t seed, uint64_t step, int half, int bead, float xi[3]) {
  float g[4];
#pragma unroll
  for (int call = 0; call < 2; ++call) {
    uint32_t c[4] = {(uint32_t)bead, (uint32_t)step, (uint32_t)(step >> 32) * 2u + (uint32_t)half,
                     0x4245414Du + (uint32_t)call};
    philox4x32_10(c, seed, 0x53454d49u);
    const float u1 = (float)(c[0] >> 8) * 5.9604644775390625e-8f;
    const float u2 = (float)(c[2] >> 8) * 5.9604644775390625e-8f;
    const float r = sqrtf(-2.0f * logf(1.0f - u1));
    float s, co;
    sincosf(6.2831853f * u2, &s, &co);
    g[2 * call] = r * co;
    g[2 * call + 1] = r * s;
  }
  xi[0] = g[0]; xi[1] = g[1]; xi[2] = g[2];
}

// Asynchronous global -> shared copies (cp.async): issued without staging
// through registers, so a thread can have its whole share of a tile in
// flight at once.  commit() closes a group, wait<n>() waits until at most n
// groups are pending.
PHAFD_D void cp_async4(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
PHAFD_D void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
PHAFD_D void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
PHAFD_D void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
PHAFD_D void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
template <typename T>
PHAFD_D void cp_async_elem(cpx<T>* smem, const cpx<T>* gmem) {
  if constexpr (sizeof(T) == 4) cp_async8(smem, gmem);
  else cp_async16(smem, gmem);
}
template <typename T>
PHAFD_D void cp_async_real(T* smem, const T* gmem) {
  if constexpr (sizeof(T) == 4) cp_async4(smem, gmem);
  else cp_async8(smem, gmem);
}

// signed wavenumber index, reference convention (fixgrid_conjugate.cpp:80-95):
// index e of N maps to e if e <= N/2, else e - N
PHAFD_HD int wrap_index(int e, int N) { return e > N / 2 ? e - N : e; }

// device status words
enum : int {
  ST_OVERFLOW = 1,
  ST_CONSTRAINT = 2,
  ST_BINRANGE = 4,
  ST_TIMEOUT = 8,  // a bounded wait of a grid pass gave up
};
