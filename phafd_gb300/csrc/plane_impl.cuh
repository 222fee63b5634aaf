// Plane-fused FFT passes: the x and y transforms of one z-plane in one
// thread-block cluster, exchanging the plane through distributed shared
// memory instead of HBM.
//
// A z-plane of the spectrum holds (Nx/2+1) x Ny complex values (264 KB at
// 256^2 in FP32), more than one CTA's shared memory, so CL CTAs of a cluster
// split it:
//   xy_fwd : phase 1, CTA r takes rows y in [r*RPC, (r+1)*RPC): Flory-Huggins
//            mu (or plain phi) on load, x r2c of row pairs, result kept in its
//            shared memory as P[kx][row]; cluster barrier; phase 2, CTA r takes
//            kx in [r*KPC, (r+1)*KPC), gathers the full y lines of those kx
//            from all CTAs (DSMEM), y FFT, writes M[kx][z][ky].
//   yx_inv : the reverse: phase 1 y ifft of kx lines (optionally times
//            i q_y), phase 2 gather of row pairs, x c2r to one or two real
//            outputs (plain and i q_x).
// This removes the HBM round trip between the x and y passes of both
// directions.  Used when Nx == Ny and the tiles fit; otherwise the separate
// passes run.
#pragma once
#include <cooperative_groups.h>

#include <algorithm>

#include "grid_impl.cuh"

namespace phafd {
namespace cg = cooperative_groups;

__host__ __device__ constexpr int odd_up(int n) { return (n & 1) ? n : n + 1; }

template <int N>
struct PlaneCfg {
  static constexpr int NXH = N / 2 + 1;
  static constexpr int CL = N <= 32 ? 1 : (N <= 64 ? 2 : (N <= 128 ? 4 : (N <= 256 ? 8 : 16)));
  static constexpr int KPC = (NXH + CL - 1) / CL;  // kx lines per CTA
  static constexpr int RPC = N / CL;               // rows per CTA
  static constexpr int PPC = RPC / 2;              // row pairs per CTA
  static constexpr int NT = 256;
};

// ------------------------------------------------------------ y ifft + x c2r
template <typename T, int N, bool YMUL, int NJOB>
__global__ void __launch_bounds__(256)
k_yx_inv(const cpx<T>* __restrict__ in, T* __restrict__ out0, T s0, T* __restrict__ out1, T s1, T dqx, T dqy,
         const cpx<T>* __restrict__ twy, const cpx<T>* __restrict__ twx, int Nz, NanArgs nan) {
  using C = PlaneCfg<N>;
  constexpr int NXH = C::NXH, KPC = C::KPC, RPC = C::RPC, PPC = C::PPC, NT = C::NT;
  constexpr int STR1 = odd_up(KPC);
  constexpr int NL2 = PPC * NJOB, STR2 = odd_up(NL2);
  constexpr int CH = RPC * STR1;  // one CTA's rows [y0, y0+RPC) of sy: contiguous
  extern __shared__ __align__(16) unsigned char smraw[];
  // [stage: CL chunks][sy: N x STR1], s2 aliases sy once every remote read is done
  cpx<T>* stage = reinterpret_cast<cpx<T>*>(smraw);
  cpx<T>* sy = stage + (size_t)C::CL * CH;
  cpx<T>* s2 = sy;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int z = blockIdx.y;
  const int k0 = r * KPC;
  // phase 1: y ifft of the kx lines [k0, k0 + KPC)
  TILE_LOOP(idx, KPC * N, NT) {
    const int l = idx / N, e = idx % N;
    const int kx = k0 + l;
    cpx<T> v = mk<T>(0, 0);
    if (kx < NXH) {
      v = in[((size_t)kx * Nz + z) * N + e];
      if constexpr (YMUL) v = deriv(v, dqy, wrap_index(e, N));
    }
    sy[e * STR1 + l] = v;
  }
  __syncthreads();
  fft::run_sub<T, N, KPC, +1, NT, STR1>(sy, twy);
  cluster.sync();
  // phase 2: copy rows [y0, y0+RPC) of every CTA's sy (one contiguous chunk
  // each) into the local stage with 16-byte DSMEM loads
  const int y0 = r * RPC;
  constexpr int CHV = CH * (int)sizeof(cpx<T>) / 16;
  static_assert((CH * sizeof(cpx<T>)) % 16 == 0, "chunk must be whole 16-byte words");
  TILE_LOOP(w, C::CL * CHV, NT) {
    const int q = w / CHV, o = w % CHV;
    const uint4* src = reinterpret_cast<const uint4*>(cluster.map_shared_rank(sy, q) + (size_t)y0 * STR1) + o;
    reinterpret_cast<uint4*>(stage + (size_t)q * CH)[o] = *src;
  }
  cluster.sync();  // every remote read done: sy may be overwritten, CTAs may exit
  TILE_LOOP(idx, PPC * NXH, NT) {
    const int p = idx % PPC, k = idx / PPC;
    const cpx<T>* ch = stage + (size_t)(k / KPC) * CH + (k % KPC);
    const cpx<T> A = ch[(2 * p) * STR1];
    const cpx<T> B = ch[(2 * p + 1) * STR1];
#pragma unroll
    for (int j = 0; j < NJOB; ++j) {
      cpx<T> a = A, b = B;
      if (j == 1) { a = deriv(a, dqx, k); b = deriv(b, dqx, k); }
      if (k == 0 || k == N / 2) { a.y = (T)0; b.y = (T)0; }
      s2[k * STR2 + j * PPC + p] = mk<T>(a.x - b.y, a.y + b.x);
      if (k > 0 && k < N / 2) s2[(N - k) * STR2 + j * PPC + p] = mk<T>(a.x + b.y, b.x - a.y);
    }
  }
  __syncthreads();
  fft::run_sub<T, N, NL2, +1, NT, STR2>(s2, twx);
  TILE_LOOP(idx, PPC * N, NT) {
    const int x = idx % N, p = idx / N;
#pragma unroll
    for (int j = 0; j < NJOB; ++j) {
      const cpx<T> v = s2[x * STR2 + j * PPC + p];
      T* out = j == 0 ? out0 : out1;
      const T sc = j == 0 ? s0 : s1;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int y = y0 + 2 * p + h;
        const T val = (h == 0 ? v.x : v.y) * sc + (j == 0 ? (T)nan.offset : (T)0);
        out[((size_t)z * N + y) * N + x] = val;
        if (j == 0 && nan.check && z == 0 && y == 0 && x == 0 && isnan(val))
          atomicCAS(reinterpret_cast<unsigned long long*>(nan.nan_step), (unsigned long long)-1LL,
                    (unsigned long long)(*nan.d_step));
      }
    }
  }
}

// ------------------------------------------------------------ x r2c + y fft
// PRO = 1: mu = deposit + FH(phi) on load (fixgrid_floryhuggins.cpp:72-82)
template <typename T, int N, int PRO>
__global__ void __launch_bounds__(256)
k_xy_fwd(const T* __restrict__ in0, const T* __restrict__ dep, cpx<T>* __restrict__ out,
         const cpx<T>* __restrict__ twx, const cpx<T>* __restrict__ twy, int Nz, FHArgs fh) {
  using C = PlaneCfg<N>;
  constexpr int NXH = C::NXH, KPC = C::KPC, RPC = C::RPC, PPC = C::PPC, NT = C::NT;
  constexpr int STRF = odd_up(PPC);   // x-FFT buffer: N (x) x PPC lines
  constexpr int STRP = RPC + 2;       // P buffer rows (kx) of RPC values; even so that chunks are 16-byte words
  constexpr int STR2 = odd_up(KPC);   // y-FFT buffer: N (y) x KPC lines
  constexpr int CH = KPC * STRP;      // one destination's kx rows of one source CTA's P: contiguous
  constexpr int RS = (C::CL * CH > N * STRF) ? C::CL * CH : N * STRF;  // sf, later the stage
  extern __shared__ __align__(16) unsigned char smraw[];
  // [sp: CL*KPC rows x STRP][sf / stage]; s2 aliases sp once every remote read is done
  cpx<T>* sp = reinterpret_cast<cpx<T>*>(smraw);
  cpx<T>* sf = sp + (size_t)C::CL * CH;
  cpx<T>* stage = sf;
  cpx<T>* s2 = sp;
  static_assert((size_t)N * STR2 <= (size_t)C::CL * CH, "s2 must fit in the P buffer");
  static_assert((CH * sizeof(cpx<T>)) % 16 == 0, "chunk must be whole 16-byte words");
  (void)RS;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int z = blockIdx.y;
  const int y0 = r * RPC;
  unsigned long long nless = 0, ngreat = 0;
  // phase 1: rows [y0, y0 + RPC) as PPC complex lines (row pairs)
  TILE_LOOP(idx, PPC * N, NT) {
    const int p = idx / N, x = idx % N;
    T v[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const size_t o = ((size_t)z * N + y0 + 2 * p + h) * N + x;
      T q = in0[o];
      if constexpr (PRO == 1) {
        T keep;
        q = fh_node(q, dep[o], fh, nless, ngreat, &keep);
        if (fh.mu_out) reinterpret_cast<T*>(fh.mu_out)[o] = keep;
      } else {
        if (fh.centered) q -= (T)fh.c;  // transform phi - c
      }
      v[h] = q;
    }
    sf[x * STRF + p] = mk<T>(v[0], v[1]);
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
  fft::run_sub<T, N, PPC, -1, NT, STRF>(sf, twx);
  TILE_LOOP(idx, PPC * NXH, NT) {
    const int p = idx % PPC, k = idx / PPC;
    const cpx<T> zk = sf[k * STRF + p];
    const cpx<T> zm = conjg(sf[((N - k) % N) * STRF + p]);
    const cpx<T> d = zk - zm;
    sp[k * STRP + 2 * p] = scale(zk + zm, (T)0.5);
    sp[k * STRP + 2 * p + 1] = mk<T>((T)0.5 * d.y, (T)-0.5 * d.x);
  }
  cluster.sync();
  // phase 2: copy the kx rows [k0, k0+KPC) of every CTA's P (one contiguous
  // chunk each) into the local stage with 16-byte DSMEM loads
  const int k0 = r * KPC;
  constexpr int CHV = CH * (int)sizeof(cpx<T>) / 16;
  TILE_LOOP(w, C::CL * CHV, NT) {
    const int q = w / CHV, o = w % CHV;
    const uint4* src = reinterpret_cast<const uint4*>(cluster.map_shared_rank(sp, q) + (size_t)k0 * STRP) + o;
    reinterpret_cast<uint4*>(stage + (size_t)q * CH)[o] = *src;
  }
  cluster.sync();  // every remote read done: sp may be overwritten, CTAs may exit
  TILE_LOOP(idx, KPC * N, NT) {
    const int l = idx % KPC, y = idx / KPC;
    s2[y * STR2 + l] = stage[(size_t)(y / RPC) * CH + l * STRP + (y % RPC)];
  }
  __syncthreads();
  fft::run_sub<T, N, KPC, -1, NT, STR2>(s2, twy);
  TILE_LOOP(idx, KPC * N, NT) {
    const int l = idx / N, e = idx % N;
    const int kx = k0 + l;
    if (kx < NXH) out[((size_t)kx * Nz + z) * N + e] = s2[e * STR2 + l];
  }
}

template <typename T, int N>
struct Plane {
  using C = PlaneCfg<N>;
  static size_t smem_inv(int njob) {
    const size_t str1 = odd_up(C::KPC), str2 = odd_up(C::PPC * njob);
    const size_t stage = (size_t)C::CL * C::RPC * str1;
    return (stage + std::max((size_t)N * str1, (size_t)N * str2)) * sizeof(cpx<T>);
  }
  static size_t smem_fwd() {
    const size_t ch = (size_t)C::KPC * (C::RPC + 2);
    const size_t sp = (size_t)C::CL * ch;
    const size_t rs = std::max((size_t)C::CL * ch, (size_t)N * odd_up(C::PPC));
    return (sp + rs) * sizeof(cpx<T>);
  }
  template <typename Kern, typename... Args>
  static int launch(Kern k, size_t sm, int nz, cudaStream_t st, Args... args) {
    if (sm > 227 * 1024) return -3;
    // the attributes belong to the current device: set once per (device, kernel)
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, int> done;
    {
      std::lock_guard<std::mutex> lock(mu);
      int& d = done[std::make_pair(dev, reinterpret_cast<const void*>(k))];
      if (!d) {
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return -1;
        if (C::CL > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
          return -3;
        d = 1;
      }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(C::CL, nz, 1);
    cfg.blockDim = dim3(C::NT, 1, 1);
    cfg.dynamicSmemBytes = sm;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C::CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k, args...) != cudaSuccess) {
      (void)cudaGetLastError();  // cluster shape not schedulable: the caller runs the separate passes
      return -3;
    }
    return 0;
  }
  static int inv(const Geom& g, const cpx<T>* in, T* out0, T s0, bool ymul, T* out1, T s1, const cpx<T>* twy,
                 const cpx<T>* twx, const NanArgs& nan, cudaStream_t st) {
    const T dqx = (T)g.kq[0], dqy = (T)g.kq[1];
    if (out1) {
      if (ymul) return -3;
      return launch(k_yx_inv<T, N, false, 2>, smem_inv(2), g.nz, st, in, out0, s0, out1, s1, dqx, dqy, twy, twx,
                    g.nz, nan);
    }
    if (ymul)
      return launch(k_yx_inv<T, N, true, 1>, smem_inv(1), g.nz, st, in, out0, s0, out1, s1, dqx, dqy, twy, twx,
                    g.nz, nan);
    return launch(k_yx_inv<T, N, false, 1>, smem_inv(1), g.nz, st, in, out0, s0, out1, s1, dqx, dqy, twy, twx, g.nz,
                  nan);
  }
  static int fwd(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* twx, const cpx<T>* twy,
                 const FHArgs& fh, cudaStream_t st) {
    if (dep) return launch(k_xy_fwd<T, N, 1>, smem_fwd(), g.nz, st, in, dep, out, twx, twy, g.nz, fh);
    return launch(k_xy_fwd<T, N, 0>, smem_fwd(), g.nz, st, in, dep, out, twx, twy, g.nz, fh);
  }
};

#define PHAFD_PLANE_SIZES(M) M(64) M(128) M(256) M(512)

template <typename T>
int GridOps<T>::yx_inv(const Geom& g, const cpx<T>* in, T* out0, T s0, bool ymul, T* out1, T s1,
                       const cpx<T>* twy, const cpx<T>* twx, const NanArgs& nan, cudaStream_t st) {
  if (g.nx != g.ny) return -3;
  switch (g.nx) {
#define CASE(n) case n: return Plane<T, n>::inv(g, in, out0, s0, ymul, out1, s1, twy, twx, nan, st);
    PHAFD_PLANE_SIZES(CASE)
#undef CASE
  }
  return -3;
}

template <typename T>
int GridOps<T>::xy_fwd(const Geom& g, const T* in, const T* dep, cpx<T>* out, const cpx<T>* twx,
                       const cpx<T>* twy, const FHArgs& fh, cudaStream_t st) {
  if (g.nx != g.ny) return -3;
  switch (g.nx) {
#define CASE(n) case n: return Plane<T, n>::fwd(g, in, dep, out, twx, twy, fh, st);
    PHAFD_PLANE_SIZES(CASE)
#undef CASE
  }
  return -3;
}

}  // namespace phafd
