// Bead-side kernels of the particle-field step.
//
// One periodic domain on one GPU replaces the reference's gathered LOCAL and
// GHOST copies (comm_brick.cpp:263-426): a periodic image of bead j is
// x_j + s*L with s in {-1, 0, 1} per axis, computed exactly as the reference
// computes a ghost coordinate (atom.cpp pack_comm: x + pbc), so distances and
// cutoff tests see the same bits.  With the rank-1 z mode, images across z
// are skipped, as borders() on one MPI rank never creates them.
//
// Neighbor rebuilds run on the device every step and exit at once unless the
// skin trigger fired (neighbor.cpp:70-97): the step is a fixed launch
// sequence that a CUDA graph can replay.
//
// Lists
//   bead list : full list, nbr[i*maxnb + k] = (j << 5) | image code
//   grid list : per bead, gl[i*maxg + k] = (node << 5) | image code,
//               node = (z*Ny + y)*Nx + x, image code applied to the bead
//   image code = (sx+1) + 3*(sy+1) + 9*(sz+1)
// As sets of unordered pairs they equal the reference's half list
// (npair_half_bin_newton.cpp:38-124) and grid list (npair_grid_bin.cpp:22-127).
#include "bead_kernels.h"

namespace phafd {

namespace {

constexpr int IMGMASK = 1023, IMGMAX = 512, IMGBITS = 10, IMG2BITS = 20;

__device__ __forceinline__ double img_shift(int code, int d, const BeadArgs& a) {
  int s = (code / (d == 0 ? 1 : d == 1 ? 3 : 9)) % 3 - 1;
  return s == 0 ? 0.0 : (s > 0 ? a.period[d] : -a.period[d]);
}

__device__ __forceinline__ int bin_coord(double x, double lo, double inv, int nb) {
  int b = (int)((x - lo) * inv);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

}  // namespace

// neighbor.cpp:79-97
// With use_cond the last block to finish (threadfence pattern) copies the
// flag into the graph conditional that gates the rebuild body.
// It also zeroes the deposit on the bead's grid-list nodes (the last pair
// stage deposited there; the pass that reads the deposit ran before this
// check), list words gathered four at a time.
__global__ void k_check(BeadArgs a, cudaGraphConditionalHandle h, int use_cond, long long* step_inc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (step_inc && i == 0) *step_inc += 1;
  if (i < a.n && a.dep && a.gl) {
    const int cnt = a.ngl[i];
    const uint32_t* __restrict__ gl = a.gl + (size_t)i * a.maxg;
    for (int k0 = 0; k0 < cnt; k0 += 4) {
      uint32_t e[4];
#pragma unroll
      for (int b = 0; b < 4; ++b) e[b] = k0 + b < cnt ? gl[k0 + b] : 0xffffffffu;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        if (e[b] == 0xffffffffu) continue;
        if (a.dep_bytes == 8) reinterpret_cast<double*>(a.dep)[e[b] >> 5] = 0.0;
        else reinterpret_cast<float*>(a.dep)[e[b] >> 5] = 0.f;
      }
    }
  }
  if (i < a.n) {
    const double d0 = a.x[3 * i] - a.xhold[3 * i];
    const double d1 = a.x[3 * i + 1] - a.xhold[3 * i + 1];
    const double d2 = a.x[3 * i + 2] - a.xhold[3 * i + 2];
    const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    if (rsq > a.triggersq) {
      atomicOr(a.flag, 1);
      __threadfence();
    }
  }
  if (!use_cond) return;
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(a.check_done, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    const int f = atomicOr(a.flag, 0);
    *a.check_done = 0;
    cudaGraphSetConditional(h, f ? 1u : 0u);
  }
}

// domain.cpp:102-163 then Domain::unmap
PHAFD_D void pbc_at(const BeadArgs& a, int i) {
  int im = a.image[i];
  double x[3] = {a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2]};
  for (int d = 0; d < 3; ++d) {
    const int sh = d == 0 ? 0 : (d == 1 ? IMGBITS : IMG2BITS);
    const double lo = a.boxlo[d], hi = a.boxhi[d], L = a.period[d];
    if (x[d] < lo) {
      x[d] = __dadd_rn(x[d], L);
      int idim = d == 2 ? (im >> IMG2BITS) : ((im >> sh) & IMGMASK);
      const int other = im ^ (idim << sh);
      idim = (idim - 1) & IMGMASK;
      im = other | (idim << sh);
    }
    if (x[d] >= hi) {
      x[d] = __dsub_rn(x[d], L);
      x[d] = x[d] > lo ? x[d] : lo;
      int idim = d == 2 ? (im >> IMG2BITS) : ((im >> sh) & IMGMASK);
      const int other = im ^ (idim << sh);
      idim = (idim + 1) & IMGMASK;
      im = other | (idim << sh);
    }
  }
  const int xbox = (im & IMGMASK) - IMGMAX;
  const int ybox = (im >> IMGBITS & IMGMASK) - IMGMAX;
  const int zbox = (im >> IMG2BITS) - IMGMAX;
  a.image[i] = im;
  for (int d = 0; d < 3; ++d) a.x[3 * i + d] = x[d];
  a.ux[3 * i + 0] = __dadd_rn(x[0], __dmul_rn((double)xbox, a.period[0]));
  a.ux[3 * i + 1] = __dadd_rn(x[1], __dmul_rn((double)ybox, a.period[1]));
  a.ux[3 * i + 2] = __dadd_rn(x[2], __dmul_rn((double)zbox, a.period[2]));
}

// pbc, then the bead's bin and its count (the counts are zero here: the
// build that used the previous ones reset the bins it had filled)
__global__ void k_pbc_bin(BeadArgs a) {
  if (!*a.flag) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  pbc_at(a, i);
  const int bx = bin_coord(a.x[3 * i], a.boxlo[0], a.bininv[0], a.nb[0]);
  const int by = bin_coord(a.x[3 * i + 1], a.boxlo[1], a.bininv[1], a.nb[1]);
  const int bz = bin_coord(a.x[3 * i + 2], a.boxlo[2], a.bininv[2], a.nb[2]);
  const int b = (bz * a.nb[1] + by) * a.nb[0] + bx;
  a.bin_of[i] = b;
  if (a.bin_off) {
    const double bs[3] = {a.period[0] / a.nb[0], a.period[1] / a.nb[1], a.period[2] / a.nb[2]};
    a.bin_off[i] = make_float4((float)(a.x[3 * i] - (a.boxlo[0] + bx * bs[0])),
                               (float)(a.x[3 * i + 1] - (a.boxlo[1] + by * bs[1])),
                               (float)(a.x[3 * i + 2] - (a.boxlo[2] + bz * bs[2])), 0.f);
  }
  atomicAdd(&a.bin_count[b], 1);
}

// exclusive scan of bin_count into bin_start, in three launches
__global__ void k_scan_block(BeadArgs a) {
  if (!*a.flag) return;
  __shared__ int warp_sums[32];
  const long long base = (long long)blockIdx.x * 1024;
  const long long i = base + threadIdx.x;
  int v = i < a.nbins ? a.bin_count[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    int s = warp_sums[lane];
    int si = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, si, off);
      if (lane >= off) si += t;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) a.scan_tmp[blockIdx.x] = si;
  }
  __syncthreads();
  if (i < a.nbins) a.bin_start[i] = incl - v + warp_sums[w];
}

// exclusive scan of the per-block sums: one block of 1024 threads, each
// thread owning a contiguous chunk of the sums
__global__ void k_scan_sums(BeadArgs a, int nblocks) {
  if (!*a.flag) return;
  __shared__ int warp_sums[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int chunk = (nblocks + 1023) / 1024;
  const int b0 = t * chunk, b1 = min(b0 + chunk, nblocks);
  int local = 0;
  for (int b = b0; b < b1; ++b) local += a.scan_tmp[b];
  int incl = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    int s = warp_sums[lane], si = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, si, off);
      if (lane >= off) si += v;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) a.bin_start[a.nbins] = si;
  }
  __syncthreads();
  int run = incl - local + warp_sums[w];
  for (int b = b0; b < b1; ++b) {
    const int v = a.scan_tmp[b];
    a.scan_tmp[b] = run;
    run += v;
  }
}

__global__ void k_scan_add(BeadArgs a) {
  if (!*a.flag) return;
  const long long i = (long long)blockIdx.x * 1024 + threadIdx.x;
  if (i < a.nbins) a.bin_start[i] += a.scan_tmp[blockIdx.x];
}

__global__ void k_bin_fill(BeadArgs a) {
  if (!*a.flag) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int b = a.bin_of[i];
  const int pos = a.bin_start[b] + atomicAdd(&a.bin_cursor[b], 1);
  a.sorted[pos] = i;
}

// order beads inside each bin by index so that the lists are deterministic;
// also clears the deposit support mask that the build then sets
__global__ void k_bin_sort(BeadArgs a) {
  if (!*a.flag) return;
  if (a.dmask)
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < a.gmask_words;
         k += (long long)gridDim.x * blockDim.x)
      a.dmask[k] = 0u;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < a.nbins; b += (long long)gridDim.x * blockDim.x) {
    const int s = a.bin_start[b], e = a.bin_start[b + 1];
    for (int p = s + 1; p < e; ++p) {
      const int v = a.sorted[p];
      int q = p - 1;
      while (q >= s && a.sorted[q] > v) { a.sorted[q + 1] = a.sorted[q]; --q; }
      a.sorted[q + 1] = v;
    }
  }
}

// the deposit support mask: the sector of a grid-list node
PHAFD_D void dmask_set(const BeadArgs& a, uint32_t node) {
  const long long sec = (long long)node / a.gmask_g;
  atomicOr(a.dmask + (sec >> 5), 1u << (sec & 31));
}
// the bin counts the next rebuild starts from: zero again in the bead's bin
// (every filled bin holds a bead, so this clears them all)
PHAFD_D void bin_reset(const BeadArgs& a, int i) {
  const int b = a.bin_of[i];
  a.bin_count[b] = 0;
  a.bin_cursor[b] = 0;
}

// stencil scans: full bead list and per-bead grid list
__global__ void k_build(BeadArgs a) {
  if (!*a.flag) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double xi[3] = {a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2]};
  // ---- bead list
  if (a.nbr) {
    const int b = a.bin_of[i];
    const int bx = b % a.nb[0], by = (b / a.nb[0]) % a.nb[1], bz = b / (a.nb[0] * a.nb[1]);
    int cnt = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      int cz = bz + dz, sz = 0;
      if (cz < 0) { cz += a.nb[2]; sz = -1; } else if (cz >= a.nb[2]) { cz -= a.nb[2]; sz = 1; }
      if (sz != 0 && !a.zperiodic) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        int cy = by + dy, sy = 0;
        if (cy < 0) { cy += a.nb[1]; sy = -1; } else if (cy >= a.nb[1]) { cy -= a.nb[1]; sy = 1; }
        for (int dx = -1; dx <= 1; ++dx) {
          int cx = bx + dx, sx = 0;
          if (cx < 0) { cx += a.nb[0]; sx = -1; } else if (cx >= a.nb[0]) { cx -= a.nb[0]; sx = 1; }
          const int nbn = (cz * a.nb[1] + cy) * a.nb[0] + cx;
          const int code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
          const double s0 = sx == 0 ? 0.0 : (sx > 0 ? a.period[0] : -a.period[0]);
          const double s1 = sy == 0 ? 0.0 : (sy > 0 ? a.period[1] : -a.period[1]);
          const double s2 = sz == 0 ? 0.0 : (sz > 0 ? a.period[2] : -a.period[2]);
          for (int p = a.bin_start[nbn]; p < a.bin_start[nbn + 1]; ++p) {
            const int j = a.sorted[p];
            if (j == i && code == 13) continue;
            const double xj0 = sx ? __dadd_rn(a.x[3 * j], s0) : a.x[3 * j];
            const double xj1 = sy ? __dadd_rn(a.x[3 * j + 1], s1) : a.x[3 * j + 1];
            const double xj2 = sz ? __dadd_rn(a.x[3 * j + 2], s2) : a.x[3 * j + 2];
            const double dx0 = __dsub_rn(xi[0], xj0), dx1 = __dsub_rn(xi[1], xj1), dx2 = __dsub_rn(xi[2], xj2);
            const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(dx0, dx0), __dmul_rn(dx1, dx1)), __dmul_rn(dx2, dx2));
            if (rsq <= a.cutneighsq) {
              if (cnt < a.maxnb) a.nbr[(size_t)i * a.maxnb + cnt] = (j << 5) | code;
              ++cnt;
            }
          }
        }
      }
    }
    if (cnt > a.maxnb) { atomicOr(a.status, ST_OVERFLOW); cnt = a.maxnb; }
    a.nnbr[i] = cnt;
  }
  // ---- grid list: nodes within cutneigh of each periodic image of bead i.
  // Candidate rows are pruned to the cutoff sphere with a margin; membership
  // is decided by the exact test in the reference's operand order.
  if (a.gl) {
    const double cutsq = a.cutneighsq;
    const double margin = 1e-9 * cutsq;
    int cnt = 0;
    const double uz = (xi[2] - a.boxlo[2]) / a.dx[2];
    const int kz0 = (int)floor(uz - a.cutneigh / a.dx[2]) - 1, kz1 = (int)ceil(uz + a.cutneigh / a.dx[2]) + 1;
    for (int kz = kz0; kz <= kz1; ++kz) {
      int wz = kz, sz = 0;
      if (wz < 0) { wz += a.N[2]; sz = 1; } else if (wz >= a.N[2]) { wz -= a.N[2]; sz = -1; }
      if (wz < 0 || wz >= a.N[2]) continue;
      if (sz != 0 && !a.zperiodic) continue;
      const double zt = __dadd_rn(__dmul_rn((double)wz, a.dx[2]), a.boxlo[2]);
      const double bz = sz ? __dadd_rn(xi[2], sz > 0 ? a.period[2] : -a.period[2]) : xi[2];
      const double dz = __dsub_rn(zt, bz);
      const double remz = cutsq - dz * dz;
      if (remz < -margin) continue;
      const double ry = sqrt(fmax(remz, 0.0)) / a.dx[1];
      const double uy = (xi[1] - a.boxlo[1]) / a.dx[1];
      const int ky0 = (int)floor(uy - ry) - 1, ky1 = (int)ceil(uy + ry) + 1;
      for (int ky = ky0; ky <= ky1; ++ky) {
        int wy = ky, sy = 0;
        if (wy < 0) { wy += a.N[1]; sy = 1; } else if (wy >= a.N[1]) { wy -= a.N[1]; sy = -1; }
        if (wy < 0 || wy >= a.N[1]) continue;
        const double yt = __dadd_rn(__dmul_rn((double)wy, a.dx[1]), a.boxlo[1]);
        const double by_ = sy ? __dadd_rn(xi[1], sy > 0 ? a.period[1] : -a.period[1]) : xi[1];
        const double dy = __dsub_rn(yt, by_);
        const double remy = remz - dy * dy;
        if (remy < -margin) continue;
        const double rx = sqrt(fmax(remy, 0.0)) / a.dx[0];
        const double ux = (xi[0] - a.boxlo[0]) / a.dx[0];
        const int kx0 = (int)floor(ux - rx) - 1, kx1 = (int)ceil(ux + rx) + 1;
        for (int kx = kx0; kx <= kx1; ++kx) {
          int wx = kx, sx = 0;
          if (wx < 0) { wx += a.N[0]; sx = 1; } else if (wx >= a.N[0]) { wx -= a.N[0]; sx = -1; }
          if (wx < 0 || wx >= a.N[0]) continue;
          const double xt = __dadd_rn(__dmul_rn((double)wx, a.dx[0]), a.boxlo[0]);
          const double bx_ = sx ? __dadd_rn(xi[0], sx > 0 ? a.period[0] : -a.period[0]) : xi[0];
          const double dxx = __dsub_rn(xt, bx_);
          const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(dxx, dxx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
          if (rsq <= cutsq) {
            const uint32_t node = (uint32_t)(((long long)wz * a.N[1] + wy) * a.N[0] + wx);
            const int code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
            if (cnt < a.maxg) {
              a.gl[(size_t)i * a.maxg + cnt] = (node << 5) | (uint32_t)code;
              if (a.dmask) dmask_set(a, node);
            }
            ++cnt;
          }
        }
      }
    }
    if (cnt > a.maxg) { atomicOr(a.status, ST_OVERFLOW); cnt = a.maxg; }
    a.ngl[i] = cnt;
  }
  bin_reset(a, i);
  // neighbor.cpp:106-109
  a.xhold[3 * i] = xi[0];
  a.xhold[3 * i + 1] = xi[1];
  a.xhold[3 * i + 2] = xi[2];
}

// FP32 list build (production precision): the same stencil scans with
// distances formed from bin-relative float offsets (bead list) and from the
// bead position in grid units split into an integer part and a fraction
// (grid list); the cutoff carries a 1e-5 relative margin, so the lists are
// supersets of the exact ones (the extra pairs lie beyond every interaction
// cutoff, which the pair kernel tests again each step).
// exclusive prefix sum over the L lanes of a group, and the group total
template <int L>
PHAFD_D int group_scan(int v, int lane, int& total) {
  int inc = v;
#pragma unroll
  for (int d = 1; d < L; d <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, inc, d, L);
    if (lane >= d) inc += t;
  }
  total = __shfl_sync(0xffffffffu, inc, L - 1, L);
  return inc - v;
}

// L lanes per bead (L = 8 while the beads alone would leave most of the GPU
// idle, else 1): lane l takes stencil bins l, l + L, ... and grid rows l,
// l + L, ... of the bead; with L > 1 each list is written in (lane, bin or
// row, member) order after a count pass and a prefix sum over the lanes, so
// the lists do not depend on timing.
template <int L>
__global__ void k_build_fp32(BeadArgs a) {
  if (!*a.flag) return;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt / L, lane = gt % L;
  const bool live = i < a.n;  // dead lanes still take part in the group shuffles
  const int ii = live ? i : 0;
  const float cut2 = (float)(a.cutneighsq * (1.0 + 1e-5));
  if (a.nbr) {
    const int b = a.bin_of[ii];
    const int bx = b % a.nb[0], by = (b / a.nb[0]) % a.nb[1], bz = b / (a.nb[0] * a.nb[1]);
    const float4 oi = a.bin_off[ii];
    const float bs[3] = {(float)(a.period[0] / a.nb[0]), (float)(a.period[1] / a.nb[1]), (float)(a.period[2] / a.nb[2])};
    // visit(write): count (write == false) or store the entries of this lane's bins
    auto visit = [&](bool write, int base) {
      int cnt = 0;
      for (int st = lane; st < 27 && live; st += L) {
        const int dx = st % 3 - 1, dy = (st / 3) % 3 - 1, dz = st / 9 - 1;
        int cz = bz + dz, sz = 0;
        if (cz < 0) { cz += a.nb[2]; sz = -1; } else if (cz >= a.nb[2]) { cz -= a.nb[2]; sz = 1; }
        if (sz != 0 && !a.zperiodic) continue;
        int cy = by + dy, sy = 0;
        if (cy < 0) { cy += a.nb[1]; sy = -1; } else if (cy >= a.nb[1]) { cy -= a.nb[1]; sy = 1; }
        int cx = bx + dx, sx = 0;
        if (cx < 0) { cx += a.nb[0]; sx = -1; } else if (cx >= a.nb[0]) { cx -= a.nb[0]; sx = 1; }
        const int nbn = (cz * a.nb[1] + cy) * a.nb[0] + cx;
        const int code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
        // x_i - (x_j + s L) = (b_i - b_j') bs + off_i - off_j, with b_j' = c + s nb
        const float ex = (float)(bx - (cx + sx * a.nb[0])) * bs[0] + oi.x;
        const float ey = (float)(by - (cy + sy * a.nb[1])) * bs[1] + oi.y;
        const float ez = (float)(bz - (cz + sz * a.nb[2])) * bs[2] + oi.z;
        const int p1 = a.bin_start[nbn + 1];
        for (int p = a.bin_start[nbn]; p < p1; ++p) {
          const int j = a.sorted[p];
          if (j == i && code == 13) continue;
          const float4 oj = a.bin_off[j];
          const float d0 = ex - oj.x, d1 = ey - oj.y, d2 = ez - oj.z;
          if (d0 * d0 + d1 * d1 + d2 * d2 <= cut2) {
            if (write && base + cnt < a.maxnb) a.nbr[(size_t)i * a.maxnb + base + cnt] = (j << 5) | code;
            ++cnt;
          }
        }
      }
      return cnt;
    };
    int total;
    if constexpr (L == 1) {
      total = visit(true, 0);
    } else {
      const int mine = visit(false, 0);
      const int off = group_scan<L>(mine, lane, total);
      visit(true, off);
    }
    if (live && lane == 0) {
      if (total > a.maxnb) { atomicOr(a.status, ST_OVERFLOW); total = a.maxnb; }
      a.nnbr[i] = total;
    }
  }
  const double xi[3] = {a.x[3 * ii], a.x[3 * ii + 1], a.x[3 * ii + 2]};
  if (a.gl) {
    int gi[3];
    float gf[3], dxf[3];
    for (int d = 0; d < 3; ++d) {
      const double ud = (xi[d] - a.boxlo[d]) * a.invdx[d];
      const double fl = floor(ud);
      gi[d] = (int)fl;
      gf[d] = (float)(ud - fl);
      dxf[d] = (float)a.dx[d];
    }
    const float cut = (float)a.cutneigh * 1.00001f;
    const int rz = (int)ceilf(cut / dxf[2]) + 1;
    const int ry = (int)ceilf(cut / dxf[1]) + 1;
    const int nrow = (2 * rz + 1) * (2 * ry + 1);
    auto visit = [&](bool write, int base) {
      int cnt = 0;
      for (int row = lane; row < nrow && live; row += L) {
        const int oz = row / (2 * ry + 1) - rz, oy = row % (2 * ry + 1) - ry;
        const int kz = gi[2] + oz;
        int wz = kz, sz = 0;
        if (wz < 0) { wz += a.N[2]; sz = 1; } else if (wz >= a.N[2]) { wz -= a.N[2]; sz = -1; }
        if (wz < 0 || wz >= a.N[2]) continue;
        if (sz != 0 && !a.zperiodic) continue;
        const float dz = ((float)oz - gf[2]) * dxf[2];
        const float remz = cut2 - dz * dz;
        if (remz < 0.f) continue;
        const int ky = gi[1] + oy;
        int wy = ky, sy = 0;
        if (wy < 0) { wy += a.N[1]; sy = 1; } else if (wy >= a.N[1]) { wy -= a.N[1]; sy = -1; }
        if (wy < 0 || wy >= a.N[1]) continue;
        const float dy = ((float)oy - gf[1]) * dxf[1];
        const float remy = remz - dy * dy;
        if (remy < 0.f) continue;
        const int rx = (int)ceilf(sqrtf(remy) / dxf[0]) + 1;
        for (int ox = -rx; ox <= rx; ++ox) {
          const int kx = gi[0] + ox;
          int wx = kx, sx = 0;
          if (wx < 0) { wx += a.N[0]; sx = 1; } else if (wx >= a.N[0]) { wx -= a.N[0]; sx = -1; }
          if (wx < 0 || wx >= a.N[0]) continue;
          const float dxx = ((float)ox - gf[0]) * dxf[0];
          if (dxx * dxx + dy * dy + dz * dz <= cut2) {
            if (write && base + cnt < a.maxg) {
              const uint32_t node = (uint32_t)(((long long)wz * a.N[1] + wy) * a.N[0] + wx);
              const int code = (sx + 1) + 3 * (sy + 1) + 9 * (sz + 1);
              a.gl[(size_t)i * a.maxg + base + cnt] = (node << 5) | (uint32_t)code;
              if (a.dmask) dmask_set(a, node);
            }
            ++cnt;
          }
        }
      }
      return cnt;
    };
    int total;
    if constexpr (L == 1) {
      total = visit(true, 0);
    } else {
      const int mine = visit(false, 0);
      const int off = group_scan<L>(mine, lane, total);
      visit(true, off);
    }
    if (live && lane == 0) {
      if (total > a.maxg) { atomicOr(a.status, ST_OVERFLOW); total = a.maxg; }
      a.ngl[i] = total;
    }
  }
  if (live && lane == 0) {
    bin_reset(a, i);
    a.xhold[3 * i] = xi[0];
    a.xhold[3 * i + 1] = xi[1];
    a.xhold[3 * i + 2] = xi[2];
  }
}

__global__ void k_build_done(BeadArgs a) {
  if (*a.flag) {
    *a.ncalls += 1;
    *a.flag = 0;
  }
}

__global__ void k_step_begin(long long* d_step) { *d_step += 1; }

// ---- pair forces: lj/cut over the bead list, gridatom over the grid list.
// PAIR_TPB threads share one bead (its list entries are split among them,
// then shuffle-reduced), so no atomics on F.  The mu deposit of the gridatom
// styles goes to `dep` with atomics.
//
// Distances.  FP64: the reference's operand order (x_i - (x_j + s);
// (k dx + lo) - (x + s)).  FP32: bead-bead separations are formed in FP64
// and rounded once; bead-node separations come from the bead's position in
// grid units split once per step into an integer part and a fraction, so the
// per-entry arithmetic is (small integer - fraction) * dx in FP32.
constexpr int PAIR_TPB = 4;
constexpr int PB = 4;  // list entries a lane gathers at once

// grid coordinates of a node index (shifts and masks for power-of-two grids)
PHAFD_D void node_coords(const BeadArgs& a, uint32_t node, int g3[3]) {
  if (a.lgN[0] >= 0) {
    g3[0] = (int)(node & (uint32_t)(a.N[0] - 1));
    g3[1] = (int)((node >> a.lgN[0]) & (uint32_t)(a.N[1] - 1));
    g3[2] = (int)(node >> (a.lgN[0] + a.lgN[1]));
  } else {
    g3[0] = (int)(node % (uint32_t)a.N[0]);
    g3[1] = (int)((node / (uint32_t)a.N[0]) % (uint32_t)a.N[1]);
    g3[2] = (int)(node / ((uint32_t)a.N[0] * (uint32_t)a.N[1]));
  }
}

template <typename T>
__global__ void k_pair(BeadArgs a, PairArgs<T> p) {
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gtid / PAIR_TPB, sub = gtid % PAIR_TPB;
  const bool live = i < a.n;
  if (p.step_inc && gtid == 0) *p.step_inc += 1;
  const int ii = live ? i : 0;
  const double xi0 = a.x[3 * ii], xi1 = a.x[3 * ii + 1], xi2 = a.x[3 * ii + 2];
  // Kahan-compensated sums (exact no-ops in double beyond round-off)
  T f[3] = {0, 0, 0}, c[3] = {0, 0, 0};
  auto add = [&](int d, T v) {
    T y = v - c[d];
    T t = f[d] + y;
    c[d] = (t - f[d]) - y;
    f[d] = t;
  };
  // the grid coupling's per-bead values, loaded ahead of the bead-bead loop
  // so that their latency overlaps it
  const bool ga = live && p.ga_style != PHAFD_GRIDATOM_NONE && a.gl;
  const int gcnt = ga ? a.ngl[i] : 0;
  const int gt = ga ? a.type[i] : 0;
  const T cutsq = ga ? (T)p.ga_cutsq[gt] : (T)0, eps = ga ? (T)p.ga_eps[gt] : (T)0,
          phit = ga ? (T)p.ga_phi[gt] : (T)0;
  // bead position in grid units: integer part + fraction (FP32 path; GB300's
  // FP64 rate makes a divide per axis and thread cost more than the rest)
  int gi[3];
  T gf[3], dxf[3];
  const double xi[3] = {xi0, xi1, xi2};
  if (ga) {
    for (int d = 0; d < 3; ++d) {
      const double ud = (xi[d] - a.boxlo[d]) * a.invdx[d];
      const double fl = floor(ud);
      gi[d] = (int)fl;
      gf[d] = (T)(ud - fl);
      dxf[d] = (T)a.dx[d];
    }
  }
  // Both loops take their entries in batches of PB per lane: the list words
  // of a batch are loaded together, then every load the batch's entries need,
  // then the arithmetic, in the entries' order k = sub, sub + PAIR_TPB, ...
  // (the compensated sums see the same sequence as one entry at a time).
  if (live && p.lj && a.nbr) {
    const int cnt = a.nnbr[i];
    const int* __restrict__ nl = a.nbr + (size_t)i * a.maxnb;
    for (int k0 = sub; k0 < cnt; k0 += PAIR_TPB * PB) {
      int e[PB];
#pragma unroll
      for (int b = 0; b < PB; ++b) e[b] = k0 + b * PAIR_TPB < cnt ? nl[k0 + b * PAIR_TPB] : -1;
      double xj[PB][3];
#pragma unroll
      for (int b = 0; b < PB; ++b) {
        const int j = e[b] >= 0 ? e[b] >> 5 : ii;
        xj[b][0] = a.x[3 * j];
        xj[b][1] = a.x[3 * j + 1];
        xj[b][2] = a.x[3 * j + 2];
      }
#pragma unroll
      for (int b = 0; b < PB; ++b) {
        if (e[b] < 0) continue;
        const int code = e[b] & 31;
        const double d0 = xi0 - (xj[b][0] + img_shift(code, 0, a));
        const double d1 = xi1 - (xj[b][1] + img_shift(code, 1, a));
        const double d2 = xi2 - (xj[b][2] + img_shift(code, 2, a));
        const T dx = (T)d0, dy = (T)d1, dz = (T)d2;
        const T rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < (T)p.lj_cutsq) {
          const T r2inv = (T)1 / rsq;
          const T r6inv = r2inv * r2inv * r2inv;
          const T forcelj = r6inv * ((T)p.lj1 * r6inv - (T)p.lj2);
          const T fpair = forcelj * r2inv;
          add(0, dx * fpair);
          add(1, dy * fpair);
          add(2, dz * fpair);
        }
      }
    }
  }
  if (ga) {
    const int cnt = gcnt;
    const bool linear = p.ga_style != PHAFD_GRIDATOM_GAUSSIAN && p.ga_style != PHAFD_GRIDATOM_LJISH;
    const uint32_t* __restrict__ gl = a.gl + (size_t)i * a.maxg;
    for (int k0 = sub; k0 < cnt; k0 += PAIR_TPB * PB) {
      uint32_t e[PB];
#pragma unroll
      for (int b = 0; b < PB; ++b) e[b] = k0 + b * PAIR_TPB < cnt ? gl[k0 + b * PAIR_TPB] : 0xffffffffu;
      // separations and the cutoff test (no loads)
      T rs[PB];
      bool in[PB];
#pragma unroll
      for (int b = 0; b < PB; ++b) {
        in[b] = false;
        rs[b] = (T)0;
        if (e[b] == 0xffffffffu) continue;
        const uint32_t node = e[b] >> 5;
        const int code = (int)(e[b] & 31u);
        int g3[3];
        node_coords(a, node, g3);
        T dd[3];
        if constexpr (sizeof(T) == 8) {
          // node coordinate k*dx + boxlo without contraction (npair_grid_bin.cpp:76-88)
          for (int d = 0; d < 3; ++d)
            dd[d] = __dadd_rn(__dmul_rn((double)g3[d], a.dx[d]), a.boxlo[d]) - (xi[d] + img_shift(code, d, a));
        } else {
          const int sc[3] = {code % 3 - 1, (code / 3) % 3 - 1, code / 9 - 1};
          for (int d = 0; d < 3; ++d) dd[d] = ((T)(g3[d] - gi[d] - sc[d] * a.N[d]) - gf[d]) * dxf[d];
        }
        const T rsq = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
        in[b] = (p.ga_style == PHAFD_GRIDATOM_GAUSSIAN) ? (rsq <= cutsq) : (rsq < cutsq);
        rs[b] = rsq / cutsq;
      }
      // the node values of the entries inside the cutoff
      T ph[PB], q0[PB], q1[PB], q2[PB];
#pragma unroll
      for (int b = 0; b < PB; ++b) {
        const uint32_t node = in[b] ? e[b] >> 5 : 0u;
        ph[b] = in[b] && !linear ? p.phi[node] : (T)0;
        q0[b] = in[b] ? p.gx[node] : (T)0;
        q1[b] = in[b] ? p.gy[node] : (T)0;
        q2[b] = in[b] ? p.gz[node] : (T)0;
      }
#pragma unroll
      for (int b = 0; b < PB; ++b) {
        if (!in[b]) continue;
        const uint32_t node = e[b] >> 5;
        const T rsq = rs[b];
        T expfac, mu_add;
        if (p.ga_style == PHAFD_GRIDATOM_GAUSSIAN) {
          // pair_gridatom_gaussian.cpp:97-107
          expfac = (exp(-rsq / (T)2.0) - exp((T)-0.5)) * exp((T)0.5) * eps;
          const T delphi = ph[b] - phit;
          mu_add = (T)2 * delphi * expfac;
          expfac = expfac * ((T)2 * delphi * (T)p.dv);
        } else if (p.ga_style == PHAFD_GRIDATOM_LJISH) {
          // pair_gridatom_lj_ish.cpp:104-176
          expfac = exp((T)-1. / ((T)1 - rsq) + (T)1) * eps;
          const T delphi = ph[b] - phit;
          mu_add = (T)2 * delphi * expfac;
          expfac = expfac * ((T)2 * delphi * (T)p.dv);
        } else {
          // pair_gridatom_lj_ish_linear.cpp:104-168
          expfac = (T)-1 * exp((T)-1. / ((T)1 - rsq) + (T)1) * eps;
          mu_add = expfac;
          expfac = expfac * (T)p.dv;
        }
        if (p.dep) atomicAdd(p.dep + node, mu_add);  // null: forces only (substeps of a macro step)
        add(0, -q0[b] * expfac);
        add(1, -q1[b] * expfac);
        add(2, -q2[b] * expfac);
      }
    }
  }
  // combine the PAIR_TPB partial sums of a bead (adjacent lanes)
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T v = f[d] - c[d];
#pragma unroll
    for (int off = 1; off < PAIR_TPB; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    f[d] = v;
  }
  if (live && sub == 0) {
    a.f[3 * i] = (double)f[0];
    a.f[3 * i + 1] = (double)f[1];
    a.f[3 * i + 2] = (double)f[2];
  }
}

// rho[node] += shape of the gridatom coupling (epsilon 1, no phi factor) of
// every bead within its cutoff: the bead-density input of the learned
// propagator.  One thread per bead, FP64 separations rounded once.
template <typename T>
__global__ void k_density(BeadArgs a, PairArgs<T> p, T* rho) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || !a.gl || p.ga_style == PHAFD_GRIDATOM_NONE) return;
  const double xi[3] = {a.x[3 * i], a.x[3 * i + 1], a.x[3 * i + 2]};
  const int cnt = a.ngl[i];
  const T cutsq = (T)p.ga_cutsq[a.type[i]];
  for (int k = 0; k < cnt; ++k) {
    const uint32_t e = a.gl[(size_t)i * a.maxg + k];
    const uint32_t node = e >> 5;
    const int code = (int)(e & 31u);
    int g3[3];
    node_coords(a, node, g3);
    T dd[3];
    for (int d = 0; d < 3; ++d) dd[d] = (T)((double)g3[d] * a.dx[d] + a.boxlo[d] - (xi[d] + img_shift(code, d, a)));
    T rsq = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
    const bool inside = (p.ga_style == PHAFD_GRIDATOM_GAUSSIAN) ? (rsq <= cutsq) : (rsq < cutsq);
    if (!inside) continue;
    rsq = rsq / cutsq;
    const T v = p.ga_style == PHAFD_GRIDATOM_GAUSSIAN ? (exp(-rsq / (T)2.0) - exp((T)-0.5)) * exp((T)0.5)
                                                      : exp((T)-1. / ((T)1 - rsq) + (T)1);
    atomicAdd(rho + node, v);
  }
}

template <typename T>
void launch_density(const BeadArgs& a, const PairArgs<T>& p, T* rho, cudaStream_t st) {
  if (a.n == 0) return;
  k_density<T><<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(a, p, rho);
}
template void launch_density<float>(const BeadArgs&, const PairArgs<float>&, float*, cudaStream_t);
template void launch_density<double>(const BeadArgs&, const PairArgs<double>&, double*, cudaStream_t);

// fixatom_drag.cpp:47-52 / 58-62
__global__ void k_drag(BeadArgs a, double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double dr = a.dragc[i];
  if (dr == 0.0) return;
  for (int d = 0; d < 3; ++d)
    a.x[3 * i + d] = __dadd_rn(a.x[3 * i + d], __dmul_rn(__dmul_rn(__dmul_rn(dr, a.f[3 * i + d]), dt), 0.5));
}

// chain model (no reference counterpart; the oracle's oracle_chain_force).
// Bond vectors are differences of FP64 positions taken in FP64, then the
// force arithmetic runs in T; positions stay FP64.
template <typename T>
PHAFD_D void chain_force_at(const BeadArgs& a, int i) {
  const int fi = a.sf_fix[i];
  if (fi < 0) return;
  const SemiDev& P = a.sf[fi];
  const int base = a.sf_start[i], n = a.sf_len[i], b = i - base;
  const double* u = a.ux + 3 * (size_t)base;
  auto bond = [&](int q, T r[3]) {  // u[q+1] - u[q]
    for (int d = 0; d < 3; ++d) r[d] = (T)(u[3 * (q + 1) + d] - u[3 * q + d]);
  };
  const T kb = (T)P.kbond, b0 = (T)P.bondlength, kap = (T)P.bending;
  T f[3] = {0, 0, 0};
  for (int side = 0; side < 2; ++side) {
    const int q = side == 0 ? b - 1 : b;
    if (q < 0 || q + 1 >= n) continue;
    T r[3];
    bond(q, r);
    const T len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const T g = kb * (len - b0) / len;
    const T sgn = (q == b) ? (T)1 : (T)-1;
    for (int d = 0; d < 3; ++d) f[d] += sgn * g * r[d];
  }
  if (P.bending != 0.0) {
    for (int cc = b - 1; cc <= b + 1; ++cc) {
      if (cc < 1 || cc + 1 >= n) continue;
      T ra[3], rb[3];
      bond(cc - 1, ra);
      bond(cc, rb);
      const T la = sqrt(ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2]);
      const T lb = sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
      const T cs = (ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2]) / (la * lb);
      for (int d = 0; d < 3; ++d) {
        const T dca = rb[d] / (la * lb) - cs * ra[d] / (la * la);
        const T dcb = ra[d] / (la * lb) - cs * rb[d] / (lb * lb);
        if (b == cc - 1) f[d] += kap * (-dca);
        else if (b == cc) f[d] += kap * (dca - dcb);
        else f[d] += kap * dcb;
      }
    }
  }
  const int lo = b > 0 ? b - 1 : b, hi = b + 1 < n ? b + 1 : b;
  T tv[3];
  for (int d = 0; d < 3; ++d) tv[d] = (T)(u[3 * hi + d] - u[3 * lo + d]);
  const T tl = sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
  for (int d = 0; d < 3; ++d) {
    a.fchain[3 * i + d] = (double)f[d];
    a.tang[3 * i + d] = (double)(tl > 0 ? tv[d] / tl : (T)0);
  }
}

template <typename T>
__global__ void k_chain_force(BeadArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) chain_force_at<T>(a, i);
}

// (nsub > 1: substep `sub` of a macro step; its noise is keyed by
// step * nsub + sub so that every substep draws fresh numbers)
template <typename T>
PHAFD_D void chain_move_at(const BeadArgs& a, int i, int half, double dt, int nsub, int sub) {
  const int fi = a.sf_fix[i];
  if (fi < 0) return;
  const SemiDev& P = a.sf[fi];
  T xi[3] = {0, 0, 0};
  const uint64_t key = nsub > 1 ? (uint64_t)(*a.d_step) * (uint64_t)nsub + (uint64_t)sub : (uint64_t)(*a.d_step);
  if (P.noise == PHAFD_NOISE_PHILOX && P.temp > 0) bead_gauss(P.seed, key, half, i, xi);
  T fc[3], fp[3], t[3];
  for (int d = 0; d < 3; ++d) {
    fc[d] = (T)a.fchain[3 * (size_t)i + d];
    fp[d] = (T)a.f[3 * (size_t)i + d];
    t[d] = (T)a.tang[3 * (size_t)i + d];
  }
  const T h = (T)(0.5 * dt);
  const T ft[3] = {fc[0] + fp[0], fc[1] + fp[1], fc[2] + fp[2]};
  const T tf = t[0] * ft[0] + t[1] * ft[1] + t[2] * ft[2];
  const T tx = t[0] * xi[0] + t[1] * xi[1] + t[2] * xi[2];
  const T aa = (T)P.inv_perp, bpar = (T)P.dinv;
  const T sa = (T)P.sinv_perp, sb = (T)P.dsinv;
  const T amp = sqrt((T)(P.temp * dt));  // sqrt(2 T h), h = dt/2
  const int im = a.image[i];
  const int box[3] = {(im & IMGMASK) - IMGMAX, (im >> IMGBITS & IMGMASK) - IMGMAX, (im >> IMG2BITS) - IMGMAX};
  bool bad = false;
  for (int d = 0; d < 3; ++d) {
    const T disp = h * (aa * ft[d] + bpar * tf * t[d]) + amp * (sa * xi[d] + sb * tx * t[d]);
    const double nu = a.ux[3 * i + d] + (double)disp;
    a.ux[3 * i + d] = nu;
    a.x[3 * i + d] = __dsub_rn(nu, __dmul_rn((double)box[d], a.period[d]));  // Domain::map, domain.cpp:180-193
    bad |= !isfinite(nu);
  }
  if (bad) atomicOr(a.status, ST_CONSTRAINT);
}

template <typename T>
__global__ void k_chain_move(BeadArgs a, int half, double dt, int nsub, int sub) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n) chain_move_at<T>(a, i, half, dt, nsub, sub);
}

// Both half-steps of the chain model in one launch: one CTA per chain (the
// chains are contiguous ranges of beads), its threads striding over the
// chain's beads; a CTA barrier separates the force and the move of each half,
// as the launch boundaries of k_chain_force / k_chain_move do.
template <typename T>
__global__ void k_chain_step(BeadArgs a, double dt, int nsub, int sub) {
  const int s = a.chain_start[blockIdx.x];
  const int len = a.sf_len[s];
  for (int half = 0; half < 2; ++half) {
    for (int b = threadIdx.x; b < len; b += blockDim.x) chain_force_at<T>(a, s + b);
    __syncthreads();
    for (int b = threadIdx.x; b < len; b += blockDim.x) chain_move_at<T>(a, s + b, half, dt, nsub, sub);
    __syncthreads();
  }
}

// ---------------------------------------------------------------- launchers
static inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

void launch_step_begin(long long* d_step, cudaStream_t st) { k_step_begin<<<1, 1, 0, st>>>(d_step); }

void launch_neighbor_check(const BeadArgs& a, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st,
                           long long* step_inc) {
  if (a.n == 0) return;
  k_check<<<nblk(a.n, 256), 256, 0, st>>>(a, h, use_cond, step_inc);
}

void launch_neighbor(const BeadArgs& a, bool force, cudaStream_t st, long long* step_inc) {
  if (a.n == 0) return;
  if (force) cudaMemsetAsync(a.flag, 0xff, sizeof(int), st);
  else launch_neighbor_check(a, 0, 0, st, step_inc);
  launch_rebuild(a, st);
}

// Node mask of the gradient.  The pair kernel reads grad phi only at nodes
// within the coupling cutoff of a bead's current position.  At each rebuild
// the mask marks every 32-byte sector (gmask_g nodes along x) holding a node
// within cutoff + skin of the bead positions of that rebuild (xhold); before the inverse transform of a step the guard
// checks that no bead has moved more than skin since, which keeps every
// node the next pair evaluation reads inside the mask.  The inverse x pass
// then stores the three gradient components at masked nodes only, unless
// the guard fired (then everywhere, until the next rebuild clears it).
__global__ void k_gmask_clear(BeadArgs a) {
  if (!*a.flag) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) *a.gmask_off = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < a.gmask_words;
       k += (long long)gridDim.x * blockDim.x)
    a.gmask[k] = 0u;
}
__global__ void k_gmask_build(BeadArgs a) {
  if (!*a.flag) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double u[3];
  for (int d = 0; d < 3; ++d) u[d] = (a.x[3 * i + d] - a.boxlo[d]) / a.dx[d];
  const double r2 = a.gmask_r * a.gmask_r;
  const int zlo = (int)floor(u[2] - a.gmask_r / a.dx[2]), zhi = (int)ceil(u[2] + a.gmask_r / a.dx[2]);
  const int ylo = (int)floor(u[1] - a.gmask_r / a.dx[1]), yhi = (int)ceil(u[1] + a.gmask_r / a.dx[1]);
  // per grid row inside the sphere: its x range, then one bit per sector
  for (int kz = zlo; kz <= zhi; ++kz) {
    const double dz = (kz - u[2]) * a.dx[2];
    const int wz = ((kz % a.N[2]) + a.N[2]) % a.N[2];
    for (int ky = ylo; ky <= yhi; ++ky) {
      const double dy = (ky - u[1]) * a.dx[1];
      const double rem = r2 - dy * dy - dz * dz;
      if (rem < 0.0) continue;
      const double h = sqrt(rem) / a.dx[0];
      const int xlo = (int)ceil(u[0] - h), xhi = (int)floor(u[0] + h);
      const int wy = ((ky % a.N[1]) + a.N[1]) % a.N[1];
      const long long row = ((long long)wz * a.N[1] + wy) * a.N[0];
      for (int x = xlo; x <= xhi;) {
        const int wx = ((x % a.N[0]) + a.N[0]) % a.N[0];
        const long long node = row + wx;
        const long long sec = node / a.gmask_g;
        atomicOr(a.gmask + (sec >> 5), 1u << (sec & 31));
        // next node of this row in another sector
        const int left = a.gmask_g - (int)(node % a.gmask_g);
        x += left < a.N[0] - wx ? left : a.N[0] - wx;
      }
    }
  }
}

__global__ void k_gmask_guard(BeadArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double d0 = a.x[3 * i] - a.xhold[3 * i];
  const double d1 = a.x[3 * i + 1] - a.xhold[3 * i + 1];
  const double d2 = a.x[3 * i + 2] - a.xhold[3 * i + 2];
  if (d0 * d0 + d1 * d1 + d2 * d2 > a.gmask_guardsq) *a.gmask_off = 1;
}

void launch_gmask_guard(const BeadArgs& a, cudaStream_t st) {
  if (a.n == 0 || !a.gmask) return;
  k_gmask_guard<<<nblk(a.n, 256), 256, 0, st>>>(a);
}

// integrate.cpp:350-370: |x_last - x_first| of the stored (wrapped)
// positions, operations in the reference's order (no contraction)
__global__ void k_touch(const double* __restrict__ x, int n, double touch_point, int delay_step,
                        const long long* __restrict__ d_step, TouchState* s) {
  const int l = 3 * (n - 1);
  const double d0 = x[l] - x[0], d1 = x[l + 1] - x[1], d2 = x[l + 2] - x[2];
  const double d = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
  const long long step = *d_step;
  if (d < touch_point) {
    if (s->since >= delay_step) {
      if (s->nev < s->maxev) {
        s->ev_kind[s->nev] = 0;
        s->ev_step[s->nev] = step;
      }
      s->nev += 1;
    }
    s->since = 0;
    s->breakflag = 1;
  } else {
    if (s->breakflag && s->since == delay_step) {
      if (s->nev < s->maxev) {
        s->ev_kind[s->nev] = 1;
        s->ev_step[s->nev] = step - delay_step;
      }
      s->nev += 1;
    }
    s->since += 1;
  }
}

void launch_touch(const double* x, int n, double touch_point, int delay_step, const long long* d_step,
                  TouchState* s, cudaStream_t st) {
  if (n <= 0) return;
  k_touch<<<1, 1, 0, st>>>(x, n, touch_point, delay_step, d_step, s);
}

void launch_rebuild(const BeadArgs& a, cudaStream_t st) {
  if (a.n == 0) return;
  const int T = 256;
  k_pbc_bin<<<nblk(a.n, T), T, 0, st>>>(a);
  const int nblocks = (int)((a.nbins + 1023) / 1024);
  k_scan_block<<<nblocks, 1024, 0, st>>>(a);
  k_scan_sums<<<1, 1024, 0, st>>>(a, nblocks);
  k_scan_add<<<nblocks, 1024, 0, st>>>(a);
  k_bin_fill<<<nblk(a.n, T), T, 0, st>>>(a);
  k_bin_sort<<<nblk(a.nbins, T) > 4096 ? 4096 : nblk(a.nbins, T), T, 0, st>>>(a);
  if (a.fp32_lists) {
    // 8-lane groups while 8 n threads stay within one wave (2048 per SM)
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if ((long long)a.n * 8 <= (long long)nsm * 2048) k_build_fp32<8><<<nblk((long long)a.n * 8, 128), 128, 0, st>>>(a);
    else k_build_fp32<1><<<nblk(a.n, 128), 128, 0, st>>>(a);
  }
  else k_build<<<nblk(a.n, 128), 128, 0, st>>>(a);
  if (a.gmask) {
    k_gmask_clear<<<1024, 256, 0, st>>>(a);
    k_gmask_build<<<nblk(a.n, 128), 128, 0, st>>>(a);
  }
  k_build_done<<<1, 1, 0, st>>>(a);
}

template <typename T>
void launch_pair(const BeadArgs& a, const PairArgs<T>& p, cudaStream_t st) {
  if (a.n == 0) return;
  k_pair<T><<<nblk((long long)a.n * PAIR_TPB, 128), 128, 0, st>>>(a, p);
}
template void launch_pair<float>(const BeadArgs&, const PairArgs<float>&, cudaStream_t);
template void launch_pair<double>(const BeadArgs&, const PairArgs<double>&, cudaStream_t);


void launch_drag(const BeadArgs& a, double dt, cudaStream_t st) {
  if (a.n == 0 || !a.any_drag) return;
  k_drag<<<nblk(a.n, 256), 256, 0, st>>>(a, dt);
}

template <typename T>
void launch_chain_half(const BeadArgs& a, int half, double dt, cudaStream_t st, int nsub, int sub) {
  if (a.n == 0 || !a.any_semi) return;
  k_chain_force<T><<<nblk(a.n, 128), 128, 0, st>>>(a);
  k_chain_move<T><<<nblk(a.n, 128), 128, 0, st>>>(a, half, dt, nsub, sub);
}
template void launch_chain_half<float>(const BeadArgs&, int, double, cudaStream_t, int, int);
template void launch_chain_half<double>(const BeadArgs&, int, double, cudaStream_t, int, int);

template <typename T>
void launch_chain_step(const BeadArgs& a, double dt, cudaStream_t st, int nsub, int sub) {
  if (a.n == 0 || !a.any_semi) return;
  k_chain_step<T><<<a.nchains, 256, 0, st>>>(a, dt, nsub, sub);
}
template void launch_chain_step<float>(const BeadArgs&, double, cudaStream_t, int, int);
template void launch_chain_step<double>(const BeadArgs&, double, cudaStream_t, int, int);

}  // namespace phafd
