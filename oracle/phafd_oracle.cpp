// PHAFD per-timestep hot path: FP64 CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py load this library, and only as the checker.
// The product (libphafd_gpu.so) never links, loads or calls it.
//
// This file restates, in plain single-threaded FP64 C++, the reference's
// algorithm for one PHAFD timestep on one MPI rank (file:line citations are
// into samueljmcameron/PHAFD's src/ directory):
//   schedule                 integrate.cpp:105-203 (double pair pass, NaN check)
//   spectral gradient        fixgrid_conjugate.cpp:62-116, fixgrid_gradphi.cpp:42-99
//   r2c mu / c2r phi         fixgrid_conjugate.cpp:120-154
//   Model-B update           conjugate.cpp:130-327 (1-rank path),
//                            conjugate_volfrac.cpp:72-144
//   Flory-Huggins mu         fixgrid_floryhuggins.cpp:65-85
//   wavenumbers              domain.cpp:206-208 (pi = 3.141592, y/z swap)
//   layout + init RNG        grid.cpp:88-113, 205-307; utility.cpp:213-235
//   gridatom pairs           pair_gridatom_gaussian.cpp:45-120,
//                            pair_gridatom_lj_ish.cpp:44-181,
//                            pair_gridatom_lj_ish_linear.cpp:46-179
//   lj/cut                   pair_lj_cut.cpp:46-119
//   neighbor                 neighbor.cpp:39-125, nbin.cpp:61-94,
//                            nbin_standard.cpp:53-229, nstencil.cpp:101-143,
//                            nstencil_half_bin_3d.cpp:26-38,
//                            nstencil_full_bin_3d.cpp:26-37,
//                            npair_half_bin_newton.cpp:38-124,
//                            npair_grid_bin.cpp:22-127, npair.cpp:125-158
//   gathered/ghost copies    comm_brick.cpp:96-426 (1-rank semantics)
//   pbc / map / unmap        domain.cpp:102-204
//   drag                     fixatom_drag.cpp:43-66
//
// Parity status: UNPINNED against reference outputs.  The reference cannot be
// built here (it needs MPI, FFTW3-MPI, Eigen3 and the un-vendored fftw_arr and
// beadrodpmer libraries) and ships no tests, fixtures or golden vectors.  This
// restatement is pinned instead against numpy.fft and analytic known answers
// (tests/test_oracle_*.py).
//
// Two deliberate, documented additions that have no reference counterpart:
//   * fix atom/semiflexible: the reference delegates the chain step to the
//     external beadrodpmer library.  The chain model here is this project's
//     own (harmonic bonds + bending + anisotropic friction + noise), shared by
//     the oracle and the GPU path.
//   * noise sources: besides the reference's own mt19937 stream, a
//     counter-based Philox4x32-10 stream (Salmon et al., SC'11) that the GPU
//     path can generate on the device, so that both sides see the same noise.
//
// The z-ghost mode: with nprocs == 1 the reference's borders() creates no
// periodic z images of beads (comm_brick.cpp:300-318); with nprocs >= 2 it
// does.  ZGHOST_RANK1 restates the former exactly, ZGHOST_PERIODIC the latter.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "phafd_oracle.h"

using cd = std::complex<double>;

namespace {

constexpr int IMGMASK = 1023;
constexpr int IMGMAX = 512;
constexpr int IMGBITS = 10;
constexpr int IMG2BITS = 20;
constexpr int OWNED = 0, LOCAL = 1, GHOST = 2;
constexpr double BIG = 1e20;
constexpr double SMALL = 1.0e-6;

// ------------------------------------------------------------------ Philox
struct Philox {
  static inline void round(uint32_t c[4], const uint32_t k[2]) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0];
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c[3] ^ k[1];
    uint32_t n3 = lo0;
    c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
  }
  static void gen(uint32_t ctr[4], uint32_t key0, uint32_t key1) {
    uint32_t k[2] = {key0, key1};
    for (int r = 0; r < 10; ++r) {
      round(ctr, k);
      k[0] += 0x9E3779B9u;
      k[1] += 0xBB67AE85u;
    }
  }
};
// 53-bit uniform in [0,1) from two words
inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// ------------------------------------------------------------------ threads
// Host threads for the grid loops (oracle_set_threads; 1 by default).  Every
// split loop writes disjoint elements with the serial loop's arithmetic, and
// integer counters are summed per thread, so results are bit-identical for
// any thread count.
int g_threads = 1;

// f(begin, end, thread) over contiguous chunks of [0, n)
template <typename F>
void par_for(long long n, F&& f) {
  const int T = (int)std::max(1LL, std::min((long long)g_threads, n));
  if (T == 1) {
    if (n > 0) f(0LL, n, 0);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 1; t < T; ++t) th.emplace_back([&f, n, t, T] { f(n * t / T, n * (t + 1) / T, t); });
  f(0LL, n / T, 0);
  for (auto& x : th) x.join();
}

// ------------------------------------------------------------------ FFT
struct Plan1D {
  int n = 0;
  std::vector<int> fac;
  std::vector<cd> twf, twb;
  std::vector<cd> buf;
  explicit Plan1D(int n_) : n(n_), buf(n_) {
    int m = n;
    while (m % 4 == 0) { fac.push_back(4); m /= 4; }
    while (m % 2 == 0) { fac.push_back(2); m /= 2; }
    for (int p = 3; m > 1; p += 2)
      while (m % p == 0) { fac.push_back(p); m /= p; }
    fac.push_back(1);
    twf.resize(n);
    twb.resize(n);
    for (int j = 0; j < n; ++j) {
      long double a = 2.0L * 3.141592653589793238462643383279502884L * j / n;
      double c = (double)std::cos(a), s = (double)std::sin(a);
      twf[j] = cd(c, -s);
      twb[j] = cd(c, s);
    }
  }
  void rec(const cd* in, cd* out, int len, int istride, const int* f,
           const cd* tw, int twstep) const {
    if (len == 1) { out[0] = in[0]; return; }
    const int p = f[0];
    const int m = len / p;
    for (int r = 0; r < p; ++r)
      rec(in + (size_t)r * istride, out + (size_t)r * m, m, istride * p, f + 1, tw, twstep * p);
    cd v[64];
    for (int k = 0; k < m; ++k) {
      for (int r = 0; r < p; ++r) v[r] = out[r * m + k] * tw[(size_t)r * k * twstep];
      for (int q = 0; q < p; ++q) {
        cd s = 0.0;
        for (int r = 0; r < p; ++r) s += v[r] * tw[(size_t)((r * q) % p) * m * twstep];
        out[k + q * m] = s;
      }
    }
  }
  // in place, unnormalised; sign -1 forward (e^{-i}), +1 backward
  void exec(cd* data, int sign) {
    const cd* tw = sign < 0 ? twf.data() : twb.data();
    if ((n & (n - 1)) == 0) {  // power of two: radix-2 Stockham autosort
      cd* x = data;
      cd* y = buf.data();
      int st = 1;
      for (int len = n; len > 1; len >>= 1) {
        const int m = len >> 1;
        for (int p = 0; p < m; ++p) {
          const cd w = tw[(size_t)p * st];
          for (int q = 0; q < st; ++q) {
            const cd a = x[q + st * p];
            const cd b = x[q + st * (p + m)];
            y[q + st * (2 * p)] = a + b;
            y[q + st * (2 * p + 1)] = (a - b) * w;
          }
        }
        std::swap(x, y);
        st <<= 1;
      }
      if (x != data) std::copy(x, x + n, data);
      return;
    }
    std::copy(data, data + n, buf.begin());
    rec(buf.data(), data, n, 1, fac.data(), tw, 1);
  }
};

// H layout: [z][y][kx], nxh = nx/2+1.  Reference k-space layout: [ky][kz][kx].
struct FFT3 {
  int nx, ny, nz, nxh;
  Plan1D px, py, pz;
  std::vector<cd> H, line;
  FFT3(int nx_, int ny_, int nz_)
      : nx(nx_), ny(ny_), nz(nz_), nxh(nx_ / 2 + 1), px(nx_), py(ny_), pz(nz_),
        H((size_t)nx_ / 2 + 1 == 0 ? 0 : (size_t)(nx_ / 2 + 1) * ny_ * nz_),
        line(std::max(nx_, std::max(ny_, nz_))) {}

  // real [z][y][x] -> complex ref layout [ky][kz][kx]   (fftw r2c, unnormalised)
  void r2c(const double* r, cd* c) {
    const int nrows = ny * nz;
    par_for((nrows + 1) / 2, [&](long long b, long long e, int) {
      Plan1D p(px);
      std::vector<cd> z(nx);
      for (int row = 2 * (int)b; row < 2 * (int)e; row += 2) {
        const double* a = r + (size_t)row * nx;
        const double* bb = (row + 1 < nrows) ? r + (size_t)(row + 1) * nx : nullptr;
        for (int x = 0; x < nx; ++x) z[x] = cd(a[x], bb ? bb[x] : 0.0);
        p.exec(z.data(), -1);
        cd* ha = &H[(size_t)row * nxh];
        cd* hb = bb ? &H[(size_t)(row + 1) * nxh] : nullptr;
        for (int k = 0; k <= nx / 2; ++k) {
          cd zk = z[k], zm = std::conj(z[(nx - k) % nx]);
          ha[k] = 0.5 * (zk + zm);
          if (hb) hb[k] = cd(0.0, -0.5) * (zk - zm);
        }
      }
    });
    ypass(-1);
    zpass(-1);
    par_for(ny, [&](long long b, long long e, int) {
      for (int ky = (int)b; ky < (int)e; ++ky)
        for (int kz = 0; kz < nz; ++kz)
          for (int k = 0; k < nxh; ++k)
            c[((size_t)ky * nz + kz) * nxh + k] = H[((size_t)kz * ny + ky) * nxh + k];
    });
  }

  // the y transforms of every (z, kx) line of H
  void ypass(int sign) {
    par_for(nz, [&](long long b, long long e, int) {
      Plan1D p(py);
      std::vector<cd> ln(ny);
      for (int zz = (int)b; zz < (int)e; ++zz)
        for (int k = 0; k < nxh; ++k) {
          for (int y = 0; y < ny; ++y) ln[y] = H[((size_t)zz * ny + y) * nxh + k];
          p.exec(ln.data(), sign);
          for (int y = 0; y < ny; ++y) H[((size_t)zz * ny + y) * nxh + k] = ln[y];
        }
    });
  }
  // the z transforms of every (y, kx) line of H
  void zpass(int sign) {
    par_for(ny, [&](long long b, long long e, int) {
      Plan1D p(pz);
      std::vector<cd> ln(nz);
      for (int y = (int)b; y < (int)e; ++y)
        for (int k = 0; k < nxh; ++k) {
          for (int zz = 0; zz < nz; ++zz) ln[zz] = H[((size_t)zz * ny + y) * nxh + k];
          p.exec(ln.data(), sign);
          for (int zz = 0; zz < nz; ++zz) H[((size_t)zz * ny + y) * nxh + k] = ln[zz];
        }
    });
  }

  // complex ref layout -> real, unnormalised.  Complex inverse along z and y,
  // then a c2r along x that uses only the real parts of the kx=0 and kx=nx/2
  // entries (the semantics of a multi-dimensional FFTW c2r).
  void c2r(const cd* c, double* r) {
    par_for(ny, [&](long long b, long long e, int) {
      for (int ky = (int)b; ky < (int)e; ++ky)
        for (int kz = 0; kz < nz; ++kz)
          for (int k = 0; k < nxh; ++k)
            H[((size_t)kz * ny + ky) * nxh + k] = c[((size_t)ky * nz + kz) * nxh + k];
    });
    zpass(+1);
    ypass(+1);
    const int nrows = ny * nz;
    par_for((nrows + 1) / 2, [&](long long b, long long e, int) {
      Plan1D p(px);
      std::vector<cd> z(nx);
      for (int row = 2 * (int)b; row < 2 * (int)e; row += 2) {
        const cd* ha = &H[(size_t)row * nxh];
        const cd* hb = (row + 1 < nrows) ? &H[(size_t)(row + 1) * nxh] : nullptr;
        for (int k = 0; k <= nx / 2; ++k) {
          cd a = ha[k], bb = hb ? hb[k] : cd(0.0, 0.0);
          if (k == 0 || k == nx / 2) { a = cd(a.real(), 0.0); bb = cd(bb.real(), 0.0); }
          z[k] = a + cd(0.0, 1.0) * bb;
          if (k > 0 && k < nx / 2) z[nx - k] = std::conj(a) + cd(0.0, 1.0) * std::conj(bb);
        }
        p.exec(z.data(), +1);
        double* ra = r + (size_t)row * nx;
        double* rb = hb ? r + (size_t)(row + 1) * nx : nullptr;
        for (int x = 0; x < nx; ++x) {
          ra[x] = z[x].real();
          if (rb) rb[x] = z[x].imag();
        }
      }
    });
  }
};

}  // namespace

// ------------------------------------------------------------------ chain model
// This project's semiflexible chain (no reference counterpart: the reference
// calls the external beadrodpmer library, fixatom_semiflexible.cpp:144-191).
//   U = kbond/2 sum (|b_i| - b0)^2 + kappa sum (1 - cos theta_i)
// Overdamped step of length h = dt/2 with anisotropic friction about the local
// tangent t:  dx = h M F + sqrt(2 T h) M^{1/2} xi,
//   M = (1/zeta_perp)(I - t t) + (1/zeta_para) t t.
extern "C" void oracle_chain_force(const double* u, int n, int b, double kbond, double b0,
                                   double kappa, double* f, double* t) {
  f[0] = f[1] = f[2] = 0.0;
  auto P = [&](int i, int d) { return u[3 * (size_t)i + d]; };
  // bonds (b-1,b) and (b,b+1)
  for (int side = 0; side < 2; ++side) {
    int a = side == 0 ? b - 1 : b;
    if (a < 0 || a + 1 >= n) continue;
    double r[3] = {P(a + 1, 0) - P(a, 0), P(a + 1, 1) - P(a, 1), P(a + 1, 2) - P(a, 2)};
    double len = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    double g = kbond * (len - b0) / len;  // force on bead a is +g r, on a+1 is -g r
    double sgn = (a == b) ? 1.0 : -1.0;
    for (int d = 0; d < 3; ++d) f[d] += sgn * g * r[d];
  }
  // bending: angles centred at c in {b-1, b, b+1}
  if (kappa != 0.0)
    for (int c = b - 1; c <= b + 1; ++c) {
      if (c < 1 || c + 1 >= n) continue;
      double ra[3], rb[3];
      for (int d = 0; d < 3; ++d) { ra[d] = P(c, d) - P(c - 1, d); rb[d] = P(c + 1, d) - P(c, d); }
      double la = std::sqrt(ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2]);
      double lb = std::sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
      double cs = (ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2]) / (la * lb);
      for (int d = 0; d < 3; ++d) {
        double dca = rb[d] / (la * lb) - cs * ra[d] / (la * la);
        double dcb = ra[d] / (la * lb) - cs * rb[d] / (lb * lb);
        if (b == c - 1) f[d] += kappa * (-dca);
        else if (b == c) f[d] += kappa * (dca - dcb);
        else f[d] += kappa * dcb;
      }
    }
  // local tangent
  int lo = b > 0 ? b - 1 : b, hi = b + 1 < n ? b + 1 : b;
  double tv[3] = {P(hi, 0) - P(lo, 0), P(hi, 1) - P(lo, 1), P(hi, 2) - P(lo, 2)};
  double tl = std::sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
  for (int d = 0; d < 3; ++d) t[d] = tl > 0 ? tv[d] / tl : 0.0;
}

extern "C" void oracle_chain_displacement(const double* fc, const double* fp, const double* t,
                                          const double* xi, double dt, double zpara, double zperp,
                                          double temp, double* disp) {
  const double h = 0.5 * dt;
  double ft[3] = {fc[0] + fp[0], fc[1] + fp[1], fc[2] + fp[2]};
  double tf = t[0] * ft[0] + t[1] * ft[1] + t[2] * ft[2];
  double tx = t[0] * xi[0] + t[1] * xi[1] + t[2] * xi[2];
  double a = 1.0 / zperp, bpar = 1.0 / zpara - 1.0 / zperp;
  double sa = 1.0 / std::sqrt(zperp), sb = 1.0 / std::sqrt(zpara) - 1.0 / std::sqrt(zperp);
  double amp = std::sqrt(2.0 * temp * h);
  for (int d = 0; d < 3; ++d)
    disp[d] = h * (a * ft[d] + bpar * tf * t[d]) + amp * (sa * xi[d] + sb * tx * t[d]);
}

extern "C" void oracle_bead_gauss(uint32_t seed, uint64_t step, int half, int bead, double* xi) {
  double g[4];
  for (int call = 0; call < 2; ++call) {
    uint32_t ctr[4] = {(uint32_t)bead, (uint32_t)step, (uint32_t)(step >> 32) * 2u + (uint32_t)half,
                       0x4245414Du + (uint32_t)call};
    Philox::gen(ctr, seed, 0x53454d49u);
    double u1 = u53(ctr[0], ctr[1]), u2 = u53(ctr[2], ctr[3]);
    double r = std::sqrt(-2.0 * std::log(1.0 - u1));
    g[2 * call] = r * std::cos(6.283185307179586 * u2);
    g[2 * call + 1] = r * std::sin(6.283185307179586 * u2);
  }
  xi[0] = g[0]; xi[1] = g[1]; xi[2] = g[2];
}

namespace {

// ------------------------------------------------------------------ state
struct Swap {
  std::vector<int> send;            // source column indices
  std::vector<double> shift;        // 3 per sent atom
  int firstrecv = 0;
};

struct Range { int start, end; };

struct DragFix { std::vector<Range> ranges; double drag; };

struct SemiFix {
  std::vector<Range> ranges;
  double bondlength = 1.0, zeta_para = 1.0, zeta_perp = 1.0, bending = 0.0, temp = 0.0;
  double kbond = 100.0;
  uint32_t seed = 0;
  int noise = PHAFD_NOISE_PHILOX;
};

}  // namespace

struct oracle_ctx {
  std::string err;
  // domain
  double boxlo[3] = {0, 0, 0}, boxhi[3] = {0, 0, 0}, period[3] = {0, 0, 0};
  double sublo[3] = {0, 0, 0}, subhi[3] = {0, 0, 0};
  bool boxset = false, gridset = false, populated = false;
  int zghost = PHAFD_ZGHOST_PERIODIC;
  // grid
  int N[3] = {0, 0, 0};
  size_t nreal = 0, ncplx = 0;
  std::vector<double> phi, chempot, grad[3];
  std::vector<cd> ft_phi, ft_chempot, ft_grad[3];
  std::unique_ptr<FFT3> fft;
  // atoms
  int nowned = 0, ngathered = 0, nlocal = 0, nghost = 0, ntypes = 0;
  std::vector<double> xs, uxs, Fs;
  std::vector<int> tags, types, labels, images, moltags;
  // comm
  std::vector<Swap> swaps;
  double cutghost = 0.0;
  // neighbor
  double skin = 0.0, cutneigh = 0.0, cutneighsq = 0.0, triggersq = 0.0;
  bool neigh_set = false;
  std::vector<double> xholds;
  int ago = 0, ncalls = 0;
  // bins
  int nbinx = 0, nbiny = 0, nbinz = 0, mbinx = 0, mbiny = 0, mbinz = 0;
  int mbinxlo = 0, mbinylo = 0, mbinzlo = 0, mbins = 0;
  double binsizex = 0, binsizey = 0, binsizez = 0, bininvx = 0, bininvy = 0, bininvz = 0;
  std::vector<int> binhead, bins, atom2bin;
  std::set<int> local_atom_indices;
  std::vector<int> stencil_half, stencil_full;
  // lists (CSR instead of pages)
  std::vector<int> half_ilist, half_off, half_nb;
  std::vector<int> grid_ilist, grid_off, grid_nb;
  // pairs
  bool have_lj = false;
  double lj_cut = 0, lj1 = 0, lj2 = 0, lj_cutsq = 0;
  int ga_style = PHAFD_GRIDATOM_NONE;
  double ga_maxcut = 0;
  std::vector<double> ga_cutsq, ga_eps, ga_phi;
  // fixes
  bool have_conj = false, have_fh = false, have_gradphi = false, gradphi_once = false;
  double c_mobility = 1, c_temp = 1, c_volFH = 1, c_gamma = 1;
  int c_seed = 0;
  int c_noise = PHAFD_NOISE_REFERENCE;
  std::mt19937 c_gen;
  std::uniform_real_distribution<double> real_dist{-0.5, 0.5};
  double normalization = 0, complexprefactor = 0, realprefactor = 0, sqrtdt = 0;
  std::vector<double> qys, qzs;
  double fh_temp = 1, fh_volFH = 1, fh_chi = 1;
  long long num_less_zero = 0, num_great_zero = 0;
  std::vector<DragFix> drags;
  std::vector<SemiFix> semis;
  // integrate
  double dt = 0.0;
  long long timestep = 0, firststep = 0;
  bool setup_done = false;
  bool images_restored = false;
  int nan_flag = 0;
  int semi_fail = 0;
  // per-stage timing (seconds) for the CPU baseline
  double t_stage[8] = {0};

  // ---------------------------------------------------------- domain helpers
  double dx() const { return period[0] / N[0]; }
  double dy() const { return period[1] / N[1]; }
  double dz() const { return period[2] / N[2]; }
  double dqx() const { return 2 * 3.141592 / period[0]; }
  double dqy() const { return 2 * 3.141592 / period[2]; }
  double dqz() const { return 2 * 3.141592 / period[1]; }

  double& X(int d, int i) { return xs[3 * (size_t)i + d]; }
  double& UX(int d, int i) { return uxs[3 * (size_t)i + d]; }
  double& F(int d, int i) { return Fs[3 * (size_t)i + d]; }
  double& PHI(int z, int y, int x) { return phi[((size_t)z * N[1] + y) * N[0] + x]; }

  int set_image() const { return (IMGMAX << IMG2BITS) | (IMGMAX << IMGBITS) | IMGMAX; }

  void unmap(int i) {
    int image = images[i];
    int xbox = (image & IMGMASK) - IMGMAX;
    int ybox = (image >> IMGBITS & IMGMASK) - IMGMAX;
    int zbox = (image >> IMG2BITS) - IMGMAX;
    UX(0, i) = X(0, i) + xbox * period[0];
    UX(1, i) = X(1, i) + ybox * period[1];
    UX(2, i) = X(2, i) + zbox * period[2];
  }
  void map(int i) {
    int image = images[i];
    int xbox = (image & IMGMASK) - IMGMAX;
    int ybox = (image >> IMGBITS & IMGMASK) - IMGMAX;
    int zbox = (image >> IMG2BITS) - IMGMAX;
    X(0, i) = UX(0, i) - xbox * period[0];
    X(1, i) = UX(1, i) - ybox * period[1];
    X(2, i) = UX(2, i) - zbox * period[2];
  }

  // domain.cpp:102-163
  void pbc() {
    int idim, otherdims;
    for (int i = 0; i < nowned; i++) {
      if (X(0, i) < boxlo[0]) {
        X(0, i) += period[0];
        idim = images[i] & IMGMASK;
        otherdims = images[i] ^ idim;
        idim--;
        idim &= IMGMASK;
        images[i] = otherdims | idim;
      }
      if (X(0, i) >= boxhi[0]) {
        X(0, i) -= period[0];
        X(0, i) = (X(0, i) > boxlo[0] ? X(0, i) : boxlo[0]);
        idim = images[i] & IMGMASK;
        otherdims = images[i] ^ idim;
        idim++;
        idim &= IMGMASK;
        images[i] = otherdims | idim;
      }
      if (X(1, i) < boxlo[1]) {
        X(1, i) += period[1];
        idim = (images[i] >> IMGBITS) & IMGMASK;
        otherdims = images[i] ^ (idim << IMGBITS);
        idim--;
        idim &= IMGMASK;
        images[i] = otherdims | (idim << IMGBITS);
      }
      if (X(1, i) >= boxhi[1]) {
        X(1, i) -= period[1];
        X(1, i) = (X(1, i) > boxlo[1] ? X(1, i) : boxlo[1]);
        idim = (images[i] >> IMGBITS) & IMGMASK;
        otherdims = images[i] ^ (idim << IMGBITS);
        idim++;
        idim &= IMGMASK;
        images[i] = otherdims | (idim << IMGBITS);
      }
      if (X(2, i) < boxlo[2]) {
        X(2, i) += period[2];
        idim = images[i] >> IMG2BITS;
        otherdims = images[i] ^ (idim << IMG2BITS);
        idim--;
        idim &= IMGMASK;
        images[i] = otherdims | (idim << IMG2BITS);
      }
      if (X(2, i) >= boxhi[2]) {
        X(2, i) -= period[2];
        X(2, i) = (X(2, i) > boxlo[2] ? X(2, i) : boxlo[2]);
        idim = images[i] >> IMG2BITS;
        otherdims = images[i] ^ (idim << IMG2BITS);
        idim++;
        idim &= IMGMASK;
        images[i] = otherdims | (idim << IMG2BITS);
      }
      unmap(i);
    }
  }

  // ---------------------------------------------------------- comm (1 rank)
  void append_copy(int src, const double sh[3], int label) {
    xs.push_back(X(0, src) + sh[0]);
    xs.push_back(X(1, src) + sh[1]);
    xs.push_back(X(2, src) + sh[2]);
    Fs.push_back(0.0); Fs.push_back(0.0); Fs.push_back(0.0);
    tags.push_back(tags[src]);
    types.push_back(types[src]);
    labels.push_back(label);
  }

  // comm_brick.cpp:263-426 for nprocs == 1
  void borders() {
    const size_t n = (size_t)nowned;
    xs.resize(3 * n); Fs.resize(3 * n);
    tags.resize(n); types.resize(n); labels.resize(n);
    ngathered = nlocal = nghost = 0;
    swaps.clear();
    // z dimension
    const double zprd = period[2];
    const int subloz = (int)sublo[2];   // comm_brick.cpp:122-123 stores bounds as int
    const int subhiz = (int)subhi[2];
    if (zghost == PHAFD_ZGHOST_RANK1) {
      const double lo = subhiz - cutghost;
      const double hi = subloz + cutghost;
      Swap s; s.firstrecv = nowned;
      std::vector<int> lab;
      for (int i = 0; i < nowned; i++) {
        double z = X(2, i);
        if (z >= subloz && z <= subhiz) {
          s.send.push_back(i); s.shift.insert(s.shift.end(), {0.0, 0.0, 0.0}); lab.push_back(LOCAL);
        } else if (z >= lo) {
          s.send.push_back(i); s.shift.insert(s.shift.end(), {0.0, 0.0, -zprd}); lab.push_back(GHOST);
        } else if (z <= hi) {
          s.send.push_back(i); s.shift.insert(s.shift.end(), {0.0, 0.0, zprd}); lab.push_back(GHOST);
        }
      }
      for (size_t m = 0; m < s.send.size(); ++m) {
        append_copy(s.send[m], &s.shift[3 * m], lab[m]);
        if (lab[m] == LOCAL) nlocal++;
      }
      ngathered += (int)s.send.size();
      swaps.push_back(std::move(s));
    } else {
      // periodic z images, as the reference's multi-rank z swaps produce them
      Swap s; s.firstrecv = nowned;
      for (int i = 0; i < nowned; i++) { s.send.push_back(i); s.shift.insert(s.shift.end(), {0.0, 0.0, 0.0}); }
      for (size_t m = 0; m < s.send.size(); ++m) append_copy(s.send[m], &s.shift[3 * m], LOCAL);
      nlocal += (int)s.send.size();
      ngathered += (int)s.send.size();
      swaps.push_back(std::move(s));
      for (int ineed = 0; ineed < 2; ++ineed) {
        Swap g; g.firstrecv = nowned + ngathered;
        for (int i = 0; i < nowned; i++) {
          double z = X(2, i);
          bool take = (ineed == 0) ? (z <= boxlo[2] + cutghost) : (z >= boxhi[2] - cutghost);
          if (take) { g.send.push_back(i); g.shift.insert(g.shift.end(), {0.0, 0.0, ineed == 0 ? zprd : -zprd}); }
        }
        for (size_t m = 0; m < g.send.size(); ++m) append_copy(g.send[m], &g.shift[3 * m], GHOST);
        ngathered += (int)g.send.size();
        swaps.push_back(std::move(g));
      }
    }
    // y then x swaps (self swaps, LAMMPS style)
    for (int dim = 1; dim >= 0; dim--) {
      int nfirst = nowned, nlast = nowned;
      for (int ineed = 0; ineed < 2; ineed++) {
        double lo, hi, sh[3] = {0, 0, 0};
        if (ineed % 2 == 0) { lo = -BIG; hi = boxlo[dim] + cutghost; sh[dim] = period[dim]; }
        else { lo = boxhi[dim] - cutghost; hi = BIG; sh[dim] = -period[dim]; }
        if (ineed % 2 == 0) { nfirst = nlast; nlast = nowned + ngathered; }
        Swap s; s.firstrecv = nowned + ngathered;
        for (int i = nfirst; i < nlast; i++)
          if (X(dim, i) >= lo && X(dim, i) <= hi) {
            s.send.push_back(i);
            s.shift.insert(s.shift.end(), {sh[0], sh[1], sh[2]});
          }
        for (size_t m = 0; m < s.send.size(); ++m) append_copy(s.send[m], &s.shift[3 * m], GHOST);
        ngathered += (int)s.send.size();
        swaps.push_back(std::move(s));
      }
    }
    nghost = ngathered - nlocal;
  }

  // comm_brick.cpp:190-224
  void forward_comm() {
    for (auto& s : swaps)
      for (size_t m = 0; m < s.send.size(); ++m) {
        int j = s.send[m], dst = s.firstrecv + (int)m;
        X(0, dst) = X(0, j) + s.shift[3 * m + 0];
        X(1, dst) = X(1, j) + s.shift[3 * m + 1];
        X(2, dst) = X(2, j) + s.shift[3 * m + 2];
      }
  }
  // comm_brick.cpp:228-258
  void reverse_comm() {
    for (int w = (int)swaps.size() - 1; w >= 0; --w) {
      auto& s = swaps[w];
      for (size_t m = 0; m < s.send.size(); ++m) {
        int j = s.send[m], src = s.firstrecv + (int)m;
        F(0, j) += F(0, src);
        F(1, j) += F(1, src);
        F(2, j) += F(2, src);
      }
    }
  }

  // ---------------------------------------------------------- bins
  void setup_bins() {  // nbin_standard.cpp:53-175
    double bsubboxlo[3], bsubboxhi[3], bbox[3];
    for (int d = 0; d < 3; ++d) {
      bsubboxlo[d] = sublo[d] - cutneigh;
      bsubboxhi[d] = subhi[d] + cutneigh;
      bbox[d] = boxhi[d] - boxlo[d];
    }
    double binsize_optimal = 0.5 * cutneigh;
    if (binsize_optimal == 0.0) binsize_optimal = bbox[0];
    double binsizeinv = 1.0 / binsize_optimal;
    nbinx = (int)(bbox[0] * binsizeinv);
    nbiny = (int)(bbox[1] * binsizeinv);
    nbinz = (int)(bbox[2] * binsizeinv);
    if (nbinx == 0) nbinx = 1;
    if (nbiny == 0) nbiny = 1;
    if (nbinz == 0) nbinz = 1;
    binsizex = bbox[0] / nbinx;
    binsizey = bbox[1] / nbiny;
    binsizez = bbox[2] / nbinz;
    bininvx = 1.0 / binsizex;
    bininvy = 1.0 / binsizey;
    bininvz = 1.0 / binsizez;
    if (binsize_optimal * bininvx > 100 || binsize_optimal * bininvy > 100 ||
        binsize_optimal * bininvz > 100)
      throw std::runtime_error("Cannot use neighbor bins - box size << cutoff");
    int mbinxhi, mbinyhi, mbinzhi;
    double coord;
    coord = bsubboxlo[0] - SMALL * bbox[0];
    mbinxlo = (int)((coord - boxlo[0]) * bininvx);
    if (coord < boxlo[0]) mbinxlo = mbinxlo - 1;
    coord = bsubboxhi[0] + SMALL * bbox[0];
    mbinxhi = (int)((coord - boxlo[0]) * bininvx);
    coord = bsubboxlo[1] - SMALL * bbox[1];
    mbinylo = (int)((coord - boxlo[1]) * bininvy);
    if (coord < boxlo[1]) mbinylo = mbinylo - 1;
    coord = bsubboxhi[1] + SMALL * bbox[1];
    mbinyhi = (int)((coord - boxlo[1]) * bininvy);
    coord = bsubboxlo[2] - SMALL * bbox[2];
    mbinzlo = (int)((coord - boxlo[2]) * bininvz);
    if (coord < boxlo[2]) mbinzlo = mbinzlo - 1;
    coord = bsubboxhi[2] + SMALL * bbox[2];
    mbinzhi = (int)((coord - boxlo[2]) * bininvz);
    mbinxlo -= 1; mbinxhi += 1; mbinx = mbinxhi - mbinxlo + 1;
    mbinylo -= 1; mbinyhi += 1; mbiny = mbinyhi - mbinylo + 1;
    mbinzlo -= 1; mbinzhi += 1; mbinz = mbinzhi - mbinzlo + 1;
    mbins = mbinx * mbiny * mbinz + 1;
    binhead.assign(mbins, -1);
  }

  // nbin.cpp:61-94 and npair.cpp:125-158 (same arithmetic)
  int coord2bin(double x, double y, double z) const {
    int ix, iy, iz;
    if (x >= boxhi[0]) ix = (int)((x - boxhi[0]) * bininvx) + nbinx;
    else if (x >= boxlo[0]) { ix = (int)((x - boxlo[0]) * bininvx); ix = std::min(ix, nbinx - 1); }
    else ix = (int)((x - boxlo[0]) * bininvx) - 1;
    if (y >= boxhi[1]) iy = (int)((y - boxhi[1]) * bininvy) + nbiny;
    else if (y >= boxlo[1]) { iy = (int)((y - boxlo[1]) * bininvy); iy = std::min(iy, nbiny - 1); }
    else iy = (int)((y - boxlo[1]) * bininvy) - 1;
    if (z >= boxhi[2]) iz = (int)((z - boxhi[2]) * bininvz) + nbinz;
    else if (z >= boxlo[2]) { iz = (int)((z - boxlo[2]) * bininvz); iz = std::min(iz, nbinz - 1); }
    else iz = (int)((z - boxlo[2]) * bininvz) - 1;
    return (iz - mbinzlo) * mbiny * mbinx + (iy - mbinylo) * mbinx + (ix - mbinxlo);
  }

  void bin_atoms() {  // nbin_standard.cpp:181-229
    std::fill(binhead.begin(), binhead.end(), -1);
    local_atom_indices.clear();
    const int nstart = nowned, nall = nowned + ngathered;
    atom2bin.assign(nall - nstart, 0);
    bins.assign(nall - nstart, -1);
    for (int i = nall - 1; i >= nstart; i--) {
      if (labels[i] == GHOST) {
        int ibin = coord2bin(X(0, i), X(1, i), X(2, i));
        if (ibin < 0 || ibin >= mbins) throw std::runtime_error("bead outside bin range");
        atom2bin[i - nstart] = ibin;
        bins[i - nstart] = binhead[ibin];
        binhead[ibin] = i;
      } else {
        local_atom_indices.insert(i);
      }
    }
    for (auto rit = local_atom_indices.rbegin(); rit != local_atom_indices.rend(); ++rit) {
      int ibin = coord2bin(X(0, *rit), X(1, *rit), X(2, *rit));
      if (ibin < 0 || ibin >= mbins) throw std::runtime_error("bead outside bin range");
      atom2bin[*rit - nstart] = ibin;
      bins[*rit - nstart] = binhead[ibin];
      binhead[ibin] = *rit;
    }
  }

  double bin_distance(int i, int j, int k) const {  // nstencil.cpp:126-143
    double delx, dely, delz;
    if (i > 0) delx = (i - 1) * binsizex; else if (i == 0) delx = 0.0; else delx = (i + 1) * binsizex;
    if (j > 0) dely = (j - 1) * binsizey; else if (j == 0) dely = 0.0; else dely = (j + 1) * binsizey;
    if (k > 0) delz = (k - 1) * binsizez; else if (k == 0) delz = 0.0; else delz = (k + 1) * binsizez;
    return delx * delx + dely * dely + delz * delz;
  }

  void create_stencils() {  // nstencil.cpp:101-120, nstencil_{half,full}_bin_3d.cpp
    int sx = (int)(cutneigh * bininvx); if (sx * binsizex < cutneigh) sx++;
    int sy = (int)(cutneigh * bininvy); if (sy * binsizey < cutneigh) sy++;
    int sz = (int)(cutneigh * bininvz); if (sz * binsizez < cutneigh) sz++;
    stencil_half.clear();
    stencil_full.clear();
    for (int k = 0; k <= sz; k++)
      for (int j = -sy; j <= sy; j++)
        for (int i = -sx; i <= sx; i++)
          if (k > 0 || j > 0 || (j == 0 && i > 0))
            if (bin_distance(i, j, k) < cutneighsq)
              stencil_half.push_back(k * mbiny * mbinx + j * mbinx + i);
    for (int k = -sz; k <= sz; k++)
      for (int j = -sy; j <= sy; j++)
        for (int i = -sx; i <= sx; i++)
          if (bin_distance(i, j, k) < cutneighsq)
            stencil_full.push_back(k * mbiny * mbinx + j * mbinx + i);
  }

  // npair_half_bin_newton.cpp:38-124
  void build_half() {
    half_ilist.clear(); half_off.assign(1, 0); half_nb.clear();
    const int nstart = nowned;
    for (int i : local_atom_indices) {
      const double xtmp = X(0, i), ytmp = X(1, i), ztmp = X(2, i);
      for (int j = bins[i - nstart]; j >= 0; j = bins[j - nstart]) {
        if (!local_atom_indices.count(j)) {
          if (X(2, j) < ztmp) continue;
          if (X(2, j) == ztmp) {
            if (X(1, j) < ytmp) continue;
            if (X(1, j) == ytmp && X(0, j) < xtmp) continue;
          }
        }
        double delx = xtmp - X(0, j), dely = ytmp - X(1, j), delz = ztmp - X(2, j);
        double rsq = delx * delx + dely * dely + delz * delz;
        if (rsq <= cutneighsq) half_nb.push_back(j);
      }
      const int ibin = atom2bin[i - nstart];
      for (int s : stencil_half)
        for (int j = binhead[ibin + s]; j >= 0; j = bins[j - nstart]) {
          double delx = xtmp - X(0, j), dely = ytmp - X(1, j), delz = ztmp - X(2, j);
          double rsq = delx * delx + dely * dely + delz * delz;
          if (rsq <= cutneighsq) half_nb.push_back(j);
        }
      half_ilist.push_back(i);
      half_off.push_back((int)half_nb.size());
    }
  }

  // npair_grid_bin.cpp:22-127
  void build_grid() {
    grid_ilist.clear(); grid_off.assign(1, 0); grid_nb.clear();
    const int nstart = nowned;
    int gridindex = 0;
    for (int k = 0; k < N[2]; k++) {
      const double ztmp = (k + 0) * dz() + boxlo[2];
      for (int j = 0; j < N[1]; j++) {
        const double ytmp = j * dy() + boxlo[1];
        for (int i = 0; i < N[0]; i++) {
          const double xtmp = i * dx() + boxlo[0];
          const size_t before = grid_nb.size();
          const int ibin = coord2bin(xtmp, ytmp, ztmp);
          for (int s : stencil_full)
            for (int ai = binhead[ibin + s]; ai >= 0; ai = bins[ai - nstart]) {
              double delx = xtmp - X(0, ai), dely = ytmp - X(1, ai), delz = ztmp - X(2, ai);
              double rsq = delx * delx + dely * dely + delz * delz;
              if (rsq <= cutneighsq) grid_nb.push_back(ai);
            }
          if (grid_nb.size() > before) {
            grid_ilist.push_back(gridindex++);
            grid_off.push_back((int)grid_nb.size());
          } else {
            gridindex++;
          }
        }
      }
    }
  }

  void neighbor_build() {  // neighbor.cpp:99-125
    ago = 0;
    ncalls++;
    xholds.assign(xs.begin(), xs.begin() + 3 * (size_t)nowned);
    bin_atoms();
    if (have_lj) build_half();
    if (ga_style != PHAFD_GRIDATOM_NONE) build_grid();
  }

  bool neighbor_decide() {  // neighbor.cpp:70-97 (delay 0, every 1, dist_check on)
    ago++;
    int flag = 0;
    for (int i = 0; i < nowned; i++) {
      double d0 = X(0, i) - xholds[3 * (size_t)i];
      double d1 = X(1, i) - xholds[3 * (size_t)i + 1];
      double d2 = X(2, i) - xholds[3 * (size_t)i + 2];
      double rsq = d0 * d0 + d1 * d1 + d2 * d2;
      if (rsq > triggersq) flag = 1;
    }
    return flag != 0;
  }

  // ---------------------------------------------------------- pairs
  void pair_lj() {  // pair_lj_cut.cpp:46-101
    for (size_t ii = 0; ii < half_ilist.size(); ++ii) {
      const int i = half_ilist[ii];
      const double xtmp = X(0, i), ytmp = X(1, i), ztmp = X(2, i);
      for (int jj = half_off[ii]; jj < half_off[ii + 1]; ++jj) {
        const int j = half_nb[jj];
        double delx = xtmp - X(0, j), dely = ytmp - X(1, j), delz = ztmp - X(2, j);
        double rsq = delx * delx + dely * dely + delz * delz;
        if (rsq < lj_cutsq) {
          double r2inv = 1.0 / rsq;
          double r6inv = r2inv * r2inv * r2inv;
          double forcelj = r6inv * (lj1 * r6inv - lj2);
          double fpair = forcelj * r2inv;
          F(0, i) += delx * fpair; F(1, i) += dely * fpair; F(2, i) += delz * fpair;
          F(0, j) -= delx * fpair; F(1, j) -= dely * fpair; F(2, j) -= delz * fpair;
        }
      }
    }
  }

  void pair_gridatom() {  // pair_gridatom_*.cpp compute()
    const double Ox = sublo[0], Oy = sublo[1], Oz = sublo[2];
    const double dv = dx() * dy() * dz();
    for (size_t iibin = 0; iibin < grid_ilist.size(); ++iibin) {
      const int gridindex = grid_ilist[iibin];
      const int i = gridindex / (N[0] * N[1]);
      const int j = (gridindex / N[0]) % N[1];
      const int k = gridindex % N[0];
      const double xtmp = k * dx() + Ox, ytmp = j * dy() + Oy, ztmp = i * dz() + Oz;
      const size_t node = ((size_t)i * N[1] + j) * N[0] + k;
      for (int ajj = grid_off[iibin]; ajj < grid_off[iibin + 1]; ++ajj) {
        const int aj = grid_nb[ajj];
        const int t = types[aj];
        double delx = xtmp - X(0, aj), dely = ytmp - X(1, aj), delz = ztmp - X(2, aj);
        double rsq = delx * delx + dely * dely + delz * delz;
        if (ga_style == PHAFD_GRIDATOM_GAUSSIAN) {
          if (rsq <= ga_cutsq[t]) {
            rsq /= ga_cutsq[t];
            double expfac = (std::exp(-rsq / 2.0) - std::exp(-0.5)) * std::exp(0.5) * ga_eps[t];
            double delphi = phi[node] - ga_phi[t];
            chempot[node] += 2 * delphi * expfac;
            expfac *= 2 * delphi * dv;
            F(0, aj) -= grad[0][node] * expfac;
            F(1, aj) -= grad[1][node] * expfac;
            F(2, aj) -= grad[2][node] * expfac;
          }
        } else if (ga_style == PHAFD_GRIDATOM_LJISH) {
          if (rsq < ga_cutsq[t]) {
            rsq /= ga_cutsq[t];
            double expfac = std::exp(-1. / (1 - rsq) + 1) * ga_eps[t];
            double delphi = phi[node] - ga_phi[t];
            chempot[node] += 2 * delphi * expfac;
            expfac *= 2 * delphi * dv;
            F(0, aj) -= grad[0][node] * expfac;
            F(1, aj) -= grad[1][node] * expfac;
            F(2, aj) -= grad[2][node] * expfac;
          }
        } else if (ga_style == PHAFD_GRIDATOM_LJISH_LINEAR) {
          if (rsq < ga_cutsq[t]) {
            rsq /= ga_cutsq[t];
            double expfac = -1 * std::exp(-1. / (1 - rsq) + 1) * ga_eps[t];
            chempot[node] += expfac;
            expfac *= dv;
            F(0, aj) -= grad[0][node] * expfac;
            F(1, aj) -= grad[1][node] * expfac;
            F(2, aj) -= grad[2][node] * expfac;
          }
        }
      }
    }
  }

  void pairs_compute() {
    if (have_lj) pair_lj();
    if (ga_style != PHAFD_GRIDATOM_NONE) pair_gridatom();
  }

  // ---------------------------------------------------------- field fixes
  void gradient() {  // fixgrid_conjugate.cpp:62-116
    fft->r2c(phi.data(), ft_phi.data());
    const int nzt = N[1];  // transposed "Nz" = ky count
    const int nyt = N[2];  // transposed "Ny" = kz count
    const int nxt = N[0] / 2 + 1;
    const int globalNy = N[2], globalNz = N[1];
    const cd idqx(0, dqx()), idqy(0, dqy()), idqz(0, dqz());
    par_for(nzt, [&](long long b, long long e, int) {
      for (int i = (int)b; i < (int)e; i++) {
        double l = (i > globalNz / 2) ? -globalNz + i : i;
        for (int j = 0; j < nyt; j++) {
          double m = (j > globalNy / 2) ? -globalNy + j : j;
          for (int k = 0; k < nxt; k++) {
            double n = k;
            size_t idx = ((size_t)i * nyt + j) * nxt + k;
            ft_grad[0][idx] = ft_phi[idx] * idqx * n;
            ft_grad[1][idx] = ft_phi[idx] * idqy * m;
            ft_grad[2][idx] = ft_phi[idx] * idqz * l;
          }
        }
      }
    });
    // grid.cpp:262-280: the y and z c2r outputs are swapped on purpose
    fft->c2r(ft_grad[0].data(), grad[0].data());
    fft->c2r(ft_grad[1].data(), grad[2].data());
    fft->c2r(ft_grad[2].data(), grad[1].data());
    const double factor = (double)N[0] * N[1] * N[2];
    for (int d = 0; d < 3; ++d)
      par_for((long long)grad[d].size(), [&](long long b, long long e, int) {
        for (long long n = b; n < e; ++n) grad[d][n] /= factor;
      });
  }

  void floryhuggins() {  // fixgrid_floryhuggins.cpp:65-85
    std::vector<long long> lt(g_threads, 0), gt(g_threads, 0);
    par_for((long long)nreal, [&](long long b, long long e, int t) {
      for (long long n = b; n < e; ++n) {
        if (phi[n] <= 0) { phi[n] = -phi[n]; lt[t] += 1; }
        else if (phi[n] >= 1) { phi[n] = 1 - (phi[n] - 1); gt[t] += 1; }
        chempot[n] += fh_temp / fh_volFH * (std::log(phi[n] / (1 - phi[n])) + fh_chi * (1 - 2 * phi[n]));
      }
    });
    for (int t = 0; t < g_threads; ++t) { num_less_zero += lt[t]; num_great_zero += gt[t]; }
  }

  void set_qs() {  // conjugate.cpp:130-161
    const int localNz = N[1], localNy = N[2];
    const int globalNy = N[2], globalNz = N[1];
    const double dyq = dqy(), dzq = dqz();
    qys.resize(localNy);
    qzs.resize(localNz);
    for (int i = 0; i < localNz; i++)
      qzs[i] = (i > globalNz / 2) ? -dzq * (globalNz - i) : dzq * i;
    for (int j = 0; j < localNy; j++)
      qys[j] = (j > globalNy / 2) ? -dyq * (globalNy - j) : dyq * j;
  }

  void reset_dt() {  // conjugate_volfrac.cpp:72-86
    double invLcubed = 1.0 / (period[0] * period[1] * period[2]);
    normalization = 1.0 / ((double)N[0] * N[2] * N[1]);
    complexprefactor = std::sqrt(12 * c_temp * c_mobility * invLcubed);
    realprefactor = std::sqrt(24 * c_temp * c_mobility * invLcubed);
    sqrtdt = std::sqrt(dt);
  }

  // Philox noise for a canonical mode (kx, ky, kz); same function on the GPU.
  // One Philox4x32-10 call serves the mode pair (kz, kz ^ 16): words (c0, c1)
  // for the mode with bit 4 of kz clear, (c2, c3) for the other; each word
  // gives a 24-bit uniform, exact in float and double.
  double philox_u(int kx, int ky, int kz, int comp) const {
    uint64_t idx = ((uint64_t)kx * N[2] + (kz & ~16)) * N[1] + ky;
    uint32_t ctr[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), (uint32_t)timestep, 0x46494c44u};
    Philox::gen(ctr, (uint32_t)c_seed, 0x434f4e4au);
    const int w = ((kz >> 4) & 1) * 2 + comp;
    return (double)(ctr[w] >> 8) * (1.0 / 16777216.0) - 0.5;
  }

  double draw(int i, int j, int k, int comp) {
    if (c_noise == PHAFD_NOISE_REFERENCE) return real_dist(c_gen);
    if (c_noise == PHAFD_NOISE_PHILOX) return philox_u(k, i, j, comp);
    return 0.0;
  }

  cd& FT(int i, int j, int k) { return ft_phi[((size_t)i * N[2] + j) * (N[0] / 2 + 1) + k]; }
  cd& FTM(int i, int j, int k) { return ft_chempot[((size_t)i * N[2] + j) * (N[0] / 2 + 1) + k]; }

  void complex_update(int i, int j, int k) {  // conjugate_volfrac.cpp:89-113
    double qz = qzs[i], qy = qys[j], qx = dqx() * k;
    double q2 = qx * qx + qy * qy + qz * qz;
    cd noise;
    noise.real(complexprefactor * std::sqrt(q2) * sqrtdt * draw(i, j, k, 0));
    noise.imag(complexprefactor * std::sqrt(q2) * sqrtdt * draw(i, j, k, 1));
    FT(i, j, k) = (FT(i, j, k) - c_mobility * q2 * dt * (FTM(i, j, k) + c_temp / c_volFH * c_gamma * q2 * FT(i, j, k))) * normalization + noise;
  }
  void real_update(int i, int j, int k) {  // conjugate_volfrac.cpp:116-136
    double qz = qzs[i], qy = qys[j], qx = dqx() * k;
    double q2 = qx * qx + qy * qy + qz * qz;
    double noise = realprefactor * std::sqrt(q2) * sqrtdt * draw(i, j, k, 0);
    FT(i, j, k) = (FT(i, j, k) - c_mobility * q2 * dt * (FTM(i, j, k) + c_temp / c_volFH * c_gamma * q2 * FT(i, j, k))) * normalization + noise;
  }

  void single(int nx) {  // conjugate.cpp:255-302
    const int localNz = N[1], localNy = N[2];
    int nz = 0;
    for (int j = 1; j < localNy / 2; j++) { complex_update(nz, j, nx); FT(nz, localNy - j, nx) = std::conj(FT(nz, j, nx)); }
    for (int i = 1; i < localNz / 2; i++)
      for (int j = 1; j < localNy / 2; j++) { complex_update(i, j, nx); FT(localNz - i, localNy - j, nx) = std::conj(FT(i, j, nx)); }
    for (int i = localNz / 2 + 1; i < localNz; i++)
      for (int j = 1; j < localNy / 2; j++) { complex_update(i, j, nx); FT(localNz - i, localNy - j, nx) = std::conj(FT(i, j, nx)); }
    nz = localNz / 2;
    for (int j = 1; j < localNy / 2; j++) { complex_update(nz, j, nx); FT(nz, localNy - j, nx) = std::conj(FT(nz, j, nx)); }
  }
  void line_single(int nx) {  // conjugate.cpp:304-327
    const int localNz = N[1], localNy = N[2];
    int ny = 0;
    for (int i = 1; i < localNz / 2; i++) { complex_update(i, ny, nx); FT(localNz - i, ny, nx) = std::conj(FT(i, ny, nx)); }
    ny = localNy / 2;
    for (int i = localNz / 2 + 1; i < localNz; i++) { complex_update(i, ny, nx); FT(localNz - i, ny, nx) = std::conj(FT(i, ny, nx)); }
  }

  void conjugate_update() {  // conjugate.cpp:163-247 (nprocs == 1)
    const int localNx = N[0] / 2 + 1, localNz = N[1], localNy = N[2];
    const int globalNz = N[1];
    // the reference generator's draws follow this loop order: split only
    // for the counter-based and the silent noise
    auto bulk = [&](long long b, long long e, int) {
      for (int nz = (int)b; nz < (int)e; nz++)
        for (int ny = 0; ny < localNy; ny++)
          for (int nx = 1; nx < localNx - 1; nx++) complex_update(nz, ny, nx);
    };
    if (c_noise == PHAFD_NOISE_REFERENCE) bulk(0, localNz, 0);
    else par_for(localNz, bulk);
    for (int nx = 0; nx < localNx; nx += localNx - 1) { single(nx); line_single(nx); }
    {
      int nx = localNx - 1;
      real_update(0, localNy / 2, 0);
      real_update(0, localNy / 2, nx);
      real_update(0, 0, nx);
      FT(0, 0, 0) *= normalization;  // origin_update
    }
    {
      int nz = globalNz / 2, nx = localNx - 1;
      real_update(nz, 0, 0);
      real_update(nz, localNy / 2, 0);
      real_update(nz, localNy / 2, nx);
      real_update(nz, 0, nx);
    }
  }

  // ---------------------------------------------------------- bead fixes
  void drag_half() {  // fixatom_drag.cpp:43-66
    for (auto& f : drags)
      for (auto& r : f.ranges)
        for (int j = r.start; j < r.end; j++)
          for (int d = 0; d < 3; ++d) X(d, j) += f.drag * F(d, j) * dt * 0.5;
  }

  void semi_half(int half) {
    for (auto& f : semis)
      for (auto& r : f.ranges) {
        const int n = r.end - r.start;
        std::vector<double> fc(3 * (size_t)n, 0.0), tang(3 * (size_t)n, 0.0);
        for (int b = 0; b < n; ++b) oracle_chain_force(&uxs[3 * (size_t)r.start], n, b, f.kbond, f.bondlength, f.bending, &fc[3 * (size_t)b], &tang[3 * (size_t)b]);
        for (int b = 0; b < n; ++b) {
          const int i = r.start + b;
          double xi[3] = {0, 0, 0};
          if (f.noise == PHAFD_NOISE_PHILOX && f.temp > 0) oracle_bead_gauss(f.seed, (uint64_t)timestep, half, i, xi);
          double disp[3];
          oracle_chain_displacement(&fc[3 * (size_t)b], &Fs[3 * (size_t)i], &tang[3 * (size_t)b], xi, dt, f.zeta_para, f.zeta_perp, f.temp, disp);
          for (int d = 0; d < 3; ++d) UX(d, i) += disp[d];
          for (int d = 0; d < 3; ++d) if (!std::isfinite(UX(d, i))) semi_fail = 1;
        }
        for (int i = r.start; i < r.end; ++i) map(i);
      }
  }

  // ---------------------------------------------------------- schedule
  void setup() {  // integrate.cpp:33-88
    if (nowned > 0) {
      if (!neigh_set) throw std::runtime_error("neighbor must be set before run");
      pbc();
      borders();
      neighbor_build();
    }
    std::fill(Fs.begin(), Fs.end(), 0.0);
    reset_dt();
    for (auto& f : semis)  // fixatom_semiflexible.cpp:114-140; skipped for beads restored from a dump
      if (!images_restored)
      for (auto& r : f.ranges)
        for (int mu = r.start + 1; mu < r.end; mu++) {
          double d0 = UX(0, mu) - UX(0, mu - 1), d1 = UX(1, mu) - UX(1, mu - 1), d2 = UX(2, mu) - UX(2, mu - 1);
          double delta = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) - f.bondlength;
          if (std::abs(delta) > 1e-3)
            throw std::runtime_error("Adjacent atom displacements do not match the FixAtomSemiFlexible bondlength specified.");
        }
    setup_done = true;
  }

  void step() {  // integrate.cpp:105-203
    timestep++;
    auto tick = []() { return std::chrono::steady_clock::now(); };
    auto t0 = tick();
    // fixgrid_gradphi.cpp:45: "once" tests timestep == firststep after the
    // increment above, which never holds inside a run
    if (have_conj || (have_gradphi && (!gradphi_once || timestep == firststep))) gradient();
    auto t1 = tick();
    if (nowned > 0 && neighbor_decide()) { pbc(); borders(); neighbor_build(); }
    else forward_comm();
    auto t2 = tick();
    std::fill(Fs.begin(), Fs.end(), 0.0);
    pairs_compute();
    reverse_comm();
    drag_half();
    semi_half(0);
    std::fill(chempot.begin(), chempot.end(), 0.0);
    std::fill(Fs.begin(), Fs.end(), 0.0);
    pairs_compute();
    reverse_comm();
    auto t3 = tick();
    if (have_fh) floryhuggins();
    auto t4 = tick();
    if (have_conj) fft->r2c(chempot.data(), ft_chempot.data());
    auto t5 = tick();
    if (have_conj) conjugate_update();
    drag_half();
    semi_half(1);
    auto t6 = tick();
    if (have_conj) fft->c2r(ft_phi.data(), phi.data());
    auto t7 = tick();
    if (std::isnan(phi[0])) nan_flag = 1;
    auto sec = [](auto a, auto b) { return std::chrono::duration<double>(b - a).count(); };
    t_stage[0] += sec(t0, t1); t_stage[1] += sec(t1, t2); t_stage[2] += sec(t2, t3);
    t_stage[3] += sec(t3, t4); t_stage[4] += sec(t4, t5); t_stage[5] += sec(t5, t6);
    t_stage[6] += sec(t6, t7);
  }
};

// ====================================================================== C ABI
#define GUARD(ctx, body)                          \
  try {                                           \
    body;                                         \
    return 0;                                     \
  } catch (const std::exception& e) {             \
    if (ctx) (ctx)->err = e.what();               \
    return PHAFD_ERR_INVALID;                     \
  }

extern "C" {

int oracle_set_threads(int n) {
  g_threads = std::max(1, std::min(n, 256));
  return 0;
}

int oracle_ctx_create(oracle_ctx** out) {
  *out = new oracle_ctx();
  return 0;
}
void oracle_ctx_destroy(oracle_ctx* c) { delete c; }
const char* oracle_last_error(oracle_ctx* c) { return c ? c->err.c_str() : "null ctx"; }

int oracle_set_zghost(oracle_ctx* c, int mode) {
  GUARD(c, {
    if (mode != PHAFD_ZGHOST_RANK1 && mode != PHAFD_ZGHOST_PERIODIC) throw std::invalid_argument("bad zghost mode");
    c->zghost = mode;
  })
}

int oracle_domain(oracle_ctx* c, const double* boxlo, const double* period) {
  GUARD(c, {
    for (int d = 0; d < 3; ++d) {
      c->period[d] = period[d];
      c->boxlo[d] = boxlo[d];
      c->boxhi[d] = boxlo[d] + period[d];
    }
    c->boxset = true;
  })
}

int oracle_grid_style(oracle_ctx* c, int nx, int ny, int nz) {
  GUARD(c, {
    if (!c->boxset) throw std::invalid_argument("grid_style before domain");
    if (nx < 4 || ny < 4 || nz < 4 || nx % 2 || ny % 2 || nz % 2) throw std::invalid_argument("grid sizes must be even and >= 4");
    c->N[0] = nx; c->N[1] = ny; c->N[2] = nz;
    c->nreal = (size_t)nx * ny * nz;
    c->ncplx = (size_t)(nx / 2 + 1) * ny * nz;
    c->phi.assign(c->nreal, 0.0);
    c->chempot.assign(c->nreal, 0.0);
    for (int d = 0; d < 3; ++d) { c->grad[d].assign(c->nreal, 0.0); c->ft_grad[d].assign(c->ncplx, 0.0); }
    c->ft_phi.assign(c->ncplx, 0.0);
    c->ft_chempot.assign(c->ncplx, 0.0);
    c->fft = std::make_unique<FFT3>(nx, ny, nz);
    // domain.cpp:78-99 with one rank
    const double dzz = c->period[2] / nz;
    c->sublo[0] = c->boxlo[0]; c->sublo[1] = c->boxlo[1]; c->sublo[2] = dzz * 0 + c->boxlo[2];
    c->subhi[0] = c->boxhi[0]; c->subhi[1] = c->boxhi[1]; c->subhi[2] = dzz * (0 + nz) + c->boxlo[2];
    c->gridset = true;
  })
}

int oracle_make_unique_seed(int baseseed) {  // utility.cpp:213-235, rank 0
  std::mt19937 gen;
  std::uniform_int_distribution<int> integer_dist;
  gen.seed(baseseed);
  return integer_dist(gen);
}

int oracle_grid_populate_constant(oracle_ctx* c, double average, double variance, int seed) {
  GUARD(c, {  // grid.cpp:120-131, 289-307
    if (!c->gridset) throw std::invalid_argument("grid_populate before grid_style");
    int s = oracle_make_unique_seed(seed);
    std::uniform_real_distribution<double> real_dist(-0.5, 0.5);
    std::mt19937 gen;
    gen.seed(s);
    for (auto& v : c->phi) v = average + variance * real_dist(gen);
    c->populated = true;
  })
}

// Grid::flat_interface (grid.cpp:310-337, seeded as in Grid::populate
// :123-134): hi + variance U for x - sublo < L (average - lo)/(hi - lo), lo +
// variance U beyond, one draw per node in [z][y][x] order
static void flat_interface_impl(oracle_ctx* c, double average, double variance, double hi, double lo, int seed) {
  {
    if (!c->gridset) throw std::invalid_argument("grid_populate before grid_style");
    std::uniform_real_distribution<double> real_dist(-0.5, 0.5);
    std::mt19937 gen;
    gen.seed(oracle_make_unique_seed(seed));
    const double Lbox = (average - lo) / (hi - lo) * c->period[0];
    const double Ox = c->sublo[0], dx = c->period[0] / c->N[0];
    size_t n = 0;
    for (int i = 0; i < c->N[2]; i++)
      for (int j = 0; j < c->N[1]; j++)
        for (int k = 0; k < c->N[0]; k++) {
          const double x = k * dx + Ox;
          if (x - Ox < Lbox) c->phi[n++] = hi + variance * real_dist(gen);
          else c->phi[n++] = lo + variance * real_dist(gen);
        }
    c->populated = true;
  }
}

int oracle_grid_populate_flat_interface(oracle_ctx* c, double average, double variance, double hi, double lo,
                                        int seed) {
  GUARD(c, { flat_interface_impl(c, average, variance, hi, lo, seed); })
}

// Grid::sphere (grid.cpp:339-425): tanh profile of `radius` and `width`
// about the origin, the outer value chosen so that the volume average is av
static void sphere_impl(oracle_ctx* c, double radius, double width, double hi, double av) {
  {
    if (!c->gridset) throw std::invalid_argument("grid_populate before grid_style");
    for (int d = 0; d < 3; d++)
      if (radius >= c->period[d] / 2.) throw std::runtime_error("Initial spherical configuration has radius > domain.");
    const double dx = c->period[0] / c->N[0], dy = c->period[1] / c->N[1], dz = c->period[2] / c->N[2];
    const double Ox = c->sublo[0], Oy = c->sublo[1], Oz = c->sublo[2];
    auto shape = [&](double r) { return std::tanh((-r + radius) / width); };
    double integral = 0;
    for (int i = 0; i < c->N[2]; i++) {
      const double z = i * dz + Oz;
      for (int j = 0; j < c->N[1]; j++) {
        const double y = j * dy + Oy;
        for (int k = 0; k < c->N[0]; k++) {
          const double x = k * dx + Ox;
          integral += shape(std::sqrt(x * x + y * y + z * z));
        }
      }
    }
    integral *= dx * dy * dz;
    const double ifrac = integral / (c->period[0] * c->period[1] * c->period[2]);
    const double lo = (2 * av - hi * (1 + ifrac)) / (1 - ifrac);
    if (lo < 0) throw std::runtime_error("Average array value is too small for specified radius.");
    if (lo > hi) throw std::runtime_error("Average array value is too large for specified radius.");
    size_t n = 0;
    for (int i = 0; i < c->N[2]; i++) {
      const double z = i * dz + Oz;
      for (int j = 0; j < c->N[1]; j++) {
        const double y = j * dy + Oy;
        for (int k = 0; k < c->N[0]; k++) {
          const double x = k * dx + Ox;
          c->phi[n++] = 0.5 * (hi - lo) * shape(std::sqrt(x * x + y * y + z * z)) + 0.5 * (hi + lo);
        }
      }
    }
    c->populated = true;
  }
}

int oracle_grid_populate_sphere(oracle_ctx* c, double radius, double width, double hi, double av) {
  GUARD(c, { sphere_impl(c, radius, width, hi, av); })
}

static void noise_state_get_impl(oracle_ctx* c, char* buf, int cap, int* len) {
  std::ostringstream os;
  os << c->c_gen;
  const std::string st = os.str();
  if (len) *len = (int)st.size() + 1;
  if (buf) {
    if (cap < (int)st.size() + 1) throw std::invalid_argument("noise state buffer too small");
    std::memcpy(buf, st.c_str(), st.size() + 1);
  }
}

// the mt19937 of the reference noise (conjugate_volfrac.cpp:64) as text
int oracle_noise_state_get(oracle_ctx* c, char* buf, int cap, int* len) {
  GUARD(c, { noise_state_get_impl(c, buf, cap, len); })
}

static void noise_state_set_impl(oracle_ctx* c, const char* state) {
  std::istringstream is(state);
  std::mt19937 g;
  is >> g;
  if (is.fail()) throw std::invalid_argument("malformed noise state");
  c->c_gen = g;
}

int oracle_noise_state_set(oracle_ctx* c, const char* state) {
  GUARD(c, { noise_state_set_impl(c, state); })
}

int oracle_grid_set(oracle_ctx* c, int field, const double* in) {
  GUARD(c, {
    std::vector<double>* dst = nullptr;
    if (field == PHAFD_FIELD_PHI) dst = &c->phi;
    else if (field == PHAFD_FIELD_CHEMPOT) dst = &c->chempot;
    else if (field >= PHAFD_FIELD_GRADX && field <= PHAFD_FIELD_GRADZ) dst = &c->grad[field - PHAFD_FIELD_GRADX];
    else throw std::invalid_argument("bad field");
    std::memcpy(dst->data(), in, c->nreal * sizeof(double));
    if (field == PHAFD_FIELD_PHI) c->populated = true;
  })
}

int oracle_grid_get(oracle_ctx* c, int field, double* out) {
  GUARD(c, {
    if (field == PHAFD_FIELD_PHI) std::memcpy(out, c->phi.data(), c->nreal * 8);
    else if (field == PHAFD_FIELD_CHEMPOT) std::memcpy(out, c->chempot.data(), c->nreal * 8);
    else if (field >= PHAFD_FIELD_GRADX && field <= PHAFD_FIELD_GRADZ) std::memcpy(out, c->grad[field - PHAFD_FIELD_GRADX].data(), c->nreal * 8);
    else if (field == PHAFD_FIELD_FT_PHI) std::memcpy(out, c->ft_phi.data(), c->ncplx * 16);
    else if (field == PHAFD_FIELD_FT_CHEMPOT) std::memcpy(out, c->ft_chempot.data(), c->ncplx * 16);
    else throw std::invalid_argument("bad field");
  })
}

int oracle_atoms_create(oracle_ctx* c, int n, const int* tags, const int* mol, const int* types, const double* x) {
  GUARD(c, {  // atom.cpp:219-252 + check_tags_and_types
    c->nowned = n;
    c->xs.assign(x, x + 3 * (size_t)n);
    c->uxs.assign(3 * (size_t)n, 0.0);
    c->Fs.assign(3 * (size_t)n, 0.0);
    c->tags.assign(tags, tags + n);
    c->types.assign(types, types + n);
    c->moltags.assign(mol ? mol : tags, (mol ? mol : tags) + n);
    c->labels.assign(n, OWNED);
    c->images.assign(n, c->set_image());
    c->images_restored = false;
    std::set<int> ts(c->tags.begin(), c->tags.end());
    if ((int)ts.size() != n) throw std::runtime_error("duplicate IDs found on processor(s).");
    int tmax = -1;
    for (int t : c->types) tmax = std::max(tmax, t);
    c->ntypes = tmax + 1;
  })
}

// the "ix" attribute of atom_populate read_dump (read_dump.cpp:239-240)
int oracle_atoms_set_images(oracle_ctx* c, const int* images) {
  GUARD(c, {
    if (c->setup_done) throw std::runtime_error("image flags are restored before setup");
    c->images.assign(images, images + c->nowned);
    c->images_restored = true;
  })
}

int oracle_atoms_get(oracle_ctx* c, double* x, double* ux, double* f, int* images) {
  GUARD(c, {
    const size_t n = c->nowned;
    if (x) std::memcpy(x, c->xs.data(), 3 * n * 8);
    if (ux) std::memcpy(ux, c->uxs.data(), 3 * n * 8);
    if (f) std::memcpy(f, c->Fs.data(), 3 * n * 8);
    if (images) std::memcpy(images, c->images.data(), n * 4);
  })
}

int oracle_pair_gridatom(oracle_ctx* c, int style, double cut) {
  GUARD(c, {  // pair_gridatom_*.cpp settings()
    if (c->ntypes <= 0) throw std::runtime_error("Cannot create pair style before atoms are made.");
    c->ga_style = style;
    c->ga_maxcut = cut;
    c->ga_cutsq.assign(c->ntypes, cut * cut);
    c->ga_eps.assign(c->ntypes, 1.0);
    c->ga_phi.assign(c->ntypes, 0.1);
  })
}

int oracle_pair_gridatom_coeff(oracle_ctx* c, int type, int has_eps, double eps, int has_w, double nucwidth, int has_phi, double phit) {
  GUARD(c, {
    if (type < 0 || type >= c->ntypes) throw std::runtime_error("Pair grid/atom atom type out of range.");
    if (has_eps) c->ga_eps[type] = eps;
    if (has_w) {
      if (nucwidth > c->ga_maxcut) throw std::runtime_error("nucwidth cannot be larger than maximum cut.");
      c->ga_cutsq[type] = nucwidth * nucwidth;
    }
    if (has_phi) c->ga_phi[type] = phit;
  })
}

int oracle_pair_lj_cut(oracle_ctx* c, double cut, double eps, double sigma) {
  GUARD(c, {  // pair_lj_cut.cpp:103-119
    c->have_lj = true;
    c->lj_cut = cut;
    c->lj1 = 48 * eps * std::pow(sigma, 12.0);
    c->lj2 = 24 * eps * std::pow(sigma, 6.0);
    c->lj_cutsq = cut * cut;
  })
}

int oracle_neighbor(oracle_ctx* c, double skin) {
  GUARD(c, {  // neighbor.cpp:39-68
    c->skin = skin;
    double cutoff = 0.0;
    if (c->have_lj) cutoff = std::max(cutoff, c->lj_cut);
    if (c->ga_style != PHAFD_GRIDATOM_NONE) cutoff = std::max(cutoff, c->ga_maxcut);
    c->triggersq = 0.25 * skin * skin;
    if (cutoff > 0.0) c->cutneigh = skin + cutoff;
    c->cutneighsq = c->cutneigh * c->cutneigh;
    c->cutghost = c->cutneigh;
    c->setup_bins();
    c->create_stencils();
    c->neigh_set = true;
  })
}

int oracle_fix_conjugate_volfrac(oracle_ctx* c, int seed, double mobility, double temp, double volFH, double gamma, int noise) {
  GUARD(c, {  // fixgrid_conjugate.cpp:21-45, conjugate_volfrac.cpp:29-70
    c->have_conj = true;
    c->c_seed = oracle_make_unique_seed(seed);
    c->c_mobility = mobility; c->c_temp = temp; c->c_volFH = volFH; c->c_gamma = gamma;
    c->c_noise = noise;
    c->c_gen.seed(c->c_seed);
    c->set_qs();
  })
}

int oracle_fix_floryhuggins(oracle_ctx* c, double temp, double volFH, double chi) {
  GUARD(c, { c->have_fh = true; c->fh_temp = temp; c->fh_volFH = volFH; c->fh_chi = chi; })
}

int oracle_fix_gradphi(oracle_ctx* c, int once) {
  GUARD(c, { c->have_gradphi = true; c->gradphi_once = once != 0; })
}

int oracle_fix_drag(oracle_ctx* c, int nranges, const int* starts, const int* ends, double drag) {
  GUARD(c, {
    DragFix f; f.drag = drag;
    for (int r = 0; r < nranges; ++r) f.ranges.push_back({starts[r], ends[r]});
    c->drags.push_back(f);
  })
}

int oracle_fix_semiflexible(oracle_ctx* c, int nranges, const int* starts, const int* ends, const phafd_semiflexible_params* p) {
  GUARD(c, {
    SemiFix f;
    for (int r = 0; r < nranges; ++r) f.ranges.push_back({starts[r], ends[r]});
    f.bondlength = p->bondlength; f.zeta_para = p->zeta_para; f.zeta_perp = p->zeta_perp;
    f.bending = p->bending; f.temp = p->temp; f.kbond = p->kbond; f.seed = (uint32_t)p->seed; f.noise = p->noise;
    c->semis.push_back(f);
  })
}

int oracle_set_dt(oracle_ctx* c, double dt) { GUARD(c, { c->dt = dt; }) }
int oracle_set_timestep(oracle_ctx* c, long long ts) { GUARD(c, { c->timestep = ts; c->firststep = ts; }) }

int oracle_setup(oracle_ctx* c) { GUARD(c, { c->setup(); }) }

int oracle_run(oracle_ctx* c, int nsteps) {
  GUARD(c, {
    if (!c->setup_done) c->setup();
    for (int s = 0; s < nsteps; ++s) {
      c->step();
      if (c->nan_flag) throw std::runtime_error("NAN encountered in phi.");
      if (c->semi_fail) throw std::runtime_error("Failed to maintain polymer bond-length constraints.");
    }
  })
}

// Integrate::run_until_touching (integrate.cpp:221-415), one rank: after
// each step the distance between the first and the last owned bead (stored,
// wrapped positions) is compared with touch_point; events are (kind, step):
// kind 0 "cyclisation occured at step", kind 1 "cyclisation interval ended
// at step" (its step already less delay_step).  Without continue_running
// the run ends after the first touching step (input.cpp:293 passes delay 0).
static void run_until_touching_impl(oracle_ctx* c, long long nsteps, double touch_point, int continue_running,
                                    int delay_step, long long* steps_done, int max_events, long long* ev_step,
                                    int* ev_kind, int* nevents) {
  if (!c->setup_done) c->setup();
  int since = delay_step, breakflag = 0, nev = 0;
  long long s = 0;
  auto record = [&](int kind, long long step) {
    if (nev < max_events) {
      ev_kind[nev] = kind;
      ev_step[nev] = step;
    }
    ++nev;
  };
  for (; s < nsteps; ++s) {
    c->step();
    if (c->nan_flag) throw std::runtime_error("NAN encountered in phi.");
    if (c->semi_fail) throw std::runtime_error("Failed to maintain polymer bond-length constraints.");
    const int last = c->nowned - 1;
    const double d0 = c->X(0, last) - c->X(0, 0), d1 = c->X(1, last) - c->X(1, 0), d2 = c->X(2, last) - c->X(2, 0);
    const double d = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    if (d < touch_point) {
      if (since >= delay_step) record(0, c->timestep);
      since = 0;
      breakflag = 1;
    } else {
      if (breakflag && since == delay_step) record(1, c->timestep - delay_step);
      since += 1;
    }
    if (!continue_running && breakflag) {
      ++s;
      break;
    }
  }
  *steps_done = s;
  *nevents = nev;
}

int oracle_run_until_touching(oracle_ctx* c, long long nsteps, double touch_point, int continue_running,
                              int delay_step, long long* steps_done, int max_events, long long* ev_step,
                              int* ev_kind, int* nevents) {
  GUARD(c, { run_until_touching_impl(c, nsteps, touch_point, continue_running, delay_step, steps_done, max_events,
                                     ev_step, ev_kind, nevents); })
}

// Stage hooks used by unit tests
int oracle_stage_gradient(oracle_ctx* c) { GUARD(c, { c->gradient(); }) }
int oracle_stage_borders_and_build(oracle_ctx* c) { GUARD(c, { c->pbc(); c->borders(); c->neighbor_build(); }) }
int oracle_stage_pairs(oracle_ctx* c) {
  GUARD(c, {
    c->forward_comm();
    std::fill(c->Fs.begin(), c->Fs.end(), 0.0);
    std::fill(c->chempot.begin(), c->chempot.end(), 0.0);
    c->pairs_compute();
    c->reverse_comm();
  })
}

// ComputePair::end_of_step (compute_pair.cpp:43-85): the forces of one pair
// style on the owned beads, from the gathered copies as the step's pair stage
// left them, the gradient arrays of the step's start and phi after the step;
// the style's chempot deposit goes into chempot as in the reference.  The
// beads' own forces are kept.
int oracle_compute_pair(oracle_ctx* c, int style, double* out3) {
  GUARD(c, {
    if (style == PHAFD_PAIR_LJ_CUT && !c->have_lj)
      throw std::invalid_argument("Cannot compute pair style lj/cut, it hasn't been created!");
    if (style == PHAFD_PAIR_GRIDATOM && c->ga_style == PHAFD_GRIDATOM_NONE)
      throw std::invalid_argument("Cannot compute pair style gridatom, it hasn't been created!");
    if (style != PHAFD_PAIR_LJ_CUT && style != PHAFD_PAIR_GRIDATOM) throw std::invalid_argument("unknown pair style");
    const std::vector<double> keep(c->Fs);
    std::fill(c->Fs.begin(), c->Fs.end(), 0.0);
    if (style == PHAFD_PAIR_LJ_CUT) c->pair_lj();
    else c->pair_gridatom();
    c->reverse_comm();
    for (int i = 0; i < c->nowned; ++i)
      for (int d = 0; d < 3; ++d) out3[3 * i + d] = c->F(d, i);
    c->Fs = keep;
  })
}

// list export: half list as (tag_i, tag_j, shift code) and grid list as (node, tag, shift code)
// shift code = (sx+1) + 3*(sy+1) + 9*(sz+1) with s in {-1,0,1} periodic images applied to j
static std::vector<int> owner_map(const oracle_ctx* c) {
  int tmax = 0;
  for (int i = 0; i < c->nowned; ++i) tmax = std::max(tmax, c->tags[i]);
  std::vector<int> own(tmax + 1, -1);
  for (int i = 0; i < c->nowned; ++i) own[c->tags[i]] = i;
  return own;
}
static int shift_code(const oracle_ctx* c, const std::vector<int>& own, int j) {
  const int owner = own[c->tags[j]];
  int code = 0, mul = 1;
  for (int d = 0; d < 3; ++d) {
    double diff = c->xs[3 * (size_t)j + d] - c->xs[3 * (size_t)owner + d];
    int s = (int)std::lround(diff / c->period[d]);
    code += (s + 1) * mul;
    mul *= 3;
  }
  return code;
}

int oracle_half_list_size(oracle_ctx* c) { return (int)c->half_nb.size(); }
int oracle_grid_list_size(oracle_ctx* c) { return (int)c->grid_nb.size(); }

int oracle_half_list(oracle_ctx* c, int* out3) {
  GUARD(c, {
    auto own = owner_map(c);
    size_t m = 0;
    for (size_t ii = 0; ii < c->half_ilist.size(); ++ii) {
      int i = c->half_ilist[ii];  // always a LOCAL copy: image code 13
      for (int jj = c->half_off[ii]; jj < c->half_off[ii + 1]; ++jj) {
        int j = c->half_nb[jj];
        out3[3 * m] = c->tags[i];
        out3[3 * m + 1] = c->tags[j];
        out3[3 * m + 2] = shift_code(c, own, j);
        ++m;
      }
    }
  })
}

int oracle_grid_list(oracle_ctx* c, int* out3) {
  GUARD(c, {
    auto own = owner_map(c);
    size_t m = 0;
    for (size_t ii = 0; ii < c->grid_ilist.size(); ++ii)
      for (int jj = c->grid_off[ii]; jj < c->grid_off[ii + 1]; ++jj) {
        int j = c->grid_nb[jj];
        out3[3 * m] = c->grid_ilist[ii];
        out3[3 * m + 1] = c->tags[j];
        out3[3 * m + 2] = shift_code(c, own, j);
        ++m;
      }
  })
}

int oracle_counters(oracle_ctx* c, long long* out) {
  GUARD(c, {
    out[0] = c->num_less_zero;
    out[1] = c->num_great_zero;
    out[2] = c->ncalls;
    out[3] = c->timestep;
    out[4] = c->nlocal;
    out[5] = c->nghost;
  })
}

int oracle_stage_times(oracle_ctx* c, double* out7) {
  GUARD(c, { for (int i = 0; i < 7; ++i) out7[i] = c->t_stage[i]; })
}

// standalone transforms (for FFT unit tests against numpy.fft)
// compute grid/cluster (compute_grid_clusters.cpp:66-229) on one periodic
// domain: label = z + (y Nx + x) Ny where phi < or > threshold, else -1
// (compute_grid_clusters.cpp:72-94); then sweeps over the nodes in (z, y, x)
// order that set a node and each labelled nearest neighbour (z, y, x wrapped;
// the reference's LEFTS/RIGHTS planes are the wrapped z neighbours of a
// one-rank domain) to the smaller of the two labels, until a sweep changes
// nothing (compute_grid_clusters.cpp:103-196).
static void grid_clusters_impl(oracle_ctx* c, double threshold, int greater, int* labels) {
  const int Nx = c->N[0], Ny = c->N[1], Nz = c->N[2];
  auto L = [&](int i, int j, int k) -> int& { return labels[((size_t)i * Ny + j) * Nx + k]; };
  for (int i = 0; i < Nz; i++)
    for (int j = 0; j < Ny; j++)
      for (int k = 0; k < Nx; k++) {
        const double v = c->PHI(i, j, k);
        const bool in = greater ? v > threshold : v < threshold;
        L(i, j, k) = in ? i + (j * Nx + k) * Ny : -1;
      }
  bool done = false;
  while (!done) {
    done = true;
    for (int i = 0; i < Nz; i++)
      for (int j = 0; j < Ny; j++)
        for (int k = 0; k < Nx; k++) {
          if (L(i, j, k) == -1) continue;
          const int nb[6][3] = {{(i + Nz - 1) % Nz, j, k}, {(i + 1) % Nz, j, k}, {i, (j + Ny - 1) % Ny, k},
                                {i, (j + 1) % Ny, k},       {i, j, (k + Nx - 1) % Nx}, {i, j, (k + 1) % Nx}};
          for (auto& q : nb) {
            int& o = L(q[0], q[1], q[2]);
            if (o == -1 || o == L(i, j, k)) continue;
            L(i, j, k) = o = std::min(L(i, j, k), o);
            done = false;
          }
        }
  }
}

int oracle_compute_grid_clusters(oracle_ctx* c, double threshold, int greater, int* labels) {
  GUARD(c, { grid_clusters_impl(c, threshold, greater, labels); })
}

int oracle_fft_r2c(int nx, int ny, int nz, const double* in, double* out_cplx) {
  try {
    FFT3 f(nx, ny, nz);
    f.r2c(in, reinterpret_cast<cd*>(out_cplx));
    return 0;
  } catch (...) { return PHAFD_ERR_INVALID; }
}
int oracle_fft_c2r(int nx, int ny, int nz, const double* in_cplx, double* out) {
  try {
    FFT3 f(nx, ny, nz);
    f.c2r(reinterpret_cast<const cd*>(in_cplx), out);
    return 0;
  } catch (...) { return PHAFD_ERR_INVALID; }
}

}  // extern "C"
