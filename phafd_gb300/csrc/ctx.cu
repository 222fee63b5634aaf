// libphafd_gpu C ABI: context, device memory, and the per-step launch
// sequence (the GB300 restatement of Integrate::run, integrate.cpp:105-203).
//
// Step, "resident" schedule (default).  State at step start: phi_hat (the
// unnormalised r2c of phi), phi and grad phi, all in HBM.
//   neighbor check / rebuild          (device flag; no host round trip)
//   pair forces + mu deposit          (lj/cut, gridatom/*)
//   drag / chain first half           (initial_integrate)
//   x-r2c fused with Flory-Huggins    (post_force + pre_final_integrate)
//   y-fft, z-fft                      -> mu_hat
//   z pass: Model-B update, z-ifft of phi_hat and of i qz phi_hat
//   y pass: y-ifft (+ i qy)           x pass: c2r -> phi, dphi/dx, dphi/dy, dphi/dz
//   drag / chain second half          (final_integrate)
// The reference recomputes phi_hat = r2c(phi) at every step start
// (fixgrid_conjugate.cpp:66); r2c(c2r(X)) equals X for the Hermitian
// spectra the update produces, so the resident schedule carries phi_hat
// across steps and saves one 3D FFT.  The "reference" schedule keeps the
// reference's order exactly (one extra r2c per step).
//
// Every launch of a step reads its parameters from device memory, so the
// whole step is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "bead_kernels.h"

using namespace phafd;

namespace {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define CK(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));    \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  void alloc(size_t b) {
    release();
    if (b == 0) return;
    CK(cudaMalloc(&p, b));
    bytes = b;
  }
  void zero(cudaStream_t st) {
    if (p) CK(cudaMemsetAsync(p, 0, bytes, st));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
  ~DevBuf() { release(); }
};

struct Range { int start, end; };

int make_unique_seed(int baseseed) {  // utility.cpp:213-235, rank 0
  std::mt19937 gen;
  std::uniform_int_distribution<int> integer_dist;
  gen.seed(baseseed);
  return integer_dist(gen);
}

// phi += scale * src
template <typename T>
__global__ void k_axpy(T* __restrict__ y, const T* __restrict__ x, T scale, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[k] += scale * x[k];
}

// F[k = 0] += v: the reference concentration's share N c of the k = 0 mode,
// after an r2c of phi - c
template <typename T>
__global__ void k_origin_add(cpx<T>* F, double v) {
  F[0].x += (T)v;
}

// shell sums of |F|^2 over the half spectrum [kx][kz][ky]; modes with
// 0 < kx < Nx/2 stand for their mirror too (weight 2)
// |q| in units of the x-axis dq (ry = dqy/dqx, rz = dqz/dqx): integer
// wavenumbers of a cubic box give exact squares, so shell edges are exact
template <typename T>
__global__ void k_shells(const cpx<T>* __restrict__ F, int Nx, int Ny, int Nz, double ry, double rz, int nbins,
                         double* __restrict__ sum, unsigned long long* __restrict__ cnt) {
  extern __shared__ double sh[];
  double* ss = sh;
  unsigned long long* sc = reinterpret_cast<unsigned long long*>(sh + nbins);
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) { ss[b] = 0.0; sc[b] = 0ull; }
  __syncthreads();
  const int Nxh = Nx / 2 + 1;
  const long long total = (long long)Nxh * Nz * Ny;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < total; m += (long long)gridDim.x * blockDim.x) {
    const int ky = (int)(m % Ny), kz = (int)((m / Ny) % Nz), kx = (int)(m / ((long long)Ny * Nz));
    if (kx == 0 && ky == 0 && kz == 0) continue;
    const double qx = (double)kx, qy = ry * wrap_index(ky, Ny), qz = rz * wrap_index(kz, Nz);
    const int b = (int)floor(sqrt(qx * qx + qy * qy + qz * qz) + 1e-9);
    if (b >= nbins) continue;
    const int w = (kx == 0 || 2 * kx == Nx) ? 1 : 2;
    const cpx<T> f = F[m];
    atomicAdd(ss + b, (double)w * ((double)f.x * f.x + (double)f.y * f.y));
    atomicAdd(sc + b, (unsigned long long)w);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
    if (sc[b]) {
      atomicAdd(sum + b, ss[b]);
      atomicAdd(cnt + b, sc[b]);
    }
  }
}

// kernel nodes at the top level of a graph (the bodies of conditional
// nodes, which run only when switched on, are not counted)
long long count_kernels(cudaGraph_t g) {
  size_t nnodes = 0;
  CK(cudaGraphGetNodes(g, nullptr, &nnodes));
  std::vector<cudaGraphNode_t> nodes(nnodes);
  if (nnodes) CK(cudaGraphGetNodes(g, nodes.data(), &nnodes));
  long long nk = 0;
  for (auto nd : nodes) {
    cudaGraphNodeType ty;
    CK(cudaGraphNodeGetType(nd, &ty));
    if (ty == cudaGraphNodeTypeKernel) ++nk;
  }
  return nk;
}

}  // namespace

struct phafd_ctx {
  std::string err;
  int device = 0, precision = PHAFD_FP32;
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;           // bead branch, forked from st inside a step
  cudaStream_t st3 = nullptr;           // Hermitian-plane branch, forked from st inside a step
  cudaStream_t stc = nullptr;           // capture of the conditional rebuild body only
  cudaEvent_t ev_fork = nullptr, ev_dep = nullptr, ev_join = nullptr;
  // pipelined read-back: per slot an event after its copies and the status
  // words copied with them into page-locked memory
  cudaEvent_t ev_slot[4] = {nullptr, nullptr, nullptr, nullptr};
  long long* slot_status = nullptr;  // [slot][2]: nan step, flag|status
  cudaEvent_t ev_pl_fork = nullptr, ev_pl_join = nullptr;
  // domain / grid
  bool boxset = false, gridset = false, populated = false;
  double boxlo[3] = {0, 0, 0}, boxhi[3] = {0, 0, 0}, period[3] = {0, 0, 0};
  int N[3] = {0, 0, 0};
  size_t nreal = 0, ncplx = 0;
  Geom geom{};
  int zghost = PHAFD_ZGHOST_PERIODIC;
  int schedule = PHAFD_SCHEDULE_RESIDENT;
  bool keep_chempot = false;
  bool chempot_from_mu = false;
  // what the last step left readable: without keep_chempot the deposit
  // buffer is reset inside the step (no real mu remains) and the resident z
  // pass stores only the Hermitian planes of mu's spectrum
  bool chempot_lost = false, muhat_stale = false, stepped = false;
  // compute pair: each step keeps the positions its pair stage used
  bool pair_snapshot = false, pair_snapped = false;
  void note_step() {
    stepped = true;
    pair_snapped = pair_snapshot && n > 0;
    chempot_lost = have_conj && !keep_chempot;
    muhat_stale = have_conj && !keep_chempot && schedule == PHAFD_SCHEDULE_RESIDENT;
  }
  bool use_plane = false;  // plane-fused x/y passes where they apply (phafd_set_plane_fusion)
  bool use_gmask = false;  // gradient stored near beads only during steps (phafd_set_gradient_mask)
  bool grad_partial = false;  // gx, gy, gz hold values at masked nodes only
  // FP32 reference concentration c (0: none), set at set-up from the mean of
  // phi: FP32 transforms of phi carry phi - c, with N c added to the k = 0
  // mode of the spectrum in FP64-exact arithmetic (the spectrum keeps its
  // meaning), and the Flory-Huggins part of mu is taken relative to f(c), so
  // that round-off scales with the fluctuations, not with the mean
  double phi_ref = 0.0;
  // which FP32 stages use c (phafd_set_fp32_centering): PHAFD_CENTER_FH the
  // Flory-Huggins part, PHAFD_CENTER_FFT the transforms of phi
  // (the transforms by default: measured, centering the Flory-Huggins part
  // costs the x pass a software log1p per node and leaves S(k) where it was)
  int center_bits = PHAFD_CENTER_FFT;
  bool centered(int bit = PHAFD_CENTER_FH | PHAFD_CENTER_FFT) const {
    return precision == PHAFD_FP32 && phi_ref > 0.0 && phi_ref < 1.0 && (center_bits & bit);
  }
  // the FP32 value of c the kernels use (0 when the stage is not centered)
  double ref_c(int bit = PHAFD_CENTER_FFT) const { return centered(bit) ? (double)(float)phi_ref : 0.0; }
  void center(FHArgs& f, int bit) const {
    if (!centered(bit)) return;
    const double c = ref_c(bit);
    f.c = c;
    f.inv_c = 1.0 / c;
    f.fconst = f.enabled ? f.tv * (std::log(c / (1.0 - c)) + f.chi * (1.0 - 2.0 * c)) : 0.0;
    f.centered = 1;
  }
  FHArgs plain_fh() const {  // r2c of phi without the Flory-Huggins prologue
    FHArgs f{0, 0, fh_counters(), 0, nullptr};
    center(f, PHAFD_CENTER_FFT);
    f.status = d_status();
    return f;
  }
  FHArgs step_fh() const {  // mu = deposit + FH(phi), fused into the x r2c of a step
    FHArgs f{fh_temp / fh_volFH, fh_chi, fh_counters(), have_fh ? 1 : 0, keep_chempot ? mu.p : nullptr};
    center(f, PHAFD_CENTER_FH);
    f.status = d_status();
    if (dmask.p && n > 0) f.dep_mask = dmask.as<uint32_t>();
    return f;
  }
  // N f(c) tv: what the k = 0 mode of a centered mu spectrum lacks
  double mu_origin_shift() const { return (double)nreal * step_fh().fconst; }
  int nsub = 1;            // substeps of one step (phafd_set_linear_substeps)
  double f2_lin = 0.0;     // dmu/dphi of the linearisation
  int graph_cur = 0;
  DevBuf phi, gx, gy, gz, dep, mu;
  DevBuf phat[2], muhat, w1, wA, wB, wC, wD, wE;
  int cur = 0;
  DevBuf tw[3][2];  // [axis][0 fwd, 1 inv]
  DevBuf uref;
  double2* uref_h = nullptr;
  // beads
  int n = 0, ntypes = 0;
  std::vector<int> tags, types, mol;
  DevBuf bx, bux, bf, bxhold, bfchain, btang, bimage, btype;
  DevBuf bin_of, bin_count, bin_cursor, bin_start, sorted, scan_tmp, bin_off;
  DevBuf nbr, nnbr, gl, ngl;
  DevBuf dragc, sf_fix, sf_start, sf_len, sf_par, chain0;
  DevBuf gmask;  // one bit per 32-byte sector of a real field (beads with a grid coupling)
  DevBuf dmask;  // the same sectors: the deposit's support, rebuilt with the grid lists
  DevBuf bx_pair, bf_tmp;  // positions of the last pair stage (phafd_set_pair_snapshot); compute pair's forces
  // run_until_touching: a check after every step while set
  DevBuf touch;
  bool touch_on = false;
  double touch_point = 0.0;
  int touch_delay = 0;
  BeadArgs ba{};
  // pairs
  bool have_lj = false;
  double lj_cut = 0, lj1 = 0, lj2 = 0;
  int ga_style = PHAFD_GRIDATOM_NONE;
  double ga_maxcut = 0;
  std::vector<double> ga_cutsq, ga_eps, ga_phi;
  DevBuf ga_dev;  // 3 * ntypes doubles
  // neighbor
  bool neigh_set = false;
  double skin = 0, cutneigh = 0;
  // fixes
  bool have_conj = false, have_fh = false, have_gradphi = false, gradphi_once = false;
  double c_mobility = 1, c_temp = 1, c_volFH = 1, c_gamma = 1;
  int c_seed = 0, c_noise = PHAFD_NOISE_PHILOX;
  std::mt19937 c_gen;
  double fh_temp = 1, fh_volFH = 1, fh_chi = 1;
  std::vector<std::pair<std::vector<Range>, double>> drags;
  std::vector<std::pair<std::vector<Range>, phafd_semiflexible_params>> semis;
  int nchains = 0;
  // integrate
  double dt = 0;
  long long timestep = 0, firststep = 0;
  bool setup_done = false;
  bool images_restored = false;  // beads restored from a dump: no initial bond check
  // device counters
  DevBuf d_counters;  // [0..1] FH counters (ull), [2] step, [3] nan_step, [4] ncalls, [5] flag|status,
                      // [6] blocks of the neighbor check done | gradient mask off
  unsigned long long* fh_counters() const { return d_counters.as<unsigned long long>(); }
  long long* d_step() const { return d_counters.as<long long>() + 2; }
  long long* d_nan() const { return d_counters.as<long long>() + 3; }
  long long* d_ncalls() const { return d_counters.as<long long>() + 4; }
  int* d_flag() const { return reinterpret_cast<int*>(d_counters.as<long long>() + 5); }
  int* d_status() const { return reinterpret_cast<int*>(d_counters.as<long long>() + 5) + 1; }
  int* d_check_done() const { return reinterpret_cast<int*>(d_counters.as<long long>() + 6); }
  int* d_gmask_off() const { return reinterpret_cast<int*>(d_counters.as<long long>() + 6) + 1; }
  // graph
  cudaGraphExec_t gexec = nullptr;
  cudaGraphExec_t gexecK = nullptr;                 // graph_steps steps (resident)
  int graph_steps = 8;
  int graph_curK = 0;
  cudaGraphExec_t gexec1[2] = {nullptr, nullptr};  // one step, per spectrum parity (resident)
  // Inside a multi-step graph the neighbor check (and conditional rebuild) of
  // every step but the first runs at the end of the previous step's bead
  // branch, where it overlaps that step's inverse chain: check_next_early is
  // set while such a step is captured, check_done_early while the step
  // whose check ran early is captured.
  bool check_next_early = false, check_done_early = false;
  bool eager_done = false;
  long long kernels_per_step = 0;
  long long rebuild_kernels = 0;  // kernels of the conditional rebuild body
  // stage profiling (eager steps only): event after each stage group
  bool profiling = false;
  std::vector<std::pair<int, cudaEvent_t>> marks;
  void mark(int stage) {
    if (!profiling) return;
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    CK(cudaEventRecord(e, st));
    marks.push_back({stage, e});
  }

  ~phafd_ctx() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (gexecK) cudaGraphExecDestroy(gexecK);
    for (auto ge : gexec1)
      if (ge) cudaGraphExecDestroy(ge);
    if (uref_h) cudaFreeHost(uref_h);
    for (cudaEvent_t e : {ev_fork, ev_dep, ev_join, ev_pl_fork, ev_pl_join}) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ev_slot) if (e) cudaEventDestroy(e);
    if (slot_status) cudaFreeHost(slot_status);
    if (stc) cudaStreamDestroy(stc);
    if (st3) cudaStreamDestroy(st3);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  }

  size_t rsz() const { return precision == PHAFD_FP64 ? 8 : 4; }

  void invalidate_graph() {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    if (gexecK) cudaGraphExecDestroy(gexecK);
    gexecK = nullptr;
    for (auto& ge : gexec1) {
      if (ge) cudaGraphExecDestroy(ge);
      ge = nullptr;
    }
    eager_done = false;
  }

  // ------------------------------------------------------------------ grid
  void build_twiddles() {
    for (int a = 0; a < 3; ++a) {
      const int n = N[a];
      for (int dir = 0; dir < 2; ++dir) {
        const double sgn = dir == 0 ? -1.0 : 1.0;
        std::vector<double> tbl(2 * (size_t)n);
        for (int m = 0; m < n; ++m) {
          long double ang = 2.0L * 3.141592653589793238462643383279502884L * m / n;
          tbl[2 * m] = (double)std::cos(ang);
          tbl[2 * m + 1] = sgn * (double)std::sin(ang);
        }
        if (precision == PHAFD_FP64) {
          tw[a][dir].alloc(tbl.size() * 8);
          CK(cudaMemcpy(tw[a][dir].p, tbl.data(), tbl.size() * 8, cudaMemcpyHostToDevice));
        } else {
          std::vector<float> f(tbl.begin(), tbl.end());
          tw[a][dir].alloc(f.size() * 4);
          CK(cudaMemcpy(tw[a][dir].p, f.data(), f.size() * 4, cudaMemcpyHostToDevice));
        }
      }
    }
  }

  void alloc_grid() {
    const size_t r = nreal * rsz(), c = ncplx * 2 * rsz();
    phi.alloc(r); gx.alloc(r); gy.alloc(r); gz.alloc(r); dep.alloc(r);
    for (auto* b : {&phi, &gx, &gy, &gz, &dep}) b->zero(st);
    phat[0].alloc(c); phat[1].alloc(c); muhat.alloc(c); w1.alloc(c);
    wA.alloc(c); wB.alloc(c); wC.alloc(c); wD.alloc(c); wE.alloc(c);
    for (auto* b : {&phat[0], &phat[1], &muhat, &w1, &wA, &wB, &wC, &wD, &wE}) b->zero(st);
    build_twiddles();
  }

  template <typename T>
  UpdateArgs<T> update_args(const cpx<T>* phi_old, const cpx<T>* mu_hat, cpx<T>* phi_new, double store_scale) {
    UpdateArgs<T> u{};
    u.phi_old = phi_old;
    u.mu_hat = mu_hat;
    u.phi_new = phi_new;
    u.uref = uref.as<double2>();
    u.mobility = (T)c_mobility;
    u.tvg = (T)(c_temp / c_volFH * c_gamma);
    u.dt = (T)dt;
    u.norm = (T)(1.0 / ((double)N[0] * N[2] * N[1]));  // conjugate_volfrac.cpp:76
    const double invLcubed = 1.0 / (period[0] * period[1] * period[2]);
    u.cpref = (T)std::sqrt(12 * c_temp * c_mobility * invLcubed);
    u.rpref = (T)std::sqrt(24 * c_temp * c_mobility * invLcubed);
    u.sqrtdt = (T)std::sqrt(dt);
    u.phi_scale = (T)1.0;
    u.store_scale = (T)store_scale;
    u.qx = (T)geom.kq[0];
    u.qy = (T)geom.kq[1];
    u.qz = (T)geom.kq[2];
    u.noise = c_noise;
    u.seed = (uint32_t)c_seed;
    u.d_step = d_step();
    u.Ny = N[1];
    u.Nz = N[2];
    u.Nxh = N[0] / 2 + 1;
    u.nsub = nsub;
    u.f2 = (T)f2_lin;
    return u;
  }

  static void chk(int rc, const char* what) {
    if (rc == -2) throw std::runtime_error(std::string("unsupported FFT length in ") + what);
    if (rc != 0) throw CudaError(std::string("launch failed: ") + what);
  }

  // r2c of a real field into `out` (unnormalised), optionally fused with FH
  template <typename T>
  void r2c(const T* in, const T* depp, cpx<T>* out, const FHArgs& fh) {
    const cpx<T>* twf[3] = {tw[0][0].as<cpx<T>>(), tw[1][0].as<cpx<T>>(), tw[2][0].as<cpx<T>>()};
    chk(GridOps<T>::xr2c(geom, in, depp, out, twf[0], fh, st), "x r2c");
    mark(4);
    chk(GridOps<T>::ypass(geom, -1, out, out, nullptr, twf[1], st), "y fft");
    mark(5);
    chk(GridOps<T>::zpass(geom, -1, out, out, nullptr, twf[2], nullptr, st), "z fft");
    if (fh.centered && !depp) k_origin_add<T><<<1, 1, 0, st>>>(out, (double)nreal * fh.c);  // phi - c was transformed
    mark(6);
  }

  // y inverse and x c2r of A (and B): phi (scale sp, optional) and grad (scale sg)
  template <typename T>
  void yx_inverse(T* phi_out, T sp, T sg, bool grad, bool nan_check, bool masked = false, double phi_off = 0.0) {
    const cpx<T>* twi[3] = {tw[0][1].as<cpx<T>>(), tw[1][1].as<cpx<T>>(), tw[2][1].as<cpx<T>>()};
    cpx<T>* A = wA.as<cpx<T>>();
    cpx<T>* B = wB.as<cpx<T>>();
    cpx<T>* Cc = wC.as<cpx<T>>();
    cpx<T>* D = wD.as<cpx<T>>();
    cpx<T>* E = wE.as<cpx<T>>();
    NanArgs nan{nan_check ? 1 : 0, d_nan(), d_step(), phi_off};
    NanArgs nonan{0, d_nan(), d_step()};
    if (grad && phi_out) {
      // one launch per direction for the whole inverse chain
      int rc = GridOps<T>::yinv2(geom, A, Cc, D, B, E, twi[1], st);
      if (rc != -3) {
        chk(rc, "y ifft");
        mark(8);
        chk(GridOps<T>::xc2r3(geom, Cc, phi_out, gx.as<T>(), D, gy.as<T>(), E, gz.as<T>(), sp, sg, twi[0], nan, nonan,
                              masked ? gmask.as<uint32_t>() : nullptr, d_gmask_off(), d_status(), st), "x c2r");
        mark(9);
        return;
      }
    }
    chk(GridOps<T>::ypass(geom, +1, A, Cc, grad ? D : nullptr, twi[1], st), "y ifft");
    if (grad) chk(GridOps<T>::ypass(geom, +1, B, E, nullptr, twi[1], st), "y ifft");
    mark(8);
    if (phi_out && grad) {
      chk(GridOps<T>::xc2r(geom, Cc, phi_out, sp, false, gx.as<T>(), sg, twi[0], nan, st), "x c2r");
    } else if (phi_out) {
      chk(GridOps<T>::xc2r(geom, Cc, phi_out, sp, false, nullptr, sg, twi[0], nan, st), "x c2r");
    } else if (grad) {
      chk(GridOps<T>::xc2r(geom, Cc, gx.as<T>(), sg, true, nullptr, sg, twi[0], nonan, st), "x c2r");
    }
    if (grad) {
      chk(GridOps<T>::xc2r(geom, D, gy.as<T>(), sg, false, nullptr, sg, twi[0], nonan, st), "x c2r");
      chk(GridOps<T>::xc2r(geom, E, gz.as<T>(), sg, false, nullptr, sg, twi[0], nonan, st), "x c2r");
    }
    mark(9);
  }

  // plane-fused y ifft + x c2r of A (phi, dphi/dx; dphi/dy) and B (dphi/dz);
  // false when the plane path does not apply to this grid
  template <typename T>
  bool yx_fused(double phi_off) {
    const cpx<T>* twy = tw[1][1].as<cpx<T>>();
    const cpx<T>* twx = tw[0][1].as<cpx<T>>();
    NanArgs nan{1, d_nan(), d_step(), phi_off};
    NanArgs nonan{0, d_nan(), d_step()};
    const int rc = GridOps<T>::yx_inv(geom, wA.as<cpx<T>>(), phi.as<T>(), (T)1, false, gx.as<T>(), (T)1, twy, twx, nan, st);
    if (rc == -3) return false;
    chk(rc, "yx inv");
    chk(GridOps<T>::yx_inv(geom, wA.as<cpx<T>>(), gy.as<T>(), (T)1, true, nullptr, (T)1, twy, twx, nonan, st), "yx inv");
    mark(8);
    chk(GridOps<T>::yx_inv(geom, wB.as<cpx<T>>(), gz.as<T>(), (T)1, false, nullptr, (T)1, twy, twx, nonan, st), "yx inv");
    mark(9);
    return true;
  }

  // from a spectrum S (z-ifft input) produce phi (scale sp, optional) and grad (scale sg)
  template <typename T>
  void inverse_chain(const cpx<T>* S, const UpdateArgs<T>* u, T* phi_out, T sp, T sg, bool grad, bool nan_check) {
    const cpx<T>* twi2 = tw[2][1].as<cpx<T>>();
    chk(GridOps<T>::zpass(geom, +1, S, wA.as<cpx<T>>(), grad ? wB.as<cpx<T>>() : nullptr, twi2, u, st), "z ifft");
    mark(7);
    yx_inverse<T>(phi_out, sp, sg, grad, nan_check);
  }

  // ------------------------------------------------------------------ beads
  void fill_bead_args() {
    BeadArgs& a = ba;
    a.n = n;
    a.x = bx.as<double>(); a.ux = bux.as<double>(); a.f = bf.as<double>(); a.xhold = bxhold.as<double>();
    a.fchain = bfchain.as<double>(); a.tang = btang.as<double>();
    a.image = bimage.as<int>(); a.type = btype.as<int>();
    for (int d = 0; d < 3; ++d) {
      a.boxlo[d] = boxlo[d]; a.boxhi[d] = boxhi[d]; a.period[d] = period[d];
      a.N[d] = N[d];
      a.dx[d] = gridset ? period[d] / N[d] : 1.0;
      a.invdx[d] = 1.0 / a.dx[d];
    }
    bool pow2 = true;
    for (int d = 0; d < 3; ++d) pow2 = pow2 && N[d] > 0 && (N[d] & (N[d] - 1)) == 0;
    for (int d = 0; d < 3; ++d) {
      int lg = 0;
      while (pow2 && (1 << lg) < N[d]) ++lg;
      a.lgN[d] = pow2 ? lg : -1;
    }
    a.triggersq = 0.25 * skin * skin;
    a.cutneigh = cutneigh;
    a.cutneighsq = cutneigh * cutneigh;
    a.flag = d_flag(); a.status = d_status(); a.ncalls = d_ncalls(); a.d_step = d_step();
    a.check_done = d_check_done();
    a.bin_of = bin_of.as<int>(); a.bin_count = bin_count.as<int>(); a.bin_cursor = bin_cursor.as<int>();
    a.bin_start = bin_start.as<int>(); a.sorted = sorted.as<int>(); a.scan_tmp = scan_tmp.as<int>();
    a.fp32_lists = precision == PHAFD_FP32 ? 1 : 0;
    a.bin_off = a.fp32_lists ? bin_off.as<float4>() : nullptr;
    a.nbr = have_lj ? nbr.as<int>() : nullptr;
    a.nnbr = nnbr.as<int>();
    a.gl = ga_style != PHAFD_GRIDATOM_NONE ? gl.as<uint32_t>() : nullptr;
    a.ngl = ngl.as<int>();
    a.zperiodic = zghost == PHAFD_ZGHOST_PERIODIC;
    a.dragc = dragc.as<double>();
    a.any_drag = !drags.empty();
    a.sf_fix = sf_fix.as<int>(); a.sf_start = sf_start.as<int>(); a.sf_len = sf_len.as<int>();
    a.sf = sf_par.as<SemiDev>();
    a.any_semi = !semis.empty();
    a.chain_start = chain0.as<int>();
    a.nchains = nchains;
    a.gmask = use_gmask && gmask.p ? gmask.as<uint32_t>() : nullptr;
    a.gmask_g = 32 / (int)rsz();
    a.gmask_words = ((long long)nreal / a.gmask_g + 32) / 32;
    a.gmask_r = ga_maxcut + skin + 1e-3 * std::min(a.dx[0], std::min(a.dx[1], a.dx[2]));
    a.gmask_guardsq = skin * skin;
    a.gmask_off = d_gmask_off();
    a.dmask = dmask.p ? dmask.as<uint32_t>() : nullptr;
    a.dep = ga_style != PHAFD_GRIDATOM_NONE ? dep.p : nullptr;
    a.dep_bytes = (int)rsz();
  }

  // steps store grad phi at masked nodes only (single-substep resident steps
  // with a grid coupling; the x pass is the merged inverse launch)
  bool gmask_steps() const {
    return use_gmask && gmask.p && nsub == 1 && schedule == PHAFD_SCHEDULE_RESIDENT && have_conj && !profiling &&
           !use_plane && n > 0;
  }

  // full gradient fields again after masked steps
  void full_gradient() {
    if (!grad_partial) return;
    if (precision == PHAFD_FP64)
      inverse_chain<double>(phat[cur].as<cpx<double>>(), nullptr, nullptr, 0.0, 1.0 / (double)nreal, true, false);
    else
      inverse_chain<float>(phat[cur].as<cpx<float>>(), nullptr, nullptr, 0.0f, (float)(1.0 / (double)nreal), true,
                           false);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    grad_partial = false;
  }

  // The gradient of the step's starting phi into gx, gy, gz.  The resident
  // schedule keeps the gradient of the current phi there: it is rebuilt from
  // the spectrum the last step read, and true is returned (restore_gradient
  // puts the current one back).  Other schedules compute it at the step's
  // start, so the buffers hold it already.
  bool load_step_start_gradient() {
    if (schedule != PHAFD_SCHEDULE_RESIDENT || !have_conj) return false;
    if (precision == PHAFD_FP64)
      inverse_chain<double>(phat[1 - cur].as<cpx<double>>(), nullptr, nullptr, 0.0, 1.0 / (double)nreal, true, false);
    else
      inverse_chain<float>(phat[1 - cur].as<cpx<float>>(), nullptr, nullptr, 0.0f, (float)(1.0 / (double)nreal), true,
                           false);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    return true;
  }
  void restore_gradient() {
    grad_partial = true;
    full_gradient();
  }

  // the gradient node mask; marked stale until the next rebuild builds it
  void alloc_gmask() {
    if (ga_style == PHAFD_GRIDATOM_NONE || !gridset || n == 0) return;
    if (!gmask.p) {
      gmask.alloc(((nreal / (32 / rsz()) + 32) / 32) * 4);
      gmask.zero(st);
    }
    const int off = 1;
    CK(cudaMemcpyAsync(d_gmask_off(), &off, sizeof(int), cudaMemcpyHostToDevice, st));
  }

  void setup_neighbor_structs() {
    // bins: at least one cutoff wide (the 27-bin stencil then covers the
    // cutoff sphere) and at most 128 per axis, at least 3 per axis
    long long nbins = 1;
    int nbd[3];
    for (int d = 0; d < 3; ++d) {
      nbd[d] = std::min(128, (int)std::floor(period[d] / cutneigh));
      if (nbd[d] < 3) throw std::runtime_error("box must span at least three neighbor cutoffs per axis");
      nbins *= nbd[d];
    }
    const long long cap = 1LL << 25;
    if (nbins > cap) {
      const double shrink = std::cbrt((double)cap / (double)nbins);
      nbins = 1;
      for (int d = 0; d < 3; ++d) {
        nbd[d] = std::max(3, (int)std::floor(nbd[d] * shrink));
        nbins *= nbd[d];
      }
    }
    for (int d = 0; d < 3; ++d) {
      ba.nb[d] = nbd[d];
      ba.bininv[d] = nbd[d] / period[d];
    }
    ba.nbins = nbins;
    bin_of.alloc(std::max(n, 1) * 4);
    bin_count.alloc(nbins * 4);
    bin_cursor.alloc(nbins * 4);
    bin_count.zero(st);  // then zero after every build (the build resets the bins it filled)
    bin_cursor.zero(st);
    bin_start.alloc((nbins + 1) * 4);
    sorted.alloc(std::max(n, 1) * 4);
    bin_off.alloc((size_t)std::max(n, 1) * sizeof(float4));
    scan_tmp.alloc(((nbins + 1023) / 1024 + 1) * 4);
    ba.maxnb = 128;
    if (have_lj) nbr.alloc((size_t)std::max(n, 1) * ba.maxnb * 4);
    nnbr.alloc(std::max(n, 1) * 4);
    int maxg = 1;
    for (int d = 0; d < 3; ++d) {
      const double dxd = gridset ? period[d] / N[d] : 1.0;
      maxg *= (int)std::floor(2.0 * cutneigh / dxd) + 3;
    }
    ba.maxg = maxg;
    if (ga_style != PHAFD_GRIDATOM_NONE) gl.alloc((size_t)std::max(n, 1) * maxg * 4);
    ngl.alloc(std::max(n, 1) * 4);
    if (ga_style != PHAFD_GRIDATOM_NONE && gridset) {  // zero until the first build: so is the deposit
      dmask.alloc(((nreal / (32 / rsz()) + 32) / 32) * 4);
      dmask.zero(st);
    }
    if (use_gmask) alloc_gmask();
    nnbr.zero(st);
    ngl.zero(st);
  }

  void upload_fix_tables() {
    std::vector<double> dc(std::max(n, 1), 0.0);
    for (auto& f : drags)
      for (auto& r : f.first)
        for (int j = r.start; j < r.end; ++j) {
          if (dc[j] != 0.0) throw std::runtime_error("a bead may belong to one atom/drag fix only");
          dc[j] = f.second;
        }
    dragc.alloc(dc.size() * 8);
    CK(cudaMemcpy(dragc.p, dc.data(), dc.size() * 8, cudaMemcpyHostToDevice));
    std::vector<int> fix(std::max(n, 1), -1), s0(std::max(n, 1), 0), ln(std::max(n, 1), 0);
    std::vector<SemiDev> par;
    std::vector<int> starts;
    for (size_t k = 0; k < semis.size(); ++k) {
      const auto& p = semis[k].second;
      SemiDev d{p.bondlength, p.zeta_para, p.zeta_perp, p.bending, p.temp, p.kbond, (uint32_t)p.seed, p.noise,
                0, 0, 0, 0};
      d.inv_perp = 1.0 / p.zeta_perp;
      d.dinv = 1.0 / p.zeta_para - 1.0 / p.zeta_perp;
      d.sinv_perp = 1.0 / std::sqrt(p.zeta_perp);
      d.dsinv = 1.0 / std::sqrt(p.zeta_para) - 1.0 / std::sqrt(p.zeta_perp);
      par.push_back(d);
      for (auto& r : semis[k].first) {
        if (r.end > r.start) starts.push_back(r.start);
        for (int j = r.start; j < r.end; ++j) {
          if (fix[j] >= 0) throw std::runtime_error("a bead may belong to one semiflexible fix only");
          fix[j] = (int)k; s0[j] = r.start; ln[j] = r.end - r.start;
        }
      }
    }
    sf_fix.alloc(fix.size() * 4); sf_start.alloc(s0.size() * 4); sf_len.alloc(ln.size() * 4);
    CK(cudaMemcpy(sf_fix.p, fix.data(), fix.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sf_start.p, s0.data(), s0.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(sf_len.p, ln.data(), ln.size() * 4, cudaMemcpyHostToDevice));
    nchains = (int)starts.size();
    chain0.alloc(std::max<size_t>(starts.size(), 1) * 4);
    if (!starts.empty()) CK(cudaMemcpy(chain0.p, starts.data(), starts.size() * 4, cudaMemcpyHostToDevice));
    sf_par.alloc(std::max<size_t>(par.size(), 1) * sizeof(SemiDev));
    if (!par.empty()) CK(cudaMemcpy(sf_par.p, par.data(), par.size() * sizeof(SemiDev), cudaMemcpyHostToDevice));
    if (ntypes > 0) {
      std::vector<double> g(3 * (size_t)ntypes, 0.0);
      for (int t = 0; t < ntypes && !ga_cutsq.empty(); ++t) {
        g[t] = ga_cutsq[t]; g[ntypes + t] = ga_eps[t]; g[2 * ntypes + t] = ga_phi[t];
      }
      ga_dev.alloc(g.size() * 8);
      CK(cudaMemcpy(ga_dev.p, g.data(), g.size() * 8, cudaMemcpyHostToDevice));
    }
  }

  template <typename T>
  PairArgs<T> pair_args() {
    PairArgs<T> p{};
    p.lj = have_lj;
    p.lj_cutsq = lj_cut * lj_cut;
    p.lj1 = lj1;
    p.lj2 = lj2;
    p.ga_style = ga_style;
    p.ga_cutsq = ga_dev.as<double>();
    p.ga_eps = ga_dev.as<double>() + ntypes;
    p.ga_phi = ga_dev.as<double>() + 2 * ntypes;
    p.phi = phi.as<T>(); p.gx = gx.as<T>(); p.gy = gy.as<T>(); p.gz = gz.as<T>();
    p.dep = dep.as<T>();
    p.dv = gridset ? (period[0] / N[0]) * (period[1] / N[1]) * (period[2] / N[2]) : 1.0;
    return p;
  }

  // ------------------------------------------------------------------ reference noise stream
  // Draw order of Conjugate::update on one rank (conjugate.cpp:163-247):
  // bulk (ky, kz, kx ascending), the kx = 0 and kx = Nx/2 planes
  // (single + line_single), then the real points.  Stored per canonical mode.
  void fill_reference_uniforms() {
    const int Nx = N[0], Ny = N[1], Nz = N[2], Nxh = Nx / 2 + 1;
    std::uniform_real_distribution<double> rd(-0.5, 0.5);
    auto at = [&](int kx, int kz, int ky) -> double2& { return uref_h[((size_t)kx * Nz + kz) * Ny + ky]; };
    auto two = [&](int ky, int kz, int kx) { double a = rd(c_gen); double b = rd(c_gen); at(kx, kz, ky) = make_double2(a, b); };
    auto one = [&](int ky, int kz, int kx) { double a = rd(c_gen); at(kx, kz, ky) = make_double2(a, 0.0); };
    for (int ky = 0; ky < Ny; ++ky)
      for (int kz = 0; kz < Nz; ++kz)
        for (int kx = 1; kx < Nxh - 1; ++kx) two(ky, kz, kx);
    for (int kx = 0; kx < Nxh; kx += Nxh - 1) {
      for (int kz = 1; kz < Nz / 2; ++kz) two(0, kz, kx);
      for (int ky = 1; ky < Ny / 2; ++ky) for (int kz = 1; kz < Nz / 2; ++kz) two(ky, kz, kx);
      for (int ky = Ny / 2 + 1; ky < Ny; ++ky) for (int kz = 1; kz < Nz / 2; ++kz) two(ky, kz, kx);
      for (int kz = 1; kz < Nz / 2; ++kz) two(Ny / 2, kz, kx);
      for (int ky = 1; ky < Ny / 2; ++ky) two(ky, 0, kx);
      for (int ky = Ny / 2 + 1; ky < Ny; ++ky) two(ky, Nz / 2, kx);
    }
    one(0, Nz / 2, 0);
    one(0, Nz / 2, Nxh - 1);
    one(0, 0, Nxh - 1);
    one(Ny / 2, 0, 0);
    one(Ny / 2, Nz / 2, 0);
    one(Ny / 2, Nz / 2, Nxh - 1);
    one(Ny / 2, 0, Nxh - 1);
  }

  // ------------------------------------------------------------------ step
  template <typename T>
  void gradient_from_phi() {
    r2c<T>(phi.as<T>(), nullptr, w1.as<cpx<T>>(), plain_fh());
    inverse_chain<T>(w1.as<cpx<T>>(), nullptr, nullptr, (T)0, (T)(1.0 / (double)nreal), true, false);
  }

  template <typename T>
  void enqueue_step() {
    mark(-1);
    const bool resident = schedule == PHAFD_SCHEDULE_RESIDENT && have_conj;
    // the neighbor check increments the step counter when it runs first
    const bool fold_step = resident && n > 0;
    if (!fold_step) launch_step_begin(d_step(), st);
    // the check may run on the previous step's bead branch when nothing
    // between the two reads the beads: no gradient mask (whose guard and
    // rebuild the inverse chain reads), no touch test at the step's end, no
    // bead substeps; the pair kernel then increments the step counter
    const bool pairs_run = n > 0 && (have_lj || ga_style != PHAFD_GRIDATOM_NONE);
    const bool early_ok = resident && !profiling && pairs_run && nsub <= 1 && !touch_on && !gmask_steps();
    const bool checked = early_ok && check_done_early;
    // fixgrid_gradphi.cpp:45: "once" tests timestep == firststep after the
    // increment, which never holds inside a run: only "every" recomputes
    if (!resident && (have_conj || (have_gradphi && !gradphi_once))) gradient_from_phi<T>();
    mark(0);
    // neighbor
    if (n > 0 && !checked) neighbor_stage(nullptr, fold_step ? d_step() : nullptr);
    mark(1);
    // pairs (computed once: the reference's second pass reproduces the first, integrate.cpp:140-146)
    PairArgs<T> pa = pair_args<T>();
    if (checked) pa.step_inc = d_step();
    if (n > 0 && pair_snapshot && bx_pair.p)
      CK(cudaMemcpyAsync(bx_pair.p, bx.p, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (n > 0 && (have_lj || ga_style != PHAFD_GRIDATOM_NONE)) launch_pair<T>(ba, pa, st);
    mark(2);
    // Bead integration needs only F: off the profiling path it runs on a
    // second stream, a parallel branch of the step, while the field passes run.
    const bool fork = !profiling && n > 0;
    cudaStream_t bs = fork ? st2 : st;
    if (fork) {
      CK(cudaEventRecord(ev_fork, st));
      CK(cudaStreamWaitEvent(st2, ev_fork, 0));
    }
    // initial_integrate, then final_integrate of the beads (independent of
    // the field update).  Without drag fixes both chain halves are one launch;
    // on the resident bead branch it follows the deposit reset, so it runs
    // beside the y and z passes rather than beside the persistent x r2c
    // (whose CTAs fill the SMs and would otherwise wait for its blocks)
    const bool one_launch = !(ba.any_drag || ba.nchains == 0);
    const bool masked = resident && gmask_steps();  // its guard reads the integrated positions
    const bool late_chain = one_launch && fork && resident && have_conj && !masked;
    if (!one_launch) {
      launch_drag(ba, dt, bs);
      launch_chain_half<T>(ba, 0, dt, bs, nsub, 0);
      launch_drag(ba, dt, bs);
      launch_chain_half<T>(ba, 1, dt, bs, nsub, 0);
    } else if (!late_chain) {
      launch_chain_step<T>(ba, dt, bs, nsub, 0);
    }
    if (masked) {
      launch_gmask_guard(ba, bs);
      grad_partial = true;
    }
    mark(3);
    if (have_conj) {
      const FHArgs fh = step_fh();
      if (resident) {
        // post_force + pre_final_integrate fused into the x r2c, y fft; then
        // z fft + update + z ifft in one pass (planes finished separately)
        const cpx<T>* twf[3] = {tw[0][0].as<cpx<T>>(), tw[1][0].as<cpx<T>>(), tw[2][0].as<cpx<T>>()};
        cpx<T>* W1 = w1.as<cpx<T>>();
        const int prc = use_plane ? GridOps<T>::xy_fwd(geom, phi.as<T>(), dep.as<T>(), W1, twf[0], twf[1], fh, st) : -3;
        if (prc == -3) {
          chk(GridOps<T>::xr2c(geom, phi.as<T>(), dep.as<T>(), W1, twf[0], fh, st), "x r2c");
          mark(4);
          dep_reset<T>(fork);
          if (late_chain) launch_chain_step<T>(ba, dt, bs, nsub, 0);
          macro_bead_substeps<T>(bs);
          if (early_ok && check_next_early && fork) neighbor_stage(st2, nullptr);
          chk(GridOps<T>::ypass(geom, -1, W1, W1, nullptr, twf[1], st), "y fft");
        } else {
          chk(prc, "xy fwd");
          mark(4);
          dep_reset<T>(fork);
          if (late_chain) launch_chain_step<T>(ba, dt, bs, nsub, 0);
          macro_bead_substeps<T>(bs);
          if (early_ok && check_next_early && fork) neighbor_stage(st2, nullptr);
        }
        mark(5);
        mark(6);
        // the state stays an unnormalised r2c spectrum: store N * update
        UpdateArgs<T> u = update_args<T>(phat[cur].as<cpx<T>>(), muhat.as<cpx<T>>(), phat[1 - cur].as<cpx<T>>(),
                                         (double)nreal);
        u.phi_off = (T)ref_c();  // the inverse chain transforms phi' - c; the c2r adds c back
        // the two Hermitian planes (kx = 0, Nx/2) on a parallel branch, the
        // bulk planes on the main stream
        cudaStream_t ps = fork ? st3 : st;
        if (fork) {
          CK(cudaEventRecord(ev_pl_fork, st));
          CK(cudaStreamWaitEvent(st3, ev_pl_fork, 0));
        }
        chk(GridOps<T>::zfwd_planes(geom, W1, muhat.as<cpx<T>>(), twf[2], ps), "z planes fwd");
        chk(GridOps<T>::zpass_planes(geom, wA.as<cpx<T>>(), wB.as<cpx<T>>(), tw[2][1].as<cpx<T>>(), u, ps), "z planes");
        chk(GridOps<T>::zfused(geom, W1, muhat.as<cpx<T>>(), wA.as<cpx<T>>(), wB.as<cpx<T>>(), twf[2],
                               tw[2][1].as<cpx<T>>(), u, keep_chempot ? 1 : 0, 1, st), "z fused");
        if (fork) {
          CK(cudaEventRecord(ev_pl_join, st3));
          CK(cudaStreamWaitEvent(st, ev_pl_join, 0));
        }
        mark(7);
        // the bead substeps read phi and grad phi, which the inverse
        // overwrites; the masked inverse reads the guard's verdict
        if (fork && (nsub > 1 || masked)) {
          CK(cudaEventRecord(ev_join, st2));
          CK(cudaStreamWaitEvent(st, ev_join, 0));
        }
        if (!use_plane || !yx_fused<T>(ref_c())) yx_inverse<T>(phi.as<T>(), (T)1, (T)1, true, true, masked, ref_c());
      } else {
        // post_force + pre_final_integrate: mu = dep + FH(phi), r2c
        r2c<T>(phi.as<T>(), dep.as<T>(), muhat.as<cpx<T>>(), fh);
        dep_reset<T>(fork);
        UpdateArgs<T> u = update_args<T>(w1.as<cpx<T>>(), muhat.as<cpx<T>>(), phat[0].as<cpx<T>>(), 1.0);
        inverse_chain<T>(nullptr, &u, phi.as<T>(), (T)1, (T)1, false, true);
      }
    }
    if (fork) {  // join the bead branch before the next step
      CK(cudaEventRecord(ev_join, st2));
      CK(cudaStreamWaitEvent(st, ev_join, 0));
    }
    if (touch_on && n > 0)
      launch_touch(bx.as<double>(), n, touch_point, touch_delay, d_step(), touch.as<TouchState>(), st);
  }

  // Neighbor::decide + build.  Inside a graph capture the rebuild kernels
  // form the body of a conditional node that the check kernel switches on,
  // so a step without a rebuild runs one kernel here instead of eleven.
  void neighbor_stage(cudaStream_t sn = nullptr, long long* step_inc = nullptr) {
    if (!sn) sn = st;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    CK(cudaStreamGetCaptureInfo(sn, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive) {
      launch_neighbor(ba, false, sn, step_inc);
      return;
    }
    cudaGraphConditionalHandle h;
    CK(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    launch_neighbor_check(ba, h, 1, sn, step_inc);
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    CK(cudaStreamGetCaptureInfo(sn, &cs, nullptr, &g, &deps, nullptr, &ndeps));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
    CK(cudaStreamUpdateCaptureDependencies(sn, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(stc, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    launch_rebuild(ba, stc);
    cudaGraph_t unused = nullptr;
    CK(cudaStreamEndCapture(stc, &unused));
    rebuild_kernels = count_kernels(body);
  }

  // Substeps 1..nsub-1 of a macro step for the beads: neighbor check, pair
  // forces against the field of the step's start (no deposit: the field's
  // linearised update uses the deposit of substep 0), integration with dt.
  // They follow the deposit reset on the bead stream, so the reset sees the
  // lists the deposit used.
  template <typename T>
  void macro_bead_substeps(cudaStream_t bs) {
    if (nsub <= 1 || n == 0) return;
    PairArgs<T> pa = pair_args<T>();
    pa.dep = nullptr;
    for (int sub = 1; sub < nsub; ++sub) {
      neighbor_stage(bs);
      if (have_lj || ga_style != PHAFD_GRIDATOM_NONE) launch_pair<T>(ba, pa, bs);
      if (ba.any_drag || ba.nchains == 0) {
        launch_drag(ba, dt, bs);
        launch_chain_half<T>(ba, 0, dt, bs, nsub, sub);
        launch_drag(ba, dt, bs);
        launch_chain_half<T>(ba, 1, dt, bs, nsub, sub);
      } else {
        launch_chain_step<T>(ba, dt, bs, nsub, sub);
      }
    }
  }

  // The deposit is zeroed by the next neighbor check (on its grid lists);
  // forked, the bead branch waits here for the x pass that reads the
  // deposit, since its check comes later on that branch.
  template <typename T>
  void dep_reset(bool fork) {
    if (n == 0 || ga_style == PHAFD_GRIDATOM_NONE || !fork) return;
    CK(cudaEventRecord(ev_dep, st));
    CK(cudaStreamWaitEvent(st2, ev_dep, 0));
  }

  void step_once() {
    if (precision == PHAFD_FP64) enqueue_step<double>();
    else enqueue_step<float>();
  }
};

// ====================================================================== helpers
#define API_BEGIN(c)                     \
  if (!(c)) return PHAFD_ERR_INVALID;    \
  try {
#define API_END(c)                                          \
  return PHAFD_OK;                                          \
  }                                                         \
  catch (const CudaError& e) {                              \
    (c)->err = e.what();                                    \
    return PHAFD_ERR_CUDA;                                  \
  }                                                         \
  catch (const std::exception& e) {                         \
    (c)->err = e.what();                                    \
    return PHAFD_ERR_INVALID;                               \
  }

static void resident_spectrum_flip(phafd_ctx* c) { c->cur = 1 - c->cur; }

template <typename T>
static void copy_real_to_host(phafd_ctx* c, const DevBuf& b, double* host) {
  std::vector<T> tmp(c->nreal);
  CK(cudaMemcpyAsync(tmp.data(), b.p, c->nreal * sizeof(T), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (size_t i = 0; i < c->nreal; ++i) host[i] = (double)tmp[i];
}

template <typename T>
static void copy_real_to_dev(phafd_ctx* c, DevBuf& b, const double* host) {
  std::vector<T> tmp(host, host + c->nreal);
  CK(cudaMemcpyAsync(b.p, tmp.data(), c->nreal * sizeof(T), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
}

// device layout [kx][kz][ky] -> reference layout [ky][kz][kx], times `scale`
template <typename T>
static void copy_spec_to_host(phafd_ctx* c, const DevBuf& b, double* host, double scale) {
  std::vector<T> tmp(2 * c->ncplx);
  CK(cudaMemcpyAsync(tmp.data(), b.p, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const int Nx = c->N[0], Ny = c->N[1], Nz = c->N[2], Nxh = Nx / 2 + 1;
  for (int kx = 0; kx < Nxh; ++kx)
    for (int kz = 0; kz < Nz; ++kz)
      for (int ky = 0; ky < Ny; ++ky) {
        const size_t s = ((size_t)kx * Nz + kz) * Ny + ky;
        const size_t d = ((size_t)ky * Nz + kz) * Nxh + kx;
        host[2 * d] = (double)tmp[2 * s] * scale;
        host[2 * d + 1] = (double)tmp[2 * s + 1] * scale;
      }
}

static int check_status(phafd_ctx* c) {
  long long h[6];
  CK(cudaMemcpyAsync(h, c->d_counters.p, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  int status = ((int*)&h[5])[1];
  if (h[3] >= 0) {
    c->err = "NAN encountered in phi. (step " + std::to_string(h[3]) + ")";
    return PHAFD_ERR_NAN;
  }
  if (status & ST_OVERFLOW) {
    c->err = "Neighbor list overflow";
    return PHAFD_ERR_OVERFLOW;
  }
  if (status & ST_CONSTRAINT) {
    c->err = "Failed to maintain polymer bond-length constraints.";
    return PHAFD_ERR_CONSTRAINT;
  }
  if (status & ST_TIMEOUT) {
    c->err = "a grid pass gave up waiting for its tensor-map loads";
    return PHAFD_ERR_TIMEOUT;
  }
  return PHAFD_OK;
}

// ====================================================================== C ABI
extern "C" {

const char* phafd_build_info(void) {
  return "libphafd_gpu: sm_103a; FFT lengths 16,32,64,96,128,160,256,512; FP32 and FP64 grid paths";
}

int phafd_ctx_create(phafd_ctx** out, int device, int precision) {
  if (!out) return PHAFD_ERR_INVALID;
  *out = nullptr;
  if (precision != PHAFD_FP32 && precision != PHAFD_FP64) return PHAFD_ERR_INVALID;
  phafd_ctx* c = new phafd_ctx();
  c->device = device;
  c->precision = precision;
  try {
    CK(cudaSetDevice(device));
    // highest priority: a step's chain of small bead kernels is scheduled
    // ahead of concurrent bulk work on other streams (the network inference
    // that overlaps a macro step)
    int plo = 0, phi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&plo, &phi));
    CK(cudaStreamCreateWithPriority(&c->st, cudaStreamNonBlocking, phi));
    CK(cudaStreamCreateWithPriority(&c->st2, cudaStreamNonBlocking, phi));
    CK(cudaStreamCreateWithPriority(&c->st3, cudaStreamNonBlocking, phi));
    CK(cudaStreamCreateWithPriority(&c->stc, cudaStreamNonBlocking, phi));
    for (cudaEvent_t* e : {&c->ev_fork, &c->ev_dep, &c->ev_join, &c->ev_pl_fork, &c->ev_pl_join})
      CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    c->d_counters.alloc(7 * sizeof(long long));
    long long init[7] = {0, 0, 0, -1, 0, 0, 0};
    CK(cudaMemcpy(c->d_counters.p, init, sizeof(init), cudaMemcpyHostToDevice));
  } catch (const std::exception& e) {
    delete c;
    return PHAFD_ERR_CUDA;
  }
  *out = c;
  return PHAFD_OK;
}

int phafd_ctx_destroy(phafd_ctx* c) {
  if (!c) return PHAFD_ERR_INVALID;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  delete c;
  return PHAFD_OK;
}

const char* phafd_last_error(phafd_ctx* c) { return c ? c->err.c_str() : "null context"; }

int phafd_set_zghost(phafd_ctx* c, int mode) {
  API_BEGIN(c)
  if (mode != PHAFD_ZGHOST_RANK1 && mode != PHAFD_ZGHOST_PERIODIC) throw std::invalid_argument("bad zghost mode");
  c->zghost = mode;
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_schedule(phafd_ctx* c, int schedule) {
  API_BEGIN(c)
  if (schedule != PHAFD_SCHEDULE_REFERENCE && schedule != PHAFD_SCHEDULE_RESIDENT) throw std::invalid_argument("bad schedule");
  if (c->setup_done) throw std::runtime_error("schedule must be chosen before setup");
  c->schedule = schedule;
  API_END(c)
}

int phafd_set_plane_fusion(phafd_ctx* c, int on) {
  API_BEGIN(c)
  c->use_plane = on != 0;
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_fp32_centering(phafd_ctx* c, int stages) {
  API_BEGIN(c)
  if (stages & ~(PHAFD_CENTER_FH | PHAFD_CENTER_FFT)) throw std::invalid_argument("unknown centering stage");
  c->center_bits = stages;
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_gradient_mask(phafd_ctx* c, int on) {
  API_BEGIN(c)
  const bool was = c->use_gmask;
  c->use_gmask = on != 0;
  if (c->use_gmask && !was && c->setup_done) {
    CK(cudaSetDevice(c->device));
    c->alloc_gmask();  // stale until the next neighbor rebuild: full stores meanwhile
    CK(cudaStreamSynchronize(c->st));
  }
  if (c->setup_done) c->fill_bead_args();
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_pair_snapshot(phafd_ctx* c, int on) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  c->pair_snapshot = on != 0;
  c->pair_snapped = false;
  if (c->pair_snapshot && c->n > 0) c->bx_pair.alloc(3 * (size_t)c->n * sizeof(double));
  c->invalidate_graph();
  API_END(c)
}

// ComputePair::end_of_step (compute_pair.cpp:43-85) after the last step: the
// style's pair loop over the gathered copies the step's pair stage formed
// (the reference integrates only the owned beads, so the copies stay there),
// with the gradient arrays of the step's start and phi after the update
int phafd_compute_pair(phafd_ctx* c, int style, int add_to_chempot, double* out) {
  API_BEGIN(c)
  if (style != PHAFD_PAIR_LJ_CUT && style != PHAFD_PAIR_GRIDATOM) throw std::invalid_argument("unknown pair style");
  if (style == PHAFD_PAIR_LJ_CUT && !c->have_lj)
    throw std::invalid_argument("Cannot compute pair style lj/cut, it hasn't been created!");
  if (style == PHAFD_PAIR_GRIDATOM && c->ga_style == PHAFD_GRIDATOM_NONE)
    throw std::invalid_argument("Cannot compute pair style gridatom, it hasn't been created!");
  if (c->n == 0) return PHAFD_OK;
  if (!c->pair_snapped || !c->bx_pair.p)
    throw std::runtime_error("compute pair needs steps taken after phafd_set_pair_snapshot(ctx, 1)");
  CK(cudaSetDevice(c->device));
  const bool loaded = style == PHAFD_PAIR_GRIDATOM && c->load_step_start_gradient();
  const size_t bytes = 3 * (size_t)c->n * sizeof(double);
  if (c->bf_tmp.bytes < bytes) c->bf_tmp.alloc(bytes);
  c->fill_bead_args();
  BeadArgs a = c->ba;
  a.x = c->bx_pair.as<double>();
  a.f = c->bf_tmp.as<double>();
  const bool dep = add_to_chempot && style == PHAFD_PAIR_GRIDATOM && c->chempot_from_mu && c->mu.p;
  if (c->precision == PHAFD_FP64) {
    PairArgs<double> p = c->pair_args<double>();
    p.lj = style == PHAFD_PAIR_LJ_CUT;
    if (style != PHAFD_PAIR_GRIDATOM) p.ga_style = PHAFD_GRIDATOM_NONE;
    p.dep = dep ? c->mu.as<double>() : nullptr;
    launch_pair<double>(a, p, c->st);
  } else {
    PairArgs<float> p = c->pair_args<float>();
    p.lj = style == PHAFD_PAIR_LJ_CUT;
    if (style != PHAFD_PAIR_GRIDATOM) p.ga_style = PHAFD_GRIDATOM_NONE;
    p.dep = dep ? c->mu.as<float>() : nullptr;
    launch_pair<float>(a, p, c->st);
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(out, c->bf_tmp.p, bytes, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (loaded) c->restore_gradient();
  API_END(c)
}

int phafd_set_keep_chempot(phafd_ctx* c, int keep) {
  API_BEGIN(c)
  c->keep_chempot = keep != 0;
  if (c->keep_chempot && c->gridset && !c->mu.p) { c->mu.alloc(c->nreal * c->rsz()); c->mu.zero(c->st); }
  c->invalidate_graph();
  API_END(c)
}

int phafd_domain(phafd_ctx* c, const double* boxlo, const double* period) {
  API_BEGIN(c)
  for (int d = 0; d < 3; ++d) {
    if (!(period[d] > 0)) throw std::invalid_argument("Bad arguments for domain_setup.");
    c->boxlo[d] = boxlo[d];
    c->period[d] = period[d];
    c->boxhi[d] = boxlo[d] + period[d];
  }
  c->boxset = true;
  API_END(c)
}

int phafd_grid_style(phafd_ctx* c, int nx, int ny, int nz) {
  API_BEGIN(c)
  if (!c->boxset) throw std::invalid_argument("CAnnot use command grid_style before domain box is set.");
  if (!fft_size_supported(nx) || !fft_size_supported(ny) || !fft_size_supported(nz))
    throw std::invalid_argument("grid sizes must be one of 16, 32, 64, 96, 128, 160, 256, 512");
  CK(cudaSetDevice(c->device));
  c->N[0] = nx; c->N[1] = ny; c->N[2] = nz;
  c->nreal = (size_t)nx * ny * nz;
  c->ncplx = (size_t)(nx / 2 + 1) * ny * nz;
  c->geom.nx = nx; c->geom.ny = ny; c->geom.nz = nz; c->geom.nxh = nx / 2 + 1;
  for (int d = 0; d < 3; ++d) c->geom.kq[d] = 2 * 3.141592 / c->period[d];  // domain.cpp:206-208
  c->alloc_grid();
  if (c->keep_chempot) { c->mu.alloc(c->nreal * c->rsz()); c->mu.zero(c->st); }
  c->gridset = true;
  API_END(c)
}

int phafd_grid_populate_constant(phafd_ctx* c, double average, double variance, int seed) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("CAnnot use command grid_populate before grid_style is set.");
  std::vector<double> h(c->nreal);
  std::uniform_real_distribution<double> rd(-0.5, 0.5);
  std::mt19937 gen;
  gen.seed(make_unique_seed(seed));  // grid.cpp:120-131, 289-307
  for (auto& v : h) v = average + variance * rd(gen);
  if (c->precision == PHAFD_FP64) copy_real_to_dev<double>(c, c->phi, h.data());
  else copy_real_to_dev<float>(c, c->phi, h.data());
  c->populated = true;
  API_END(c)
}

static void upload_phi(phafd_ctx* c, const std::vector<double>& h) {
  if (c->precision == PHAFD_FP64) copy_real_to_dev<double>(c, c->phi, h.data());
  else copy_real_to_dev<float>(c, c->phi, h.data());
  c->populated = true;
}

int phafd_grid_populate_flat_interface(phafd_ctx* c, double average, double variance, double hi, double lo,
                                       int seed) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("CAnnot use command grid_populate before grid_style is set.");
  std::vector<double> h(c->nreal);
  std::uniform_real_distribution<double> rd(-0.5, 0.5);
  std::mt19937 gen;
  gen.seed(make_unique_seed(seed));  // grid.cpp:123-134, 310-337
  const double Lbox = (average - lo) / (hi - lo) * c->period[0];
  const double Ox = c->boxlo[0], dx = c->period[0] / c->N[0];
  size_t n = 0;
  for (int i = 0; i < c->N[2]; i++)
    for (int j = 0; j < c->N[1]; j++)
      for (int k = 0; k < c->N[0]; k++) {
        const double x = k * dx + Ox;
        h[n++] = (x - Ox < Lbox ? hi : lo) + variance * rd(gen);
      }
  upload_phi(c, h);
  API_END(c)
}

int phafd_grid_populate_sphere(phafd_ctx* c, double radius, double width, double hi, double average) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("CAnnot use command grid_populate before grid_style is set.");
  for (int d = 0; d < 3; d++)  // grid.cpp:339-425
    if (radius >= c->period[d] / 2.) throw std::runtime_error("Initial spherical configuration has radius > domain.");
  const double h3[3] = {c->period[0] / c->N[0], c->period[1] / c->N[1], c->period[2] / c->N[2]};
  std::vector<double> f(c->nreal);  // tanh((radius - r) / width) at every node, [z][y][x]
  double integral = 0;
  size_t n = 0;
  for (int i = 0; i < c->N[2]; i++) {
    const double z = i * h3[2] + c->boxlo[2];
    for (int j = 0; j < c->N[1]; j++) {
      const double y = j * h3[1] + c->boxlo[1];
      for (int k = 0; k < c->N[0]; k++) {
        const double x = k * h3[0] + c->boxlo[0];
        f[n] = std::tanh((-std::sqrt(x * x + y * y + z * z) + radius) / width);
        integral += f[n++];
      }
    }
  }
  integral *= h3[0] * h3[1] * h3[2];
  const double ifrac = integral / (c->period[0] * c->period[1] * c->period[2]);
  const double lo = (2 * average - hi * (1 + ifrac)) / (1 - ifrac);
  if (lo < 0) throw std::runtime_error("Average array value is too small for specified radius.");
  if (lo > hi) throw std::runtime_error("Average array value is too large for specified radius.");
  for (auto& v : f) v = 0.5 * (hi - lo) * v + 0.5 * (hi + lo);
  upload_phi(c, f);
  API_END(c)
}

int phafd_noise_state_get(phafd_ctx* c, char* buf, int cap, int* len) {
  API_BEGIN(c)
  std::ostringstream os;
  os << c->c_gen;  // the 624 words and position of the host generator, as text
  const std::string st = os.str();
  if (len) *len = (int)st.size() + 1;
  if (buf) {
    if (cap < (int)st.size() + 1) throw std::invalid_argument("noise state buffer too small");
    std::memcpy(buf, st.c_str(), st.size() + 1);
  }
  API_END(c)
}

int phafd_noise_state_set(phafd_ctx* c, const char* state) {
  API_BEGIN(c)
  if (!state) throw std::invalid_argument("null noise state");
  if (!c->have_conj) throw std::runtime_error("noise state needs fix grid/conjugate/volfrac");
  std::istringstream is(state);
  std::mt19937 g;
  is >> g;
  if (is.fail()) throw std::invalid_argument("malformed noise state");
  c->c_gen = g;
  API_END(c)
}

int phafd_grid_set(phafd_ctx* c, int field, const double* host) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("grid not created");
  DevBuf* b = field == PHAFD_FIELD_PHI ? &c->phi : field == PHAFD_FIELD_GRADX ? &c->gx
            : field == PHAFD_FIELD_GRADY ? &c->gy : field == PHAFD_FIELD_GRADZ ? &c->gz : nullptr;
  if (!b) throw std::invalid_argument("field cannot be set");
  if (field != PHAFD_FIELD_PHI) c->full_gradient();  // the other two components stay complete
  if (c->precision == PHAFD_FP64) copy_real_to_dev<double>(c, *b, host);
  else copy_real_to_dev<float>(c, *b, host);
  if (field == PHAFD_FIELD_PHI) c->populated = true;
  API_END(c)
}

int phafd_grid_get(phafd_ctx* c, int field, double* host) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("grid not created");
  const bool f64 = c->precision == PHAFD_FP64;
  if ((field == PHAFD_FIELD_CHEMPOT && c->chempot_lost) || (field == PHAFD_FIELD_FT_CHEMPOT && c->muhat_stale))
    throw std::runtime_error("chempot after a run is kept only when phafd_set_keep_chempot(ctx, 1) precedes the steps");
  if (field >= PHAFD_FIELD_GRADX_STEP_START && field <= PHAFD_FIELD_GRADZ_STEP_START) {
    if (!c->stepped) {
      std::fill(host, host + c->nreal, 0.0);
    } else {
      const bool loaded = c->load_step_start_gradient();
      const DevBuf& b = field == PHAFD_FIELD_GRADX_STEP_START ? c->gx : field == PHAFD_FIELD_GRADY_STEP_START ? c->gy : c->gz;
      if (f64) copy_real_to_host<double>(c, b, host);
      else copy_real_to_host<float>(c, b, host);
      if (loaded) c->restore_gradient();
    }
  } else if (field == PHAFD_FIELD_FT_PHI_STEP_START) {
    if (c->schedule != PHAFD_SCHEDULE_RESIDENT || !c->have_conj)
      throw std::invalid_argument("the step-start spectrum is kept by the resident schedule");
    if (!c->stepped) {
      std::fill(host, host + 2 * c->ncplx, 0.0);
    } else if (f64) {  // the ping-pong buffer the last step read
      copy_spec_to_host<double>(c, c->phat[1 - c->cur], host, 1.0);
    } else {
      copy_spec_to_host<float>(c, c->phat[1 - c->cur], host, 1.0);
    }
  } else if (field == PHAFD_FIELD_FT_PHI || field == PHAFD_FIELD_FT_CHEMPOT) {
    const DevBuf* b;
    double sc = 1.0;
    if (field == PHAFD_FIELD_FT_CHEMPOT) b = &c->muhat;
    else if (c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj) b = &c->phat[c->cur];
    else if (c->have_conj && c->setup_done) { b = &c->phat[0]; sc = (double)c->nreal; }
    else b = &c->w1;
    if (f64) copy_spec_to_host<double>(c, *b, host, sc);
    else copy_spec_to_host<float>(c, *b, host, sc);
    // an FP32 context transforms mu - tv f(c) (see FHArgs): restore its k = 0 mode
    if (field == PHAFD_FIELD_FT_CHEMPOT) host[0] += c->mu_origin_shift();
  } else {
    const DevBuf* b = field == PHAFD_FIELD_PHI ? &c->phi : field == PHAFD_FIELD_GRADX ? &c->gx
                    : field == PHAFD_FIELD_GRADY ? &c->gy : field == PHAFD_FIELD_GRADZ ? &c->gz
                    : field == PHAFD_FIELD_CHEMPOT ? (c->chempot_from_mu ? &c->mu : &c->dep) : nullptr;
    if (!b) throw std::invalid_argument("bad field");
    if (field == PHAFD_FIELD_GRADX || field == PHAFD_FIELD_GRADY || field == PHAFD_FIELD_GRADZ) c->full_gradient();
    if (f64) copy_real_to_host<double>(c, *b, host);
    else copy_real_to_host<float>(c, *b, host);
  }
  API_END(c)
}

int phafd_atoms_create(phafd_ctx* c, int n, const int* tags, const int* mol, const int* types, const double* x) {
  API_BEGIN(c)
  if (n < 0) throw std::invalid_argument("negative bead count");
  CK(cudaSetDevice(c->device));
  c->n = n;
  c->images_restored = false;
  c->tags.assign(tags, tags + n);
  c->types.assign(types, types + n);
  c->mol.assign(mol ? mol : tags, (mol ? mol : tags) + n);
  std::vector<int> sorted_tags(c->tags);
  std::sort(sorted_tags.begin(), sorted_tags.end());
  if (std::adjacent_find(sorted_tags.begin(), sorted_tags.end()) != sorted_tags.end())
    throw std::runtime_error("duplicate IDs found on processor(s).");
  int tmax = -1;
  for (int t : c->types) tmax = std::max(tmax, t);
  c->ntypes = tmax + 1;
  const size_t nn = std::max(n, 1);
  for (auto* b : {&c->bx, &c->bux, &c->bf, &c->bxhold, &c->bfchain, &c->btang}) { b->alloc(3 * nn * 8); b->zero(c->st); }
  c->bimage.alloc(nn * 4);
  c->btype.alloc(nn * 4);
  if (n > 0) {
    CK(cudaMemcpy(c->bx.p, x, 3 * (size_t)n * 8, cudaMemcpyHostToDevice));
    std::vector<int> img(n, (512 << 20) | (512 << 10) | 512);  // Domain::set_image
    CK(cudaMemcpy(c->bimage.p, img.data(), n * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->btype.p, types, n * 4, cudaMemcpyHostToDevice));
  }
  API_END(c)
}

int phafd_atoms_get(phafd_ctx* c, double* x, double* ux, double* f, int* images) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  const size_t n = c->n;
  if (n == 0) return PHAFD_OK;
  if (x) CK(cudaMemcpy(x, c->bx.p, 3 * n * 8, cudaMemcpyDeviceToHost));
  if (ux) CK(cudaMemcpy(ux, c->bux.p, 3 * n * 8, cudaMemcpyDeviceToHost));
  if (f) CK(cudaMemcpy(f, c->bf.p, 3 * n * 8, cudaMemcpyDeviceToHost));
  if (images) CK(cudaMemcpy(images, c->bimage.p, n * 4, cudaMemcpyDeviceToHost));
  API_END(c)
}

int phafd_atoms_get_async(phafd_ctx* c, double* x, double* ux, double* f, int* images, int slot) {
  API_BEGIN(c)
  if (slot < 0 || slot > 3) throw std::invalid_argument("slot: 0..3");
  CK(cudaSetDevice(c->device));
  if (!c->ev_slot[slot]) CK(cudaEventCreateWithFlags(&c->ev_slot[slot], cudaEventDisableTiming));
  if (!c->slot_status) CK(cudaHostAlloc(reinterpret_cast<void**>(&c->slot_status), 8 * sizeof(long long), 0));
  const size_t n = c->n;
  if (n > 0) {
    if (x) CK(cudaMemcpyAsync(x, c->bx.p, 3 * n * 8, cudaMemcpyDeviceToHost, c->st));
    if (ux) CK(cudaMemcpyAsync(ux, c->bux.p, 3 * n * 8, cudaMemcpyDeviceToHost, c->st));
    if (f) CK(cudaMemcpyAsync(f, c->bf.p, 3 * n * 8, cudaMemcpyDeviceToHost, c->st));
    if (images) CK(cudaMemcpyAsync(images, c->bimage.p, n * 4, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaMemcpyAsync(c->slot_status + 2 * slot, c->d_counters.as<long long>() + 3, sizeof(long long),
                     cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->slot_status + 2 * slot + 1, c->d_counters.as<long long>() + 5, sizeof(long long),
                     cudaMemcpyDeviceToHost, c->st));
  CK(cudaEventRecord(c->ev_slot[slot], c->st));
  API_END(c)
}

int phafd_wait_slot(phafd_ctx* c, int slot) {
  API_BEGIN(c)
  if (slot < 0 || slot > 3 || !c->ev_slot[slot]) throw std::invalid_argument("no read-back enqueued on this slot");
  CK(cudaEventSynchronize(c->ev_slot[slot]));
  const long long nan_step = c->slot_status[2 * slot];
  const int status = reinterpret_cast<const int*>(c->slot_status + 2 * slot + 1)[1];
  if (nan_step >= 0) {
    c->err = "NAN encountered in phi. (step " + std::to_string(nan_step) + ")";
    return PHAFD_ERR_NAN;
  }
  if (status & ST_OVERFLOW) {
    c->err = "Neighbor list overflow";
    return PHAFD_ERR_OVERFLOW;
  }
  if (status & ST_CONSTRAINT) {
    c->err = "Failed to maintain polymer bond-length constraints.";
    return PHAFD_ERR_CONSTRAINT;
  }
  if (status & ST_TIMEOUT) {
    c->err = "a grid pass gave up waiting for its tensor-map loads";
    return PHAFD_ERR_TIMEOUT;
  }
  API_END(c)
}

int phafd_host_register(void* ptr, size_t bytes) {
  if (!ptr || bytes == 0) return PHAFD_ERR_INVALID;
  return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? PHAFD_OK : PHAFD_ERR_CUDA;
}

int phafd_host_unregister(void* ptr) {
  if (!ptr) return PHAFD_ERR_INVALID;
  return cudaHostUnregister(ptr) == cudaSuccess ? PHAFD_OK : PHAFD_ERR_CUDA;
}

int phafd_atoms_set_images(phafd_ctx* c, const int* images) {
  API_BEGIN(c)
  if (!images && c->n > 0) throw std::invalid_argument("null images");
  if (c->setup_done) throw std::runtime_error("image flags are restored before setup");
  CK(cudaSetDevice(c->device));
  if (c->n > 0) CK(cudaMemcpy(c->bimage.p, images, (size_t)c->n * 4, cudaMemcpyHostToDevice));
  c->images_restored = true;
  API_END(c)
}

int phafd_pair_gridatom(phafd_ctx* c, int style, double cut) {
  API_BEGIN(c)
  if (c->ntypes <= 0) throw std::runtime_error("Cannot create pair style before atoms are made.");
  if (style < PHAFD_GRIDATOM_GAUSSIAN || style > PHAFD_GRIDATOM_LJISH_LINEAR) throw std::invalid_argument("Unrecognised pair style.");
  c->ga_style = style;
  c->ga_maxcut = cut;
  c->ga_cutsq.assign(c->ntypes, cut * cut);  // pair_gridatom_gaussian.cpp:127-141
  c->ga_eps.assign(c->ntypes, 1.0);
  c->ga_phi.assign(c->ntypes, 0.1);
  API_END(c)
}

int phafd_pair_gridatom_coeff(phafd_ctx* c, int type, int has_eps, double eps, int has_w, double nucwidth, int has_phi, double phit) {
  API_BEGIN(c)
  if (c->ga_style == PHAFD_GRIDATOM_NONE) throw std::runtime_error("pairCoeffs before a gridatom pair");
  if (type < 0 || type >= c->ntypes) throw std::runtime_error("Pair grid/atom atom type out of range.");
  if (has_eps) c->ga_eps[type] = eps;
  if (has_w) {
    if (nucwidth > c->ga_maxcut) throw std::runtime_error("nucwidth cannot be larger than maximum cut.");
    c->ga_cutsq[type] = nucwidth * nucwidth;
  }
  if (has_phi) c->ga_phi[type] = phit;
  API_END(c)
}

int phafd_pair_lj_cut(phafd_ctx* c, double cut, double eps, double sigma) {
  API_BEGIN(c)
  c->have_lj = true;  // pair_lj_cut.cpp:103-119
  c->lj_cut = cut;
  c->lj1 = 48 * eps * std::pow(sigma, 12.0);
  c->lj2 = 24 * eps * std::pow(sigma, 6.0);
  API_END(c)
}

int phafd_neighbor(phafd_ctx* c, double skin) {
  API_BEGIN(c)
  if (!c->gridset) throw std::runtime_error("Must call neighbor after subboxes are set (via grid style).");
  c->skin = skin;  // neighbor.cpp:39-68
  double cutoff = 0.0;
  if (c->have_lj) cutoff = std::max(cutoff, c->lj_cut);
  if (c->ga_style != PHAFD_GRIDATOM_NONE) cutoff = std::max(cutoff, c->ga_maxcut);
  c->cutneigh = cutoff > 0.0 ? skin + cutoff : 0.0;
  if (c->cutneigh <= 0.0) c->cutneigh = skin > 0 ? skin : 1.0;
  c->neigh_set = true;
  API_END(c)
}

int phafd_fix_conjugate_volfrac(phafd_ctx* c, int seed, double mobility, double temp, double volFH, double gamma, int noise) {
  API_BEGIN(c)
  if (!c->populated) throw std::runtime_error("Fix requires grid to be populated.");
  if (noise != PHAFD_NOISE_OFF && noise != PHAFD_NOISE_REFERENCE && noise != PHAFD_NOISE_PHILOX) throw std::invalid_argument("bad noise mode");
  c->have_conj = true;
  c->c_seed = make_unique_seed(seed);  // fixgrid_conjugate.cpp:33
  c->c_mobility = mobility; c->c_temp = temp; c->c_volFH = volFH; c->c_gamma = gamma;
  c->c_noise = noise;
  c->c_gen.seed(c->c_seed);  // conjugate_volfrac.cpp:64
  if (noise == PHAFD_NOISE_REFERENCE) {
    c->uref.alloc(c->ncplx * sizeof(double2));
    c->uref.zero(c->st);
    if (c->uref_h) cudaFreeHost(c->uref_h);
    CK(cudaMallocHost(&c->uref_h, c->ncplx * sizeof(double2)));
    std::memset(c->uref_h, 0, c->ncplx * sizeof(double2));
  }
  API_END(c)
}

int phafd_fix_floryhuggins(phafd_ctx* c, double temp, double volFH, double chi) {
  API_BEGIN(c)
  if (!c->populated) throw std::runtime_error("Fix requires grid to be populated.");
  c->have_fh = true;
  c->fh_temp = temp; c->fh_volFH = volFH; c->fh_chi = chi;
  API_END(c)
}

int phafd_fix_gradphi(phafd_ctx* c, int once) {
  API_BEGIN(c)
  c->have_gradphi = true;
  c->gradphi_once = once != 0;
  API_END(c)
}

int phafd_fix_drag(phafd_ctx* c, int nranges, const int* starts, const int* ends, double drag) {
  API_BEGIN(c)
  std::vector<Range> r;
  for (int k = 0; k < nranges; ++k) {
    if (starts[k] < 0 || ends[k] > c->n || starts[k] > ends[k]) throw std::invalid_argument("bad group range");
    r.push_back({starts[k], ends[k]});
  }
  c->drags.push_back({r, drag});
  API_END(c)
}

int phafd_fix_semiflexible(phafd_ctx* c, int nranges, const int* starts, const int* ends, const phafd_semiflexible_params* p) {
  API_BEGIN(c)
  std::vector<Range> r;
  for (int k = 0; k < nranges; ++k) {
    if (starts[k] < 0 || ends[k] > c->n || starts[k] > ends[k]) throw std::invalid_argument("bad group range");
    r.push_back({starts[k], ends[k]});
  }
  if (!(p->zeta_para > 0) || !(p->zeta_perp > 0)) throw std::invalid_argument("zeta must be positive");
  c->semis.push_back({r, *p});
  API_END(c)
}

int phafd_set_dt(phafd_ctx* c, double dt) {
  API_BEGIN(c)
  c->dt = dt;
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_timestep(phafd_ctx* c, long long step) {
  API_BEGIN(c)
  c->timestep = c->firststep = step;
  CK(cudaMemcpyAsync(c->d_step(), &c->timestep, sizeof(long long), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  API_END(c)
}

int phafd_setup(phafd_ctx* c) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (c->have_fh && !c->have_conj)
    throw std::runtime_error("fix grid/floryhuggins/gpu runs fused with fix grid/conjugate/volfrac/gpu; define both");
  if (!c->neigh_set && c->n > 0 && (c->have_lj || c->ga_style)) throw std::runtime_error("neighbor must be set before run");
  if (c->have_conj && c->dt <= 0.0) throw std::runtime_error("Cannot run simulation without setting dt > 0.");
  if (c->have_conj && c->geom.nx == 0) throw std::runtime_error("grid not created");
  // FixAtomSemiFlexible::check_bonds, fixatom_semiflexible.cpp:114-140 (on positions as given)
  if (!c->semis.empty() && !c->images_restored) {
    // FixAtomSemiFlexible::check_bonds on the unwrapped positions
    // (fixatom_semiflexible.cpp:114-140)
    std::vector<double> x(3 * (size_t)c->n);
    std::vector<int> img(c->n);
    CK(cudaMemcpy(x.data(), c->bx.p, x.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(img.data(), c->bimage.p, img.size() * 4, cudaMemcpyDeviceToHost));
    for (int i = 0; i < c->n; ++i) {
      const int box[3] = {(img[i] & 1023) - 512, (img[i] >> 10 & 1023) - 512, (img[i] >> 20) - 512};
      for (int d = 0; d < 3; ++d) x[3 * i + d] += box[d] * c->period[d];
    }
    for (auto& f : c->semis)
      for (auto& r : f.first)
        for (int mu = r.start + 1; mu < r.end; ++mu) {
          double d0 = x[3 * mu] - x[3 * (mu - 1)], d1 = x[3 * mu + 1] - x[3 * (mu - 1) + 1], d2 = x[3 * mu + 2] - x[3 * (mu - 1) + 2];
          if (std::abs(std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) - f.second.bondlength) > 1e-3)
            throw std::runtime_error("Adjacent atom displacements do not match the FixAtomSemiFlexible bondlength specified.");
        }
  }
  if (c->pair_snapshot && c->n > 0 && c->bx_pair.bytes < 3 * (size_t)c->n * sizeof(double))
    c->bx_pair.alloc(3 * (size_t)c->n * sizeof(double));
  c->pair_snapped = false;
  if (c->n > 0) {
    if (!c->neigh_set) {  // no lists: bins only serve Domain::pbc on every step
      c->cutneigh = std::min(c->period[0], std::min(c->period[1], c->period[2])) / 3.0;
      c->skin = 0.0;
    }
    c->setup_neighbor_structs();
    c->upload_fix_tables();
    c->fill_bead_args();
    c->dep.zero(c->st);  // the lists about to be built replace those the next check would zero on
    launch_neighbor(c->ba, true, c->st);  // Integrate::setup: pbc, borders, build
    c->bf.zero(c->st);
  }
  // FP32 reference concentration: the mean of phi, from the k = 0 mode of an
  // uncentered r2c
  if (c->gridset && c->precision == PHAFD_FP32) {
    c->phi_ref = 0.0;
    c->r2c<float>(c->phi.as<float>(), nullptr, c->w1.as<cpx<float>>(), c->plain_fh());
    float origin[2];
    CK(cudaMemcpyAsync(origin, c->w1.p, sizeof(origin), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    const double mean = (double)origin[0] / (double)c->nreal;
    c->phi_ref = std::isfinite(mean) && mean > 0.0 && mean < 1.0 ? mean : 0.0;
  }
  // field state
  if (c->gridset && (c->have_conj || c->have_gradphi)) {
    if (c->precision == PHAFD_FP64) {
      if (c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj) {
        c->r2c<double>(c->phi.as<double>(), nullptr, c->phat[c->cur].as<cpx<double>>(), c->plain_fh());
        c->inverse_chain<double>(c->phat[c->cur].as<cpx<double>>(), nullptr, nullptr, 0.0, 1.0 / (double)c->nreal, true, false);
      }
    } else {
      if (c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj) {
        c->r2c<float>(c->phi.as<float>(), nullptr, c->phat[c->cur].as<cpx<float>>(), c->plain_fh());
        c->inverse_chain<float>(c->phat[c->cur].as<cpx<float>>(), nullptr, nullptr, 0.0f, (float)(1.0 / (double)c->nreal), true, false);
      }
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  c->invalidate_graph();
  c->grad_partial = false;
  c->stepped = false;
  c->setup_done = true;
  int rc = check_status(c);
  if (rc) return rc;
  API_END(c)
}

static void enqueue_run(phafd_ctx* c, int nsteps);

int phafd_run(phafd_ctx* c, int nsteps) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  enqueue_run(c, nsteps);
  CK(cudaStreamSynchronize(c->st));
  if (c->keep_chempot && c->have_conj && nsteps > 0) c->chempot_from_mu = true;
  int rc = check_status(c);
  if (rc) return rc;
  API_END(c)
}

static void apply_variants(phafd_ctx* c, int flags) {
  c->use_plane = (flags & PHAFD_TUNE_PLANE) != 0;
  c->geom.generic256 = (flags & PHAFD_TUNE_GENERIC256) ? 1 : 0;
  c->geom.xc2r_tma = (flags & PHAFD_TUNE_XC2R_TMA) ? 1 : 0;
  c->geom.xr2c_tma = (flags & PHAFD_TUNE_XR2C_TMA) ? 1 : 0;
  c->invalidate_graph();
}

int phafd_set_graph_steps(phafd_ctx* c, int steps) {
  API_BEGIN(c)
  if (steps < 2 || (steps & 1)) throw std::invalid_argument("graph steps: an even number >= 2");
  c->graph_steps = steps;
  c->invalidate_graph();
  API_END(c)
}

int phafd_set_variants(phafd_ctx* c, int flags) {
  API_BEGIN(c)
  if (flags & ~(PHAFD_TUNE_PLANE | PHAFD_TUNE_GENERIC256 | PHAFD_TUNE_XC2R_TMA | PHAFD_TUNE_XR2C_TMA))
    throw std::invalid_argument("unknown kernel variant");
  apply_variants(c, flags);
  API_END(c)
}

int phafd_autotune(phafd_ctx* c, int steps, int* best, double* ms) {
  API_BEGIN(c)
  if (steps < 1 || !best || !ms) throw std::invalid_argument("autotune: steps >= 1 and output arrays needed");
  CK(cudaSetDevice(c->device));
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  const bool has256 = c->N[0] == 256 || c->N[1] == 256 || c->N[2] == 256;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  double best_ms = 1e300;
  int best_flags = 0;
  int rc = PHAFD_OK;
  // the tensor-map x passes replace the register-resident x passes only
  const bool tma_ok = c->precision == PHAFD_FP32 && c->N[0] == 256 && c->N[1] % 32 == 0;
  const int tma_bits = PHAFD_TUNE_XC2R_TMA | PHAFD_TUNE_XR2C_TMA;
  for (int f = 0; f < 16 && rc == PHAFD_OK; ++f) {
    ms[f] = -1.0;
    if ((f & PHAFD_TUNE_GENERIC256) && !has256) continue;
    if ((f & PHAFD_TUNE_PLANE) && (c->N[0] != c->N[1] || !c->have_conj)) continue;
    if ((f & tma_bits) && (!tma_ok || (f & (PHAFD_TUNE_PLANE | PHAFD_TUNE_GENERIC256)))) continue;
    apply_variants(c, f);
    enqueue_run(c, 4);  // an eager step, then the graphs' captures
    CK(cudaStreamSynchronize(c->st));
    rc = check_status(c);
    if (rc) break;
    const int timed = steps + (steps & 1);  // whole two-step graphs
    CK(cudaEventRecord(e0, c->st));
    enqueue_run(c, timed);
    CK(cudaEventRecord(e1, c->st));
    CK(cudaEventSynchronize(e1));
    rc = check_status(c);
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, e0, e1));
    ms[f] = (double)t / timed;
    if (ms[f] < best_ms) {
      best_ms = ms[f];
      best_flags = f;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  apply_variants(c, best_flags);
  *best = best_flags;
  if (c->keep_chempot && c->have_conj) c->chempot_from_mu = true;
  if (rc) return rc;
  API_END(c)
}

int phafd_run_until_touching(phafd_ctx* c, long long nsteps, double touch_point, int continue_running,
                             int delay_step, long long* steps_done, int max_events, long long* event_steps,
                             int* event_kinds, int* nevents) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (c->n < 1) throw std::invalid_argument("run_until_touching needs beads");
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  if (!continue_running) delay_step = 0;  // input.cpp:293
  TouchState init{};
  init.since = delay_step;
  init.maxev = 1024;
  c->touch.alloc(sizeof(TouchState));
  CK(cudaMemcpy(c->touch.p, &init, sizeof(init), cudaMemcpyHostToDevice));
  c->touch_on = true;
  c->touch_point = touch_point;
  c->touch_delay = delay_step;
  c->invalidate_graph();
  long long done = 0;
  int rc = 0;
  try {
    if (continue_running) {
      for (long long left = nsteps; left > 0 && rc == 0;) {
        const int chunk = (int)std::min<long long>(left, 1 << 20);
        enqueue_run(c, chunk);
        CK(cudaStreamSynchronize(c->st));
        rc = check_status(c);
        left -= chunk;
        done += chunk;
      }
    } else {
      // one step at a time: the run ends right after the first touching step
      for (; done < nsteps && rc == 0;) {
        enqueue_run(c, 1);
        int flag = 0;
        CK(cudaMemcpyAsync(&flag, (char*)c->touch.p + offsetof(TouchState, breakflag), sizeof(int),
                           cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        rc = check_status(c);
        ++done;
        if (flag) break;
      }
    }
  } catch (...) {
    c->touch_on = false;
    c->invalidate_graph();
    throw;
  }
  TouchState out{};
  CK(cudaMemcpy(&out, c->touch.p, sizeof(out), cudaMemcpyDeviceToHost));
  c->touch_on = false;
  c->invalidate_graph();
  if (steps_done) *steps_done = done;
  if (nevents) *nevents = out.nev;
  for (int k = 0; k < std::min(out.nev, std::min(max_events, out.maxev)); ++k) {
    if (event_steps) event_steps[k] = out.ev_step[k];
    if (event_kinds) event_kinds[k] = out.ev_kind[k];
  }
  if (rc) return rc;
  API_END(c)
}

int phafd_run_async(phafd_ctx* c, int nsteps) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  if (c->have_conj && c->c_noise == PHAFD_NOISE_REFERENCE)
    throw std::runtime_error("the reference noise stream is generated on the host: use phafd_run");
  enqueue_run(c, nsteps);
  if (c->keep_chempot && c->have_conj && nsteps > 0) c->chempot_from_mu = true;
  API_END(c)
}

static void enqueue_run(phafd_ctx* c, int nsteps) {
  {
  c->check_done_early = c->check_next_early = false;  // set only while a multi-step graph is captured
  const bool use_graph = c->c_noise != PHAFD_NOISE_REFERENCE || !c->have_conj;
  const bool resident = c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj;
  for (int s = 0; s < nsteps; ++s) {
    if (c->have_conj && c->c_noise == PHAFD_NOISE_REFERENCE) {
      CK(cudaStreamSynchronize(c->st));
      c->fill_reference_uniforms();
      CK(cudaMemcpyAsync(c->uref.p, c->uref_h, c->ncplx * sizeof(double2), cudaMemcpyHostToDevice, c->st));
    }
    if (!use_graph || !c->eager_done) {
      c->step_once();
      CK(cudaGetLastError());
      if (use_graph) c->eager_done = true;
    } else {
      // Graphs: graph_steps steps, then two (both spectrum parities of the
      // resident schedule), one step per parity for the rest.
      bool launched = false;
      for (const int k : {c->graph_steps, 2}) {
        if (k == c->graph_steps && k == 2) continue;  // the two-step graph comes next
        cudaGraphExec_t& ge = k == 2 ? c->gexec : c->gexecK;
        int& gcur = k == 2 ? c->graph_cur : c->graph_curK;
        if (!(resident && nsteps - s >= k && (!ge || c->cur == gcur))) continue;
        if (!ge) {
          gcur = c->cur;
          cudaGraph_t g;
          CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed));
          for (int j = 0; j < k; ++j) {
            c->check_done_early = j > 0;
            c->check_next_early = j + 1 < k;
            c->step_once();
            resident_spectrum_flip(c);
          }
          c->check_done_early = c->check_next_early = false;
          CK(cudaStreamEndCapture(c->st, &g));
          c->kernels_per_step = count_kernels(g) / k;
          CK(cudaGraphInstantiate(&ge, g, 0));
          cudaGraphDestroy(g);
        }
        CK(cudaGraphLaunch(ge, c->st));
        s += k - 1;
        c->timestep += k;
        c->note_step();
        launched = true;
        break;
      }
      if (launched) continue;  // an even number of steps leaves cur unchanged
      const int par = resident ? c->cur : 0;
      if (!c->gexec1[par]) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeRelaxed));
        c->step_once();
        CK(cudaStreamEndCapture(c->st, &g));
        if (!c->kernels_per_step) c->kernels_per_step = count_kernels(g);
        CK(cudaGraphInstantiate(&c->gexec1[par], g, 0));
        cudaGraphDestroy(g);
      }
      CK(cudaGraphLaunch(c->gexec1[par], c->st));
    }
    c->timestep += 1;
    c->note_step();
    if (resident) resident_spectrum_flip(c);
  }
  }
}

int phafd_run_timed(phafd_ctx* c, int nsteps, double* ms) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaStreamSynchronize(c->st));
  CK(cudaEventRecord(e0, c->st));
  int rc = phafd_run(c, nsteps);
  CK(cudaEventRecord(e1, c->st));
  CK(cudaEventSynchronize(e1));
  float f = 0;
  CK(cudaEventElapsedTime(&f, e0, e1));
  *ms = f;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  API_END(c)
}

int phafd_profile_stages(phafd_ctx* c, int nsteps, double* stage_ms, int nstage) {
  API_BEGIN(c)
  CK(cudaSetDevice(c->device));
  if (!c->setup_done) {
    int rc = phafd_setup(c);
    if (rc) return rc;
  }
  if (c->have_conj && c->c_noise == PHAFD_NOISE_REFERENCE) throw std::runtime_error("profiling needs device noise");
  for (int k = 0; k < nstage; ++k) stage_ms[k] = 0.0;
  const bool resident = c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj;
  for (int s = 0; s < nsteps; ++s) {
    c->profiling = true;
    c->step_once();
    c->profiling = false;
    c->note_step();
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->st));
    for (size_t k = 1; k < c->marks.size(); ++k) {
      float f = 0;
      CK(cudaEventElapsedTime(&f, c->marks[k - 1].second, c->marks[k].second));
      const int id = c->marks[k].first;
      if (id >= 0 && id < nstage) stage_ms[id] += f;
    }
    for (auto& m : c->marks) cudaEventDestroy(m.second);
    c->marks.clear();
    c->timestep += 1;
    if (resident) resident_spectrum_flip(c);
  }
  int rc = check_status(c);
  if (rc) return rc;
  API_END(c)
}

int phafd_synchronize(phafd_ctx* c) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  int rc = check_status(c);
  if (rc) return rc;
  API_END(c)
}

int phafd_counters_get(phafd_ctx* c, phafd_counters* out) {
  API_BEGIN(c)
  long long h[6];
  CK(cudaMemcpyAsync(h, c->d_counters.p, sizeof(h), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  out->num_less_zero = h[0];
  out->num_great_zero = h[1];
  out->timestep = h[2];
  out->nan_step = h[3];
  out->neighbor_calls = h[4];
  out->status = ((int*)&h[5])[1];
  out->kernels_per_step = c->kernels_per_step;
  out->kernels_per_rebuild = c->rebuild_kernels;
  API_END(c)
}

int phafd_half_list_size(phafd_ctx* c, long long* nout) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  long long tot = 0;
  if (c->have_lj && c->n > 0) {
    std::vector<int> nn(c->n), nb((size_t)c->n * c->ba.maxnb);
    CK(cudaMemcpy(nn.data(), c->nnbr.p, c->n * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nb.data(), c->nbr.p, nb.size() * 4, cudaMemcpyDeviceToHost));
    for (int i = 0; i < c->n; ++i)
      for (int k = 0; k < nn[i]; ++k) if ((nb[(size_t)i * c->ba.maxnb + k] >> 5) > i) ++tot;
  }
  *nout = tot;
  API_END(c)
}

int phafd_half_list(phafd_ctx* c, int* out3) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  if (c->have_lj && c->n > 0) {
    std::vector<int> nn(c->n), nb((size_t)c->n * c->ba.maxnb);
    CK(cudaMemcpy(nn.data(), c->nnbr.p, c->n * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(nb.data(), c->nbr.p, nb.size() * 4, cudaMemcpyDeviceToHost));
    size_t m = 0;
    for (int i = 0; i < c->n; ++i)
      for (int k = 0; k < nn[i]; ++k) {
        const int e = nb[(size_t)i * c->ba.maxnb + k], j = e >> 5;
        if (j <= i) continue;  // each unordered pair once
        out3[3 * m] = c->tags[i];
        out3[3 * m + 1] = c->tags[j];
        out3[3 * m + 2] = e & 31;
        ++m;
      }
  }
  API_END(c)
}

int phafd_grid_list_size(phafd_ctx* c, long long* nout) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  long long tot = 0;
  if (c->ga_style != PHAFD_GRIDATOM_NONE && c->n > 0) {
    std::vector<int> nn(c->n);
    CK(cudaMemcpy(nn.data(), c->ngl.p, c->n * 4, cudaMemcpyDeviceToHost));
    for (int v : nn) tot += v;
  }
  *nout = tot;
  API_END(c)
}

int phafd_grid_list(phafd_ctx* c, int* out3) {
  API_BEGIN(c)
  CK(cudaStreamSynchronize(c->st));
  if (c->ga_style != PHAFD_GRIDATOM_NONE && c->n > 0) {
    std::vector<int> nn(c->n);
    std::vector<uint32_t> g((size_t)c->n * c->ba.maxg);
    CK(cudaMemcpy(nn.data(), c->ngl.p, c->n * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(g.data(), c->gl.p, g.size() * 4, cudaMemcpyDeviceToHost));
    size_t m = 0;
    for (int i = 0; i < c->n; ++i)
      for (int k = 0; k < nn[i]; ++k) {
        const uint32_t e = g[(size_t)i * c->ba.maxg + k];
        out3[3 * m] = (int)(e >> 5);
        out3[3 * m + 1] = c->tags[i];
        out3[3 * m + 2] = (int)(e & 31u);
        ++m;
      }
  }
  API_END(c)
}

int phafd_stage_gradient(phafd_ctx* c) {
  API_BEGIN(c)
  if (c->precision == PHAFD_FP64) c->gradient_from_phi<double>();
  else c->gradient_from_phi<float>();
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  API_END(c)
}

int phafd_stage_borders_and_build(phafd_ctx* c) {
  API_BEGIN(c)
  if (c->n == 0) return PHAFD_OK;
  if (c->ba.nbins == 0) {
    c->setup_neighbor_structs();
    c->upload_fix_tables();
  }
  c->fill_bead_args();
  c->dep.zero(c->st);  // the lists about to be built replace those the next check would zero on
  launch_neighbor(c->ba, true, c->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  int rc = check_status(c);
  if (rc) return rc;
  API_END(c)
}

int phafd_compute_complex(phafd_ctx* c, int field, int quant, double* out) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("grid not created");
  if (field != PHAFD_FIELD_FT_PHI && field != PHAFD_FIELD_FT_CHEMPOT && field != PHAFD_FIELD_FT_PHI_STEP_START)
    throw std::invalid_argument("Invalid array to compute in compute modulus.");
  if (quant < PHAFD_COMPLEX_REAL || quant > PHAFD_COMPLEX_NORM) throw std::invalid_argument("Invalid argument in compute complex.");
  std::vector<double> spec(2 * c->ncplx);
  int rc = phafd_grid_get(c, field, spec.data());
  if (rc) return rc;
  // compute_complex.cpp:50: prefac = 1 / (dx dy dz)
  const double prefac = 1.0 / ((c->period[0] / c->N[0]) * (c->period[1] / c->N[1]) * (c->period[2] / c->N[2]));
  for (size_t m = 0; m < c->ncplx; ++m) {
    const double re = spec[2 * m], im = spec[2 * m + 1];
    switch (quant) {
      case PHAFD_COMPLEX_REAL: out[m] = re * prefac; break;
      case PHAFD_COMPLEX_IMAG: out[m] = im * prefac; break;
      case PHAFD_COMPLEX_MODULUS: out[m] = std::sqrt(re * re + im * im) * prefac; break;
      default: out[m] = (re * re + im * im) * prefac * prefac; break;
    }
  }
  API_END(c)
}

int phafd_structure_factor(phafd_ctx* c, int nbins, double* sk, long long* counts) {
  API_BEGIN(c)
  if (!c->gridset || nbins <= 0 || !sk) throw std::invalid_argument("structure factor: grid and bins needed");
  CK(cudaSetDevice(c->device));
  DevBuf acc;
  acc.alloc((size_t)nbins * 16);
  acc.zero(c->st);
  double* dsum = acc.as<double>();
  unsigned long long* dcnt = reinterpret_cast<unsigned long long*>(dsum + nbins);
  const FHArgs none = c->plain_fh();  // phi - c in FP32: the k = 0 mode is not binned
  const double ry = c->period[0] / c->period[1], rz = c->period[0] / c->period[2];
  const size_t shm = (size_t)nbins * 16;
  if (c->precision == PHAFD_FP64) {
    c->r2c<double>(c->phi.as<double>(), nullptr, c->w1.as<cpx<double>>(), none);
    k_shells<double><<<1024, 256, shm, c->st>>>(c->w1.as<cpx<double>>(), c->N[0], c->N[1], c->N[2], ry, rz, nbins,
                                                dsum, dcnt);
  } else {
    c->r2c<float>(c->phi.as<float>(), nullptr, c->w1.as<cpx<float>>(), none);
    k_shells<float><<<1024, 256, shm, c->st>>>(c->w1.as<cpx<float>>(), c->N[0], c->N[1], c->N[2], ry, rz, nbins,
                                               dsum, dcnt);
  }
  CK(cudaGetLastError());
  std::vector<double> hs(nbins);
  std::vector<unsigned long long> hc(nbins);
  CK(cudaMemcpyAsync(hs.data(), dsum, nbins * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(hc.data(), dcnt, nbins * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int b = 0; b < nbins; ++b) {
    sk[b] = hc[b] ? hs[b] / (double)hc[b] / (double)c->nreal : 0.0;
    if (counts) counts[b] = (long long)hc[b];
  }
  API_END(c)
}

int phafd_set_linear_substeps(phafd_ctx* c, int nsub, double f2) {
  API_BEGIN(c)
  if (nsub < 1) throw std::invalid_argument("substeps must be >= 1");
  if (nsub > 1 && c->c_noise == PHAFD_NOISE_REFERENCE)
    throw std::invalid_argument("macro steps draw Philox noise (the reference stream has one draw per substep)");
  if (nsub > 1 && c->schedule != PHAFD_SCHEDULE_RESIDENT)
    throw std::invalid_argument("macro steps need the resident schedule");
  c->nsub = nsub;
  c->f2_lin = f2;
  c->invalidate_graph();
  API_END(c)
}

int phafd_grid_device(phafd_ctx* c, int field, void** dev) {
  API_BEGIN(c)
  if (!c->gridset || !dev) throw std::invalid_argument("grid not created");
  const DevBuf* b = field == PHAFD_FIELD_PHI ? &c->phi : field == PHAFD_FIELD_GRADX ? &c->gx
                  : field == PHAFD_FIELD_GRADY ? &c->gy : field == PHAFD_FIELD_GRADZ ? &c->gz
                  : field == PHAFD_FIELD_CHEMPOT ? &c->dep : nullptr;
  if (!b) throw std::invalid_argument("bad field");
  if (field == PHAFD_FIELD_GRADX || field == PHAFD_FIELD_GRADY || field == PHAFD_FIELD_GRADZ) c->full_gradient();
  *dev = b->p;
  API_END(c)
}

int phafd_grid_copy_device(phafd_ctx* c, int field, void* dst) {
  API_BEGIN(c)
  if (!c->gridset || !dst) throw std::invalid_argument("grid not created");
  if (field == PHAFD_FIELD_GRADX || field == PHAFD_FIELD_GRADY || field == PHAFD_FIELD_GRADZ) c->full_gradient();
  const DevBuf* b = field == PHAFD_FIELD_PHI ? &c->phi : field == PHAFD_FIELD_GRADX ? &c->gx
                  : field == PHAFD_FIELD_GRADY ? &c->gy : field == PHAFD_FIELD_GRADZ ? &c->gz
                  : field == PHAFD_FIELD_CHEMPOT ? &c->dep : nullptr;
  if (!b) throw std::invalid_argument("bad field");
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(dst, b->p, c->nreal * c->rsz(), cudaMemcpyDeviceToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  API_END(c)
}

int phafd_compute_grid_clusters(phafd_ctx* c, double threshold, int greater, int* labels, int* nclusters) {
  API_BEGIN(c)
  if (!c->gridset) throw std::invalid_argument("grid not created");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->st));
  DevBuf lab;
  lab.alloc(c->nreal * sizeof(int));
  const int rc = c->precision == PHAFD_FP64
                     ? grid_clusters<double>(c->phi.as<double>(), c->N[0], c->N[1], c->N[2], threshold, greater,
                                             lab.as<int>(), nclusters, c->st)
                     : grid_clusters<float>(c->phi.as<float>(), c->N[0], c->N[1], c->N[2], threshold, greater,
                                            lab.as<int>(), nclusters, c->st);
  if (rc == -8) {
    c->err = "compute grid/cluster: an iteration limit was reached";
    return PHAFD_ERR_TIMEOUT;
  }
  if (rc == -7) throw std::bad_alloc();
  if (rc != 0) throw CudaError("compute grid/cluster failed");
  if (labels) CK(cudaMemcpy(labels, lab.p, c->nreal * sizeof(int), cudaMemcpyDeviceToHost));
  API_END(c)
}

int phafd_deposit_density(phafd_ctx* c, void* rho) {
  API_BEGIN(c)
  if (!c->gridset || !rho) throw std::invalid_argument("grid not created");
  if (!c->setup_done) throw std::invalid_argument("density needs the neighbor lists of setup");
  CK(cudaSetDevice(c->device));
  CK(cudaMemsetAsync(rho, 0, c->nreal * c->rsz(), c->st));
  if (c->n > 0 && c->ga_style != PHAFD_GRIDATOM_NONE) {
    c->fill_bead_args();
    if (c->precision == PHAFD_FP64) launch_density<double>(c->ba, c->pair_args<double>(), (double*)rho, c->st);
    else launch_density<float>(c->ba, c->pair_args<float>(), (float*)rho, c->st);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  API_END(c)
}

int phafd_grid_add_device(phafd_ctx* c, const void* src, double scale) {
  API_BEGIN(c)
  if (!c->gridset || !src) throw std::invalid_argument("grid not created");
  CK(cudaSetDevice(c->device));
  const bool resident = c->schedule == PHAFD_SCHEDULE_RESIDENT && c->have_conj && c->setup_done;
  const FHArgs none = c->plain_fh();
  if (c->precision == PHAFD_FP64) {
    k_axpy<double><<<1024, 256, 0, c->st>>>(c->phi.as<double>(), (const double*)src, scale, (long long)c->nreal);
    if (resident) {
      c->r2c<double>(c->phi.as<double>(), nullptr, c->phat[c->cur].as<cpx<double>>(), none);
      c->inverse_chain<double>(c->phat[c->cur].as<cpx<double>>(), nullptr, nullptr, 0.0, 1.0 / (double)c->nreal, true, false);
    }
  } else {
    k_axpy<float><<<1024, 256, 0, c->st>>>(c->phi.as<float>(), (const float*)src, (float)scale, (long long)c->nreal);
    if (resident) {
      c->r2c<float>(c->phi.as<float>(), nullptr, c->phat[c->cur].as<cpx<float>>(), none);
      c->inverse_chain<float>(c->phat[c->cur].as<cpx<float>>(), nullptr, nullptr, 0.0f, (float)(1.0 / (double)c->nreal), true, false);
    }
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  if (resident) c->grad_partial = false;
  API_END(c)
}

int phafd_ctx_copy_state(phafd_ctx* dst, phafd_ctx* src) {
  if (!dst || !src) return PHAFD_ERR_INVALID;
  phafd_ctx* c = dst;
  API_BEGIN(c)
  if (dst->device != src->device || dst->precision != src->precision || !dst->setup_done || !src->setup_done ||
      dst->nreal != src->nreal || dst->n != src->n || dst->schedule != src->schedule)
    throw std::invalid_argument("copy_state: contexts differ in device, precision, grid, beads or schedule");
  CK(cudaSetDevice(src->device));
  CK(cudaStreamSynchronize(dst->st));
  CK(cudaStreamSynchronize(src->st));
  auto cp = [&](DevBuf& d, const DevBuf& s) {
    if (d.bytes != s.bytes) throw std::invalid_argument("copy_state: buffer sizes differ");
    if (s.bytes) CK(cudaMemcpyAsync(d.p, s.p, s.bytes, cudaMemcpyDeviceToDevice, src->st));
  };
  for (auto pr : {std::make_pair(&dst->phi, &src->phi), std::make_pair(&dst->gx, &src->gx),
                  std::make_pair(&dst->gy, &src->gy), std::make_pair(&dst->gz, &src->gz),
                  std::make_pair(&dst->dep, &src->dep), std::make_pair(&dst->phat[0], &src->phat[0]),
                  std::make_pair(&dst->phat[1], &src->phat[1]), std::make_pair(&dst->bx, &src->bx),
                  std::make_pair(&dst->bux, &src->bux), std::make_pair(&dst->bf, &src->bf),
                  std::make_pair(&dst->bxhold, &src->bxhold), std::make_pair(&dst->bfchain, &src->bfchain),
                  std::make_pair(&dst->btang, &src->btang), std::make_pair(&dst->bimage, &src->bimage),
                  std::make_pair(&dst->bin_of, &src->bin_of), std::make_pair(&dst->bin_count, &src->bin_count),
                  std::make_pair(&dst->bin_start, &src->bin_start), std::make_pair(&dst->sorted, &src->sorted),
                  std::make_pair(&dst->bin_off, &src->bin_off), std::make_pair(&dst->nbr, &src->nbr),
                  std::make_pair(&dst->nnbr, &src->nnbr), std::make_pair(&dst->gl, &src->gl),
                  std::make_pair(&dst->ngl, &src->ngl), std::make_pair(&dst->d_counters, &src->d_counters),
                  std::make_pair(&dst->dmask, &src->dmask)})
    cp(*pr.first, *pr.second);
  // the gradient node mask travels with the counters (its stale flag) only
  // when both contexts keep one; otherwise dst's mask is stale until its
  // next rebuild
  if (dst->gmask.p) {
    if (src->gmask.p && src->use_gmask && dst->gmask.bytes == src->gmask.bytes) {
      cp(dst->gmask, src->gmask);
    } else {
      const int off = 1;
      CK(cudaMemcpyAsync(dst->d_gmask_off(), &off, sizeof(int), cudaMemcpyHostToDevice, src->st));
    }
  }
  CK(cudaStreamSynchronize(src->st));
  dst->cur = src->cur;
  dst->grad_partial = src->grad_partial;
  dst->timestep = src->timestep;
  API_END(c)
}

int phafd_stage_pairs(phafd_ctx* c) {
  API_BEGIN(c)
  if (c->n == 0) return PHAFD_OK;
  c->fill_bead_args();
  if (c->precision == PHAFD_FP64) {
    c->dep.zero(c->st);
    launch_pair<double>(c->ba, c->pair_args<double>(), c->st);
  } else {
    c->dep.zero(c->st);
    launch_pair<float>(c->ba, c->pair_args<float>(), c->st);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->st));
  API_END(c)
}

}  // extern "C"
