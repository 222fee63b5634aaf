// Bead-side device arguments and launchers.
#pragma once
#include "internal.h"

namespace phafd {

struct SemiDev {
  double bondlength, zeta_para, zeta_perp, bending, temp, kbond;
  uint32_t seed;
  int noise;
  // per-fix constants of the displacement, precomputed on the host:
  // 1/zeta_perp, 1/zeta_para - 1/zeta_perp, their square-root forms, and
  // sqrt(2 T h) is formed with h = dt/2 on the device
  double inv_perp, dinv, sinv_perp, dsinv;
};

struct BeadArgs {
  int n;
  double *x, *ux, *f, *xhold, *fchain, *tang;
  int *image, *type;
  double boxlo[3], boxhi[3], period[3];
  double invdx[3];      // 1 / grid spacing (FP32 pair path: one FP64 multiply instead of a divide)
  int lgN[3];           // log2 N[d] when every N[d] is a power of two, else -1 (node index decode)
  double triggersq, cutneigh, cutneighsq;
  int* flag;            // rebuild requested (device)
  uint32_t* gmask;      // bit per 32-byte sector of a grid field (gmask_g nodes) holding a node within gmask_r
                        // of a bead's position at the last rebuild (null: none)
  long long gmask_words;
  int gmask_g;
  double gmask_r;       // radius of the mask: coupling cutoff + skin (+ a round-off margin)
  double gmask_guardsq; // squared displacement since the last rebuild up to which the mask covers every read
  int* gmask_off;       // set: the mask does not cover the current positions (cleared by a rebuild)
  uint32_t* dmask;      // bit per 32-byte sector (gmask_g nodes) holding a node of the grid lists, rebuilt with
                        // them: the deposit's support (null: none)
  void* dep;            // the mu deposit (dep_bytes per node): the check zeroes the nodes of the current grid
  int dep_bytes;        // lists, which hold the last pair stage's deposits (null: nothing to zero)
  int* check_done;      // blocks of k_check finished (last one sets the graph condition)
  int* status;          // sticky ST_* bits
  long long* ncalls;    // Neighbor::ncalls
  const long long* d_step;
  // bins
  int nb[3];
  double bininv[3];
  long long nbins;
  int *bin_of, *bin_count, *bin_cursor, *bin_start, *sorted, *scan_tmp;
  float4* bin_off;   // position minus the corner of its bin (FP32 lists)
  int fp32_lists;    // 1: list membership in FP32 with a superset margin
  // lists
  int* nbr;
  int* nnbr;
  int maxnb;
  uint32_t* gl;
  int* ngl;
  int maxg;
  int N[3];
  double dx[3];
  int zperiodic;
  // fixes
  double* dragc;
  int any_drag;
  int *sf_fix, *sf_start, *sf_len;
  const SemiDev* sf;
  int any_semi;
  const int* chain_start;  // first bead of every chain of the semiflexible fixes
  int nchains;
};

template <typename T>
struct PairArgs {
  int lj;
  double lj_cutsq, lj1, lj2;
  int ga_style;
  const double *ga_cutsq, *ga_eps, *ga_phi;  // per type, device
  const T *phi, *gx, *gy, *gz;
  T* dep;
  double dv;
  // the step counter, incremented by the kernel when the step's neighbor
  // check (which otherwise increments it) ran early, on the previous step's
  // bead branch (null: no increment)
  long long* step_inc;
};

void launch_step_begin(long long* d_step, cudaStream_t st);
// step_inc (optional): counter the check kernel increments (the step counter,
// saving a launch of its own)
void launch_neighbor(const BeadArgs& a, bool force, cudaStream_t st, long long* step_inc = nullptr);
// the two halves of launch_neighbor: the displacement check (optionally
// setting a graph conditional to the rebuild flag) and the rebuild kernels
void launch_neighbor_check(const BeadArgs& a, cudaGraphConditionalHandle h, int use_cond, cudaStream_t st,
                           long long* step_inc = nullptr);
void launch_rebuild(const BeadArgs& a, cudaStream_t st);

// Integrate::run_until_touching state (integrate.cpp:221-415), on the device
struct TouchState {
  int since, breakflag, nev, maxev;
  long long ev_step[1024];
  int ev_kind[1024];  // 0: cyclisation at step, 1: cyclisation interval ended at step
};
// after a step: distance between the first and the last bead against touch_point
void launch_touch(const double* x, int n, double touch_point, int delay_step, const long long* d_step,
                  TouchState* s, cudaStream_t st);
// sets *gmask_off when a bead moved more than sqrt(gmask_guardsq) since the last rebuild
void launch_gmask_guard(const BeadArgs& a, cudaStream_t st);
template <typename T> void launch_pair(const BeadArgs& a, const PairArgs<T>& p, cudaStream_t st);
template <typename T> void launch_density(const BeadArgs& a, const PairArgs<T>& p, T* rho, cudaStream_t st);
void launch_drag(const BeadArgs& a, double dt, cudaStream_t st);
template <typename T>
void launch_chain_half(const BeadArgs& a, int half, double dt, cudaStream_t st, int nsub = 1, int sub = 0);
// both halves (force, move, force, move) in one launch, one CTA per chain
template <typename T>
void launch_chain_step(const BeadArgs& a, double dt, cudaStream_t st, int nsub = 1, int sub = 0);

}  // namespace phafd
