/*
 * phafd_gpu.h -- C ABI of libphafd_gpu.so, the GB300 (sm_103a) implementation
 * of PHAFD's per-timestep particle-field hot path.
 *
 * The reference (samueljmcameron/PHAFD, src/) exposes this path as C++ style
 * classes constructed by name from an input script (input.cpp:48-299) and
 * driven through Fix / Pair / NPair hooks by Integrate::run
 * (integrate.cpp:105-203).  Each entry point below replaces one of those
 * hooks or commands; the citation on each line names the reference interface
 * it stands in for.  All state lives on one GPU: the library owns device
 * memory, the caller only passes host pointers and sizes.
 *
 * Conventions
 *   - every call returns 0 on success or a negative PHAFD_ERR_* code;
 *     phafd_last_error() gives the message (the reference throws
 *     std::runtime_error with the same text at the same point);
 *   - real grids are [z][y][x] row-major, x fastest, no padding;
 *   - k-space arrays are exchanged in the reference's transposed FFTW-MPI
 *     layout [ky][kz][kx] with kx in [0, Nx/2], interleaved (re, im) doubles
 *     (grid.cpp:96-97);
 *   - bead arrays are owned beads in creation order, xyz interleaved
 *     (Eigen::Matrix3Xd column layout, atom.hpp:38);
 *   - one context per host thread; calls are ordered on the context's stream.
 */
#ifndef PHAFD_GPU_H
#define PHAFD_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PHAFD_OK 0
#define PHAFD_ERR_INVALID -1      /* bad argument / order of commands        */
#define PHAFD_ERR_CUDA -2         /* CUDA runtime error                      */
#define PHAFD_ERR_NAN -3          /* phi(0,0,0) is NaN (integrate.cpp:190)   */
#define PHAFD_ERR_OVERFLOW -4     /* neighbor capacity exceeded              */
#define PHAFD_ERR_CONSTRAINT -5   /* chain step failed (non-finite / stretch)*/
#define PHAFD_ERR_UNSUPPORTED -6  /* size or option not built                */
#define PHAFD_ERR_NOMEM -7
#define PHAFD_ERR_TIMEOUT -8      /* a bounded device wait gave up           */

/* ---- precision of the grid path ---- */
#define PHAFD_FP64 64
#define PHAFD_FP32 32

/* ---- grid fields (grid.hpp:29-36) ---- */
#define PHAFD_FIELD_PHI 0
#define PHAFD_FIELD_CHEMPOT 1
#define PHAFD_FIELD_GRADX 2
#define PHAFD_FIELD_GRADY 3
#define PHAFD_FIELD_GRADZ 4
#define PHAFD_FIELD_FT_PHI 5
#define PHAFD_FIELD_FT_CHEMPOT 6
/* the spectrum of the last step's starting phi (unnormalised, reference
 * layout): what the reference's compute complex ft_phi sees at a dump step,
 * evaluated inside the step before the update (integrate.cpp:157-165).
 * Resident schedule; zeros before the first step after set-up. */
#define PHAFD_FIELD_FT_PHI_STEP_START 7
/* the gradient of the step's starting phi (read only): what the reference's
 * gradphi arrays hold after a step, since FixGridConjugate::start_of_step
 * computes them before the update (fixgrid_conjugate.cpp:62-114); the grid
 * dump's gradphi_x/y/z attributes (dump.cpp:976-981).  Zeros before the
 * first step, as the reference's arrays start. */
#define PHAFD_FIELD_GRADX_STEP_START 8
#define PHAFD_FIELD_GRADY_STEP_START 9
#define PHAFD_FIELD_GRADZ_STEP_START 10

/* ---- gridatom pair styles (input.cpp:107-116) ---- */
#define PHAFD_GRIDATOM_NONE 0
#define PHAFD_GRIDATOM_GAUSSIAN 1      /* pair gridatom/gaussian     */
#define PHAFD_GRIDATOM_LJISH 2         /* pair gridatom/LJish        */
#define PHAFD_GRIDATOM_LJISH_LINEAR 3  /* pair gridatom/LJish/linear */

/* ---- noise sources ---- */
#define PHAFD_NOISE_OFF 0        /* zero noise, all other terms unchanged            */
#define PHAFD_NOISE_REFERENCE 1  /* the reference's mt19937 + uniform_real stream    */
#define PHAFD_NOISE_PHILOX 2     /* counter-based Philox4x32-10, generated on device */

/* ---- periodic z images of beads ---- */
#define PHAFD_ZGHOST_RANK1 0     /* reference with 1 MPI rank: no z images (comm_brick.cpp:300-318) */
#define PHAFD_ZGHOST_PERIODIC 1  /* reference with >= 2 ranks: fully periodic                     */

/* ---- step schedule of the field ---- */
#define PHAFD_SCHEDULE_REFERENCE 0 /* r2c(phi) at every step start, as fixgrid_conjugate.cpp:62   */
#define PHAFD_SCHEDULE_RESIDENT 1  /* phi-hat carried across steps (same maths, one FFT fewer)   */

typedef struct phafd_semiflexible_params {
  double bondlength; /* rest length of a bond                              */
  double zeta_para;  /* friction along the local chain tangent             */
  double zeta_perp;  /* friction across the local chain tangent            */
  double bending;    /* bending energy: bending * sum (1 - cos theta)      */
  double temp;       /* kT of the bead noise                               */
  double kbond;      /* harmonic bond constant                             */
  int seed;          /* Philox key of the bead noise                       */
  int noise;         /* PHAFD_NOISE_OFF or PHAFD_NOISE_PHILOX              */
} phafd_semiflexible_params;

typedef struct phafd_counters {
  long long num_less_zero;   /* FH reflections phi <= 0 (fixgrid_floryhuggins.cpp:74) */
  long long num_great_zero;  /* FH reflections phi >= 1 (fixgrid_floryhuggins.cpp:77) */
  long long neighbor_calls;  /* Neighbor::ncalls (neighbor.cpp:103)                    */
  long long timestep;        /* Integrate::timestep                                    */
  long long status;          /* sticky PHAFD_ERR_* raised on the device, 0 if none     */
  long long nan_step;        /* first step whose phi(0,0,0) was NaN, -1 if none        */
  long long kernels_per_step; /* kernel launches of one step in the captured graph, 0 before capture */
  long long kernels_per_rebuild; /* launches added by a neighbor rebuild inside the graph          */
} phafd_counters;

typedef struct phafd_ctx phafd_ctx;

/* ---- context (replaces PHAFD::PHAFD / PHAFD::create, phafd.cpp:21-121) ---- */
int phafd_ctx_create(phafd_ctx** out, int device, int precision);
int phafd_ctx_destroy(phafd_ctx* ctx);
const char* phafd_last_error(phafd_ctx* ctx);
const char* phafd_build_info(void);

/* ---- domain / grid (input.cpp:67-80) ---- */
int phafd_domain(phafd_ctx* ctx, const double boxlo[3], const double period[3]); /* Domain::set_box, domain.cpp:30-76 */
int phafd_grid_style(phafd_ctx* ctx, int nx, int ny, int nz);   /* Grid::create + create_concentration, grid.cpp:88-113,205-286 */
int phafd_grid_populate_constant(phafd_ctx* ctx, double average, double variance, int seed); /* Grid::noisy_constant, grid.cpp:289-307 */
/* Grid::flat_interface (grid.cpp:310-337): hi + variance*U(-1/2,1/2) for
 * x - boxlo < Lx (average - lo)/(hi - lo), lo + variance*U beyond */
int phafd_grid_populate_flat_interface(phafd_ctx* ctx, double average, double variance, double hi, double lo,
                                       int seed);
/* Grid::sphere (grid.cpp:339-425): 0.5 (hi - lo) tanh((radius - r)/width) +
 * 0.5 (hi + lo) about the origin, lo chosen for the volume average; `width`
 * is the profile width itself (the script's argument is its square,
 * grid.cpp:153-162) */
int phafd_grid_populate_sphere(phafd_ctx* ctx, double radius, double width, double hi, double average);
int phafd_grid_set(phafd_ctx* ctx, int field, const double* host);   /* upload a real field, [z][y][x]              */
/* download a real field ([z][y][x]) or a k-space field (complex, the
 * reference's [ky][kz][kx] layout, unnormalised r2c convention: ft_phi is the
 * spectrum of the current phi, ft_chempot the r2c of the last step's mu).
 * chempot and ft_chempot after steps exist only if phafd_set_keep_chempot(ctx,
 * 1) preceded them: the step reuses mu's buffers, so such a read is refused */
int phafd_grid_get(phafd_ctx* ctx, int field, double* host);
int phafd_set_zghost(phafd_ctx* ctx, int mode);                      /* CommBrick::borders z swaps, comm_brick.cpp:283-352 */
int phafd_set_schedule(phafd_ctx* ctx, int schedule);
int phafd_set_keep_chempot(phafd_ctx* ctx, int keep);               /* also store mu = deposit + FH (grid->chempot) each step */
int phafd_set_plane_fusion(phafd_ctx* ctx, int on);                 /* x and y passes fused per z-plane in thread-block clusters (Nx == Ny) */
/* on (off by default): single-substep resident steps store grad phi only at grid
 * nodes within (gridatom cutoff + skin) of the beads' positions at the last
 * neighbor rebuild -- the only nodes the pair forces read while no bead has
 * moved more than skin since; a step after which some bead has moved further
 * stores it everywhere.  Reads of the gradient fields (phafd_grid_get,
 * phafd_grid_device) first recompute them everywhere from the current phi. */
int phafd_set_gradient_mask(phafd_ctx* ctx, int on);
/* FP32 contexts only (no effect in FP64; PHAFD_CENTER_FFT by default): the
 * stages that work relative to a reference concentration c, the mean of phi
 * found at set-up.  PHAFD_CENTER_FFT: the transforms of phi carry phi - c
 * (N c goes back into the k = 0 mode, c back into phi after the inverse), so
 * their round-off scales with the fluctuations of phi, not with its mean.
 * PHAFD_CENTER_FH: the Flory-Huggins part of mu is formed as
 * tv (f(phi) - f(c)) with one log1p; the constant tv f(c) moves only the
 * k = 0 mode of mu, which the update does not read (a kept chempot and its
 * spectrum include it); it costs a software log1p per node in the x pass
 * and, measured at 256^3, does not change the S(k) error.  Takes effect at
 * the next step.  No counterpart in the
 * reference, which is FP64 throughout; switching stages off gives the FP32
 * error budget. */
/* ---- autotuner (no counterpart in the reference, which leaves its
 * transforms to FFTW's planner, grid.cpp:236-280) ----
 * Kernel variants of the step, each parity-tested, which give the same
 * trajectory up to round-off:
 *   PHAFD_TUNE_PLANE       the x and y passes fused per z-plane (thread-block
 *                          clusters exchanging through distributed shared
 *                          memory; where Nx == Ny and the plane fits)
 *   PHAFD_TUNE_GENERIC256  the shared-memory tile transforms on 256-point
 *                          axes in place of the register-resident ones
 *   PHAFD_TUNE_XC2R_TMA    FP32, Nx = 256, Ny a multiple of 32: the merged
 *                          x c2r of the inverse chain as a persistent grid fed
 *                          by tensor-map loads, each CTA's next tile landing
 *                          while it transforms the current one (in place of
 *                          the non-persistent grid that loads its own tiles)
 *   PHAFD_TUNE_XR2C_TMA    the same for the x r2c (with the Flory-Huggins
 *                          prologue) of phi's rows
 * phafd_set_variants selects a combination; a new context starts with
 * PHAFD_TUNE_XC2R_TMA | PHAFD_TUNE_XR2C_TMA (no effect where they do not
 * apply).
 * phafd_autotune times every applicable combination over `steps` steps (rounded
 * up to even) of the run itself, after four warm-up steps that capture its
 * graphs, keeps the
 * fastest (*best) and writes the milliseconds per step of each combination
 * to ms[16], indexed by the flags (-1 where a combination does not apply).
 * The tuning steps advance the run like phafd_run. */
#define PHAFD_TUNE_PLANE 1
#define PHAFD_TUNE_GENERIC256 2
#define PHAFD_TUNE_XC2R_TMA 4
#define PHAFD_TUNE_XR2C_TMA 8
int phafd_set_variants(phafd_ctx* ctx, int flags);
/* Steps per CUDA graph of a run (no counterpart in the reference; even, >= 2;
 * default 8): runs launch graphs
 * of this many steps, then two-step and one-step graphs for the rest.  Long
 * graphs keep a single system's neighbor checks off its critical path (every
 * step but a graph's first checks on the previous step's bead branch); many
 * contexts sharing one GPU interleave better with two-step graphs. */
int phafd_set_graph_steps(phafd_ctx* ctx, int steps);
int phafd_autotune(phafd_ctx* ctx, int steps, int* best, double* ms);
#define PHAFD_CENTER_FH 1
#define PHAFD_CENTER_FFT 2
int phafd_set_fp32_centering(phafd_ctx* ctx, int stages);

/* ---- beads (atom_style / atom_populate, atom.cpp:26-110,219-252) ---- */
int phafd_atoms_create(phafd_ctx* ctx, int n, const int* tags, const int* mol, const int* types, const double* x);
int phafd_atoms_get(phafd_ctx* ctx, double* x, double* ux, double* f, int* images);
/* Read-back pipelined with the steps (no counterpart in the reference, whose
 * dumps are written inside its step loop, integrate.cpp:178-186):
 * phafd_atoms_get_async enqueues the
 * copies of x, ux, F and the image flags (NULL skips one) into host memory
 * at the current end of the context's stream, after the steps enqueued so
 * far, and returns; slot (0..3) names the copy.  phafd_wait_slot waits for
 * that copy only (later steps may still run) and reports the device status
 * as of the copy (NaN step, overflow, constraint failure).  With page-locked
 * host buffers (phafd_host_register) the copies run on the copy engine
 * while the next steps compute, so a caller that reads every step's beads
 * can enqueue step k + 1 before it waits for step k's copy. */
int phafd_atoms_get_async(phafd_ctx* ctx, double* x, double* ux, double* f, int* images, int slot);
int phafd_wait_slot(phafd_ctx* ctx, int slot);
/* page-lock (and release) a caller's host buffer for asynchronous copies */
int phafd_host_register(void* ptr, size_t bytes);
int phafd_host_unregister(void* ptr);
/* image flags of every bead, packed as Domain::set_image (x in bits 0-9, y in
 * 10-19, z from 20, each offset by 512): the "ix" attribute that
 * atom_populate read_dump restores (read_dump.cpp:239-240); called after
 * phafd_atoms_create and before phafd_setup, which rebuilds the unwrapped
 * positions from x and these flags.  Setup then skips the initial bond-length
 * check of the chain fixes (|bond - bondlength| <= 1e-3): the harmonic
 * chain's bonds stretch during a run, so a restored state need not pass it */
int phafd_atoms_set_images(phafd_ctx* ctx, const int* images);

/* ---- pairs (input.cpp:99-153) ---- */
int phafd_pair_gridatom(phafd_ctx* ctx, int style, double cut);  /* PairGridAtom*::settings, pair_gridatom_gaussian.cpp:123-142 */
int phafd_pair_gridatom_coeff(phafd_ctx* ctx, int type, int has_eps, double eps, int has_width, double nucwidth,
                              int has_phi, double phi);           /* PairGridAtom*::coeff, pair_gridatom_gaussian.cpp:145-181 */
int phafd_pair_lj_cut(phafd_ctx* ctx, double cut, double eps, double sigma); /* PairLJCut::settings, pair_lj_cut.cpp:103-119 */

/* ---- neighbor (input.cpp:154-164) ---- */
int phafd_neighbor(phafd_ctx* ctx, double skin);                  /* Neighbor::setup, neighbor.cpp:39-68 */

/* ---- fixes (input.cpp:177-229) ---- */
int phafd_fix_conjugate_volfrac(phafd_ctx* ctx, int seed, double mobility, double temp, double volFH, double gamma,
                                int noise);                       /* FixGridConjugate<ConjugateVolFrac>::init, fixgrid_conjugate.cpp:21-45 */
int phafd_fix_floryhuggins(phafd_ctx* ctx, double temp, double volFH, double chi); /* FixGridFloryHuggins::init, fixgrid_floryhuggins.cpp:22-56 */
int phafd_fix_gradphi(phafd_ctx* ctx, int once);                  /* FixGridGradPhi, fixgrid_gradphi.cpp:42-99 */
int phafd_fix_drag(phafd_ctx* ctx, int nranges, const int* starts, const int* ends, double drag); /* FixAtomDrag, fixatom_drag.cpp:24-66 */
int phafd_fix_semiflexible(phafd_ctx* ctx, int nranges, const int* starts, const int* ends,
                           const phafd_semiflexible_params* p);  /* FixAtomSemiFlexible<NoTether>, fixatom_semiflexible.cpp:27-191 */

/* ---- integrate (input.cpp:256-273) ---- */
int phafd_set_dt(phafd_ctx* ctx, double dt);                      /* "dt" command */
int phafd_set_timestep(phafd_ctx* ctx, long long step);           /* "timestep" command */
/* State of the host generator behind PHAFD_NOISE_REFERENCE (the reference's
 * std::mt19937 of conjugate_volfrac.cpp:64, drawn in its order every step),
 * as text (about 7 KB): saved with a restart, it continues that stream
 * exactly, which the reference cannot do.  get: *len = bytes needed
 * (NUL included), buf may be NULL.  set: after
 * phafd_fix_conjugate_volfrac, which seeds the generator.  The Philox noise
 * is keyed by (seed, step) and needs no state. */
int phafd_noise_state_get(phafd_ctx* ctx, char* buf, int cap, int* len);
int phafd_noise_state_set(phafd_ctx* ctx, const char* state);
int phafd_setup(phafd_ctx* ctx);                                  /* Integrate::setup, integrate.cpp:33-88 */
int phafd_run(phafd_ctx* ctx, int nsteps);                        /* Integrate::run, integrate.cpp:90-219 */
int phafd_run_async(phafd_ctx* ctx, int nsteps);
/* Integrate::run_until_touching (integrate.cpp:221-415): after every step the
 * distance between the first and the last bead (stored positions) is compared
 * with touch_point on the device.  Events: kinds[k] = 0 "cyclisation occured at
 * step steps[k]", 1 "cyclisation interval ended at step steps[k]" (already less
 * delay_step).  Without continue_running the run ends after the first touching
 * step (delay_step is then 0, input.cpp:293); steps_done = the steps taken;
 * nevents may exceed max_events (only the first max_events are stored). */
int phafd_run_until_touching(phafd_ctx* ctx, long long nsteps, double touch_point, int continue_running,
                             int delay_step, long long* steps_done, int max_events, long long* event_steps,
                             int* event_kinds, int* nevents);                  /* enqueue the steps and return; phafd_synchronize
                                                                     waits and reports device status (replicas overlap) */
int phafd_counters_get(phafd_ctx* ctx, phafd_counters* out);      /* Integrate::finalise counters, integrate.cpp:418-443 */
int phafd_synchronize(phafd_ctx* ctx);
int phafd_run_timed(phafd_ctx* ctx, int nsteps, double* ms);      /* run, timed by CUDA events on the context's stream */
/* per-stage device time over `nsteps` eager steps (events between stage
 * groups): 0 gradient (reference schedule), 1 neighbor, 2 pairs, 3 bead
 * integration, 4 x r2c + Flory-Huggins, 5 y fft, 6 z fft, 7 z pass with the
 * Model-B update, 8 y ifft, 9 x c2r; stage_ms has nstage entries */
int phafd_profile_stages(phafd_ctx* ctx, int nsteps, double* stage_ms, int nstage);

/* ---- spectra (compute complex, compute_complex.cpp:54-91) ----
 * quant: real, imag, modulus |F| or norm |F|^2 of ft_phi / ft_chempot times
 * 1/(dx dy dz) (squared for norm), one value per mode in the reference's
 * transposed layout [ky][kz][kx], kx in [0, Nx/2] */
#define PHAFD_COMPLEX_REAL 0
#define PHAFD_COMPLEX_IMAG 1
#define PHAFD_COMPLEX_MODULUS 2
#define PHAFD_COMPLEX_NORM 3
int phafd_compute_complex(phafd_ctx* ctx, int field, int quant, double* out);
/* structure factor of the current phi (no reference counterpart: the shell
 * average of compute complex ft_phi norm): S[b] = mean of |phi_hat(q)|^2 / N
 * over the modes with b <= |q| / dq < b + 1, dq = 2 pi / L of the x axis,
 * q != 0, every mode of the full spectrum counted once (the half spectrum
 * with its mirror modes).  counts[b] = modes in shell b (may be NULL). */
int phafd_structure_factor(phafd_ctx* ctx, int nbins, double* sk, long long* counts);
/* compute grid/cluster phi THRESHOLD gt|lt (compute_grid_clusters.cpp:66-229) on the
 * current phi of the one periodic domain: labels (host, nx*ny*nz int, [z][y][x]) =
 * the smallest z + (y*nx + x)*ny over the node's 6-connected periodic component of
 * phi > threshold (greater = 1) or phi < threshold (greater = 0), -1 elsewhere;
 * nclusters (optional) = the number of components.  Either pointer may be null. */
int phafd_compute_grid_clusters(phafd_ctx* ctx, double threshold, int greater, int* labels, int* nclusters);

/* ---- learned macro step support (no reference counterpart) ----
 * nsub > 1 makes each step a macro step (resident schedule): the Model-B
 * update of nsub linearised substeps (dmu/dphi = f2 about the mean, the rest
 * of mu frozen at the step's start) and nsub bead substeps of dt against the
 * field of the step's start; nsub = 1 restores the plain step.  phafd_grid_device returns the device address of a real field (FP32
 * or FP64 as the context); phafd_deposit_density writes to the device array
 * rho (nx*ny*nz, context precision) the sum over beads of the gridatom shape
 * function (pair_gridatom_*.cpp without epsilon and the phi factor);
 * phafd_grid_add_device adds scale * src (device, context precision) to phi
 * and re-derives the spectrum and gradient the next step starts from. */
int phafd_set_linear_substeps(phafd_ctx* ctx, int nsub, double f2);
/* copy the dynamic state (fields, spectra, beads, lists, step counters) of
 * src into dst; both set up with the same grid, beads and schedule on one
 * device (fix parameters such as noise may differ) */
int phafd_ctx_copy_state(phafd_ctx* dst, phafd_ctx* src);
int phafd_grid_device(phafd_ctx* ctx, int field, void** dev);
/* copy a real field into the device array dst (nx*ny*nz, context precision) */
int phafd_grid_copy_device(phafd_ctx* ctx, int field, void* dst);
int phafd_deposit_density(phafd_ctx* ctx, void* rho);
int phafd_grid_add_device(phafd_ctx* ctx, const void* src, double scale);

/* ---- neighbor-list export (NeighList ilist/firstneigh, neigh_list.hpp) ----
 * half list: (tag_i, tag_j, image code of j relative to i)
 * grid list: (node index (z*Ny+y)*Nx+x, tag, image code of the bead)
 * image code = (sx+1) + 3*(sy+1) + 9*(sz+1), s in {-1,0,1} periods added to the bead */
int phafd_half_list_size(phafd_ctx* ctx, long long* n);
int phafd_half_list(phafd_ctx* ctx, int* out3);
int phafd_grid_list_size(phafd_ctx* ctx, long long* n);
int phafd_grid_list(phafd_ctx* ctx, int* out3);

/* ---- compute pair (compute_pair.cpp:43-85) ----
 * The forces of one pair style on every bead as the reference's compute
 * evaluates them after a step: bead copies where the step's pair stage left
 * them, grad phi of the step's starting phi, phi after the step.  style is
 * PHAFD_PAIR_LJ_CUT or PHAFD_PAIR_GRIDATOM (the context's gridatom style);
 * out: 3 doubles per bead in phafd_atoms_create order.  The reference's
 * compute also adds that style's mu deposit to its chempot array once more (a
 * side effect its chempot dumps show); add_to_chempot != 0 does the same to
 * the kept chempot (phafd_set_keep_chempot).  Needs phafd_set_pair_snapshot(ctx,
 * 1) before the steps: each step then keeps the positions of its pair stage. */
#define PHAFD_PAIR_LJ_CUT 1
#define PHAFD_PAIR_GRIDATOM 2
int phafd_set_pair_snapshot(phafd_ctx* ctx, int on);
int phafd_compute_pair(phafd_ctx* ctx, int style, int add_to_chempot, double* out);

/* ---- stage hooks for unit tests and partial pipelines ---- */
int phafd_stage_gradient(phafd_ctx* ctx);          /* FixGridConjugate::start_of_step               */
int phafd_stage_borders_and_build(phafd_ctx* ctx); /* Domain::pbc + CommBrick::borders + Neighbor::build */
int phafd_stage_pairs(phafd_ctx* ctx);             /* Fs = 0, chempot = 0, pair->compute(), reverse_comm */

/* ---- allocation-free gradient (no counterpart in the reference) ----
 * grad phi of a device-resident phi for callers that cannot allocate device
 * memory inside a time step (a host code that owns the device heap, or one
 * that forbids cudaMalloc/cudaFree mid-step because they synchronise the
 * device).  phi, gradx, grady, gradz are caller-owned device arrays
 * [z][y][x] of FP64; period is a host array of the three box lengths;
 * stream is a cudaStream_t (NULL = default stream).  Same result as
 * phafd_stage_gradient on the same phi and box.  The scratch spectra live in
 * a fixed 6.5 MB device array inside the library, so every axis must be 16,
 * 32 or 64 points (larger: PHAFD_ERR_UNSUPPORTED, nothing done).  All calls
 * share that array (and the library's twiddle tables): calls that overlap on
 * the GPU race; calls ordered on one stream need no synchronisation.  The
 * first call on a device looks up the arrays' device addresses and fills the
 * twiddle tables with a synchronous copy; make it before any stream capture
 * on that device.  Later calls only enqueue kernels.  Allocates no device
 * memory. */
int phafd_gradphi_noalloc(const double* phi, double* gradx, double* grady, double* gradz, int nx, int ny, int nz,
                          const double* period, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PHAFD_GPU_H */
