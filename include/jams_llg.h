/*
 * jams_llg.h - C ABI of the GB300 (sm_103a) stochastic Landau-Lifshitz-Gilbert
 * step library (libjams_llg.so).
 *
 * The library replaces the GPU LLG hot path of JAMS (stonerlab/jams):
 *   CUDAHeunLLGSolver::run        src/jams/solvers/cuda_llg_heun.cu:64-122
 *   CudaRK4BaseSolver::run        src/jams/solvers/cuda_rk4_base.cu:50-108
 *   CudaSolver::compute_fields    src/jams/cuda/cuda_solver.cc:11-26
 *   SparseInteractionHamiltonian::calculate_fields
 *                                 src/jams/hamiltonian/sparse_interaction.cc:36-45
 *   CudaUniaxialAnisotropyHamiltonian / CubicAnisotropyHamiltonian /
 *   CudaAppliedFieldHamiltonian::calculate_fields
 *                                 src/jams/hamiltonian/cuda_uniaxial_anisotropy.cu:28-32,
 *                                 src/jams/hamiltonian/cubic_anisotropy.cc:197-226,
 *                                 src/jams/hamiltonian/cuda_applied_field.cu:10-23
 *   CudaThermostatClassical::update
 *                                 src/jams/thermostats/cuda_thermostat_classical.cc:47-56
 * with one fused pass per integrator stage (field of every term + thermal
 * noise + LLG update) and a batched form over independent replicas.
 *
 * Conventions (those of the reference):
 *   spins   N x 3 row-major doubles, site index ((i*L2 + j)*L3 + k)*nb + m
 *           (src/jams/core/lattice.cc:617-651)
 *   energy  meV; fields of the terms in meV (-dE/dS, not divided by mu_s)
 *   mu_s    meV/T, gamma rad/ps/T, dt ps, temperature K, B tesla
 *
 * Every function returns 0 on success or a negative LLG_ERR_* code; the
 * message is available from llg_last_error(handle) (or with a NULL handle for
 * failures before a handle exists).  Nothing here throws across the ABI.
 */
#ifndef JAMS_LLG_H
#define JAMS_LLG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LLG_ABI_VERSION 3

/* status codes */
enum {
  LLG_OK = 0,
  LLG_ERR_BAD_DESC = -1,     /* invalid descriptor or argument */
  LLG_ERR_OOM = -2,          /* device or host allocation failed */
  LLG_ERR_CUDA = -3,         /* CUDA launch or runtime error */
  LLG_ERR_TIMEOUT = -4,      /* a device-side wait ran out of iterations */
  LLG_ERR_NONFINITE = -5,    /* a spin became NaN or infinite */
  LLG_ERR_NO_DEVICE = -6,    /* no usable sm_103 device */
  LLG_ERR_UNSUPPORTED = -7,  /* combination not implemented */
  LLG_ERR_IO = -8,           /* a file could not be read, written or parsed */
  LLG_ERR_BOUNDS = -9        /* bounds-checked build: a kernel met an index outside its array (the access was
                                skipped) */
};

/* arithmetic form */
enum {
  LLG_FP64 = 0,   /* plain FP64, same association order as the reference CPU
                     path: results equal the CPU solver's bit for bit */
  LLG_FP32C = 1   /* FP32 spins/fields, compensated neighbour sums, FP64
                     noise prefactors and reductions */
};

enum { LLG_HEUN = 0, LLG_RK4 = 1 };

/* Hamiltonian term kinds, summed in list order like Solver::compute_fields
   (src/jams/core/solver.cc:43-57) */
enum {
  LLG_TERM_EXCHANGE = 0,      /* module "exchange": bilinear 3x3 tensors */
  LLG_TERM_UNIAXIAL = 1,      /* module "uniaxial": -K (S.a)^p, p = 2, 4, 6 */
  LLG_TERM_CUBIC = 2,         /* module "cubic": K1 or K2 cubic anisotropy */
  LLG_TERM_APPLIED_FIELD = 3, /* module "applied-field": mu_s B f(t), with
                                 f = 1 or a sinc / sinc-cos pulse */
  LLG_TERM_DIPOLE = 4,        /* modules "dipole-fft" (and its brute-force,
                                 tensor, neighbour-list, near-tree twins):
                                 magnetic dipole-dipole field within a cutoff */
  LLG_TERM_ZEEMAN = 5         /* module "zeeman": mu_s (B_dc + B_ac cos(w t))
                                 per basis site */
};

/* time dependence of an applied-field term (src/jams/hamiltonian/
   applied_field.cc:10-103), t in ps at the stage's time (Heun: t0, t0 + dt;
   RK4: t0, t0 + dt/2, t0 + dt/2, t0 + dt; t0 = iteration * dt) */
enum {
  LLG_PULSE_STATIC = 0,   /* B */
  LLG_PULSE_SINC = 1,     /* B sinc(pi f_bw (t - t_c)) */
  LLG_PULSE_SINC_COS = 2  /* B sinc(pi f_bw (t - t_c)) cos(2 pi f_c (t - t_c)) */
};

typedef struct {
  int32_t kind;
  int32_t order;          /* uniaxial power (2, 4, 6); cubic order (1, 2) */
  /* exchange template: entry e couples basis site bi[e] of cell c to basis
     site bj[e] of cell c + T[3e..3e+2] with tensor J[9e..9e+8] (meV,
     row-major) - the post-symmetry interaction list of
     src/jams/core/interactions.cc:292-348 */
  int32_t n_int;
  const int32_t *bi;
  const int32_t *bj;
  const int32_t *T;
  const double *J;
  /* anisotropy: magnitude per basis site (meV) and unit axes per basis site
     (uniaxial: 3 doubles; cubic: 9 doubles u, v, w) */
  const double *K;
  const double *axis;
  double B[3];            /* applied field (T) */
  /* dipole: h_i = mu_i sum_j mu_j mu0 (3 r (r.S_j) - r^2 S_j) / (4 pi a^3 |r|^5)
     over every site pair closer than r_cutoff + distance_tolerance
     (src/jams/hamiltonian/dipole_fft.cc:205-265, dipole_bruteforce.cc:80-119):
     r in lattice parameters from the lattice vectors (rows a1, a2, a3, in
     lattice parameters) and the fractional basis positions, minimum image
     along periodic axes; r_cutoff must not exceed the inradius of the
     periodic supercell.  lattice_parameter a in metres. */
  double r_cutoff;
  double distance_tolerance;
  double lattice_parameter;
  const double *lattice_vectors;  /* 9 */
  const double *positions;        /* 3 nb */
  /* applied field: LLG_PULSE_* and its centre time (ps), bandwidth and
     centre frequency (THz) */
  int32_t pulse;
  double time_center;
  double freq_bandwidth;
  double freq_center;
  /* zeeman (src/jams/hamiltonian/zeeman.cc:12-71,106-121): per basis site
     the dc field (T, 3 nb), the ac field (T, 3 nb; null: none) and its
     frequency (THz, nb; the angular frequency is 2 pi times it) */
  const double *dc_field;
  const double *ac_field;
  const double *ac_frequency;
} llg_term;

typedef struct {
  int32_t L[3];           /* unit cells along a1, a2, a3 */
  double temperature;     /* K */
  double B[3];            /* replaces the applied-field term's B if use_B */
  int32_t use_B;
} llg_replica;

typedef struct {
  int32_t abi_version;    /* LLG_ABI_VERSION */
  int32_t nb;             /* basis sites per cell (one material each) */
  int32_t periodic[3];
  const double *mus;      /* nb: mu_s (meV/T) */
  const double *gyro;     /* nb: gamma (rad/ps/T), gilbert prefactor applied */
  const double *alpha;    /* nb */
  int32_t n_terms;
  const llg_term *terms;
  double dt;              /* ps (t_step / 1e-12) */
  int32_t gilbert_prefactor; /* noise amplitude / (1 + alpha^2) */
  int32_t integrator;     /* LLG_HEUN or LLG_RK4 */
  int32_t precision;      /* LLG_FP64 or LLG_FP32C */
  int32_t rk4_normalise_stages; /* FP32C RK4: renormalise every stage */
  uint64_t seed;          /* Philox key of the thermal noise */
  int32_t n_replicas;
  const llg_replica *replicas;
  int32_t device;         /* CUDA ordinal */
  int32_t steps_per_graph;/* steps captured per CUDA graph (0: 100) */
} llg_desc;

typedef struct llg_handle llg_handle;

/* Creates the solver state on the device (Solver::initialize +
   Hamiltonian::create for the listed terms, src/jams/core/solver.cc:60-77,
   src/jams/core/hamiltonian.cc:80-115).  Spins start at +z. */
int llg_create(const llg_desc *desc, llg_handle **out);

/* Creates a solver from the text of a JAMS config file and an optional patch
   string merged over it (src/jams/core/jams++.cc:48-84,
   src/jams/interface/config.cc:15-167): materials, unitcell, lattice,
   hamiltonians (exchange with inline interactions and symmetry operations,
   uniaxial, cubic, applied-field, zeeman dc field), solver (llg-heun-gpu,
   llg-rk4-gpu; t_step, t_max in seconds; gilbert_prefactor), physics
   (temperature), sim (seed).  Initial spins from the materials' spin
   settings ("random": uniform directions drawn from sim.seed). */
int llg_create_from_config(const char *config_text, const char *patch_text,
                           int32_t precision, int32_t device, llg_handle **out);

/* The model a config file describes, as JSON (lattice, per-basis-site
   parameters, every term with its interaction template), without touching
   a GPU; for checking a config.  LLG_ERR_BAD_DESC when the config is invalid
   or json_len is too small (the message gives the size needed). */
int llg_config_describe(const char *config_text, const char *patch_text,
                        char *json, int64_t json_len);

/* int(t_max / t_step) of the solver section a handle was created from
   (src/jams/solvers/cuda_llg_heun.cu:23-29); -1 for llg_create handles. */
int64_t llg_max_steps(const llg_handle *h);

void llg_destroy(llg_handle *h);

/* message of the last failure on h (thread-local when h is NULL) */
const char *llg_last_error(const llg_handle *h);

int64_t llg_num_spins(const llg_handle *h, int32_t replica);
int32_t llg_num_replicas(const llg_handle *h);

/* Spin state of one replica (replica < 0: all replicas back to back), host
   buffers of N x 3 doubles.  Set normalises nothing (the reference loads
   spins as given, src/jams/core/lattice.cc:741-748). */
int llg_set_state(llg_handle *h, int32_t replica, const double *s_host);
int llg_get_state(llg_handle *h, int32_t replica, double *s_host);

/* Same with device buffers (the globals::s.device_data() of the reference). */
int llg_set_state_device(llg_handle *h, int32_t replica, const double *s_dev);
int llg_get_state_device(llg_handle *h, int32_t replica, double *s_dev);

/* Advances every replica nsteps steps (Solver::run called nsteps times;
   src/jams/core/jams++.cc:333-347).  Asynchronous on the handle's stream;
   full blocks of steps_per_graph steps run as one CUDA graph launch. */
int llg_step(llg_handle *h, int32_t nsteps);

/* Waits for the handle's stream and reports device-side status
   (LLG_ERR_NONFINITE when a spin became NaN or infinite). */
int llg_synchronize(llg_handle *h);

int64_t llg_iteration(const llg_handle *h);
int llg_set_iteration(llg_handle *h, int64_t iteration);

/* Per-replica physics (Physics::temperature, applied-field B). */
int llg_set_temperature(llg_handle *h, int32_t replica, double temperature);
int llg_set_field(llg_handle *h, int32_t replica, const double B[3]);

/* Total field (meV) at the current spins, N x 3, summed over the terms in
   order (CudaSolver::compute_fields, src/jams/cuda/cuda_solver.cc:11-26). */
int llg_fields(llg_handle *h, int32_t replica, double *h_host);

/* The field of one term (index into the descriptor's term list, or the
   config's Hamiltonian order) at the current spins and solver time, meV,
   N x 3 in site order: what Hamiltonian::calculate_fields(t) leaves in that
   term's field_ (src/jams/core/hamiltonian.h:15-78; e.g.
   SparseInteractionHamiltonian::calculate_fields,
   src/jams/hamiltonian/sparse_interaction.cc:36-45).  The FP64 form gives
   the reference's values bit for bit; the FP32C form computes the term
   from its FP32 state.  The _device variant writes to device memory (a
   Hamiltonian's dev_ptr_field()) on the handle's stream and returns when
   the copy is done. */
int llg_term_fields(llg_handle *h, int32_t replica, int32_t term, double *h_host);
int llg_term_fields_device(llg_handle *h, int32_t replica, int32_t term, double *h_dev);

/* FP64 on-device reductions of one replica: m4 = (Mx, My, Mz, |M|) with
   M = sum mu_s S / sum mu_s (src/jams/monitors/magnetisation.cc:77-104);
   e_terms[n_terms] = total energy of each term in meV
   (Hamiltonian::calculate_total_energy). */
int llg_observables(llg_handle *h, int32_t replica, double *m4, double *e_terms);

/* Magnetisation by groups of basis sites, as MagnetisationMonitor
   (src/jams/monitors/magnetisation.cc:20-104): group_of_basis[b] in
   [0, ngroups) is the group of basis site b (grouping "materials": its
   material; "positions": b; "none": 0).  m4[4g..4g+2] = sum mu_s S over the
   spins of group g and m4[4g+3] = |sum mu_s S|, divided by the group's
   sum mu_s (normalize != 0) or by the Bohr magneton in meV/T (normalize = 0,
   moments in Bohr magnetons).  Synchronous. */
int llg_magnetisation_groups(llg_handle *h, int32_t replica, const int32_t *group_of_basis, int32_t ngroups,
                             int32_t normalize, double *m4);

/* Geometric topological charge of a one-basis-site triangular monolayer
   replica (src/jams/monitors/topological_charge_geometrical_def.cc:159-181). */
int llg_topological_charge(llg_handle *h, int32_t replica, double *q);

/* Uses a caller-owned cudaStream_t (NULL: the handle's own stream). */
int llg_set_stream(llg_handle *h, void *cuda_stream);

/* Number of kernel launches issued by the last llg_step or
   llg_profile_stages call. */
int64_t llg_last_launch_count(const llg_handle *h);

/* Advances nsteps steps like llg_step, without graphs, with CUDA events
   around every stage; ms holds 2 x stages values: ms[k] = mean duration (ms)
   of the kernel of stage k (Heun: predictor, corrector; RK4: stages 1-4),
   ms[stages + k] = the dipole-field evaluation (FFT convolution) before it,
   0 without a dipole term.  Synchronous. */
int llg_profile_stages(llg_handle *h, int32_t nsteps, double *ms);

/* Kernel selection of the handle: info[0] stencil family of the tiled FP32
   kernels (0: generic gather kernels; 1 simple cubic, 2 bcc nearest
   neighbours, 3 bcc three shells, 4 triangular monolayer, 5 fcc nearest
   neighbours, 6 fcc two shells), info[1] planes
   streamed per CTA, info[2] 1 when the Heun predictor stores the corrector's
   partial sum s0 + dt/2 rhs(s0) (else the corrector recomputes rhs(s0)), info[3..4] CTA tile
   (cells along the contiguous axis, rows), info[5] 1 for FP64, info[6] the
   occupancy variant (CTAs per SM the tiled kernels were compiled for),
   info[7] rows computed per thread (1 or 2; 0 without tiled kernels),
   info[8] 1 when each Heun step is one fused kernel (predictor and
   corrector in one sweep), info[9] 1 with TMA plane loads, info[10] 1 in
   stored-noise mode.  info holds 11 values. */
int llg_kernel_info(const llg_handle *h, int32_t *info);

/* Tiling choice of the tiled FP32 kernels (no effect on other kernels):
   planes streamed per CTA (rounded up to even: the thermal noise of planes
   x and x + 1, x even, comes from one draw); flags bit 0: the Heun
   predictor stores the corrector's partial sum s0 + dt/2 rhs(s0); bit 1:
   the narrow tile (half the rows, twice the CTAs, for lattices too small
   to fill the GPU); bit 2: two rows per thread (wide tile of sc, bcc and
   fcc lattices, no dipole term; occupancy 2 only); bit 3:
   the fused Heun step, one kernel per step that computes
   the predictor of its tile and a one-reach halo in shared memory and the
   corrector in the same sweep (sc, bcc and fcc lattices, no dipole term;
   bits 0 and 2 clear; bit 1 picks its narrow tile); flags >> 4: occupancy
   variant, 2 (<= 128 registers), 3 (<= 80) or 4 (<= 64); for the fused
   step 2 or 4 x 256 resident threads per SM; bit 8: TMA plane loads; bit
   9: stored noise (with bit 0: the predictor also stores the step's thermal
   field, which the corrector reads instead of drawing it again); bit 10:
   the half-width tile of simple-cubic lattices, 16 cells along z (fewer
   idle lanes where z extents are not multiples of 32; wide rows, no dipole
   term, not with TMA or the fused step).  Every choice gives the same
   results bit for bit. */
int llg_set_tuning(llg_handle *h, int32_t planes_per_cta, int32_t flags);

/* Times every tiling candidate (planes per CTA 2..64; stored or recomputed
   rhs; occupancy; narrow tile; two rows per thread; the fused Heun step;
   TMA plane loads; stored noise above 0 K; the half-width simple-cubic
   tile: the llg_set_tuning choices that
   apply to the handle) for trial_steps steps on a copy of the state and
   keeps the fastest; the state and iteration are restored.  With use_cache the choice is read
   from / appended to the file named by $JAMS_LLG_TUNE_CACHE (default
   ~/.cache/jams_llg_tuning.txt), keyed by device, lattice and terms. */
int llg_autotune(llg_handle *h, int32_t trial_steps, int32_t use_cache);

/* No counterpart in the reference.  Magnetisation m4 = (Mx, My, Mz, |M|),
   M = sum mu_s S / sum mu_s, of n_spins spins already on the device (N x 3
   doubles, basis site of spin i = i % nb, mu_s per basis site in mus[nb]),
   written to m4_dev (4 doubles of device memory) on cuda_stream - without
   allocating anything.  It exists for callers that cannot call cudaMalloc
   when they need the value: host loops that must not synchronise the device
   (cudaMalloc and cudaFree can), and callers whose device memory belongs to
   an external pool or arena.  Its reduction scratch is a fixed 32 KiB
   device array inside the library (held on every GPU that loads it until
   exit); n_spins above 2^30 or not a multiple of nb, nb outside [1, 4] and
   a mu_s that is not positive and finite are rejected with
   LLG_ERR_BAD_DESC.  The first call on a device looks up that array's
   device address (set-up done once per device, with the device current);
   make that first call before any stream capture, and do not call
   cudaDeviceReset after it.  All calls share the array: calls that overlap
   on the GPU race.  Errors are reported through llg_last_error(NULL). */
int llg_magnetisation_noalloc(const double *spins_dev, int64_t n_spins, int32_t nb, const double *mus,
                              double *m4_dev, void *cuda_stream);

/* ---- spin files and checkpoints ------------------------------------ */

/* Writes a rows x cols array (row-major doubles) to `path`: HDF5 when the
   name ends in ".h5" (one contiguous float64 dataset named `dataset` in the
   root group, the file the reference's HDF5 monitor writes with
   HighFive's createDataSet<double>, src/jams/monitors/hdf5.cc:292-307),
   else text, one row per line, 17 significant digits.  Needs no device. */
int llg_write_array_file(const char *path, const char *dataset, const double *data, int64_t rows, int64_t cols);

/* Reads an array the way the reference loads spins and per-spin parameters
   (load_array_from_file, src/jams/helpers/load.h:14-60): HDF5 dataset
   `dataset` of a ".h5" file (float64/float32, contiguous, compact or
   chunked with the shuffle and deflate filters of the HDF5 monitor's
   "compressed" option; other filters and version-4 chunk indexes give
   LLG_ERR_IO), else every number of a text file
   ('#' and '//' comment lines skipped) with rows = count, cols = 1.
   With data == NULL only *rows and *cols are set; LLG_ERR_BAD_DESC when
   rows x cols exceeds capacity.  Needs no device. */
int llg_read_array_file(const char *path, const char *dataset, double *data, int64_t capacity, int64_t *rows,
                        int64_t *cols);

/* /spins of one replica (N x 3, reference site order) to / from a file in
   the formats above: the HDF5 monitor's spin output
   (src/jams/monitors/hdf5.cc:94-150) and init_h5's "spins" input
   (src/jams/initializer/init_h5.cc:10-34).  Reading requires exactly 3N
   values, as the reference does. */
int llg_write_spins(llg_handle *h, int32_t replica, const char *path);
int llg_read_spins(llg_handle *h, int32_t replica, const char *path);

/* Checkpoint: every replica's state (FP64, exact for both precisions), the
   iteration (which is also the noise step counter), each replica's
   temperature and applied field, and a fingerprint of the model (replica
   count and sizes, basis, precision, integrator, dt, seed).  Loading it into
   a solver created from the same description continues the trajectory bit
   for bit, thermal noise included.  The file is written beside `path` and
   renamed into place; a checksum guards the load, which changes nothing
   unless the whole file verifies.  The reference restarts from the HDF5
   monitor's spins through init_h5 and a fresh noise stream; this call has
   no single reference counterpart. */
int llg_save_checkpoint(llg_handle *h, const char *path);
int llg_load_checkpoint(llg_handle *h, const char *path);

#ifdef __cplusplus
}
#endif

#endif /* JAMS_LLG_H */
