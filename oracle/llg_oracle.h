/*
 * CPU oracle for the stochastic LLG step: a plain-C, FP64 restatement of the
 * JAMS (stonerlab/jams) CPU path.  TEST INFRASTRUCTURE ONLY: the GPU library
 * never links, loads or calls this code; tests, the smoke check and the CPU
 * baseline leg of the benchmark use it as the checker.
 *
 * What it restates (file:line in the reference project):
 *   - neighbour list from an interaction template:
 *       src/jams/core/interactions.cc:350-396 (neighbour_list_from_interactions)
 *       src/jams/core/lattice.cc:987-1007      (apply_boundary_conditions)
 *       src/jams/core/lattice.cc:617-651       (site numbering i,j,k,m)
 *   - exchange as a 3N x 3N CSR matrix and its row sums:
 *       src/jams/hamiltonian/sparse_interaction.cc:25-34 (insert_interaction_tensor)
 *       src/jams/hamiltonian/exchange.cc:162-169        (max_abs(J) > cutoff)
 *       src/jams/containers/sparse_matrix_builder.h:108-248 (sort, merge, CSR)
 *       src/jams/interface/sparse_blas.h:13-27,57-81     (Xcsrmv_general)
 *   - uniaxial field/energy: src/jams/hamiltonian/uniaxial_anisotropy.cc:126-172
 *   - cubic field/energy:    src/jams/hamiltonian/cubic_anisotropy.cc:135-226
 *   - applied field:         src/jams/hamiltonian/applied_field.cc:10-148
 *                            (static, sinc and sinc-cos pulses at the
 *                            solver time; src/jams/helpers/maths.h:437-446)
 *   - zeeman field:          src/jams/hamiltonian/zeeman.cc:12-71,106-121
 *   - stage times:           src/jams/solvers/cpu_llg_heun.cc:45-148 (t0,
 *                            t0 + dt), src/jams/solvers/cuda_rk4_base.cu:50-108
 *                            (t0, t0 + dt/2, t0 + dt/2, t0 + dt), with
 *                            t0 = iteration * dt
 *   - field summation:       src/jams/core/solver.cc:43-57 (copy + daxpy)
 *   - Heun step:             src/jams/solvers/cpu_llg_heun.cc:28-148
 *   - RK4 step (no CPU version exists in the reference; restated from the
 *     GPU path): src/jams/solvers/cuda_rk4_base.cu:50-108,
 *                src/jams/solvers/cuda_llg_rk4_kernel.cuh:26-53,
 *                src/jams/solvers/cuda_rk4_base_kernel.cuh:1-18,
 *                src/jams/cuda/cuda_spin_ops.cu:4-27
 *   - thermal noise amplitude: src/jams/solvers/cpu_llg_heun.cc:36-43,
 *                src/jams/thermostats/cuda_thermostat_classical.cc:33-45
 *   - dipole field and energy, as the sum the FFT term convolves:
 *       src/jams/hamiltonian/dipole_fft.cc:205-265 (tensor within
 *       r_cutoff + distance_tolerance, self term excluded),
 *       src/jams/hamiltonian/dipole_bruteforce.cc:80-119 (field formula),
 *       src/jams/core/lattice.cc:1155-1200 (cutoff <= supercell inradius)
 *   - magnetisation / energies: src/jams/monitors/magnetisation.cc:77-104,
 *                src/jams/hamiltonian/sparse_interaction.cc:86-100
 *
 * The reference draws its Gaussian noise from pcg32 + std::normal_distribution
 * (CPU) or cuRAND XORWOW (GPU); neither stream can be reproduced bit for bit on
 * another device, so the noise here is a counter-based Philox4x32-10
 * (Salmon et al., SC'11) with a Box-Muller transform built only from IEEE
 * operations (see llg_oracle.c).  At T = 0 no noise is drawn.
 *
 * Compile with -ffp-contract=off: every product and sum is rounded on its own,
 * exactly as the reference's x86-64 build (no FMA) evaluates it.
 */
#ifndef LLG_ORACLE_H
#define LLG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_TERM_EXCHANGE = 0,
  ORC_TERM_UNIAXIAL = 1,
  ORC_TERM_CUBIC = 2,
  ORC_TERM_APPLIED_FIELD = 3,
  ORC_TERM_DIPOLE = 4,
  ORC_TERM_ZEEMAN = 5
};

enum { ORC_PULSE_STATIC = 0, ORC_PULSE_SINC = 1, ORC_PULSE_SINC_COS = 2 };

enum { ORC_HEUN = 0, ORC_RK4 = 1 };

typedef struct {
  int32_t kind;
  int32_t order;            /* uniaxial power 2/4/6, cubic order 1/2 */
  /* exchange template: entry e couples basis site bi[e] of cell c to basis
     site bj[e] of cell c + T[3e..3e+2] with the 3x3 tensor J[9e..9e+8] (meV) */
  int32_t n_int;
  const int32_t *bi;
  const int32_t *bj;
  const int32_t *T;
  const double *J;
  /* anisotropy magnitude per basis site (meV) and axes per basis site:
     uniaxial 3 doubles, cubic 9 doubles (u, v, w) */
  const double *K;
  const double *axis;
  /* applied field in tesla */
  double B[3];
  /* dipole: cutoff and tolerance in lattice parameters, lattice parameter in
     metres, lattice vectors (rows, lattice parameters), fractional basis
     positions (3 nb) */
  double r_cutoff;
  double distance_tolerance;
  double lattice_parameter;
  const double *lattice_vectors;
  const double *positions;
  /* applied field: ORC_PULSE_*, centre time (ps), bandwidth and centre
     frequency (THz) */
  int32_t pulse;
  double time_center;
  double freq_bandwidth;
  double freq_center;
  /* zeeman: per basis site dc field and ac field (T, 3 nb; ac may be null),
     ac frequency (THz, nb) */
  const double *dc_field;
  const double *ac_field;
  const double *ac_frequency;
} orc_term;

typedef struct {
  int32_t L[3];
  int32_t periodic[3];
  int32_t nb;
  const double *mus;        /* per basis site, meV/T */
  const double *gyro;       /* per basis site, rad/ps/T */
  const double *alpha;      /* per basis site */
  int32_t n_terms;
  const orc_term *terms;
  double dt;                /* ps */
  double temperature;       /* K */
  int32_t gilbert_prefactor;/* 1: noise amplitude divided by (1 + alpha^2) */
  int32_t integrator;       /* ORC_HEUN or ORC_RK4 */
  uint64_t seed;
  uint32_t replica;
  int32_t serial_noise;     /* 1: draw noise on one thread, as the reference does */
} orc_model;

typedef struct orc_sim orc_sim;

int orc_create(const orc_model *m, orc_sim **out);
void orc_destroy(orc_sim *s);
const char *orc_last_error(void);
int64_t orc_num_spins(const orc_sim *s);

/* advance nsteps steps from iteration `first_step` (the noise counter) */
int orc_run(orc_sim *s, double *spins, int64_t first_step, int32_t nsteps);

/* total effective field (meV, not divided by mu_s) at time t */
int orc_fields(orc_sim *s, const double *spins, double t, double *h);

/* total energy of each term (meV), in term order */
int orc_energies(orc_sim *s, const double *spins, double t, double *e_terms);

/* M = sum mu_s s / sum mu_s (3 values) and |M| */
int orc_magnetisation(const orc_sim *s, const double *spins, double *m4);

/* CSR of exchange term `term` (pointers stay owned by the oracle) */
int orc_exchange_csr(const orc_sim *s, int32_t term, int64_t *nnz,
                     const int64_t **rows, const int32_t **cols,
                     const double **vals);

/* the three unit normals used for spin `spin` at iteration `step` */
void orc_noise_normals(uint64_t seed, uint32_t replica, uint64_t step,
                       uint32_t spin, float out[3]);

/* noise amplitude sigma_i for basis site b (before the sqrt(T) factor) */
double orc_sigma(const orc_sim *s, int32_t b);

/* geometric topological charge of a triangulated monolayer (a1, a2 at 60
   degrees, one basis site): sum over up and down triangles of the signed
   solid angle / 4 pi */
double orc_topological_charge_triangular(const double *spins, int32_t L1,
                                         int32_t L2);

void orc_set_threads(int32_t n);

#ifdef __cplusplus
}
#endif

#endif
