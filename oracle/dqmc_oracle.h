/*
 * dqmc_oracle.h — CPU oracle for the DQMC sweep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, on the CPU and in plain
 * C++17, the algorithm of the reference implementation (dqmc-framework) so
 * that the CUDA path can be checked against it.  Only tests/, the smoke entry
 * point and the CPU-baseline leg of bench.py may load it.  The product never
 * links or calls it.
 *
 * Every exported routine names the reference file:line it follows.  Matrices
 * crossing this interface are column-major N x N doubles; fields are int8
 * +/-1 laid out [t][i] (time-major), t = 0..Lt-1.
 */
#ifndef DQMC_ORACLE_H
#define DQMC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_REPULSIVE = 0, ORC_ATTRACTIVE = 1 };
enum { ORC_STACK_SVD = 0, ORC_STACK_QRP = 1 };
enum { ORC_SQUARE = 0, ORC_CUBIC = 1 };

/* Observable slots (equal-time); order fixed for the C interface. */
enum {
  ORC_OBS_FILLING = 0,
  ORC_OBS_DOUBLE_OCC = 1,
  ORC_OBS_KINETIC = 2,
  ORC_OBS_MOMENTUM_DIST = 3,
  ORC_OBS_LOCAL_SPIN = 4,
  ORC_OBS_SDW = 5,
  ORC_OBS_CDW = 6,
  ORC_OBS_SWAVE = 7,
  ORC_OBS_SIGN = 8,
  ORC_NUM_OBS = 9
};

typedef struct orc_params {
  int model;          /* ORC_REPULSIVE / ORC_ATTRACTIVE */
  int L;              /* lattice side, N = L*L (square) or L*L*L (cubic) */
  double hopping_t;
  double onsite_u;    /* |U| (attractive takes |U|, reference asserts U >= 0) */
  double mu;
  double beta;
  int Lt;             /* time slices, dtau = beta / Lt */
  int pace;           /* stabilization pace */
  int checkerboard;   /* 0 dense exp(-dtau K), 1 checkerboard break-up (square lattice only) */
  int stack_kind;     /* ORC_STACK_SVD (reference) / ORC_STACK_QRP (device algorithm) */
  int momentum_index; /* k-star index for SDW/CDW/n(k); -1 -> the last k star, (pi, ..., pi):
                         the M point of the square lattice, the R point of the cubic one */
  int record_greens;  /* 1: keep the Lt-slice G series and measure from it */
  int lattice;        /* ORC_SQUARE (src/lattice/square.cpp) / ORC_CUBIC (src/lattice/cubic.cpp) */
} orc_params;

/* BLAS/LAPACK hooks (Fortran calling convention).  When unset the oracle
 * uses its own FP64 routines (Jacobi SVD, blocked loops).  Set from Python
 * with the function pointers that scipy.linalg.cython_{blas,lapack} export. */
typedef void (*orc_dgemm_t)(const char*, const char*, const int*, const int*, const int*,
                            const double*, const double*, const int*, const double*, const int*,
                            const double*, double*, const int*);
typedef void (*orc_dgesvd_t)(const char*, const char*, const int*, const int*, double*, const int*,
                             double*, double*, const int*, double*, const int*, double*, const int*,
                             int*);
void orc_set_lapack(orc_dgemm_t gemm, orc_dgesvd_t gesvd);

/* NULL when the parameters are rejected (checkerboard on the cubic lattice, L < 1, ...). */
void* orc_create(const orc_params* p);
void orc_destroy(void* h);
int orc_space_size(void* h);

/* RNG: std::minstd_rand0 seeded like Utils::Random::set_seed (src/random.cpp:8-10). */
void orc_seed(void* h, unsigned seed);
/* Draw one canonical uniform exactly as std::bernoulli_distribution consumes it. */
double orc_draw_uniform(void* h);
/* Optional injected uniform stream (one per site attempt); NULL -> engine. */
void orc_set_uniforms(void* h, const double* u, size_t n);

/* Fields. */
void orc_fields_random(void* h);                       /* repulsive_hubbard.cpp:86-99 */
void orc_set_fields(void* h, const int8_t* f);         /* [Lt][N] */
void orc_get_fields(void* h, int8_t* f);

/* Walker set-up: initial_svd_stacks + initial_greens_functions + initial_config_sign
 * (src/dqmc_walker.cpp:109-163). */
void orc_init(void* h);

/* Half-sweeps (src/dqmc_walker.cpp:246-325 and 334-412). */
void orc_sweep_0_to_beta(void* h);
void orc_sweep_beta_to_0(void* h);

/* Dynamic half-sweep 0 -> beta with the fields fixed (src/dqmc_walker.cpp:424-524),
 * accumulating G(k, tau) of the walker's momentum at the listed tau
 * (measure_methods.cpp:278-308).  Needs the stacks of t = 0 (after init or a
 * backward half-sweep); 0 on success, -1 otherwise.  The trace records G(t,0)
 * after each stabilization. */
int orc_sweep_dynamic(void* h, const int* taus, int ntau);
void orc_get_dynamic(void* h, double* sums, int64_t* counts);          /* [ntau] */
void orc_get_green_dynamic(void* h, int which, int spin, double* out); /* 0: G(t,0), 1: G(0,t) */
/* density of states, dynamic spin susceptibility, superfluid-stiffness contribution [ntau] each */
void orc_get_dynamic_obs(void* h, double* dos, double* chi, double* rho);
/* per-displacement sums [ntau][N] (see dqmc_get_dynamic_r) */
void orc_get_dynamic_r(void* h, double* out);

/* Equal-time measurement over the recorded series (measure_handler.cpp:136-150). */
void orc_measure(void* h);
/* Normalise the temporaries into bin b and clear them (measure_handler.cpp:170-240,261-277). */
void orc_write_bin(void* h, int b, double* out_values /* ORC_NUM_OBS */);
void orc_get_accumulators(void* h, double* sums /* ORC_NUM_OBS */, int* counts /* ORC_NUM_OBS */);

/* State access. */
void orc_get_green(void* h, int spin, double* out);    /* spin 0 up, 1 down */
void orc_set_green(void* h, int spin, const double* in);
double orc_wrap_error(void* h);
double orc_config_sign(void* h);
/* Test hook: overwrite the configuration sign (the reference's initial sign,
 * sgn(det G_up det G_dn) of src/dqmc_walker.cpp:162, is not fixed by FP64 once
 * G has eigenvalues below its rounding; a test may adopt the device's value). */
void orc_set_config_sign(void* h, double s);
int64_t orc_accept_count(void* h);
/* G after every stabilization of the last half-sweep(s) since the last clear. */
int orc_trace_count(void* h);
void orc_trace_get(void* h, int k, int spin, double* out);
void orc_trace_clear(void* h);
void orc_trace_enable(void* h, int on);

/* Model-level pieces for unit tests. */
double orc_update_ratio(void* h, int eff_t, int i);
void orc_update_greens(void* h, int eff_t, int i);
void orc_mult_B(void* h, int which, double* mat, int t, int spin);
/* which: 0 B from left, 1 B from right, 2 invB from left, 3 invB from right, 4 transB from left */
void orc_mult_expK(void* h, int which, double* mat);
/* which: 0 expK left, 1 expK right, 2 inv left, 3 inv right, 4 trans left */
void orc_get_expK(void* h, int which, double* out);    /* dense matrices: 0 expK, 1 inv, 2 hopping H */
double orc_alpha(void* h);

/* Linear-algebra pieces for unit tests. */
void orc_svd(int n, const double* a, double* u, double* s, double* v);
void orc_qrp_udt(int n, const double* a, double* u, double* d, double* t);
void orc_greens_from_udv(int n, const double* u, const double* d, const double* f, double* g);

/* Lattice tables (src/lattice/square.cpp, src/lattice/cubic.cpp). */
int orc_num_k_stars(void* h);
int orc_m_point_index(void* h);                     /* the last k star, (pi, ..., pi) */
double orc_fourier_factor(void* h, int disp, int k);
int orc_space_dim(void* h);
int orc_nearest_neighbour(void* h, int i, int dir); /* dir < 2 dim: +x, +y (, +z), -x, -y (, -z) */
int orc_displacement(void* h, int i, int j);        /* index of the displacement from site i to j */
void orc_k_star(void* h, int k, double* out);       /* momentum of k star k, SpaceDim components */

#ifdef __cplusplus
}
#endif
#endif
