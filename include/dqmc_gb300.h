/*
 * dqmc_gb300.h — C-ABI of the GB300 (sm_103a) DQMC sweep library.
 *
 * The reference (dqmc-framework) has no FFI: its operator interface is the
 * C++ virtual set ModelBase / CheckerBoardBase / DqmcWalker / MeasureHandler.
 * Each entry point below replaces one call of that interface, for a batch of
 * independent walkers (the reference runs one walker per MPI rank).  The
 * reference interface each one stands in for is cited beside it.
 *
 * Conventions
 *   - Every call returns a status (DQMC_OK = 0).  The library never exits.
 *     dqmc_last_error() gives a one-line message for the last failure.
 *   - Matrices crossing the ABI are column-major N x N doubles (Eigen's
 *     layout in the reference); fields are int8 +/-1 laid out [t][i].
 *   - A batch owns all its device memory and is bound to one CUDA stream.
 *     Calls on one batch are not thread-safe; distinct batches are
 *     independent.  Host buffers passed in are copied.
 *   - The CUDA kernels are the only compute path; there is no CPU fallback.
 */
#ifndef DQMC_GB300_H
#define DQMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DQMC_ABI_VERSION 3

enum dqmc_status {
  DQMC_OK = 0,
  DQMC_ERR_ARG = 1,         /* invalid argument or unsupported size */
  DQMC_ERR_CUDA = 2,        /* CUDA runtime error (no device, launch failure) */
  DQMC_ERR_NUMERIC = 3,     /* non-finite Green's function / factorisation breakdown */
  DQMC_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
  DQMC_ERR_STATE = 5        /* call out of order (e.g. sweep before init) */
};

enum dqmc_model { DQMC_REPULSIVE_HUBBARD = 0, DQMC_ATTRACTIVE_HUBBARD = 1 };

/* Lattice::Square (src/lattice/square.cpp) and Lattice::Cubic (src/lattice/cubic.cpp),
 * periodic, side L: N = L^2 or L^3 sites, site index x + L y (+ L^2 z). */
enum dqmc_lattice { DQMC_SQUARE = 0, DQMC_CUBIC = 1 };

enum dqmc_rng {
  DQMC_RNG_MINSTD = 0,  /* parity mode: per-walker std::minstd_rand0 on the host,
                           consumed exactly as std::bernoulli_distribution does */
  DQMC_RNG_PHILOX = 1   /* throughput mode: Philox4x32-10 on the device */
};

enum dqmc_precision {
  DQMC_FP64 = 0,  /* plain method: every product in FP64 */
  DQMC_MIXED = 1  /* tensor-core path: wraps and B-chain products on the BF16 tensor cores
                     (tcgen05), split into exact integer slices and recombined to 49 bits
                     (48 for N > 256); Metropolis by submatrix updates with 42-bit block
                     flushes; for 128 <= N <= 768 the UDT push and Green's assembly by
                     blocked Householder QR whose products carry 56 bits (FP64 class),
                     FP64 panels; Metropolis ratios and all reductions in FP64 */
};

/* Observable slots, the equal-time list of src/measure/observable_handler.cpp:11-20
 * followed by the equal-time sign. */
enum dqmc_observable {
  DQMC_OBS_FILLING = 0,
  DQMC_OBS_DOUBLE_OCCUPANCY = 1,
  DQMC_OBS_KINETIC_ENERGY = 2,
  DQMC_OBS_MOMENTUM_DISTRIBUTION = 3,
  DQMC_OBS_LOCAL_SPIN_CORR = 4,
  DQMC_OBS_SDW_STRUCTURE_FACTOR = 5,
  DQMC_OBS_CDW_STRUCTURE_FACTOR = 6,
  DQMC_OBS_S_WAVE_PAIRING = 7,
  DQMC_OBS_SIGN = 8,
  DQMC_NUM_OBS = 9
};

/* One walker: the parameters the reference spreads over
 * Model::set_model_params (include/model/model_base.h:111-163),
 * Lattice::Square / Lattice::Cubic::set_lattice_params (src/lattice/square.cpp:16-28,
 * src/lattice/cubic.cpp:17-32),
 * DqmcWalker::set_physical_params / set_stabilization_pace
 * (src/dqmc_walker.cpp:25-38) and the checkerboard link
 * (src/model/model_base.cpp:38-55). */
typedef struct dqmc_walker_desc {
  int model;           /* enum dqmc_model */
  int L;               /* lattice side: N = L*L sites (square) or L*L*L (cubic) */
  double hopping_t;
  double onsite_u;     /* |U|; the attractive model takes |U| (attractive_hubbard.cpp:37) */
  double mu;
  double beta;
  int Lt;              /* imaginary-time slices, dtau = beta / Lt */
  int pace;            /* stabilization pace */
  int checkerboard;    /* 0: dense exp(-dtau K); 1: checkerboard break-up (even L, square only) */
  int momentum_index;  /* k-star index for SDW/CDW/n(k); -1 = the last star, (pi, pi) or (pi, pi, pi) */
  uint64_t seed;       /* minstd seed (parity) or Philox key (throughput) */
  int lattice;         /* enum dqmc_lattice (0 = square) */
} dqmc_walker_desc;

typedef struct dqmc_batch_options {
  int rng;             /* enum dqmc_rng */
  int precision;       /* enum dqmc_precision */
  int trace;           /* 1: keep G after every stabilization of the last half-sweep
                          (parity tests; costs device memory) */
  int graphs;          /* 1: capture each kind of half-sweep once into a CUDA graph and replay
                          it (ignored while tracing or profiling) */
  int hbm;             /* 1: every walker on the HBM path, whatever its size (N <= 64 walkers
                          otherwise live in shared memory) */
} dqmc_batch_options;

typedef struct dqmc_batch dqmc_batch;

const char* dqmc_last_error(void);
int dqmc_abi_version(void);

/* Create / destroy a batch of walkers on the current CUDA device.
 * Replaces DqmcInitializer::initial_modules (src/dqmc_initializer.cpp:341-392)
 * for n_walkers independent chains. */
int dqmc_batch_create(const dqmc_walker_desc* descs, int n_walkers,
                      const dqmc_batch_options* opt, dqmc_batch** out);
int dqmc_batch_destroy(dqmc_batch* b);

/* Bind the batch to a caller-owned cudaStream_t (NULL = the batch's own stream). */
int dqmc_set_stream(dqmc_batch* b, void* cuda_stream);
int dqmc_synchronize(dqmc_batch* b);

/* Fields.  dqmc_fields_random replaces Model::set_bosonic_fields_to_random
 * (src/model/repulsive_hubbard.cpp:86-99) with the walker's own engine;
 * set/get replace DqmcIO::read_bosonic_fields_from_file / output_bosonic_fields
 * (include/dqmc_io.h:479-629) for in-memory arrays. */
int dqmc_fields_random(dqmc_batch* b, int walker);
int dqmc_set_fields(dqmc_batch* b, int walker, const int8_t* fields);
int dqmc_get_fields(dqmc_batch* b, int walker, int8_t* fields);

/* DqmcWalker::initial_svd_stacks + initial_greens_functions + initial_config_sign
 * (src/dqmc_walker.cpp:109-163), for every walker. */
int dqmc_init_greens(dqmc_batch* b);

/* DqmcWalker::sweep_from_0_to_beta (src/dqmc_walker.cpp:246-325) and
 * sweep_from_beta_to_0 (:334-412) for every walker.  measure != 0 fuses
 * MeasureHandler::equaltime_measure (src/measure/measure_handler.cpp:136-150)
 * over the half-sweep's Lt slices, exactly as the reference measures the
 * recorded G(t,t) series after the half-sweep. */
int dqmc_sweep_0_to_beta(dqmc_batch* b, int measure);
int dqmc_sweep_beta_to_0(dqmc_batch* b, int measure);

/* Dynamic (time-displaced) half-sweep: DqmcWalker::sweep_for_dynamic_greens
 * (src/dqmc_walker.cpp:424-524) with MeasureHandler::dynamic_measure's
 * measure_greens_functions (src/measure/measure_methods.cpp:278-308).  Replaces
 * a 0 -> beta half-sweep (src/dqmc.cpp:53-57): the fields stay fixed, G(t,0)
 * and G(0,t) are carried besides G(t,t) and recomputed stably at every
 * stabilization (their differences enter the wrap error, which here also
 * includes the equal-time G), and G(k,tau) = sign/N sum_ij FF(r_j - r_i)
 * (G_up(tau,0)(j,i) + G_dn(tau,0)(j,i))/2 is accumulated for the walker's
 * momentum at each listed tau in [0, Lt) (tau = 0 from G(beta,beta)).  Needs
 * the stacks of t = 0 (after dqmc_init_greens or dqmc_sweep_beta_to_0).  Any
 * walker: dense or checkerboard exp(-dtau K), shared-memory walkers (N <= 64)
 * included (they run this half-sweep on the HBM path's kernels).  On the
 * DQMC_MIXED path the G(t,0), G(0,t) steps run on the tensor cores and walkers
 * with 128 <= N <= 768 stabilize with the blocked Householder QR (one
 * factorization of M for both right-hand sides); the others with the FP64
 * kernels.  A new tau list (at most 256 entries) restarts the accumulators. */
int dqmc_sweep_dynamic(dqmc_batch* b, const int* taus, int ntau);
/* Sums of sign * G(k,tau) and their counts, in the order of the last tau list. */
int dqmc_get_dynamic(dqmc_batch* b, int walker, double* sums, int64_t* counts);
int dqmc_clear_dynamic(dqmc_batch* b);
/* Dqmc::measure (src/dqmc.cpp:108-151) with the binning on the device: nbins bins of
 * bin_size / 2 forth-and-back half-sweep pairs with equal-time measurements, each bin
 * normalised and stored by a kernel (MeasureHandler::normalize_stats and
 * write_stats_to_bins, src/measure/measure_handler.cpp:170-277), sweeps_between / 2
 * unmeasured pairs between bins; one copy out at the end.  out: [walker][nbins][9] in
 * the order of dqmc_get_observables, the last entry |<sign>|. */
int dqmc_measure_bins(dqmc_batch* b, int nbins, int bin_size, int sweeps_between, double* out);
/* Sums per listed tau of the other dynamic observables of the reference
 * (src/measure/measure_methods.cpp:315-461): the density of states D(tau)
 * (measure_density_of_states), the local dynamic spin susceptibility
 * (measure_dynamic_spin_susceptibility) and the superfluid-stiffness
 * contribution of that tau (measure_superfluid_stiffness sums it over all tau),
 * each sign-weighted like the reference's tmp_value; counts as dqmc_get_dynamic.
 * Any output may be null. */
int dqmc_get_dynamic_obs(dqmc_batch* b, int walker, double* dos, double* chi, double* rho);
/* Sums per listed tau of sign * 0.5 * sum_i (G_up + G_dn)(i + r, i) / N for every
 * displacement r (site index of the displacement vector), out[tau][r]: G(k,tau) of
 * measure_greens_functions for any momentum k is sum_r FourierFactor(r, k) out[tau][r]. */
int dqmc_get_dynamic_r(dqmc_batch* b, int walker, double* out);
/* G(beta,0) (which = 0) or G(0,beta) (which = 1) after the last dynamic half-sweep
 * (DqmcWalker::Greent0Up/Dn, Green0tUp/Dn at t = Lt), column-major N x N. */
int dqmc_get_green_dynamic(dqmc_batch* b, int walker, int which, int spin, double* out);

/* Accessors: DqmcWalker::GreenttUp/GreenttDn, ConfigSign, WrapError
 * (include/dqmc_walker.h:150-184). spin 0 = up, 1 = down. */
int dqmc_get_green(dqmc_batch* b, int walker, int spin, double* out);
/* Overwrite the equal-time G of one walker and spin (column-major N x N; the
 * attractive model's walkers use spin 0).  The reference's walker owns G and has no
 * setter: this is a restart and test hook (the tests inject a non-finite entry this
 * way and check that only that walker's status word reports it). */
int dqmc_set_green(dqmc_batch* b, int walker, int spin, const double* g);
int dqmc_get_config_sign(dqmc_batch* b, int walker, double* out);
int dqmc_get_wrap_error(dqmc_batch* b, int walker, double* out);
int dqmc_get_accept_count(dqmc_batch* b, int walker, int64_t* out);
/* Per-walker status word, 0 when healthy; bits: 1 non-finite G, 2 zero pivot
 * in a factorization, 4 non-finite Metropolis ratio, 8 a bounded device-side
 * wait gave up (that kernel skipped its output). */
int dqmc_get_status(dqmc_batch* b, int walker, int* out);

/* Equal-time accumulators of a walker: sums[k] = sum over measured slices of
 * sign * O_k (Observable::tmp_value) and counts[k] (Observable::counts),
 * src/measure/measure_methods.cpp:22-255. */
int dqmc_get_observables(dqmc_batch* b, int walker, double* sums, int64_t* counts);
int dqmc_clear_observables(dqmc_batch* b);
/* All walkers at once (one device-to-host copy): sums/counts [n_walkers][DQMC_NUM_OBS];
 * the per-rank bin gather of include/utils/mpi.hpp:68-104 becomes this read. */
int dqmc_get_observables_all(dqmc_batch* b, double* sums, int64_t* counts);

/* Trace (options.trace = 1): G after the k-th stabilization of the most recent
 * half-sweep(s) since the last clear; count is per walker. */
int dqmc_trace_count(dqmc_batch* b, int* count);
int dqmc_trace_get(dqmc_batch* b, int walker, int k, int spin, double* out);
int dqmc_trace_clear(dqmc_batch* b);

/* Statistics of the last half-sweep for throughput accounting. */
int dqmc_batch_info(dqmc_batch* b, int* n_walkers, int64_t* updates_per_half_sweep);

/* The autotuner's choice for walkers whose G lives in HBM (N > 64 or the mixed
 * path): delayed-update block size k and the update kind tc_flush (0 delayed
 * updates with an FP64 flush, 1 with a tensor-core flush, 2 submatrix updates in
 * one kernel per walker, 3 submatrix updates split per 32-site block into a
 * decision kernel and a flush kernel of several CTAs per walker), with every
 * candidate's time for one slice of the whole batch (arrays sized 8).
 * dqmc_init_greens runs the tuner on the batch's own state. */
int dqmc_tuning(dqmc_batch* b, int* kd, int* tc_flush, int* n_candidates, int* cand_kd, int* cand_tc,
                float* cand_ms);
/* The autotuner's tile shape for the tensor-core wrap and chain products of a DQMC_MIXED
 * batch: 0 = 128 x 32 output tiles for N <= 256 (7 slices) and 128 x 64 above (8 slices),
 * 1 = the other way round; with each candidate's time for one slice's products of the whole
 * batch (arrays sized 2; no candidates for FP64 or checkerboard-only batches).  No reference
 * counterpart: the reference's products are MKL calls. */
int dqmc_tuning_products(dqmc_batch* b, int* shape, int* n_candidates, int* cand_shape, float* cand_ms);

/* Kernels launched by this batch since creation (graph replays count every
 * kernel node of the replayed graph). */
int dqmc_launch_count(dqmc_batch* b, int64_t* launches);

/* Kernel-class timing with CUDA events on the batch's stream (the reference
 * has only a whole-run wall-clock timer, src/dqmc.cpp:37-41).  Classes:
 * 0 segment, 1 push, 2 greens, 3 measure.  Enabling resets the totals. */
enum { DQMC_KCLASS_SEGMENT = 0, DQMC_KCLASS_PUSH = 1, DQMC_KCLASS_GREENS = 2, DQMC_KCLASS_MEASURE = 3,
       DQMC_KCLASS_PRODUCT = 4,     /* HBM walkers: dense products of a slice (wraps, B-chain step) */
       DQMC_KCLASS_METROPOLIS = 5,  /* HBM walkers: Metropolis updates of a slice (+ fused measurement) */
       DQMC_KCLASS_DYNAMIC = 6,     /* dynamic half-sweep: the G(t,0), G(0,t) steps and G(k,tau) measurement */
       DQMC_KCLASS_DYN_STAB = 7,    /* dynamic half-sweep: G(t,0), G(0,t) recomputed at a stabilization */
       DQMC_NUM_KCLASS = 8 };
int dqmc_profile_enable(dqmc_batch* b, int on);
/* Test hook of the failure detection (no reference counterpart): the iteration limit of
 * the waits in which the tensor-core wrap and B-chain products wait for their operands to
 * land (default 2^24; 0 gives up at once).  A product whose wait runs out drains the copies
 * it issued, skips its output and sets status bit 8 of its walker; the batch's other work
 * and other batches are unaffected.  limit < 0 restores the default. */
int dqmc_set_wait_limit(dqmc_batch* b, int limit);
int dqmc_profile_read(dqmc_batch* b, int kclass, double* total_ms, int64_t* launches);

/* The mixed-precision product engine on host matrices: C = A B for column-major
 * N x N doubles, computed exactly as the DQMC_MIXED sweep computes its wraps
 * (no reference counterpart: it exposes the engine for validation). */
int dqmc_product_check(int n, const double* a, const double* b, double* c);

/* The same product for callers that cannot allocate device memory: a host
 * framework that owns every device buffer through its own pool, or a time loop
 * that forbids allocation once it runs.  a, b, c are the caller's device buffers
 * (column-major n x n doubles) and the BF16 slice scratch is a fixed 1.75 MB
 * array in the library's device image, so the call allocates nothing.  Limit:
 * n <= 256 (larger n is rejected with DQMC_ERR_ARG).  All calls on a device share
 * that scratch: calls that overlap on the GPU race, so the caller serialises them.
 * The first call on a device resolves the scratch address; make it before any
 * stream capture.  A CUDA error already pending from the caller's own work is
 * reported (DQMC_ERR_CUDA) before anything is launched.
 * No counterpart in the reference (it has no device code). */
int dqmc_product_device_noalloc(int n, const double* a, const double* b, double* c, void* cuda_stream);

/* FP64 FMA throughput of the current device (GFLOP/s), measured by a
 * register-resident FMA loop over all SMs: the FP64 roofline denominator. */
int dqmc_microbench_fp64(double* gflops);

#ifdef __cplusplus
}
#endif
#endif
