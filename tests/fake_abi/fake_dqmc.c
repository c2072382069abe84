/*
 * fake_dqmc.c — a stand-in for libdqmc_gb300.so, for host tests only.
 *
 * It implements every entry point of include/dqmc_gb300.h without a device and
 * answers with deterministic values that depend on the walker, the bin, tau and
 * the displacement, so that a driver's binning, normalisation, pooling and file
 * output can be compared between the Python driver (dqmc_gb300.run over ctypes)
 * and the native one (apps/dqmc_main.cpp linked against this file).  Entry points
 * the drivers do not use return DQMC_ERR_STATE.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "dqmc_gb300.h"

struct dqmc_batch {
  int n, lt, N, ntau;
  int *ecount, *dcount, *ebins, *dbins;
  signed char* fields;
};

static double sign_of(int w) { return (w % 2) ? -0.5 : 0.75; }
static double eq_val(const dqmc_batch* b, int w, int k) { return 0.1 * (k + 1) + w + 0.01 * b->ebins[w]; }

const char* dqmc_last_error(void) { return "fake library"; }
int dqmc_abi_version(void) { return DQMC_ABI_VERSION; }

int dqmc_batch_create(const dqmc_walker_desc* d, int n, const dqmc_batch_options* o, dqmc_batch** out) {
  (void)o;
  if (!d || n <= 0 || !out) return DQMC_ERR_ARG;
  dqmc_batch* b = (dqmc_batch*)calloc(1, sizeof *b);
  b->n = n;
  b->lt = d[0].Lt;
  b->N = d[0].L * d[0].L * (d[0].lattice == DQMC_CUBIC ? d[0].L : 1);
  b->ecount = (int*)calloc(n, sizeof(int));
  b->dcount = (int*)calloc(n, sizeof(int));
  b->ebins = (int*)calloc(n, sizeof(int));
  b->dbins = (int*)calloc(n, sizeof(int));
  b->fields = (signed char*)calloc((size_t)n * b->lt * b->N, 1);
  *out = b;
  return DQMC_OK;
}
int dqmc_batch_destroy(dqmc_batch* b) {
  if (b) {
    free(b->ecount), free(b->dcount), free(b->ebins), free(b->dbins), free(b->fields), free(b);
  }
  return DQMC_OK;
}
int dqmc_set_stream(dqmc_batch* b, void* s) { (void)b, (void)s; return DQMC_OK; }
int dqmc_synchronize(dqmc_batch* b) { (void)b; return DQMC_OK; }

int dqmc_fields_random(dqmc_batch* b, int w) {
  const size_t m = (size_t)b->lt * b->N;
  for (size_t k = 0; k < m; ++k) b->fields[(size_t)w * m + k] = ((k + (size_t)w) % 3 == 0) ? -1 : 1;
  return DQMC_OK;
}
int dqmc_set_fields(dqmc_batch* b, int w, const int8_t* f) {
  const size_t m = (size_t)b->lt * b->N;
  memcpy(b->fields + (size_t)w * m, f, m);
  return DQMC_OK;
}
int dqmc_get_fields(dqmc_batch* b, int w, int8_t* f) {
  const size_t m = (size_t)b->lt * b->N;
  for (size_t k = 0; k < m; ++k) f[k] = (int8_t)(-b->fields[(size_t)w * m + k]);  /* the "final" fields */
  return DQMC_OK;
}
int dqmc_init_greens(dqmc_batch* b) { (void)b; return DQMC_OK; }

static void measure_all(dqmc_batch* b, int measure) {
  if (measure)
    for (int w = 0; w < b->n; ++w) b->ecount[w] += 1;
}
int dqmc_sweep_0_to_beta(dqmc_batch* b, int measure) { measure_all(b, measure); return DQMC_OK; }
int dqmc_sweep_beta_to_0(dqmc_batch* b, int measure) { measure_all(b, measure); return DQMC_OK; }

int dqmc_get_config_sign(dqmc_batch* b, int w, double* v) { (void)b; *v = sign_of(w); return DQMC_OK; }
int dqmc_get_wrap_error(dqmc_batch* b, int w, double* v) { (void)b; *v = 1e-9 * (w + 1); return DQMC_OK; }

int dqmc_clear_observables(dqmc_batch* b) {
  for (int w = 0; w < b->n; ++w) b->ecount[w] = 0, b->ebins[w] += 1;
  return DQMC_OK;
}
int dqmc_get_observables(dqmc_batch* b, int w, double* sums, int64_t* counts) {
  for (int k = 0; k < DQMC_NUM_OBS; ++k) {
    counts[k] = (int64_t)b->ecount[w] * b->lt;
    sums[k] = (double)counts[k] * (k == DQMC_OBS_SIGN ? 1.0 : eq_val(b, w, k)) * sign_of(w);
  }
  return DQMC_OK;
}
int dqmc_get_observables_all(dqmc_batch* b, double* sums, int64_t* counts) {
  for (int w = 0; w < b->n; ++w) dqmc_get_observables(b, w, sums + (size_t)w * DQMC_NUM_OBS, counts + (size_t)w * DQMC_NUM_OBS);
  return DQMC_OK;
}
int dqmc_measure_bins(dqmc_batch* b, int nbins, int bin_size, int sweeps_between, double* out) {
  (void)sweeps_between;
  for (int bin = 0; bin < nbins; ++bin) {
    dqmc_clear_observables(b);
    for (int s = 0; s < bin_size / 2; ++s) measure_all(b, 1), measure_all(b, 1);
    for (int w = 0; w < b->n; ++w) {
      double* o = out + ((size_t)w * nbins + bin) * DQMC_NUM_OBS;
      for (int k = 0; k < DQMC_OBS_SIGN; ++k) o[k] = eq_val(b, w, k);
      o[DQMC_OBS_SIGN] = fabs(sign_of(w));
    }
  }
  return DQMC_OK;
}

int dqmc_sweep_dynamic(dqmc_batch* b, const int* taus, int ntau) {
  (void)taus;
  b->ntau = ntau;
  for (int w = 0; w < b->n; ++w) b->dcount[w] += 1;
  return DQMC_OK;
}
int dqmc_clear_dynamic(dqmc_batch* b) {
  for (int w = 0; w < b->n; ++w) b->dcount[w] = 0, b->dbins[w] += 1;
  return DQMC_OK;
}
int dqmc_get_dynamic(dqmc_batch* b, int w, double* sums, int64_t* counts) {
  for (int t = 0; t < b->ntau; ++t) {
    counts[t] = b->dcount[w];
    sums[t] = b->dcount[w] * sign_of(w) * (t / 100.0 + w);
  }
  return DQMC_OK;
}
int dqmc_get_dynamic_r(dqmc_batch* b, int w, double* out) {
  for (int t = 0; t < b->ntau; ++t)
    for (int r = 0; r < b->N; ++r)
      out[(size_t)t * b->N + r] =
          b->dcount[w] * sign_of(w) * ((r + 1.0) / b->N + 0.01 * t + 0.1 * w + 0.001 * b->dbins[w]);
  return DQMC_OK;
}
int dqmc_get_dynamic_obs(dqmc_batch* b, int w, double* dos, double* chi, double* rho) {
  for (int t = 0; t < b->ntau; ++t) {
    const double f = b->dcount[w] * sign_of(w);
    if (dos) dos[t] = f * (1.0 + t + w + 0.01 * b->dbins[w]);
    if (chi) chi[t] = f * (2.0 * t + 0.5 * w);
    if (rho) rho[t] = f * 0.01 * (t + 1);
  }
  return DQMC_OK;
}

/* not used by the drivers */
int dqmc_get_green(dqmc_batch* b, int w, int s, double* o) { (void)b, (void)w, (void)s, (void)o; return DQMC_ERR_STATE; }
int dqmc_set_green(dqmc_batch* b, int w, int s, const double* g) { (void)b, (void)w, (void)s, (void)g; return DQMC_ERR_STATE; }
int dqmc_get_green_dynamic(dqmc_batch* b, int w, int x, int s, double* o) {
  (void)b, (void)w, (void)x, (void)s, (void)o;
  return DQMC_ERR_STATE;
}
int dqmc_get_accept_count(dqmc_batch* b, int w, int64_t* v) { (void)b, (void)w; *v = 0; return DQMC_OK; }
int dqmc_get_status(dqmc_batch* b, int w, int* v) { (void)b, (void)w; *v = 0; return DQMC_OK; }
int dqmc_trace_count(dqmc_batch* b, int* n) { (void)b; *n = 0; return DQMC_OK; }
int dqmc_trace_get(dqmc_batch* b, int w, int k, int s, double* o) { (void)b, (void)w, (void)k, (void)s, (void)o; return DQMC_ERR_STATE; }
int dqmc_trace_clear(dqmc_batch* b) { (void)b; return DQMC_OK; }
int dqmc_batch_info(dqmc_batch* b, int* nw, int64_t* upd) {
  if (nw) *nw = b->n;
  if (upd) *upd = (int64_t)b->n * b->N * b->lt;
  return DQMC_OK;
}
int dqmc_profile_enable(dqmc_batch* b, int on) { (void)b, (void)on; return DQMC_ERR_STATE; }
int dqmc_set_wait_limit(dqmc_batch* b, int limit) { (void)b, (void)limit; return DQMC_ERR_STATE; }
int dqmc_tuning_products(dqmc_batch* b, int* shape, int* n, int* cs, float* cm) {
  (void)b, (void)cs, (void)cm;
  if (shape) *shape = 0;
  if (n) *n = 0;
  return DQMC_OK;
}
int dqmc_profile_read(dqmc_batch* b, int k, double* ms, int64_t* n) { (void)b, (void)k, (void)ms, (void)n; return DQMC_ERR_STATE; }
int dqmc_microbench_fp64(double* t) { (void)t; return DQMC_ERR_STATE; }
int dqmc_product_check(int n, const double* a, const double* b, double* c) { (void)n, (void)a, (void)b, (void)c; return DQMC_ERR_STATE; }
int dqmc_product_device_noalloc(int n, const double* a, const double* b, double* c, void* s) {
  (void)n, (void)a, (void)b, (void)c, (void)s;
  return DQMC_ERR_STATE;
}
int dqmc_launch_count(dqmc_batch* b, int64_t* n) { (void)b; *n = 0; return DQMC_OK; }
int dqmc_tuning(dqmc_batch* b, int* kd, int* flush, int* nc, int* ckd, int* cfl, float* cms) {
  (void)b, (void)kd, (void)flush, (void)nc, (void)ckd, (void)cfl, (void)cms;
  return DQMC_ERR_STATE;
}
