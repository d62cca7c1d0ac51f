/*
 * riga_oracle.h — CPU oracle for the riga-flow Phoenix scenario hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the reference's CPU algorithm
 * (crates/riga-engine/src/{qmc,note,lib}.rs, crates/riga-market/src/{lib,correlation}.rs,
 * crates/riga-risk/src/lib.rs), generalised from two to N assets so that it reduces exactly to
 * the reference at N = 2.  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it; the product library never links or calls it.
 *
 * Parity status: pinned against the reference's own known-answer tests (probit quantiles,
 * van der Corput, bridge variance, Cholesky closed form and reconstruction, PSD clamp, flat-smile
 * Dupire, the termsheet1 calibrated local-vol nodes, KO-gates-put) — see tests/test_oracle.py.
 * The reference (Rust) cannot be compiled in this environment, so no output of the reference
 * itself is available for the QMC lane.
 */
#ifndef RIGA_ORACLE_H
#define RIGA_ORACLE_H

#include <stdint.h>
#include "../include/riga_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* --- elementary functions: libm (default, reproduces the golden) or the portable deterministic
 * exp/log the engine's FP64 parity kernel uses (bit-identical on CPU and GPU) --- */
void or_set_portable_math(int on);
double or_pexp(double x);
double or_plog(double x);

/* --- qmc.rs restatement --- */
double or_probit(double p);
double or_radical_inverse(uint64_t index, uint32_t base);
uint64_t or_mix64(uint64_t z);
double or_halton_hashed_u(uint32_t n, uint32_t b, uint64_t seed, uint64_t dim);
uint32_t or_owen_scramble(uint32_t x, uint64_t dim, uint64_t seed);
uint32_t or_digital_shift(uint64_t dim, uint64_t seed);
/* Fills masks[0..count) with the first `count` primitive GF(2) polynomials of degree >= 2. */
void or_primitive_polynomials(int64_t count, uint32_t* masks);
void or_direction_numbers(uint32_t mask, uint32_t* v32);
/* Direction table v[dim][32] for `dimension` dims (dim 0 = van der Corput). */
void or_sobol_table(int64_t dimension, uint32_t* v);
/* Gray-code Sobol integer of 1-based point n in `dim` (row = dim % dimension), unscrambled. */
uint32_t or_sobol_int(const uint32_t* v, int64_t dimension, uint64_t n, uint64_t dim);
void or_bridge_increments(const double* normals, int64_t n, double dt, double* out);
int32_t or_first_primes(int32_t count, uint32_t* out);
void or_halton_permutation(uint32_t base, uint64_t seed, uint32_t* perm);

/* --- the pseudo-random lane: ChaCha8Rng + StandardNormal (rand_chacha 0.9.0, rand_distr 0.5.1) --- */
void or_chacha8_normals(uint64_t seed, uint64_t count, double* out);
void or_chacha8_u64(uint64_t seed, uint64_t count, uint64_t* out);

/* --- correlation.rs restatement --- */
double or_min_eigenvalue(const double* c, int32_t n);
void or_psd_clamp(const double* c, int32_t n, double floor_, double* out);
/* L with L·Lᵀ = C (PSD-clamped first when min eig < -1e-10); returns RG_OK or an error. */
int32_t or_cholesky(const double* c, int32_t n, double* l);

/* --- riga-market/src/lib.rs restatement --- */
typedef struct or_lv_surface {
  int32_t n_t, gx;
  double* t_axis; /* [n_t] */
  double* log_s;  /* [gx] */
  double* v;      /* [n_t * gx] */
} or_lv_surface;
int32_t or_lv_calibrate(const rg_implied_vol_grid* grid, double spot, double rate, int32_t gx,
                        or_lv_surface* out);
double or_lv_sigma(const or_lv_surface* s, double t, double spot);
void or_lv_free(or_lv_surface* s);

/* --- lib.rs validate + note.rs price_full_phoenix --- */
int32_t or_validate(const rg_price_request* req);
/* threads <= 1: one sequential pass in path order (the reference's own order). */
int32_t or_price_put_leg(const rg_price_request* req, int32_t threads, rg_price_result* out);
/* explain.rs run_paths over [first, first + count). */
int32_t or_run_paths(const rg_price_request* req, uint64_t first, uint64_t count,
                     rg_path_record* out);
/* run_paths plus the f32 spot cube [count][steps][n] (spots after each step); records may be null. */
int32_t or_materialize_paths(const rg_price_request* req, uint64_t first, uint64_t count, float* cube,
                             rg_path_record* records);
/* Scenario batch: each scenario re-priced with the request's seed (CRN). */
int32_t or_price_scenarios(const rg_price_request* req, const rg_scenario* sc, int32_t n,
                           int32_t threads, rg_price_result* out);
/* --- pathcube.rs: the correlated ChaCha8 Brownian block and gbm_evolve --- */
void or_generate_correlated_block(uint64_t seed, int64_t paths, int64_t times, int32_t factors,
                                  const double* chol, float* out);
int32_t or_gbm_evolve(const double* s0, const double* vols, double rate, const double* q, int32_t factors,
                      double dt, const float* block, int64_t paths, int64_t times, float* out);

/* --- books: one universe path set, many trades, a common scenario set (threads >= 1) --- */
int32_t or_price_book(const rg_book_request* req, const rg_market_snapshot* sc, int32_t n_scen,
                      int32_t threads, rg_price_result* out /* [n_trades * S] */);
int32_t or_book_run_paths(const rg_book_request* req, const rg_market_snapshot* sc, int32_t n_scen,
                          uint64_t first, uint64_t count, rg_path_record* out);
/* riga-risk price_risk_batch (+ price_central_greeks). */
int32_t or_price_risk_batch(const rg_price_request* req, const rg_central_difference_config* cfg,
                            int32_t threads, rg_batch_risk_report* out);

/* Last error message of the calling thread. */
const char* or_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
