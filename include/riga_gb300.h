/*
 * riga_gb300.h — C ABI of the GB300 Monte Carlo engine for riga-flow's scenario hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and POD structs, and returns an
 * int32 status (0 = success).  A non-zero status maps 1:1 onto the reference's
 * `RigaError { code, message }` (crates/riga-core/src/lib.rs:5-19): `rg_status_code()` gives the
 * stable `code` string, `rg_last_error()` the thread's last `message`.  No C++ exception crosses
 * this boundary and there is no CPU fallback: without a usable sm_103a device every compute entry
 * point fails with RG_ERR_GPU_UNAVAILABLE ("gpu_unavailable"), as the reference's `gpu` build does
 * (crates/riga-engine/src/lib.rs:188-202, crates/riga-engine/src/gpu.rs:490-512).
 *
 * Structs mirror the reference's serde types field by field.  `Option<T>` fields become a
 * `has_<field>` flag plus the value.  Asset arrays are length `n_assets`; the reference accepts
 * exactly two assets (crates/riga-engine/src/lib.rs:234-245) and this engine accepts
 * 1..RG_MAX_ASSETS, reducing exactly to the reference at two.
 */
#ifndef RIGA_GB300_H
#define RIGA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_ABI_VERSION 1
#define RG_MAX_ASSETS 5
#define RG_TRACE_EVENT_CAP 64 /* crates/riga-engine/src/note.rs:57 */
#define RG_N_TRANSITIONS 3    /* daily_global_ko, final_fixing_eki, memory_coupon */

/* ------------------------------------------------------------------ status codes -------------- */
/* Stable error codes; the strings returned by rg_status_code() are the reference's RigaError.code
 * values (crates/riga-engine/src/lib.rs:209-321, gpu.rs:78-80,143-144,173-176,
 * crates/riga-risk/src/lib.rs:338-457). */
enum {
  RG_OK = 0,
  RG_ERR_MISSING_AS_OF = 1,          /* "missing_as_of" */
  RG_ERR_AS_OF_MISMATCH = 2,         /* "as_of_mismatch" */
  RG_ERR_INVALID_PATHS = 3,          /* "invalid_paths" */
  RG_ERR_INVALID_SCHEDULE = 4,       /* "invalid_schedule" */
  RG_ERR_INVALID_MARKET_SHAPE = 5,   /* "invalid_market_shape" */
  RG_ERR_INVALID_MARKET = 6,         /* "invalid_market" */
  RG_ERR_INVALID_TRADE = 7,          /* "invalid_trade" */
  RG_ERR_INVALID_LOCAL_VOL = 8,      /* "invalid_local_vol" */
  RG_ERR_SHAPE_MISMATCH = 9,         /* "shape_mismatch" */
  RG_ERR_GPU_UNAVAILABLE = 10,       /* "gpu_unavailable" */
  RG_ERR_GPU_ERROR = 11,             /* "gpu_error" */
  RG_ERR_NO_CRN_REJECTED = 12,       /* "no_crn_rejected" */
  RG_ERR_INVALID_SPOT_BUMP = 13,     /* "invalid_spot_bump" */
  RG_ERR_INVALID_VOLATILITY_BUMP = 14, /* "invalid_volatility_bump" */
  RG_ERR_INVALID_RATE_BUMP = 15,     /* "invalid_rate_bump" */
  RG_ERR_INVALID_CORRELATION_BUMP = 16, /* "invalid_correlation_bump" */
  RG_ERR_RISK_INPUT_SHAPE = 17,      /* "risk_input_shape" */
  RG_ERR_RISK_PATHS_REQUIRED = 18,   /* "risk_paths_required" */
  RG_ERR_PATH_OUT_OF_RANGE = 19,     /* "path_out_of_range" */
  RG_ERR_INVALID_ARGUMENT = 20,      /* "invalid_argument" (null pointer, bad enum, size limit) */
  RG_ERR_UNSUPPORTED = 21,           /* "unsupported" (a lane this engine does not run) */
  RG_ERR_INVALID_PERCENTILE = 22,    /* "invalid_percentile" */
  RG_ERR_CANCELLED = 23,             /* "cancelled" */
  RG_ERR_TIMEOUT = 24                /* "device_timeout": a bounded device wait expired */
};

/* ------------------------------------------------------------------ enums --------------------- */
/* TraceLevel, crates/riga-core/src/lib.rs:21-28 */
enum { RG_TRACE_OFF = 0, RG_TRACE_AGGREGATED = 1, RG_TRACE_SAMPLED = 2, RG_TRACE_FULL = 3 };
/* VarianceReduction, crates/riga-core/src/lib.rs:88-106 */
enum { RG_VR_NONE = 0, RG_VR_HALTON = 1, RG_VR_SOBOL = 2 };
/* Engine knobs that the reference does not have.  The defaults (all zero) reproduce the
 * reference: Owen scrambling (qmc.rs:292-308), FP64 arithmetic, dimension clamp+wrap at 512
 * (qmc.rs:9,249,271), the 96-point Dupire log-strike axis (riga-market/src/lib.rs:28). */
enum { RG_SCRAMBLE_OWEN = 0, RG_SCRAMBLE_DIGITAL_SHIFT = 1 };
enum { RG_PRECISION_FP64_PARITY = 0, RG_PRECISION_FP32 = 1 };
enum { RG_DIM_WRAP_REFERENCE = 0, RG_DIM_FULL = 1 };

/* ------------------------------------------------------------------ request types ------------- */
/* PhoenixTrade, crates/riga-core/src/lib.rs:57-75 */
typedef struct rg_phoenix_trade {
  const char* trade_id;
  int32_t n_assets;
  const double* initial_spots; /* [n_assets] */
  double maturity_years;
  int64_t steps;
  double strike;
  double knock_in_barrier;
  int32_t has_knock_out_barrier;
  double knock_out_barrier;
  int32_t has_coupon_barrier;
  double coupon_barrier;
  int32_t has_coupon_rate;
  double coupon_rate;
  int32_t memory_coupon;
  int32_t has_coupon_periods;
  int64_t coupon_periods;
  int32_t fixed_first_coupon;
  int32_t has_call_start_step;
  int64_t call_start_step;
} rg_phoenix_trade;

/* MarketSnapshot, crates/riga-core/src/lib.rs:37-45 */
typedef struct rg_market_snapshot {
  const char* as_of;
  int32_t n_assets;
  const double* spots;           /* [n_assets] */
  const double* vols;            /* [n_assets] */
  double risk_free_rate;
  const double* dividend_yields; /* [n_assets] */
  const double* correlation;     /* [n_assets * n_assets], row-major */
} rg_market_snapshot;

/* SimulationConfig, crates/riga-core/src/lib.rs:77-86, plus this engine's knobs. */
typedef struct rg_simulation_config {
  uint64_t paths;
  uint64_t path_block_size;
  uint64_t seed;
  int32_t trace_level;        /* RG_TRACE_* */
  int32_t variance_reduction; /* RG_VR_* */
  uint64_t qmc_dimension;     /* VarianceReduction::{Halton,Sobol}{dimension} */
  int32_t scrambler;          /* RG_SCRAMBLE_* (Sobol only) */
  int32_t precision;          /* RG_PRECISION_* */
  int32_t dim_mode;           /* RG_DIM_* */
  int32_t lv_grid_x;          /* Dupire log-strike points; 0 = 96 (riga-market/src/lib.rs:28) */
  uint64_t first_path;        /* global index of this request's path 0 (path-range sharding);
                                 path i uses QMC point first_path + i + 1 (qmc.rs:286) */
} rg_simulation_config;

/* ImpliedVolGrid, crates/riga-market/src/lib.rs:83-91 */
typedef struct rg_implied_vol_grid {
  int32_t n_maturities;
  int32_t n_strikes;
  const double* maturities_years; /* [n_maturities], strictly increasing */
  const double* strikes;          /* [n_strikes], strictly increasing */
  const double* vols;             /* [n_maturities * n_strikes], row-major */
} rg_implied_vol_grid;

/* PriceRequest, crates/riga-engine/src/lib.rs:36-46.  n_local_vol == 0 is `local_vol: None`. */
typedef struct rg_price_request {
  rg_phoenix_trade trade;
  rg_market_snapshot market;
  rg_simulation_config config;
  const char* as_of;
  int32_t n_local_vol;
  const rg_implied_vol_grid* local_vol; /* [n_local_vol] */
} rg_price_request;

/* ------------------------------------------------------------------ result types -------------- */
/* LegAttribution, crates/riga-core/src/lib.rs:209-217 */
typedef struct rg_leg_attribution {
  double par_redemption, coupon, memory_coupon, down_and_in_put, funding, discounting, total;
} rg_leg_attribution;

/* TransitionStats, crates/riga-core/src/lib.rs:219-229 (transition_id implied by the index:
 * 0 daily_global_ko, 1 final_fixing_eki, 2 memory_coupon; note.rs:277-308) */
typedef struct rg_transition_stats {
  uint64_t input_count, output_count;
  double probability, mean_payoff, variance_payoff, mean_delta, mean_vega;
} rg_transition_stats;

/* LedgerEntry numeric fields, crates/riga-core/src/lib.rs:231-241 (note.rs:314-354); the
 * condition and evidence strings are formatted by the caller from the request. */
typedef struct rg_ledger_entry {
  uint64_t population_before, population_after;
  double pv_impact, delta_impact, vega_impact;
} rg_ledger_entry;

/* One `daily_global_ko:path={path_id}:t={time:.6}` trace event (note.rs:174-180). */
typedef struct rg_trace_event {
  uint64_t path_id;
  double time;
} rg_trace_event;

/* FP64 path sums behind a result, in this slot order (pv and KO funding are shifted by -1):
 * sum(pv-1), sum((pv-1)^2), sum(KO funding-1), sum((KO funding-1)^2), sum(KI put), sum(KI put^2),
 * sum(coupon | paid), sum(coupon^2 | paid), sum(put), sum(funding), sum(coupon quote - memory
 * quote), sum(memory quote), #KO, #KI, #put eligible, #paid a coupon. */
#define RG_PATH_SUMS 16

/* PriceResult, crates/riga-core/src/lib.rs:243-255 */
typedef struct rg_price_result {
  double pv, mc_error, ki_probability;
  rg_leg_attribution legs;
  rg_transition_stats stats[RG_N_TRANSITIONS];
  rg_ledger_entry ledger[RG_N_TRANSITIONS];
  uint64_t seed;
  uint64_t ko_count, ki_count, put_eligible_count, coupon_path_count;
  int32_t n_trace_events;
  rg_trace_event trace_events[RG_TRACE_EVENT_CAP];
  double path_sums[RG_PATH_SUMS]; /* merged exactly by rg_merge_results */
} rg_price_result;

/* One scenario of a common-random-number batch: a complete market plus an optional parallel
 * implied-vol shift per asset (sticky strike, crates/riga-risk/src/lib.rs:260-279).  Every
 * scenario of a batch reuses the request's seed, trade and simulation config. */
typedef struct rg_scenario {
  rg_market_snapshot market;
  const double* implied_vol_shift; /* [n_assets] or NULL */
} rg_scenario;

/* CentralDifferenceConfig, crates/riga-risk/src/lib.rs:24-49 */
enum { RG_CRN = 0, RG_NO_CRN = 1 };
typedef struct rg_central_difference_config {
  double spot_relative_bump;
  double volatility_absolute_bump;
  double rate_absolute_bump;
  double correlation_absolute_bump;
  int32_t random_number_policy; /* RG_CRN; RG_NO_CRN is rejected */
} rg_central_difference_config;

/* FiniteDifferenceEstimate, crates/riga-risk/src/lib.rs:63-72 */
typedef struct rg_fd_estimate {
  double value, mc_error_upper_bound;
} rg_fd_estimate;

/* AssetGreeks + BatchAssetGreeks, crates/riga-risk/src/lib.rs:74-94, 468-476 */
typedef struct rg_asset_greeks {
  int32_t asset_index;
  double spot_bump, volatility_bump;
  rg_fd_estimate delta, gamma, vega;
  double spot_up_pv, spot_down_pv, vol_up_pv, vol_down_pv;
  double spot_up_mc_error, spot_down_mc_error, vol_up_mc_error, vol_down_mc_error;
} rg_asset_greeks;

/* TransitionRisk, crates/riga-risk/src/lib.rs:478-493 (index as in rg_transition_stats) */
typedef struct rg_transition_risk {
  double pv_impact, delta_impact, vega_impact;
} rg_transition_risk;

/* BatchRiskReport, crates/riga-risk/src/lib.rs:495-516.  `base` is the full base-case result. */
typedef struct rg_batch_risk_report {
  rg_price_result base;
  uint64_t scenario_count;
  uint64_t seed;
  int32_t n_assets;
  rg_asset_greeks assets[RG_MAX_ASSETS];
  rg_transition_risk transitions[RG_N_TRANSITIONS];
  double rate_up_pv, rate_down_pv, correlation_up_pv, correlation_down_pv;
  double rate_bump, correlation_bump, pv_mc_error;
} rg_batch_risk_report;

/* PathRecord scalar fields, crates/riga-engine/src/explain.rs:57-74 */
typedef struct rg_path_record {
  uint64_t path_id, rng_seed, sobol_index;
  double worst_final;
  int32_t knocked_out;
  int32_t ko_step;      /* -1 when the path never knocked out */
  double ko_time;       /* NaN when the path never knocked out */
  int32_t ki_hit;
  int32_t qualified_steps; /* qualifying coupon observations while alive (explain.rs:226) */
  int32_t paid_periods;    /* period ends and KO dates that paid a coupon */
  double put_payoff, coupon_pv, memory_coupon_pv, funding, pv;
} rg_path_record;

/* ------------------------------------------------------------------ errors -------------------- */
/* The RigaError.code string for a status (crates/riga-core/src/lib.rs:5-19). */
const char* rg_status_code(int32_t status);
/* Copies the calling thread's last error message (NUL-terminated, truncated to len); returns
 * the full message length. */
int32_t rg_last_error(char* buf, size_t len);
int32_t rg_abi_version(void);

/* ------------------------------------------------------------------ device -------------------- */
/* gpu::ensure_available, crates/riga-engine/src/gpu.rs:500-503 */
int32_t rg_ensure_available(void);
/* gpu::device_name, crates/riga-engine/src/gpu.rs:505-508 */
int32_t rg_device_name(char* buf, size_t len);
/* gpu::arch, crates/riga-engine/src/gpu.rs:510-512 ("sm_103" on GB300) */
int32_t rg_arch(char* buf, size_t len);

/* ------------------------------------------------------------------ engine -------------------- */
/* An engine owns one CUDA stream, its device workspace and cached tables.  Calls on one engine
 * are serialised by the engine; separate engines run concurrently.  Replaces the process-wide
 * `OnceLock<Gpu>` of crates/riga-engine/src/gpu.rs:490-497. */
typedef struct rg_engine rg_engine;
int32_t rg_engine_create(int32_t device, rg_engine** out);
void rg_engine_destroy(rg_engine* engine);

/* riga_engine::price_put_leg, crates/riga-engine/src/lib.rs:183-186 (-> note::price_full_phoenix,
 * note.rs:38-373).  Runs the fused generation+step+payoff kernel on the device. */
int32_t rg_price_put_leg(rg_engine* engine, const rg_price_request* request, rg_price_result* out);

/* rg_price_put_leg without any device allocation (this entry point has no counterpart in the
 * reference).  For callers that may not allocate device memory: hosts whose memory pool owns every
 * byte of the device, processes under a hard device-memory budget, and plugins that must not call
 * cudaMalloc or cudaFree behind their host's back (cudaFree synchronises the whole device; both
 * take memory outside the host's accounting).  It needs no engine: every device buffer comes from
 * one static 16 MiB region of the library, a module global that stays reserved on each GPU where
 * the library's module is loaded until the process exits (with lazy module loading, the CUDA
 * default, only GPUs where the library's kernels run; with CUDA_MODULE_LOADING=EAGER every context
 * that loads the library).  Requests that need more — e.g. many paths with trace events on, or
 * long local-vol grids — fail with RG_ERR_INVALID_ARGUMENT.  Runs on the current device and the
 * legacy default stream and returns when the result is ready.  The first call on a device
 * resolves the region's address (cudaGetSymbolAddress) with that device current, so make that
 * first call before any stream capture.  Calls on one device share the region, which keeps the
 * last call's contents: they are serialised by a per-device lock, because GPU work of two calls
 * that overlapped would race on it.  Same results as rg_price_put_leg for the same request. */
int32_t rg_price_put_leg_static(const rg_price_request* request, rg_price_result* out);

/* A CRN scenario batch in one fused launch: out[i] is the request priced under scenarios[i] with
 * the request's seed (crates/riga-risk/src/lib.rs:253-258; crates/riga-engine/src/dispatch.rs:23-70). */
int32_t rg_price_scenarios(rg_engine* engine, const rg_price_request* request,
                           const rg_scenario* scenarios, int32_t n_scenarios,
                           rg_price_result* out);

/* Calibrates, on the device in FP64, the Dupire surfaces a local-vol request needs — one per
 * (asset, market) of the request and of its `n_scenarios` CRN scenarios with their implied-vol
 * shifts (crates/riga-market/src/lib.rs:210-299, crates/riga-risk/src/lib.rs:260-279) — and keeps
 * them resident on the engine, so that pricing calls with the same inputs copy them instead of
 * recalibrating.  The engine keeps the 64 most recently used surfaces (pricing calls add theirs
 * too); a resident surface is byte-identical to a fresh calibration.  `*resident` (optional)
 * receives the number of distinct surfaces.  A request without local vol uploads nothing. */
int32_t rg_surfaces_upload(rg_engine* engine, const rg_price_request* request, const rg_scenario* scenarios,
                           int32_t n_scenarios, int32_t* resident);

/* riga_risk::price_risk_batch, crates/riga-risk/src/lib.rs:573-626 (with the central Greeks of
 * price_central_greeks, :117-186): base + spot/vol up/down per asset + rate up/down +
 * correlation up/down, all priced in one CRN launch. */
int32_t rg_price_risk_batch(rg_engine* engine, const rg_price_request* request,
                            const rg_central_difference_config* config,
                            rg_batch_risk_report* out);

/* Merges the results of disjoint path shards (in shard order: fixed-order FP64 sums, trace
 * events concatenated up to the cap) into the result of all their paths — the one gather of the
 * multi-GPU path.  `paths` is the total path count. */
int32_t rg_merge_results(const rg_price_result* parts, int32_t n_parts, uint64_t paths,
                         rg_price_result* out);

/* Device-time breakdown of the engine's last call, from CUDA events on the engine's stream. */
typedef struct rg_timing {
  double h2d_ms, prologue_ms, kernel_ms, reduce_ms, d2h_ms, device_ms;
  uint64_t h2d_bytes, d2h_bytes;
  int32_t kernel_launches; /* kernels this call launched (prologue + fused + reduce) */
  int32_t grid, block, smem_bytes; /* launch shape of the fused kernel */
  int32_t tile_steps; /* steps per time tile of the tiled FP32 kernel (0 for the other kernels) */
  int32_t paths_per_thread; /* paths each thread of the tiled FP32 kernel steps (1 or 2) */
} rg_timing;
int32_t rg_engine_last_timing(rg_engine* engine, rg_timing* out);

/* The tiled FP32 kernel's autotuner (on by default, process-wide).  The first pricing call of a
 * launch shape (asset count, local vol, scenario slots, steps, QMC lane, grid width) with at least
 * eight waves of path tiles times every candidate schedule — one or two paths per thread (two:
 * packed FP32x2 stepping on 512 threads) and the time-tile depths — on a prefix of its paths and
 * keeps the fastest for that shape; later calls reuse it.  Neither knob changes a path's arithmetic
 * or the 32-path chunks of the sums, so prices are the same with the autotuner on or off.  Calls
 * through rg_price_put_leg_static never tune.  Disabling also clears the tuned shapes.  No
 * counterpart in the reference. */
int32_t rg_set_autotune(int32_t enabled);
/* Forces every tiled FP32 launch of the process onto one schedule: paths per thread 1 or 2, a tile
 * depth among the autotuner's candidates (24, 32, 48, 64, 80, 96, 128) and a block of
 * paths_per_block paths per CTA tile (0 = the formula block of 1024 / scenario slots; otherwise a
 * power of two of at least 32 × paths per thread); (0, 0, 0) returns to the formula shape or the
 * autotuner.  A forced shape that does not fit (shared memory, 1024 threads) fails the pricing
 * call with RG_ERR_INVALID_ARGUMENT.  For callers that need a fixed schedule, and for checking
 * that schedules do not change prices.  No counterpart in the reference. */
int32_t rg_set_tiled_shape(int32_t paths_per_thread, int32_t tile_steps, int32_t paths_per_block);
/* Clock cycles the tiled FP32 kernel's CTAs spent in generation, bridge, stepping and path close
 * (out[0..3], summed over CTAs since the last reset), for profiling.  Only a library built with
 * RG_PHASE_CLOCKS=1 records them; others return RG_ERR_UNSUPPORTED.  No counterpart in the
 * reference. */
int32_t rg_phase_clocks(uint64_t out[4], int32_t reset);

/* explain::run_paths restricted to [first_path, first_path + count),
 * crates/riga-engine/src/explain.rs:90-316 (reconstruct_path :319-333 is count == 1). */
int32_t rg_run_paths(rg_engine* engine, const rg_price_request* request, uint64_t first_path,
                     uint64_t count, rg_path_record* out);

/* Replay materialisation of a priced trade: the spot paths of [first_path, first_path + count)
 * under the request's base scenario as an f32 cube in PathCube's [path][time][factor] layout
 * (crates/riga-engine/src/pathcube.rs:19-35): cube[(i * steps + t) * n + f] = S_f after step t
 * (the state explain::run_paths holds after its multiplicative step, explain.rs:183-193; spots
 * keep evolving after a knock-out there and here).  `records` (optional, may be null) receives
 * the same paths' PathRecord fields.  Always computed by the FP64 kernel (the precision setting
 * is ignored), each spot rounded to f32 on store; the cube is produced and copied out in chunks
 * of at most 1 GiB, so `count` is bounded only by the host buffer. */
int32_t rg_materialize_paths(rg_engine* engine, const rg_price_request* request, uint64_t first_path,
                             uint64_t count, float* cube, rg_path_record* records);

/* ------------------------------------------------------------------ books --------------------- */
/* A book: many Phoenix trades on one asset universe, priced under one common CRN scenario set.
 * This entry point has no single counterpart in the reference, which prices one trade per
 * request (price_put_leg, crates/riga-engine/src/lib.rs:183) and each risk scenario by a full
 * re-simulation (crates/riga-risk/src/lib.rs:573-626).
 *
 * Semantics — one universe path set on a common grid of `universe_steps` steps of
 * dt = universe_maturity_years / universe_steps: path i draws the universe's normals at QMC
 * point first_path + i + 1, dimension U·step + u for universe asset u (the reference's
 * N·step + f numbering with N = U), correlates them with the Cholesky factor of the universe
 * correlation and bridges every asset over the whole grid (note.rs:83-106 with N = U and
 * T = universe_steps).  A trade on universe assets a_0..a_{n-1} with `steps` = T_j <=
 * universe_steps runs the reference's step and Phoenix scan (note.rs:129-259) on the first T_j
 * steps of those assets' increments with the universe dt.  So a book holding one trade on every
 * universe asset in order, with T_j = universe_steps, prices exactly that trade's
 * price_put_leg; a shorter trade reads a truncation of the same Brownian paths. */
#define RG_BOOK_MAX_UNIVERSE 32

typedef struct rg_book_trade {
  rg_phoenix_trade terms;     /* maturity_years must be steps × the universe dt (1e-12 relative) */
  const int32_t* underlyings; /* [terms.n_assets] distinct universe indices */
} rg_book_trade;

typedef struct rg_book_request {
  rg_market_snapshot universe; /* base market, n_assets = U <= RG_BOOK_MAX_UNIVERSE, U×U correlation */
  int64_t universe_steps;
  double universe_maturity_years;
  int32_t n_trades;
  const rg_book_trade* trades; /* [n_trades] */
  rg_simulation_config config; /* Sobol or Halton; trace_level must be RG_TRACE_OFF */
} rg_book_request;

/* Prices every trade of the book under every scenario: out[j * S + s] is trade j under
 * scenarios[s], S = n_scenarios (scenarios NULL and n_scenarios 0: the base market alone, S = 1).
 * A scenario is a market of the universe (n_assets = U) that keeps the base correlation — its
 * `correlation` is NULL or equal to the base — so every scenario reads the same paths; spots,
 * vols, dividend yields and the rate may differ. */
int32_t rg_price_book(rg_engine* engine, const rg_book_request* request,
                      const rg_market_snapshot* scenarios, int32_t n_scenarios,
                      rg_price_result* out);

/* Per-trade bump sets (this scenario layout has no single counterpart in the reference, which bumps
 * one trade's own underlyings per risk call: crates/riga-risk/src/lib.rs:117-186, 573-626, and the
 * cross-gamma corners of crates/riga-mcp/src/main.rs:1366-1393).  Every trade of a book is priced
 * under RG_BOOK_TRADE_SCENARIOS scenarios on its own underlyings, all on the same universe paths:
 * scenario 0 is the base market and scenarios 1..15 are bumps, taken in this order until there are
 * 15 (h = spot_relative, v = vol_absolute, r = rate_absolute; underlying positions within the
 * trade, pairs in the order (0,1), (0,2), (1,2), (0,3), (1,3), (2,3), (0,4), ...):
 *   spot ×(1 + h) and ×(1 - h) of each underlying; vol + v of each underlying; rate + r;
 *   spot ×(1 + h) of both underlyings of each pair (cross-gamma corner); vol - v of each underlying;
 *   rate - r; spot ×(1 - h) of both of each pair; spot ×(1 ± 2h), ×(1 ± 5h), ×(1 ± 10h) of each
 *   underlying; vol ± 2v of each underlying; rate ± 2r.
 * So a 5-underlying trade gets spot ± and vol + of every underlying, a 3-underlying trade also the
 * rate, the three ++ corners, and vol - of two underlyings.  Vols are floored at 0. */
#define RG_BOOK_TRADE_SCENARIOS 16
typedef struct rg_book_bumps {
  double spot_relative; /* 0 = 0.01 */
  double vol_absolute;  /* 0 = 0.01 */
  double rate_absolute; /* 0 = 1e-4 */
} rg_book_bumps;
enum { RG_BUMP_BASE = 0, RG_BUMP_SPOT = 1, RG_BUMP_VOL = 2, RG_BUMP_RATE = 3, RG_BUMP_SPOT_PAIR = 4 };
typedef struct rg_book_bump_spec {
  int32_t kind;          /* RG_BUMP_* */
  int32_t first, second; /* underlying positions within the trade (-1 when unused) */
  double size;           /* relative spot move, absolute vol or rate move (signed) */
} rg_book_bump_spec;
/* The bump of scenario `scenario` (0..15) of a trade with n_underlyings underlyings. */
int32_t rg_book_trade_bump(int32_t n_underlyings, int32_t scenario, const rg_book_bumps* sizes,
                           rg_book_bump_spec* out);
/* Prices every trade of the book under its own 16 scenarios: out[j * 16 + k] is trade j under its
 * scenario k.  sizes NULL = the defaults. */
int32_t rg_price_book_trade_bumps(rg_engine* engine, const rg_book_request* request,
                                  const rg_book_bumps* sizes, rg_price_result* out);

/* Per-path records of book paths [first_path, first_path + count) for every (trade, scenario):
 * out[(p * n_trades + j) * S + s] (explain.rs:90-316 applied to each trade of the book). */
int32_t rg_book_run_paths(rg_engine* engine, const rg_book_request* request,
                          const rg_market_snapshot* scenarios, int32_t n_scenarios,
                          uint64_t first_path, uint64_t count, rg_path_record* out);

/* A resident book: trades uploaded once, then priced under many scenario sets.  rg_book_create
 * uploads the book to the engine's device once — trade tables, QMC tables, bridge schedule, the
 * universe Cholesky factor and the universe's FP32 increments of every path (they do not depend on
 * the scenarios; up to 96 GiB).  rg_book_price prices it under a new scenario set: host planning of
 * the scenario tables, then the replay of a CUDA graph of the device work (scenario upload, scans,
 * reduction, download) captured on the first call for that scenario count, after an autotuner has
 * timed the scan's stage depth (time steps per TMA stage) on a prefix of the paths.  Results equal
 * rg_price_book's for the same book and scenarios bit for bit (the tuned stage depth changes the
 * schedule, not the arithmetic).  FP32 books only; the engine must outlive the book. */
typedef struct rg_book rg_book;
int32_t rg_book_create(rg_engine* engine, const rg_book_request* request, rg_book** out);
int32_t rg_book_price(rg_book* book, const rg_market_snapshot* scenarios, int32_t n_scenarios,
                      rg_price_result* out);
/* The resident book under per-trade bump sets (rg_price_book_trade_bumps): out[j * 16 + k]. */
int32_t rg_book_price_trade_bumps(rg_book* book, const rg_book_bumps* sizes, rg_price_result* out);
/* The stage depth the autotuner chose for n_scenarios (0 before the first price at that count). */
int32_t rg_book_tuned_stage(rg_book* book, int32_t n_scenarios, int32_t* steps_per_stage);
void rg_book_destroy(rg_book* book);

/* ------------------------------------------------------------------ serving ------------------- */
/* A continuous-batching request server on one GPU (the engine side of the reference's MCP task
 * loop, crates/riga-mcp/src/main.rs:1000-1042, with its tasks/get, tasks/result and tasks/cancel
 * semantics).  It owns `slots` engines, each with its own CUDA stream and workspace.  Submitted
 * requests are deep-copied and queued in arrival order; a request is admitted as soon as a slot is
 * free and its device-memory estimate fits in the budget beside the slots' current holdings (idle
 * slots release their buffers when that makes room), so requests that arrive while others run are
 * admitted as slots and memory free up and run concurrently with them on the device.  A request's
 * results do not depend on what runs beside it.  Requests whose estimate exceeds the whole budget
 * are rejected at submission (RG_ERR_INVALID_ARGUMENT). */
typedef struct rg_server rg_server;

typedef struct rg_server_config {
  int32_t device;
  int32_t slots;                 /* concurrent requests (engines); 0 = 4 */
  uint64_t device_memory_budget; /* bytes for the slots' workspaces; 0 = 80% of free memory */
  int32_t max_large_slots;       /* slots large requests may hold at once; 0 = half the slots */
  uint64_t large_work;           /* paths × steps × scenarios (summed over a book's trades, plus its
                                    universe generation) at which a request is large; 0 = 2^31 */
  int32_t large_max_sms;         /* SMs a large request's kernels are sized for, leaving the rest to
                                    small requests, whose streams also have the highest priority;
                                    0 = two thirds of the SMs, negative = all */
} rg_server_config;

enum { RG_JOB_QUEUED = 0, RG_JOB_RUNNING = 1, RG_JOB_DONE = 2, RG_JOB_FAILED = 3, RG_JOB_CANCELLED = 4 };
enum { RG_JOB_PRICE = 0, RG_JOB_RISK = 1, RG_JOB_BOOK = 2, RG_JOB_BOOK_BUMPS = 3 };

typedef struct rg_job_info {
  int32_t state;          /* RG_JOB_* */
  int32_t status;         /* RG_OK or the failure's status code once FAILED */
  int32_t kind;           /* RG_JOB_PRICE / RISK / BOOK */
  int32_t slot;           /* slot that ran it, -1 before admission */
  uint64_t n_results;     /* rg_price_result entries the request produces */
  uint64_t device_bytes;  /* admission estimate */
  double submit_s, start_s, end_s; /* seconds since the server started (0 until reached) */
} rg_job_info;

typedef struct rg_server_stats {
  uint64_t submitted, completed, failed, cancelled, queued, running;
  uint64_t device_bytes_held, device_memory_budget;
  double p50_ms, p99_ms, max_ms; /* submit-to-completion latency of completed requests */
  double busy_s;                 /* wall time with at least one request running */
  uint64_t memory_waits;         /* requests that waited at the head of the queue because their
                                    device-memory estimate did not fit beside the running ones */
  uint64_t peak_reserved_bytes;  /* largest reservation seen: the slots' holdings and the running
                                    requests' estimates */
} rg_server_stats;

int32_t rg_server_create(const rg_server_config* config, rg_server** out);
/* Waits for running requests, cancels queued ones and frees the engines. */
void rg_server_destroy(rg_server* server);
/* A price request, optionally over a CRN scenario batch (n_scenarios 0 = the request's market). */
int32_t rg_server_submit_price(rg_server* server, const rg_price_request* request,
                               const rg_scenario* scenarios, int32_t n_scenarios, uint64_t* ticket);
/* riga_risk::price_risk_batch (crates/riga-risk/src/lib.rs:573-626). */
int32_t rg_server_submit_risk(rg_server* server, const rg_price_request* request,
                              const rg_central_difference_config* config, uint64_t* ticket);
/* A book under a common scenario set (rg_price_book). */
int32_t rg_server_submit_book(rg_server* server, const rg_book_request* request,
                              const rg_market_snapshot* scenarios, int32_t n_scenarios, uint64_t* ticket);
/* A book with every trade under its own 16 scenarios (rg_price_book_trade_bumps; sizes NULL = the
 * defaults): n_results = n_trades * 16, out[j * 16 + k]. */
int32_t rg_server_submit_book_trade_bumps(rg_server* server, const rg_book_request* request,
                                          const rg_book_bumps* sizes, uint64_t* ticket);
/* Current state without blocking. */
int32_t rg_server_poll(rg_server* server, uint64_t ticket, rg_job_info* info);
/* Blocks until the request is DONE, FAILED or CANCELLED, or `timeout_ms` passes (negative = no
 * limit; RG_ERR_TIMEOUT when it passes first).  Returns RG_OK with the final state in *info; a
 * FAILED request's status and message are also the calling thread's rg_last_error. */
int32_t rg_server_wait(rg_server* server, uint64_t ticket, int64_t timeout_ms, rg_job_info* info);
/* Copies a DONE price or book request's results (n_results entries) into out[capacity]. */
int32_t rg_server_results(rg_server* server, uint64_t ticket, rg_price_result* out, uint64_t capacity);
/* Copies a DONE risk request's report. */
int32_t rg_server_risk_report(rg_server* server, uint64_t ticket, rg_batch_risk_report* out);
/* A queued request is dropped; a running one finishes on the device and is reported CANCELLED. */
int32_t rg_server_cancel(rg_server* server, uint64_t ticket);
/* Forgets a finished request and its results. */
int32_t rg_server_release(rg_server* server, uint64_t ticket);
int32_t rg_server_get_stats(rg_server* server, rg_server_stats* out);

/* ------------------------------------------------------------------ host tables --------------- */
/* The Sobol direction table v[dim][32] the engine uses for `dim` dimensions: dimension 0 is van
 * der Corput, dimension d >= 1 the Joe–Kuo recurrence with unit initial values on the d-th
 * primitive polynomial of degree >= 2 (crates/riga-engine/src/qmc.rs:247-262, 316-430). */
int32_t rg_sobol_directions(int64_t dim, uint32_t* out /* [dim * 32] */);

/* The streamed Brownian-bridge schedule for `steps` steps of length dt: node_off[steps + 1]
 * (first node consumed at each step), node_k[steps] (the preorder index of each node, i.e. the
 * QMC step whose normals it reads; node 0 is the terminal point) and node_c[steps] (its
 * conditional standard deviation) — the in-order traversal of the reference's depth-first
 * bisection (crates/riga-engine/src/qmc.rs:155-191).  Returns the anchor-stack depth in
 * *stack_depth. */
int32_t rg_bridge_schedule(int64_t steps, double dt, int32_t* node_off, int32_t* node_k,
                           double* node_c, int32_t* stack_depth);

/* ------------------------------------------------------------------ pseudo-random lane ------- */
/* The reference's MC lane draws ChaCha8Rng::seed_from_u64(seed) -> rand_distr::StandardNormal
 * (rand_chacha 0.9.0, rand_distr 0.5.1; note.rs:58,123-127): one sequential stream in which path p,
 * step s, factor f is draw (p·T + s)·n + f.  The engine generates that stream on the device (a
 * parallel parse of the ziggurat's variable consumption), so VarianceReduction::None prices on the
 * GPU through rg_price_put_leg / rg_price_scenarios / rg_price_risk_batch / rg_run_paths (always
 * with the FP64 kernel) and the PathCube functions below exist.  Not available through
 * rg_price_put_leg_static (RG_ERR_UNSUPPORTED). */

/* Draws [first, first + count) of the stream for `seed` (count <= 2^31). */
int32_t rg_chacha8_normals(uint64_t seed, uint64_t first, uint64_t count, double* out);

/* pathcube::generate_correlated_block, crates/riga-engine/src/pathcube.rs:37-66: out[path][time]
 * [factor] = (f32)(L·z) with z the stream's draws in (path, time, factor) order and `chol` the
 * factors × factors Cholesky factor (row-major, lower triangle read). */
int32_t rg_generate_correlated_block(uint64_t seed, int64_t paths, int64_t times, int32_t factors,
                                     const double* chol, float* out);

/* pathcube::gbm_evolve, crates/riga-engine/src/pathcube.rs:146-187: out[path][time][factor] =
 * (f32)exp(ln s0 + Σ_{i<=time} ((rate - q - vol²/2)·dt + vol·√dt·block[path][i][factor])). */
int32_t rg_gbm_evolve(const double* s0, const double* vols, double rate, const double* dividend_yields,
                      int32_t factors, double dt, const float* block, int64_t paths, int64_t times,
                      float* out);

/* ------------------------------------------------------------------ gpu backend drop-in ------- */
/* gpu::worst_of, crates/riga-engine/src/gpu.rs:171-205 / :515-517 (out = min(a, b)). */
int32_t rg_worst_of(const float* a, const float* b, float* out, int64_t n);

/* gpu::lv_terminal_spots, crates/riga-engine/src/gpu.rs:209-277 / :538-564.  normals
 * [paths, steps, 2], rows [2, steps, gx], ls_axis [2 * gx], s0/references/dividends [2];
 * writes terminal spots [paths, 2] and the first autocall step (or -1) [paths]. */
int32_t rg_lv_terminal_spots(const float* normals, const float* rows, const float* ls_axis,
                             int64_t gx, const float* s0, const float* references,
                             float call_barrier, int64_t paths, int64_t steps, float dt,
                             float rate, const float* dividends, float* out_terminal,
                             int32_t* out_ko);

/* gpu::resident_lv / ResidentLv::{run, download, synchronize}, crates/riga-engine/src/gpu.rs:
 * 283-327, 409-488, 525-534: upload the scenario-independent buffers once, re-run per bump. */
typedef struct rg_resident_lv rg_resident_lv;
int32_t rg_resident_lv_create(const float* normals, const float* rows, const float* ls_axis,
                              int64_t gx, int64_t paths, int64_t steps, float dt,
                              rg_resident_lv** out);
int32_t rg_resident_lv_run(rg_resident_lv* lv, const float* s0, const float* references,
                           float call_barrier, float rate, const float* dividends);
int32_t rg_resident_lv_download(rg_resident_lv* lv, float* out_terminal, int32_t* out_ko);
int32_t rg_resident_lv_synchronize(rg_resident_lv* lv);
void rg_resident_lv_destroy(rg_resident_lv* lv);

/* gpu::resident_worst_of / ResidentWorstOf::{reduce, download, synchronize},
 * crates/riga-engine/src/gpu.rs:362-405. */
typedef struct rg_resident_worst_of rg_resident_worst_of;
int32_t rg_resident_worst_of_create(const float* a, const float* b, int64_t n,
                                    rg_resident_worst_of** out);
int32_t rg_resident_worst_of_reduce(rg_resident_worst_of* w);
int32_t rg_resident_worst_of_download(rg_resident_worst_of* w, float* out);
int32_t rg_resident_worst_of_synchronize(rg_resident_worst_of* w);
void rg_resident_worst_of_destroy(rg_resident_worst_of* w);

#ifdef __cplusplus
}
#endif

#endif /* RIGA_GB300_H */
