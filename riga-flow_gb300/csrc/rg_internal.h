// rg_internal.h — host-side structures shared by the C ABI, the request preparation and the
// kernel launchers.  Nothing here crosses the C ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <memory>
#include <vector>

#include "rg_common.cuh"

namespace rg {

// Error raised inside the host layer; converted to a status code at the ABI boundary.
struct Error {
  int32_t status;
  std::string message;
};

[[noreturn]] void raise(int32_t status, const std::string& message);
// PriceResult from the FP64 path sums of one scenario (note.rs:262-372).
void finish(const double* sums, uint64_t paths, uint64_t seed, rg_price_result* out);
void set_last_error(const std::string& message);
void cuda_check(cudaError_t e, const char* what);

// A device buffer that only grows.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  void ensure(size_t n);
  void release();
  ~DevBuf() { release(); }
};

// A pinned host buffer that only grows.
struct HostBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  void ensure(size_t n);
  void release();
  ~HostBuf() { release(); }
};

// Packs many small tables into one host staging area, copied to the device in one transfer.
struct Pack {
  std::vector<uint8_t> host;
  template <class T>
  size_t add(const T* data, size_t count) {
    size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + sizeof(T) * count);
    if (count) memcpy(host.data() + off, data, sizeof(T) * count);
    return off;
  }
  template <class T>
  size_t add(const std::vector<T>& v) { return add(v.data(), v.size()); }
  size_t reserve(size_t bytes) {
    size_t off = (host.size() + 255) & ~size_t(255);
    host.resize(off + bytes);
    return off;
  }
};

// One Dupire surface to calibrate: asset index, the market spot and rate it is calibrated
// against and the parallel implied-vol shift (crates/riga-risk/src/lib.rs:260-279).
struct SurfaceKey {
  int asset;
  double spot, rate, shift;
  bool operator==(const SurfaceKey& o) const {
    return asset == o.asset && spot == o.spot && rate == o.rate && shift == o.shift;
  }
};

// FP32 scenario constants for the CRN kernel, one per scenario.
struct DevScen32 {
  float x0[RG_NMAX];      // ln(spot / initial_spot)
  float mu_dt[RG_NMAX];   // (r - q) dt
  float sig[RG_NMAX];     // flat vol
  float a_u[RG_NMAX];     // (ln initial_spot - log_lo) / h
  float inv_h[RG_NMAX];   // 1 / h on the Dupire log-strike axis
  int32_t surf_off[RG_NMAX];  // first FP32 step row of the scenario's surface: surface·T·gx
  float L[RG_NMAX * RG_NMAX]; // the scenario's Cholesky factor rounded to FP32 (written by cholesky_kernel)
};

// Everything one request needs on the device, after preparation.
struct Prepared {
  DevTrade trade{};
  int n = 0;
  int64_t T = 0;
  int n_scen = 0;
  int n_surf = 0;
  int lv_nt_max = 0;
  int stack_max = 0;
  double ln_ko = 0, ln_cb = 0, ln_ki = 0;  // log barriers for the FP32 kernel
  std::vector<uint32_t> step_flags;
  std::vector<int32_t> step_period;
  std::vector<double> accr_inc;
  std::vector<float> accr_f;  // accr_inc in FP32 (the FP32 kernels read no FP64 per step)
  std::vector<int32_t> node_off, node_k;
  std::vector<double> node_c;
  std::vector<float> node_cf;
  std::vector<int32_t> nf_row;   // [node][n] Sobol row (dim % sob_dim) or Halton base index
  std::vector<uint32_t> nf_shift;  // [node][n] digital-shift mask of that dimension
  std::vector<int32_t> lv_ti;   // [n][T][2] (row, next row)
  std::vector<double> lv_tw;    // [n][T]
  std::vector<float> lv_twf;    // [n][T]
  std::vector<DevScenario> scen;
  std::vector<DevScen32> scen32;
  std::vector<double> df, df_mat;
  std::vector<float> df_f, df_mat_f;  // the same in FP32
  std::vector<SurfaceKey> surfaces;
  std::vector<int32_t> surf_nt;  // tenor count of each surface
  std::vector<double> asset_log_lo, asset_log_hi;
  // host copies of the request inputs the calibration kernel reads
  std::vector<const rg_implied_vol_grid*> grids;
};

struct Engine;

// The device and host memory one pricing call draws on: the engine's growable buffers, or a fixed
// region.  Slots are requested in this order within each fused launch.
enum WsSlot {
  WS_ARENA = 0, WS_CALIB, WS_LVROWS, WS_PARTIAL, WS_SUMS, WS_KOSTEPS, WS_RECORDS,
  WS_MCZ, WS_MCKEYS, WS_MCAUX,  // the pseudo-random lane's normals, keystream and parse tables
  WS_CUBE,                      // f32 spot cube of a materialised path range
  WS_NSLOTS
};
struct SurfaceCache;
struct Workspace {
  cudaStream_t stream = nullptr;
  cudaEvent_t* ev = nullptr;    // six events for the timing breakdown, or null
  rg_timing* timing = nullptr;  // or null
  int sm_count = 0;
  virtual void begin_launch() {}
  virtual void* device(int slot, size_t bytes) = 0;
  virtual void* host(size_t bytes) = 0;  // landing area of the FP64 sums
  // whether slots keep their contents across fused launches (false for a bump allocator)
  virtual bool persistent() const { return true; }
  // whether extra timed launches (the tile-depth autotuner) may run on this stream; not for the
  // static entry point, which may be called under stream capture
  virtual bool may_tune() const { return true; }
  // the engine's resident calibrated surfaces, or null (the static entry point keeps none)
  virtual SurfaceCache* surfaces() { return nullptr; }
  virtual ~Workspace() = default;
};
// validate → host tables → H2D → prologue → fused kernel → reduce → D2H → PriceResults
void price_with(Workspace& W, const rg_price_request* req, const rg_scenario* sc, int n_scen,
                rg_price_result* out);
int device_sm_count();

// Request preparation (host, FP64): validation already done.
void prepare(const rg_price_request* req, const rg_scenario* scen, int n_scen, Prepared& P);
// The streamed bridge schedule (node_off, node_k, node_c, stack_max) of T steps.
void bridge_schedule_into(int64_t T, double dt, Prepared& P);
// The Sobol direction table for `dim` dimensions (process-wide cache).
const std::vector<uint32_t>& sobol_table(int64_t dim);
std::vector<double> calib_axes(const rg_implied_vol_grid& g, double spot, double rate, int gx);
// The FP32 kernels' consumption-order Sobol tables for points starting at offset o within a
// 32-point block (host_prep.cu): transposed directions st[32][n·T] and the lanes' low-bit terms
// lut[n·T][32]; built once per (directions, assets, steps, seed, scrambler, o) and shared
// process-wide.
struct SobolLut {
  std::vector<uint32_t> st, lut;
};
std::shared_ptr<const SobolLut> sobol_lut_tables(const Prepared& P, int64_t sob_dim, uint32_t o, bool shift);
// The first `count` primes (a copy of a process-wide cache; at least `count` entries).
std::vector<uint32_t> first_primes(int count);
// Halton bases and permutations.
void halton_tables(int dim, uint64_t seed, std::vector<uint32_t>& base, std::vector<uint32_t>& off,
                   std::vector<uint32_t>& perm);

// Validation of lib.rs:209-321, generalised to N assets.
void validate_request(const rg_price_request* r);

// Kernel launchers (defined in the .cu files).
struct CalibJob {
  int32_t n_t, n_k, gx, pad;
  const double* mats;
  const double* strikes;
  const double* vols;
  double spot, rate, shift;
  double* out_v;
  float2* out_vf;
  double* out_logs;
  double* scratch;  // 4 * n_t * gx + gx + 6 * n_t * n_k doubles
  // the calibration's logarithms, evaluated on the host with the platform libm (calib_axes):
  // [log-strike axis, gx][log(K_j / F_k), n_t * n_k][log(S_i / F_k) before clamping, n_t * gx]
  const double* ax;
  // resident-surface cache entry ([v][logs][vf], surface_entry_bytes): copy the surface from it
  // instead of calibrating (cache_src), or calibrate and also store it there (cache_dst)
  const double* cache_src;
  double* cache_dst;
};
inline size_t surface_entry_bytes(int n_t, int gx) {
  return (size_t)n_t * gx * sizeof(double) + (size_t)gx * sizeof(double) + (size_t)n_t * gx * sizeof(float2);
}

// Calibrated Dupire surfaces kept on the device between calls of one engine, keyed by every input
// of the calibration (implied grid, spot, rate, implied-vol shift, grid width).  A copy is
// bit-identical to a recalibration.  Entries found by a call become usable only when the call
// completes (commit), so a failed call never leaves a half-written surface behind.
struct SurfaceCache {
  struct Entry {
    std::vector<uint8_t> key;
    DevBuf buf;
    uint64_t used = 0;
    bool ready = false;
  };
  static constexpr int kEntries = 64;
  Entry entries[kEntries];
  uint64_t tick = 0;
  std::vector<int> pending;  // entries this call fills
  std::vector<int> in_use;   // entries this call reads or fills (never evicted during it)
  // The entry for `key`: `hit` says whether it holds the calibrated surface already.
  // (null when every entry is in use by this call: then the surface is only calibrated)
  double* lookup(const std::vector<uint8_t>& key, size_t bytes, bool& hit);
  void begin_call();  // forget the entries of a call that did not complete
  void commit();      // the entries this call filled hold their surfaces now
  size_t device_bytes() const;
  void release();
};
void launch_calibrate(const CalibJob* jobs_dev, int n_jobs, cudaStream_t s);
void launch_cholesky(DevScenario* scen_dev, DevScen32* scen32_dev, int n_scen, int n, cudaStream_t s);
// Per surface and step, the Dupire row interpolated to the step's time, as FP32 (v_j, v_j+1 - v_j).
void launch_lvrows(const double* lv_v, const int32_t* surf_cell_off, const int32_t* surf_asset,
                   const int2* lv_ti, const double* lv_tw, int n_surf, int T, int gx, float2* rows,
                   cudaStream_t s);

struct LaunchOut {
  double* partial;      // [grid][n_scen][RG_ACC] (FP64 kernel), [32-path chunk][n_scen][RG_ACC] (FP32)
  int32_t* ko_steps;    // [npaths] (scenario 0) or null
  rg_path_record* records;  // [npaths] or null
  int grid;
  const double* mcz = nullptr;  // pseudo-random lane: normals [npaths][T][n] of the launch's paths
  float* cube = nullptr;        // [npaths][T][n] spots after each step (base scenario), or null
};
// StandardNormal draws [first, first + count) of ChaCha8Rng::seed_from_u64(seed) into d_out.
void mc_normals(uint64_t seed, uint64_t first, uint64_t count, double* d_out, Workspace& W);
int phoenix64_grid(const Prepared& P, uint64_t npaths);
void launch_phoenix64(const Prepared& P, const DevTables& tb, const DevScenario* scen_dev,
                      uint64_t path0, uint64_t npaths, const LaunchOut& out, cudaStream_t s);
struct Fp32Shape {
  int Sb, Pb, TT, threads, grid, smem;
  int ppt;     // paths per thread of the tiled kernel (1 or 2)
  int tuned;   // 1: Pb, ppt and TT came from the autotuner's cache (or were forced)
  int direct;  // 1: the per-thread kernel of phoenix32d.cu; then only grid and threads are used
};
// Scenario counts up to this value run on the direct kernel (phoenix32d.cu), when the launch has
// at least p32_direct_min_paths(n) paths: one path per thread needs enough warps to fill the GPU
// (measured crossover against the tiled kernel: about 2^18 paths for 1-3 assets, 2^16 for 4-5).
constexpr int kP32DirectMaxScen = 1;
inline uint64_t p32_direct_min_paths(int n) { return n >= 4 ? (uint64_t(1) << 16) : (uint64_t(3) << 16); }
inline bool p32_direct(const Prepared& P, uint64_t npaths) {
  return P.n_scen <= kP32DirectMaxScen && npaths >= p32_direct_min_paths(P.n);
}
int phoenix32d_grid(const Prepared& P, uint64_t npaths, int sm_count);
void launch_phoenix32d(const Prepared& P, const DevTables& tb, const DevScenario* scen, const DevScen32* scen32,
                       uint64_t path0, uint64_t npaths, int grid, const LaunchOut& out, cudaStream_t st);
Fp32Shape phoenix32_shape(const Prepared& P, uint64_t npaths, int sm_count);
// Rows of the FP32 kernels' partial sums partial[chunk][scenario][RG_ACC]: one per 32 paths.
uint64_t p32_chunks(uint64_t npaths);
// The level-ordered evaluation plans of the streamed Brownian bridge for every tile depth the tiled
// FP32 kernel may launch with (its formula depth and the autotuner's candidates): packed words,
// and per depth its value and word offset.
struct BridgePlans {
  std::vector<uint32_t> words;
  int32_t tt[RG_BPLAN_MAX], at[RG_BPLAN_MAX];
  int n = 0;
};
// A plan depends only on the step count (the node schedule and stack depth) and the tile depths,
// so the plans are built once per (steps, formula depth) and shared process-wide.
std::shared_ptr<const BridgePlans> p32_bridge_plans(const Prepared& P);
// The tiled kernel's step tiling from the autotuner: a cached choice for the launch's shape, or —
// when `may_tune` and the launch is large enough to amortise it — one tuning pass that times the
// candidate tile depths on a prefix of the paths (their results are discarded; the tile depth
// changes the schedule, never the arithmetic) and caches the fastest.  Returns `sh` with TT set.
// Enables or disables the autotuner process-wide; either way its cache is cleared.
void p32_set_autotune(bool enabled);
void p32_force_shape(int ppt, int tt, int pb);
// Phase clocks of the tiled FP32 kernel (a build option); 0 when the build has none.
int p32_phase_clocks(unsigned long long out[4], bool reset);
Fp32Shape phoenix32_tune(const Prepared& P, const DevTables& tb, const DevScenario* scen,
                         const DevScen32* scen32, uint64_t path0, uint64_t npaths, Fp32Shape sh,
                         const LaunchOut& out, bool may_tune, int sm_count, cudaStream_t st);
void launch_phoenix32(const Prepared& P, const DevTables& tb, const DevScenario* scen_dev,
                      const DevScen32* scen32_dev, uint64_t path0, uint64_t npaths,
                      const Fp32Shape& shape, const LaunchOut& out, cudaStream_t s);
// out[S][RG_ACC] = Σ over rows of partial[rows][S][RG_ACC] in a fixed order; `out` must hold
// reduce_scratch_doubles(rows, S) more doubles after its S·RG_ACC (the first pass's group sums).
void launch_reduce(const double* partial, int rows, int n_scen, double* out, cudaStream_t s);
size_t reduce_scratch_doubles(int rows, int n_scen);

// The 32-bit Sobol integers at which the inverse normal switches between its central and tail
// branches (computed in FP64 so the FP32 kernels branch exactly as the reference does).
// Cholesky factor (with the reference's PSD clamp) of one n×n correlation, n <= RG_BOOK_MAX_UNIVERSE,
// by one device thread; `work` holds 2·n·n doubles.
void launch_cholesky_big(const double* c, int n, double* l, double* work, cudaStream_t s);

// ------------------------------------------------------------------ books ---------------------
// One book trade's constants on the device.
struct BookTradeDev {
  int32_t n, T, periods, call_start;
  int32_t idx[RG_NMAX];   // universe asset of each underlying
  int32_t fixed_first, memory;
  double init[RG_NMAX];
  double maturity, call_barrier, coupon_barrier, coupon_rate, strike, ki;
  float ln_ko, ln_cb, ln_ki, coupon_f, strike_f;
  // the FP32 coupon increment coupon_rate / period_steps: a period has ps_a = max(1, T / periods)
  // steps (inc_a) or ps_a + 1 (inc_b)
  float inc_a, inc_b;
  int32_t ps_a;
};
// One scenario of a book: a market of the universe.
struct BookScenDev {
  double rate;
  double spots[RG_BOOK_MAX_UNIVERSE], vols[RG_BOOK_MAX_UNIVERSE], q[RG_BOOK_MAX_UNIVERSE];
  int32_t dfrow;  // row of the discount tables for this market's rate
};
// One (trade, scenario) pair: its market (index into the book's markets), the discount-table row
// of that market's rate, and the FP32 constants ln(S/S0), the log drift per step and the vol.
struct BookPair32 {
  float x0[RG_NMAX], drift[RG_NMAX], sig[RG_NMAX];
  int32_t mkt, dfrow;
};
// Device pointers of a staged book.
struct BookDev {
  int32_t U, S, n_trades;
  int64_t TU;
  const BookTradeDev* trades;  // [n_trades]
  const BookScenDev* scen;     // the markets the pairs price under
  const BookPair32* pair32;    // [n_trades][S]
  const double* df;            // [rate row][TU]  exp(-r (t+1) dt)
  const double* dfm;           // [n_trades][S] exp(-r_s maturity_j)
  const float* df_f;           // df and dfm rounded to FP32 for the FP32 scan
  const float* dfm_f;
  const double* L;             // [U][U] universe Cholesky factor (FP64)
  const float* L32;            // [U][U] the same in FP32
  const int32_t* order;        // [n_trades] trade order of the work items (longest first)
};
// Universe increments of paths [path0, path0 + npaths): incr[t][u][p], FP64 ΔW/√dt (parity) or
// FP32 ΔW (production, rows of `rowlen` >= npaths floats so that tensor-map strides are aligned).
void launch_book_gen64(const DevTrade& gen, const DevTables& tb, const double* L, int U,
                       uint64_t path0, uint64_t npaths, double* incr, cudaStream_t s);
void launch_book_gen32(const DevTrade& gen, const DevTables& tb, const float* L32, int U,
                       uint64_t path0, uint64_t npaths, uint64_t rowlen, float* incr, cudaStream_t s);
// FP64 scan of every (trade, scenario) on the chunk's increments: one thread per (pair, path);
// partial[pair][block][RG_ACC] over `blocks` blocks of 128 paths; records[p][pair] when given.
// partial[pair][block][RG_ACC] with `blocks` blocks of 128 paths per pair.
void launch_book_trade64(const DevTrade& gen, const BookDev& bk, const double* incr, uint64_t path0,
                         uint64_t npaths, double* partial, int blocks, rg_path_record* records,
                         cudaStream_t s);
// FP32 persistent scan: work items (path block, trade) with block-major order; every item's
// FP64 sums land in partial[(block0 + b) * n_trades + j][S][RG_ACC].
struct Book32Shape {
  int threads, Sb, Pb, TT, grid, blk_paths, smem;
};
// `paths`: the book's path count; `min_group_trades`: trades in its smallest underlying-count group.
Book32Shape book32_shape(int S, int sm_count, uint64_t paths, int min_group_trades);
// `tmap` views the chunk's increments as [TU][U][npaths] floats (boxes of Pb paths × 1 asset × TT
// steps) for the kernel's TMA stages.
// One persistent launch per underlying count n with trades order[group_lo[n-1], + group_n[n-1]).
// `maps[n - 1]`: the increments' tensor map with boxes of book_stage_steps(n, sh.TT) steps.
void launch_book_trade32(const BookDev& bk, const Book32Shape& sh, const CUtensorMap* maps, uint64_t npaths,
                         uint64_t block0, const int* group_lo, const int* group_n, double* partial,
                         int32_t* counter, int* status, cudaStream_t s);
int book_stage_steps(int n, int base);
// The FP32 copy of the universe Cholesky factor.
void launch_book_l32(const double* L, int U, float* L32, cudaStream_t s);
// Fixed-order sums over path blocks: out[pair][k] = Σ_b partial[b·stride_b + pair·stride_pair + k].
void launch_book_reduce_strided(const double* partial, int64_t blocks, int64_t stride_b, int64_t stride_pair,
                                int pairs, double* out, cudaStream_t s);

}  // namespace rg

// Body of every C entry point: rg::Error and allocation failures become status codes.
#define RG_TRY(...)                              \
  try {                                           \
    __VA_ARGS__;                                  \
    return RG_OK;                                 \
  } catch (const rg::Error& e) {                  \
    rg::set_last_error(e.message);                \
    return e.status;                              \
  } catch (const std::bad_alloc&) {               \
    rg::set_last_error("host allocation failed"); \
    return RG_ERR_GPU_ERROR;                      \
  }

int32_t rg_guard_device();

struct rg_engine;
namespace rg {
// Device bytes an engine's workspace holds, and releasing them (the engine must be idle).
size_t engine_device_bytes(rg_engine* E);
void engine_trim(rg_engine* E);
// Before a request on an idle engine: its streams' priority (high or default) and the SMs its
// grids are sized for (0: all), so a server's large requests leave SMs and priority to small ones.
void engine_set_class(rg_engine* E, bool high_priority, int sm_cap);
// The SM count the engine's launches size their grids for.
int engine_sm_count(const rg_engine* E);
// Device bytes one call will hold at its peak (workspace buffers; upper estimates).
size_t estimate_price_bytes(const rg_price_request* r, int n_scen);
size_t estimate_book_bytes(const rg_book_request* r, int n_scen);
size_t estimate_book_trade_bumps_bytes(const rg_book_request* r);
}  // namespace rg

// The engine behind the opaque C handle.
struct rg_engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t gen_stream = nullptr;  // book path generation, overlapped with the scan
  // the two stream pairs stream/gen_stream point to: default priority (direct calls and a server's
  // large requests) and the device's highest priority (a server's small requests)
  cudaStream_t stream_lo = nullptr, gen_stream_lo = nullptr;
  cudaStream_t stream_hi = nullptr, gen_stream_hi = nullptr;
  int sm_cap = 0;  // SMs the engine's grids are sized for (0: every SM of the device)
  std::mutex mu;
  rg::DevBuf bufs[rg::WS_NSLOTS];
  rg::DevBuf book_bufs[8];
  rg::HostBuf host_sums;
  std::vector<uint8_t> host_pack;
  rg::SurfaceCache surfaces;
  // the universe increments held in the first book increment buffer (a book of one path chunk),
  // by the bytes of every input of their generation; empty when the buffer holds anything else
  std::vector<uint8_t> universe_key;
  const void* universe_ptr = nullptr;
  cudaEvent_t ev[6] = {};
  cudaEvent_t book_ev[4] = {};
  rg_timing timing{};
};
