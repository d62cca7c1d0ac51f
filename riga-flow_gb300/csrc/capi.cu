// capi.cu — the C ABI of the engine: errors, device discovery, the engine object, pricing,
// scenario batches, the CRN risk batch and per-path replay records.
//
// The pipeline of one request, all on the engine's stream:
//   validate (host) → host tables (host_prep.cu) → one packed H2D copy → FP64 prologue kernels
//   (Dupire calibration per distinct surface, Cholesky per scenario) → fused path kernel
//   (FP64 parity or FP32 CRN) → fixed-order reduction → one D2H copy of the FP64 sums →
//   PriceResult assembly on the host (note.rs:262-372).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "rg_internal.h"

namespace rg {

static thread_local std::string g_last_error;

void set_last_error(const std::string& m) { g_last_error = m; }

[[noreturn]] void raise(int32_t status, const std::string& message) { throw Error{status, message}; }

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear a non-sticky error so the context stays usable
    raise(RG_ERR_GPU_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

// Capacity for n bytes: below 1 GiB the next power of two, so that requests of growing size
// re-allocate a few times rather than at every step (cudaFree waits for the whole device).
static size_t grown(size_t n) {
  if (n < 256) return 256;
  if (n >= (size_t(1) << 30)) return n;
  size_t c = 256;
  while (c < n) c <<= 1;
  return c;
}
void DevBuf::ensure(size_t n) {
  if (n <= bytes && ptr) return;
  release();
  const size_t want = grown(n);
  cuda_check(cudaMalloc(&ptr, want), "cudaMalloc");
  bytes = want;
}
void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}
void HostBuf::ensure(size_t n) {
  if (n <= bytes && ptr) return;
  release();
  const size_t want = grown(n);
  cuda_check(cudaMallocHost(&ptr, want), "cudaMallocHost");
  bytes = want;
}
void HostBuf::release() {
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  bytes = 0;
}

// ------------------------------------------------------------------ device guard --------------
struct DeviceInfo {
  int32_t status = RG_OK;
  std::string message, name, arch;
  int sm_count = 0;
  int count = 0;
};

static const DeviceInfo& device_info() {
  static std::once_flag once;
  static DeviceInfo info;
  std::call_once(once, [] {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
      cudaGetLastError();
      info.status = RG_ERR_GPU_UNAVAILABLE;
      info.message = std::string("CUDA device 0: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "no device");
      return;
    }
    info.count = count;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
      cudaGetLastError();
      info.status = RG_ERR_GPU_UNAVAILABLE;
      info.message = "CUDA device 0: properties unavailable";
      return;
    }
    info.name = p.name;
    info.arch = "sm_" + std::to_string(p.major) + std::to_string(p.minor);
    info.sm_count = p.multiProcessorCount;
    if (!(p.major == 10 && p.minor == 3)) {
      info.status = RG_ERR_GPU_UNAVAILABLE;
      info.message = "the library holds sm_103a code only; device 0 is " + info.arch;
    }
  });
  return info;
}

}  // namespace rg

using namespace rg;

int32_t rg_guard_device() {
  const DeviceInfo& d = device_info();
  if (d.status) set_last_error(d.message);
  return d.status;
}


static const char* const kCodes[] = {
    "ok", "missing_as_of", "as_of_mismatch", "invalid_paths", "invalid_schedule",
    "invalid_market_shape", "invalid_market", "invalid_trade", "invalid_local_vol", "shape_mismatch",
    "gpu_unavailable", "gpu_error", "no_crn_rejected", "invalid_spot_bump", "invalid_volatility_bump",
    "invalid_rate_bump", "invalid_correlation_bump", "risk_input_shape", "risk_paths_required",
    "path_out_of_range", "invalid_argument", "unsupported", "invalid_percentile", "cancelled",
    "device_timeout"};

extern "C" const char* rg_status_code(int32_t status) {
  if (status < 0 || status >= (int32_t)(sizeof kCodes / sizeof kCodes[0])) return "unknown";
  return kCodes[status];
}

extern "C" int32_t rg_last_error(char* buf, size_t len) {
  const std::string& m = g_last_error;
  if (buf && len) {
    size_t n = m.size() < len - 1 ? m.size() : len - 1;
    memcpy(buf, m.data(), n);
    buf[n] = 0;
  }
  return (int32_t)m.size();
}

extern "C" int32_t rg_abi_version(void) { return RG_ABI_VERSION; }

static int32_t copy_str(const std::string& s, char* buf, size_t len) {
  if (!buf || !len) return RG_ERR_INVALID_ARGUMENT;
  size_t n = s.size() < len - 1 ? s.size() : len - 1;
  memcpy(buf, s.data(), n);
  buf[n] = 0;
  return RG_OK;
}

extern "C" int32_t rg_ensure_available(void) { return rg_guard_device(); }

extern "C" int32_t rg_device_name(char* buf, size_t len) {
  int32_t g = rg_guard_device();
  if (g) return g;
  return copy_str(device_info().name, buf, len);
}

extern "C" int32_t rg_arch(char* buf, size_t len) {
  int32_t g = rg_guard_device();
  if (g) return g;
  return copy_str(device_info().arch, buf, len);
}

// ------------------------------------------------------------------ engine --------------------

extern "C" int32_t rg_engine_create(int32_t device, rg_engine** out) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    int32_t g = rg_guard_device();
    if (g) raise(g, device_info().message);
    if (device < 0 || device >= device_info().count)
      raise(RG_ERR_INVALID_ARGUMENT, "device index out of range");
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    std::unique_ptr<rg_engine> e(new rg_engine());
    e->device = device;
    cuda_check(cudaStreamCreateWithFlags(&e->stream_lo, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaStreamCreateWithFlags(&e->gen_stream_lo, cudaStreamNonBlocking), "cudaStreamCreate");
    int least = 0, greatest = 0;
    cuda_check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    cuda_check(cudaStreamCreateWithPriority(&e->stream_hi, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    cuda_check(cudaStreamCreateWithPriority(&e->gen_stream_hi, cudaStreamNonBlocking, greatest), "cudaStreamCreate");
    e->stream = e->stream_lo;
    e->gen_stream = e->gen_stream_lo;
    for (cudaEvent_t& ev : e->ev) cuda_check(cudaEventCreate(&ev), "cudaEventCreate");
    for (cudaEvent_t& ev : e->book_ev)
      cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    *out = e.release();
  })
}

extern "C" void rg_engine_destroy(rg_engine* e) {
  if (!e) return;
  for (cudaStream_t s : {e->stream_lo, e->gen_stream_lo, e->stream_hi, e->gen_stream_hi})
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  for (cudaEvent_t ev : e->ev)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : e->book_ev)
    if (ev) cudaEventDestroy(ev);
  delete e;
}

namespace rg {

// Builds the device tables of a prepared request into the engine arena.
struct Staged {
  DevTables tb{};
  DevScenario* scen = nullptr;
  DevScen32* scen32 = nullptr;
};

// Every input of one surface's calibration, as bytes: the cache key of a resident surface.
static std::vector<uint8_t> surface_key_bytes(const rg_implied_vol_grid& g, const SurfaceKey& k, int gx) {
  std::vector<uint8_t> b;
  auto put = [&b](const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  };
  const int32_t dims[3] = {g.n_maturities, g.n_strikes, gx};
  const double mkt[3] = {k.spot, k.rate, k.shift};
  put(dims, sizeof dims);
  put(mkt, sizeof mkt);
  put(g.maturities_years, sizeof(double) * (size_t)g.n_maturities);
  put(g.strikes, sizeof(double) * (size_t)g.n_strikes);
  put(g.vols, sizeof(double) * (size_t)g.n_maturities * (size_t)g.n_strikes);
  return b;
}

double* SurfaceCache::lookup(const std::vector<uint8_t>& key, size_t bytes, bool& hit) {
  ++tick;
  hit = false;
  int victim = -1;
  for (int i = 0; i < kEntries; ++i) {
    Entry& e = entries[i];
    if (e.ready && e.key == key && e.buf.bytes >= bytes) {
      e.used = tick;
      hit = true;
      in_use.push_back(i);
      return static_cast<double*>(e.buf.ptr);
    }
    // an entry this call reads or fills is not available: one launch serves all of them
    if (std::find(in_use.begin(), in_use.end(), i) != in_use.end()) continue;
    if (victim < 0 || e.used < entries[victim].used) victim = i;
  }
  if (victim < 0) return nullptr;  // more surfaces in one call than entries: calibrate only
  // not resident: the least recently used entry takes this surface once the call completes
  Entry& e = entries[victim];
  e.ready = false;
  e.key = key;
  e.used = tick;
  e.buf.ensure(bytes);
  in_use.push_back(victim);
  pending.push_back(victim);
  return static_cast<double*>(e.buf.ptr);
}

void SurfaceCache::begin_call() {
  pending.clear();
  in_use.clear();
}

void SurfaceCache::commit() {
  for (int i : pending) entries[i].ready = true;
  pending.clear();
  in_use.clear();
}

size_t SurfaceCache::device_bytes() const {
  size_t b = 0;
  for (const Entry& e : entries) b += e.buf.bytes;
  return b;
}

void SurfaceCache::release() {
  for (Entry& e : entries) {
    e.buf.release();
    e.key.clear();
    e.ready = false;
    e.used = 0;
  }
  pending.clear();
  in_use.clear();
}

static Staged stage(Workspace& W, const rg_price_request* req, Prepared& P) {
  Pack pk;
  const DevTrade& tr = P.trade;
  // QMC tables
  size_t o_sobol = 0, o_hb = 0, o_ho = 0, o_hp = 0;
  std::vector<uint32_t> hb, ho, hp;
  if (tr.vr == RG_VR_SOBOL) {
    const std::vector<uint32_t>& v = sobol_table(tr.sob_dim);
    o_sobol = pk.add(v);
  } else if (tr.vr == RG_VR_HALTON && tr.hal_hash) {
    o_hb = pk.add(first_primes(tr.hal_dim).data(), (size_t)tr.hal_dim);  // no permutation tables
    o_ho = o_hp = o_hb;
  } else if (tr.vr == RG_VR_HALTON) {
    halton_tables(tr.hal_dim, tr.seed, hb, ho, hp);
    o_hb = pk.add(hb);
    o_ho = pk.add(ho);
    o_hp = pk.add(hp);
  }
  size_t o_flags = pk.add(P.step_flags), o_per = pk.add(P.step_period), o_acc = pk.add(P.accr_inc);
  size_t o_noff = pk.add(P.node_off), o_nk = pk.add(P.node_k), o_nc = pk.add(P.node_c),
         o_ncf = pk.add(P.node_cf), o_nfr = pk.add(P.nf_row), o_nfs = pk.add(P.nf_shift);
  size_t o_ti = pk.add(P.lv_ti), o_tw = pk.add(P.lv_tw), o_twf = pk.add(P.lv_twf);
  size_t o_df = pk.add(P.df), o_dfm = pk.add(P.df_mat);
  size_t o_acf = pk.add(P.accr_f), o_dff = pk.add(P.df_f), o_dfmf = pk.add(P.df_mat_f);
  // the FP32 tiled kernel's bridge plans, one per tile depth it may launch with
  std::shared_ptr<const BridgePlans> bp;
  size_t o_bplan = 0;
  if (req->config.precision == RG_PRECISION_FP32) {
    bp = p32_bridge_plans(P);
    o_bplan = pk.add(bp->words);
  }
  // the FP32 kernels' consumption-order Sobol tables (1.1 MB per 1,000 steps of 3 assets), for
  // launches long enough that generating from them pays for their upload
  size_t o_sobt = 0, o_slut = 0;
  int32_t lut_o = -1;
  if (req->config.precision == RG_PRECISION_FP32 && tr.vr == RG_VR_SOBOL && req->config.paths >= (uint64_t(1) << 16)) {
    lut_o = (int32_t)((req->config.first_path + 1) & 31);
    std::shared_ptr<const SobolLut> t =
        sobol_lut_tables(P, tr.sob_dim, (uint32_t)lut_o, tr.scrambler == RG_SCRAMBLE_DIGITAL_SHIFT);
    o_sobt = pk.add(t->st);
    o_slut = pk.add(t->lut);
  }
  size_t o_scen = pk.add(P.scen), o_s32 = pk.add(P.scen32);
  // local-vol surfaces: inputs (grids) and outputs
  const int gx = tr.gx;
  size_t o_lv = 0, o_lvf = 0, o_logs = 0, o_jobs = 0, o_celloff = 0, o_sasset = 0;
  std::vector<size_t> o_mats, o_ks, o_vs, o_ax;
  size_t cells = 0, scratch = 0;
  std::vector<CalibJob> jobs;
  if (tr.has_lv) {
    for (int j = 0; j < P.n_surf; ++j) cells += (size_t)P.surf_nt[j] * gx;
    o_lv = pk.reserve(cells * sizeof(double));
    o_lvf = pk.reserve(cells * sizeof(float2));
    o_logs = pk.reserve((size_t)P.n_surf * gx * sizeof(double));
    for (int f = 0; f < P.n; ++f) {
      const rg_implied_vol_grid& g = req->local_vol[f];
      o_mats.push_back(pk.add(g.maturities_years, (size_t)g.n_maturities));
      o_ks.push_back(pk.add(g.strikes, (size_t)g.n_strikes));
      o_vs.push_back(pk.add(g.vols, (size_t)g.n_maturities * g.n_strikes));
    }
    for (int j = 0; j < P.n_surf; ++j) {
      const rg_implied_vol_grid& g = req->local_vol[P.surfaces[j].asset];
      scratch += (size_t)4 * g.n_maturities * gx + gx + (size_t)6 * g.n_maturities * g.n_strikes;
    }
    jobs.resize(P.n_surf);
    o_jobs = pk.reserve(sizeof(CalibJob) * (size_t)P.n_surf);
    std::vector<int32_t> cell_off(P.n_surf), sasset(P.n_surf);
    int32_t co = 0;
    for (int j = 0; j < P.n_surf; ++j) {
      cell_off[j] = co;
      co += P.surf_nt[j] * gx;
      sasset[j] = P.surfaces[j].asset;
    }
    o_celloff = pk.add(cell_off);
    o_sasset = pk.add(sasset);
    // the calibration's host-libm logarithms, once per (asset, spot, rate): vol bumps share them
    o_ax.resize(P.n_surf);
    for (int j = 0; j < P.n_surf; ++j) {
      const SurfaceKey& key = P.surfaces[j];
      int same = -1;
      for (int i = 0; i < j && same < 0; ++i)
        if (P.surfaces[i].asset == key.asset && P.surfaces[i].spot == key.spot && P.surfaces[i].rate == key.rate)
          same = i;
      o_ax[j] = same >= 0 ? o_ax[same] : pk.add(calib_axes(req->local_vol[key.asset], key.spot, key.rate, gx));
    }
  }
  uint8_t* base = static_cast<uint8_t*>(W.device(WS_ARENA, pk.host.size()));
  if (tr.has_lv) {
    if (SurfaceCache* cache = W.surfaces()) cache->begin_call();
    double* sc = static_cast<double*>(W.device(WS_CALIB, scratch * sizeof(double)));
    size_t cell_off = 0, sc_off = 0;
    for (int j = 0; j < P.n_surf; ++j) {
      const SurfaceKey& key = P.surfaces[j];
      const rg_implied_vol_grid& g = req->local_vol[key.asset];
      CalibJob& J = jobs[j];
      J.n_t = g.n_maturities;
      J.n_k = g.n_strikes;
      J.gx = gx;
      J.mats = reinterpret_cast<const double*>(base + o_mats[key.asset]);
      J.strikes = reinterpret_cast<const double*>(base + o_ks[key.asset]);
      J.vols = reinterpret_cast<const double*>(base + o_vs[key.asset]);
      J.spot = key.spot;
      J.rate = key.rate;
      J.shift = key.shift;
      J.out_v = reinterpret_cast<double*>(base + o_lv) + cell_off;
      J.out_vf = reinterpret_cast<float2*>(base + o_lvf) + cell_off;
      J.out_logs = reinterpret_cast<double*>(base + o_logs) + (size_t)j * gx;
      J.scratch = sc + sc_off;
      J.ax = reinterpret_cast<const double*>(base + o_ax[j]);
      J.cache_src = nullptr;
      J.cache_dst = nullptr;
      if (SurfaceCache* cache = W.surfaces()) {
        bool hit = false;
        double* e = cache->lookup(surface_key_bytes(g, key, gx), surface_entry_bytes(J.n_t, gx), hit);
        if (hit) J.cache_src = e;
        else J.cache_dst = e;
      }
      cell_off += (size_t)J.n_t * gx;
      sc_off += (size_t)4 * J.n_t * gx + gx + (size_t)6 * J.n_t * J.n_k;
    }
    memcpy(pk.host.data() + o_jobs, jobs.data(), sizeof(CalibJob) * jobs.size());
  }
  if (W.ev) cuda_check(cudaEventRecord(W.ev[0], W.stream), "event");
  cuda_check(cudaMemcpyAsync(base, pk.host.data(), pk.host.size(), cudaMemcpyHostToDevice, W.stream),
             "H2D request tables");
  if (W.ev) cuda_check(cudaEventRecord(W.ev[1], W.stream), "event");
  if (W.timing) W.timing->h2d_bytes += pk.host.size();
  Staged S;
  DevTables& tb = S.tb;
  tb.sobol = reinterpret_cast<const uint32_t*>(base + o_sobol);
  tb.hal_base = reinterpret_cast<const uint32_t*>(base + o_hb);
  tb.hal_off = reinterpret_cast<const uint32_t*>(base + o_ho);
  tb.hal_perm = reinterpret_cast<const uint32_t*>(base + o_hp);
  tb.step_flags = reinterpret_cast<const uint32_t*>(base + o_flags);
  tb.step_period = reinterpret_cast<const int32_t*>(base + o_per);
  tb.accr_inc = reinterpret_cast<const double*>(base + o_acc);
  tb.node_off = reinterpret_cast<const int32_t*>(base + o_noff);
  tb.node_k = reinterpret_cast<const int32_t*>(base + o_nk);
  tb.node_c = reinterpret_cast<const double*>(base + o_nc);
  tb.node_cf = reinterpret_cast<const float*>(base + o_ncf);
  tb.nf_row = reinterpret_cast<const int32_t*>(base + o_nfr);
  tb.nf_shift = reinterpret_cast<const uint32_t*>(base + o_nfs);
  tb.lv_ti = reinterpret_cast<const int2*>(base + o_ti);
  tb.lv_tw = reinterpret_cast<const double*>(base + o_tw);
  tb.lv_twf = reinterpret_cast<const float*>(base + o_twf);
  tb.lv_v = reinterpret_cast<const double*>(base + o_lv);
  tb.lv_vf = reinterpret_cast<const float2*>(base + o_lvf);
  tb.lv_logs = reinterpret_cast<const double*>(base + o_logs);
  tb.df = reinterpret_cast<const double*>(base + o_df);
  tb.df_mat = reinterpret_cast<const double*>(base + o_dfm);
  tb.accr_f = reinterpret_cast<const float*>(base + o_acf);
  tb.df_f = reinterpret_cast<const float*>(base + o_dff);
  tb.df_mat_f = reinterpret_cast<const float*>(base + o_dfmf);
  tb.bplan = reinterpret_cast<const uint32_t*>(base + o_bplan);
  tb.n_bplan = bp ? bp->n : 0;
  for (int i = 0; i < RG_BPLAN_MAX; ++i) {
    tb.bplan_tt[i] = i < tb.n_bplan ? bp->tt[i] : 0;
    tb.bplan_at[i] = i < tb.n_bplan ? bp->at[i] : 0;
  }
  tb.lv_nt = P.lv_nt_max;
  tb.sob_t = lut_o >= 0 ? reinterpret_cast<const uint32_t*>(base + o_sobt) : nullptr;
  tb.sob_lut = lut_o >= 0 ? reinterpret_cast<const uint32_t*>(base + o_slut) : nullptr;
  tb.sob_nq = (int32_t)(P.T * P.n);
  tb.sob_lut_o = lut_o;
  S.scen = reinterpret_cast<DevScenario*>(base + o_scen);
  S.scen32 = reinterpret_cast<DevScen32*>(base + o_s32);
  if (tr.has_lv) {
    launch_calibrate(reinterpret_cast<const CalibJob*>(base + o_jobs), P.n_surf, W.stream);
    if (W.timing) W.timing->kernel_launches += 1;
    if (req->config.precision == RG_PRECISION_FP32) {
      float2* rows = static_cast<float2*>(W.device(WS_LVROWS, (size_t)P.n_surf * P.T * gx * sizeof(float2)));
      launch_lvrows(tb.lv_v, reinterpret_cast<const int32_t*>(base + o_celloff),
                    reinterpret_cast<const int32_t*>(base + o_sasset), tb.lv_ti, tb.lv_tw, P.n_surf,
                    (int)P.T, gx, rows, W.stream);
      tb.lv_rows = rows;
      if (W.timing) W.timing->kernel_launches += 1;
    }
  }
  launch_cholesky(S.scen, S.scen32, P.n_scen, P.n, W.stream);
  if (W.timing) W.timing->kernel_launches += 1;
  if (W.ev) cuda_check(cudaEventRecord(W.ev[2], W.stream), "event");
  return S;
}

// PriceResult from the FP64 sums (note.rs:262-372); counts are exact in FP64.
void finish(const double* a, uint64_t paths, uint64_t seed, rg_price_result* out) {
  memset(out, 0, sizeof *out);
  const double P = (double)paths;
  auto var = [](double s1, double s2, double n) {
    return n > 1.0 ? (s2 - s1 * s1 / n) / (n - 1.0) : 0.0;
  };
  const double ko = a[ACC_NKO], ki = a[ACC_NKI], pe = a[ACC_NPUT], cp = a[ACC_NCPN];
  const double mean_put = a[ACC_PUT] / P, mean_funding = a[ACC_FUND] / P;
  const double mean_cq = a[ACC_CQ] / P, mean_mq = a[ACC_MQ] / P;
  const double total = mean_funding + (mean_cq + mean_mq) / 10.0 - mean_put;
  out->pv = total;
  out->mc_error = std::sqrt(var(a[ACC_PV], a[ACC_PV2], P) / P);
  out->ki_probability = ki / P;
  out->legs.coupon = mean_cq;
  out->legs.memory_coupon = mean_mq;
  out->legs.down_and_in_put = mean_put;
  out->legs.funding = mean_funding;
  out->legs.total = total;
  rg_transition_stats* s = out->stats;
  s[0].input_count = paths;
  s[0].output_count = (uint64_t)ko;
  s[0].probability = ko / P;
  s[0].mean_payoff = ko > 0 ? 1.0 + a[ACC_KOF] / ko : 0.0;
  s[0].variance_payoff = var(a[ACC_KOF], a[ACC_KOF2], ko);
  s[1].input_count = paths;
  s[1].output_count = (uint64_t)ki;
  s[1].probability = ki / P;
  s[1].mean_payoff = ki > 0 ? a[ACC_KIPUT] / ki : 0.0;
  s[1].variance_payoff = var(a[ACC_KIPUT], a[ACC_KIPUT2], ki);
  s[2].input_count = paths;
  s[2].output_count = (uint64_t)cp;
  s[2].probability = cp / P;
  s[2].mean_payoff = cp > 0 ? a[ACC_CPN] / cp : 0.0;
  s[2].variance_payoff = var(a[ACC_CPN], a[ACC_CPN2], cp);
  rg_ledger_entry* l = out->ledger;
  l[0].population_before = paths;
  l[0].population_after = (uint64_t)ko;
  l[0].pv_impact = mean_funding * (ko / P);
  l[1].population_before = paths - (uint64_t)ko;
  l[1].population_after = (uint64_t)pe;
  l[1].pv_impact = -mean_put;
  l[2].population_before = paths;
  l[2].population_after = (uint64_t)cp;
  l[2].pv_impact = (mean_cq + mean_mq) / 10.0;
  out->seed = seed;
  out->ko_count = (uint64_t)ko;
  out->ki_count = (uint64_t)ki;
  out->put_eligible_count = (uint64_t)pe;
  out->coupon_path_count = (uint64_t)cp;
  for (int k = 0; k < RG_ACC; ++k) out->path_sums[k] = a[k];
}

// First RG_TRACE_EVENT_CAP knocked-out paths in path order (note.rs:174-180), read back in
// growing chunks of the per-path KO steps.
static void collect_trace(Workspace& W, const int32_t* dev_ko, uint64_t paths, uint64_t first_path,
                          double dt, rg_price_result* out) {
  std::vector<int32_t> buf;
  uint64_t done = 0, chunk = 4096;
  while (done < paths && out->n_trace_events < RG_TRACE_EVENT_CAP) {
    uint64_t n = paths - done < chunk ? paths - done : chunk;
    buf.resize(n);
    cuda_check(cudaMemcpyAsync(buf.data(), dev_ko + done, n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               W.stream), "D2H ko steps");
    cuda_check(cudaStreamSynchronize(W.stream), "trace sync");
    for (uint64_t i = 0; i < n && out->n_trace_events < RG_TRACE_EVENT_CAP; ++i)
      if (buf[i] >= 0) {
        out->trace_events[out->n_trace_events].path_id = first_path + done + i;
        out->trace_events[out->n_trace_events].time = (double)(buf[i] + 1) * dt;
        out->n_trace_events++;
      }
    done += n;
    chunk *= 4;
  }
}

// The pseudo-random lane (VarianceReduction::None, note.rs:58,123-127): the slice of the ChaCha8
// normal stream that paths [first, first + count) of the request draw, generated on the device;
// null for the QMC lanes.  The lane always runs the FP64 kernel.
static const double* mc_lane_normals(Workspace& W, const rg_price_request* req, uint64_t first, uint64_t count) {
  if (req->config.variance_reduction != RG_VR_NONE) return nullptr;
  if (!W.persistent())
    raise(RG_ERR_UNSUPPORTED, "the pseudo-random lane needs an engine: its normal stream does not fit the static region");
  const uint64_t per_path = (uint64_t)req->trade.steps * (uint64_t)req->market.n_assets;
  const uint64_t n = count * per_path;
  if (n > (uint64_t(1) << 31))
    raise(RG_ERR_UNSUPPORTED, "the pseudo-random lane holds at most 2^31 normals per call (fewer paths or steps)");
  double* z = static_cast<double*>(W.device(WS_MCZ, n * sizeof(double)));
  mc_normals(req->config.seed, (req->config.first_path + first) * per_path, n, z, W);
  return z;
}

// Prices `n_scen` scenarios (0 = the request's own market) into out[max(1, n_scen)].
void price_with(Workspace& W, const rg_price_request* req, const rg_scenario* sc, int n_scen,
                rg_price_result* out) {
  validate_request(req);
  for (int i = 0; i < n_scen; ++i) {
    rg_price_request r2 = *req;
    r2.market = sc[i].market;
    r2.market.as_of = req->market.as_of;
    validate_request(&r2);
  }
  const int total = n_scen ? n_scen : 1;
  const double* mcz = mc_lane_normals(W, req, 0, req->config.paths);
  const bool fp32 = req->config.precision == RG_PRECISION_FP32 && !mcz;
  const int per_launch = fp32 ? 32 : 1;
  const uint64_t paths = req->config.paths;
  const bool trace = req->config.trace_level != RG_TRACE_OFF;
  if (W.timing) *W.timing = rg_timing{};
  for (int first = 0; first < total; first += per_launch) {
    const int cnt = total - first < per_launch ? total - first : per_launch;
    Prepared P;
    prepare(req, n_scen ? sc + first : nullptr, n_scen ? cnt : 0, P);
    W.begin_launch();
    Staged S = stage(W, req, P);
    LaunchOut lo{};
    lo.mcz = mcz;
    // rows of partial sums: one per block of the FP64 kernel, one per 32-path chunk of the FP32 kernels
    uint64_t rows;
    Fp32Shape sh{};
    if (fp32) {
      sh = phoenix32_shape(P, paths, W.sm_count);
      rows = p32_chunks(paths);
    } else {
      rows = (uint64_t)phoenix64_grid(P, paths);
    }
    if (rows > (uint64_t)INT32_MAX) raise(RG_ERR_INVALID_PATHS, "too many paths for one launch");
    const int grid = (int)rows;
    const size_t sums_bytes = (size_t)P.n_scen * RG_ACC * sizeof(double);
    lo.partial = static_cast<double*>(W.device(WS_PARTIAL, rows * P.n_scen * RG_ACC * sizeof(double)));
    double* dsums = static_cast<double*>(
        W.device(WS_SUMS, sums_bytes + reduce_scratch_doubles(grid, P.n_scen) * sizeof(double)));
    lo.grid = grid;
    if (trace) {
      // KO trace events are recorded for the first scenario of each fused launch
      lo.ko_steps = static_cast<int32_t*>(W.device(WS_KOSTEPS, paths * sizeof(int32_t)));
    }
    const uint64_t path0 = req->config.first_path;
    if (fp32) {
      sh = phoenix32_tune(P, S.tb, S.scen, S.scen32, path0, paths, sh, lo, W.may_tune(), W.sm_count, W.stream);
      launch_phoenix32(P, S.tb, S.scen, S.scen32, path0, paths, sh, lo, W.stream);
    } else {
      launch_phoenix64(P, S.tb, S.scen, path0, paths, lo, W.stream);
    }
    if (W.timing) {
      W.timing->block = fp32 ? sh.threads : 128;
      W.timing->smem_bytes = fp32 ? sh.smem : 0;
      W.timing->tile_steps = fp32 && !sh.direct ? sh.TT : 0;
      W.timing->paths_per_thread = fp32 && !sh.direct ? sh.ppt : 1;
      W.timing->grid = fp32 ? sh.grid : grid;
      W.timing->kernel_launches += 2;
      W.timing->d2h_bytes += sums_bytes;
    }
    if (W.ev) cuda_check(cudaEventRecord(W.ev[3], W.stream), "event");
    launch_reduce(lo.partial, grid, P.n_scen, dsums, W.stream);
    if (W.ev) cuda_check(cudaEventRecord(W.ev[4], W.stream), "event");
    double* hs = static_cast<double*>(W.host(sums_bytes));
    cuda_check(cudaMemcpyAsync(hs, dsums, sums_bytes, cudaMemcpyDeviceToHost, W.stream), "D2H sums");
    if (W.ev) cuda_check(cudaEventRecord(W.ev[5], W.stream), "event");
    cuda_check(cudaStreamSynchronize(W.stream), "pricing");
    if (SurfaceCache* cache = W.surfaces()) cache->commit();
    if (W.ev && W.timing) {
      float ms[5];
      for (int k = 0; k < 5; ++k) cuda_check(cudaEventElapsedTime(&ms[k], W.ev[k], W.ev[k + 1]), "event time");
      W.timing->h2d_ms += ms[0];
      W.timing->prologue_ms += ms[1];
      W.timing->kernel_ms += ms[2];
      W.timing->reduce_ms += ms[3];
      W.timing->d2h_ms += ms[4];
      W.timing->device_ms += ms[0] + ms[1] + ms[2] + ms[3] + ms[4];
    }
    if (fp32) {
      // the FP32 kernel poisons its sums with NaN when it was given too little shared memory
      for (size_t k = 0; k < (size_t)cnt * RG_ACC; ++k)
        if (!std::isfinite(hs[k])) raise(RG_ERR_GPU_ERROR, "phoenix32: non-finite path sums (launch shape check failed)");
    }
    for (int i = 0; i < cnt; ++i) finish(hs + (size_t)i * RG_ACC, paths, req->config.seed, &out[first + i]);
    if (trace) collect_trace(W, lo.ko_steps, paths, req->config.first_path, P.trade.dt, &out[first]);
  }
}

int device_sm_count() { return device_info().sm_count; }

int engine_sm_count(const rg_engine* E) {
  const int sms = device_info().sm_count;
  return E->sm_cap > 0 && E->sm_cap < sms ? E->sm_cap : sms;
}

void engine_set_class(rg_engine* E, bool high_priority, int sm_cap) {
  std::lock_guard<std::mutex> lock(E->mu);
  E->stream = high_priority ? E->stream_hi : E->stream_lo;
  E->gen_stream = high_priority ? E->gen_stream_hi : E->gen_stream_lo;
  E->sm_cap = sm_cap;
}

// The engine's workspace: growable device buffers, pinned host sums, timing events.
struct EngineWorkspace : Workspace {
  rg_engine* E;
  explicit EngineWorkspace(rg_engine* e) : E(e) {
    stream = e->stream;
    ev = e->ev;
    timing = &e->timing;
    sm_count = engine_sm_count(e);
  }
  void* device(int slot, size_t bytes) override {
    E->bufs[slot].ensure(bytes);
    return E->bufs[slot].ptr;
  }
  void* host(size_t bytes) override {
    E->host_sums.ensure(bytes);
    return E->host_sums.ptr;
  }
  SurfaceCache* surfaces() override { return &E->surfaces; }
};

size_t estimate_price_bytes(const rg_price_request* r, int n_scen) {
  const size_t S = n_scen > 0 ? (size_t)n_scen : 1;
  const size_t n = (size_t)(r->market.n_assets > 0 ? r->market.n_assets : 1);
  const size_t T = (size_t)(r->trade.steps > 0 ? r->trade.steps : 1);
  const bool fp32 = r->config.precision == RG_PRECISION_FP32;
  size_t sob_rows = r->config.dim_mode == RG_DIM_FULL ? n * T : 512;
  size_t b = sob_rows * 128 + n * T * 64 + S * T * 12 + S * 1024 + (size_t(64) << 10);  // tables
  if (r->n_local_vol) {
    const size_t gx = (size_t)(r->config.lv_grid_x > 0 ? r->config.lv_grid_x : 96);
    size_t nt = 1, nk = 1;
    for (int f = 0; f < r->n_local_vol; ++f) {
      nt = std::max(nt, (size_t)r->local_vol[f].n_maturities);
      nk = std::max(nk, (size_t)r->local_vol[f].n_strikes);
    }
    const size_t surf = S * n;
    b += surf * ((2 * nt * gx + gx) * 8 + (4 * nt * gx + gx + 6 * nt * nk) * 8);  // calibration
    if (fp32) b += surf * T * gx * 8;                                            // step rows
  }
  if (fp32) b += T * 160;  // bridge plans of the tiled kernel
  // rows of partial sums: one per 32-path chunk (FP32 kernels) or per block (FP64 kernel)
  const size_t grid = fp32 ? (size_t)p32_chunks(r->config.paths) : 152 * 16;
  b += grid * std::min<size_t>(S, 32) * RG_ACC * 8 + S * RG_ACC * 8;  // partial and reduced sums
  b += reduce_scratch_doubles((int)std::min<size_t>(grid, INT32_MAX), (int)std::min<size_t>(S, 32)) * 8;
  if (r->config.trace_level != RG_TRACE_OFF) b += (size_t)r->config.paths * 4;
  return b + b / 4 + (size_t(1) << 20);
}

size_t engine_device_bytes(rg_engine* E) {
  size_t b = 0;
  for (const DevBuf& d : E->bufs) b += d.bytes;
  for (const DevBuf& d : E->book_bufs) b += d.bytes;
  return b + E->surfaces.device_bytes();
}

void engine_trim(rg_engine* E) {
  std::lock_guard<std::mutex> lock(E->mu);
  cuda_check(cudaSetDevice(E->device), "cudaSetDevice");
  cuda_check(cudaStreamSynchronize(E->stream), "trim");
  cuda_check(cudaStreamSynchronize(E->gen_stream), "trim");
  for (DevBuf& d : E->bufs) d.release();
  for (DevBuf& d : E->book_bufs) d.release();
  E->surfaces.release();
  E->universe_key.clear();
  E->universe_ptr = nullptr;
}

static void price(rg_engine* E, const rg_price_request* req, const rg_scenario* sc, int n_scen,
                  rg_price_result* out) {
  std::lock_guard<std::mutex> lock(E->mu);
  cuda_check(cudaSetDevice(E->device), "cudaSetDevice");
  EngineWorkspace W(E);
  price_with(W, req, sc, n_scen, out);
}

}  // namespace rg

extern "C" int32_t rg_price_put_leg(rg_engine* e, const rg_price_request* req, rg_price_result* out) {
  RG_TRY({
    if (!e || !req || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    price(e, req, nullptr, 0, out);
  })
}

extern "C" int32_t rg_price_scenarios(rg_engine* e, const rg_price_request* req, const rg_scenario* sc,
                                      int32_t n, rg_price_result* out) {
  RG_TRY({
    if (!e || !req || !out || (n > 0 && !sc)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    if (n <= 0) raise(RG_ERR_INVALID_ARGUMENT, "at least one scenario is required");
    for (int i = 0; i < n; ++i)
      if (sc[i].market.n_assets != req->market.n_assets)
        raise(RG_ERR_INVALID_MARKET_SHAPE, "scenario asset count differs from the request's");
    price(e, req, sc, n, out);
  })
}

extern "C" int32_t rg_surfaces_upload(rg_engine* e, const rg_price_request* req, const rg_scenario* sc,
                                      int32_t n, int32_t* resident) {
  RG_TRY({
    if (!e || !req || (n > 0 && !sc) || n < 0) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    for (int i = 0; i < n; ++i) {
      if (sc[i].market.n_assets != req->market.n_assets)
        raise(RG_ERR_INVALID_MARKET_SHAPE, "scenario asset count differs from the request's");
      rg_price_request r2 = *req;
      r2.market = sc[i].market;
      r2.market.as_of = req->market.as_of;
      validate_request(&r2);
    }
    if (resident) *resident = 0;
    if (req->n_local_vol == 0) return RG_OK;
    std::lock_guard<std::mutex> lock(e->mu);
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    EngineWorkspace W(e);
    int total = 0;
    // the same staging as a pricing call (tables, calibration into the resident entries), no kernel
    for (int first = 0; first < (n > 0 ? n : 1); first += 32) {
      const int cnt = n > 0 ? std::min(32, n - first) : 0;
      Prepared P;
      prepare(req, n > 0 ? sc + first : nullptr, cnt, P);
      W.begin_launch();
      stage(W, req, P);
      cuda_check(cudaStreamSynchronize(e->stream), "surface upload");
      e->surfaces.commit();
      total += P.n_surf;
    }
    if (resident) *resident = total;
  })
}

namespace rg {
// validate_configuration, crates/riga-risk/src/lib.rs:338-457 (N-asset form).
static void validate_risk(const rg_price_request* r, const rg_central_difference_config* c) {
  if (c->random_number_policy == RG_NO_CRN)
    raise(RG_ERR_NO_CRN_REJECTED,
          "central finite differences require CommonRandomNumbers; independent streams are rejected");
  if (!std::isfinite(c->spot_relative_bump) || c->spot_relative_bump <= 0.0 || c->spot_relative_bump >= 1.0)
    raise(RG_ERR_INVALID_SPOT_BUMP, "spot_relative_bump must be finite, positive, and less than one");
  if (!std::isfinite(c->volatility_absolute_bump) || c->volatility_absolute_bump <= 0.0)
    raise(RG_ERR_INVALID_VOLATILITY_BUMP, "volatility_absolute_bump must be finite and positive");
  if (!std::isfinite(c->rate_absolute_bump) || c->rate_absolute_bump <= 0.0)
    raise(RG_ERR_INVALID_RATE_BUMP, "rate_absolute_bump must be finite and positive");
  if (!std::isfinite(c->correlation_absolute_bump) || c->correlation_absolute_bump <= 0.0)
    raise(RG_ERR_INVALID_CORRELATION_BUMP, "correlation_absolute_bump must be finite and positive");
  const int n = r->market.n_assets;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (i == j) continue;
      double rho = r->market.correlation[i * n + j];
      if (!std::isfinite(rho) || rho - c->correlation_absolute_bump <= -1.0 ||
          rho + c->correlation_absolute_bump >= 1.0)
        raise(RG_ERR_INVALID_CORRELATION_BUMP,
              "correlation up/down scenarios must remain strictly inside (-1, 1)");
    }
  for (int f = 0; f < n; ++f) {
    double s = r->market.spots[f], v = r->market.vols[f];
    if (!std::isfinite(s) || s <= 0.0) raise(RG_ERR_INVALID_SPOT_BUMP, "spot must be finite and positive");
    double h = s * c->spot_relative_bump;
    if (!std::isfinite(h) || h == 0.0 || s - h <= 0.0)
      raise(RG_ERR_INVALID_SPOT_BUMP, "spot bump is not representable and positive");
    if (!std::isfinite(v) || v < c->volatility_absolute_bump)
      raise(RG_ERR_INVALID_VOLATILITY_BUMP, "volatility must be finite and at least volatility_absolute_bump");
  }
  if (r->config.paths < 2)
    raise(RG_ERR_RISK_PATHS_REQUIRED, "at least two paths are required to report Monte Carlo risk uncertainty");
  for (int f = 0; f < r->n_local_vol; ++f) {
    const rg_implied_vol_grid& g = r->local_vol[f];
    for (int i = 0; i < g.n_maturities * g.n_strikes; ++i)
      if (!std::isfinite(g.vols[i]) || g.vols[i] < c->volatility_absolute_bump)
        raise(RG_ERR_INVALID_VOLATILITY_BUMP,
              "local-vol surface must align with assets and every implied-vol node must remain "
              "non-negative under the down bump");
  }
}
}  // namespace rg

// Scenario order: base, per asset {spot+, spot-, vol+, vol-}, rate+, rate-, corr+, corr-
// (crates/riga-risk/src/lib.rs:117-186, 573-626; scenario_count = 1 + 4n + 4).
extern "C" int32_t rg_price_risk_batch(rg_engine* e, const rg_price_request* req,
                                       const rg_central_difference_config* cfg,
                                       rg_batch_risk_report* out) {
  RG_TRY({
    if (!e || !req || !cfg || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    validate_risk(req, cfg);
    const int n = req->market.n_assets;
    const int ns = 1 + 4 * n + 4;
    std::vector<std::vector<double>> spots(ns), vols(ns), corr(ns), shift(ns);
    std::vector<rg_scenario> sc(ns);
    for (int s = 0; s < ns; ++s) {
      spots[s].assign(req->market.spots, req->market.spots + n);
      vols[s].assign(req->market.vols, req->market.vols + n);
      corr[s].assign(req->market.correlation, req->market.correlation + n * n);
      shift[s].assign(n, 0.0);
      sc[s].market = req->market;
    }
    for (int f = 0; f < n; ++f) {
      double h = req->market.spots[f] * cfg->spot_relative_bump;
      spots[1 + 4 * f][f] += h;
      spots[2 + 4 * f][f] -= h;
      vols[3 + 4 * f][f] += cfg->volatility_absolute_bump;
      vols[4 + 4 * f][f] += -cfg->volatility_absolute_bump;
      shift[3 + 4 * f][f] = cfg->volatility_absolute_bump;
      shift[4 + 4 * f][f] = -cfg->volatility_absolute_bump;
    }
    const int ir = 1 + 4 * n;
    sc[ir].market.risk_free_rate += cfg->rate_absolute_bump;
    sc[ir + 1].market.risk_free_rate += -cfg->rate_absolute_bump;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        if (i != j) {
          corr[ir + 2][i * n + j] += cfg->correlation_absolute_bump;
          corr[ir + 3][i * n + j] += -cfg->correlation_absolute_bump;
        }
    for (int s = 0; s < ns; ++s) {
      sc[s].market.spots = spots[s].data();
      sc[s].market.vols = vols[s].data();
      sc[s].market.correlation = corr[s].data();
      sc[s].implied_vol_shift = req->n_local_vol ? shift[s].data() : nullptr;
    }
    std::vector<rg_price_result> res(ns);
    price(e, req, sc.data(), ns, res.data());
    memset(out, 0, sizeof *out);
    out->base = res[0];
    out->scenario_count = (uint64_t)ns;
    out->seed = req->config.seed;
    out->n_assets = n;
    for (int f = 0; f < n; ++f) {
      const rg_price_result &su = res[1 + 4 * f], &sd = res[2 + 4 * f], &vu = res[3 + 4 * f], &vd = res[4 + 4 * f];
      const double h = req->market.spots[f] * cfg->spot_relative_bump, hv = cfg->volatility_absolute_bump;
      rg_asset_greeks& g = out->assets[f];
      g.asset_index = f;
      g.spot_bump = h;
      g.volatility_bump = hv;
      g.delta = {(su.pv - sd.pv) / (2.0 * h), (su.mc_error + sd.mc_error) / (2.0 * h)};
      g.gamma = {(su.pv - 2.0 * res[0].pv + sd.pv) / (h * h),
                 (su.mc_error + 2.0 * res[0].mc_error + sd.mc_error) / (h * h)};
      g.vega = {(vu.pv - vd.pv) / (2.0 * hv), (vu.mc_error + vd.mc_error) / (2.0 * hv)};
      g.spot_up_pv = su.pv;
      g.spot_down_pv = sd.pv;
      g.vol_up_pv = vu.pv;
      g.vol_down_pv = vd.pv;
      g.spot_up_mc_error = su.mc_error;
      g.spot_down_mc_error = sd.mc_error;
      g.vol_up_mc_error = vu.mc_error;
      g.vol_down_mc_error = vd.mc_error;
    }
    // transition_risk, crates/riga-risk/src/lib.rs:519-554
    for (int k = 0; k < RG_N_TRANSITIONS; ++k) {
      double d = 0.0, v = 0.0;
      for (int f = 0; f < n; ++f) {
        const double h = out->assets[f].spot_bump, hv = out->assets[f].volatility_bump;
        if (h > 0.0) d += (res[1 + 4 * f].ledger[k].pv_impact - res[2 + 4 * f].ledger[k].pv_impact) / (2.0 * h);
        if (hv > 0.0) v += (res[3 + 4 * f].ledger[k].pv_impact - res[4 + 4 * f].ledger[k].pv_impact) / (2.0 * hv);
      }
      out->transitions[k] = {res[0].ledger[k].pv_impact, d, v};
    }
    out->rate_up_pv = res[ir].pv;
    out->rate_down_pv = res[ir + 1].pv;
    out->correlation_up_pv = res[ir + 2].pv;
    out->correlation_down_pv = res[ir + 3].pv;
    out->rate_bump = cfg->rate_absolute_bump;
    out->correlation_bump = cfg->correlation_absolute_bump;
    out->pv_mc_error = res[0].mc_error;
  })
}

// One path range of the base scenario: records (FP32 or FP64 kernel per the request) or, when
// `cube` is non-null, the FP64 kernel's spot cube (and records) in chunks of at most 1 GiB of cube.
static void run_path_range(rg_engine* e, const rg_price_request* req, uint64_t first, uint64_t count,
                           rg_path_record* out, float* cube) {
  if (first > req->config.paths || count > req->config.paths - first)
    raise(RG_ERR_PATH_OUT_OF_RANGE, "path range is outside the configured path count");
  if (count == 0) return;
  std::lock_guard<std::mutex> lock(e->mu);
  cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
  Prepared P;
  prepare(req, nullptr, 0, P);
  EngineWorkspace W(e);
  Staged S = stage(W, req, P);
  const uint64_t cube_row = (uint64_t)P.trade.steps * (uint64_t)P.n;  // floats per path
  const uint64_t chunk_cap = cube ? std::max<uint64_t>(1, (uint64_t(1) << 28) / cube_row) : count;
  for (uint64_t done = 0; done < count;) {
    const uint64_t m = std::min(chunk_cap, count - done);
    const double* mcz = mc_lane_normals(W, req, first + done, m);
    const bool fp32 = req->config.precision == RG_PRECISION_FP32 && !mcz && !cube;
    LaunchOut lo{};
    lo.mcz = mcz;
    Fp32Shape sh{};
    if (fp32) sh = phoenix32_shape(P, m, engine_sm_count(e));
    lo.grid = fp32 ? (int)p32_chunks(m) : phoenix64_grid(P, m);
    lo.partial = static_cast<double*>(W.device(WS_PARTIAL, (size_t)lo.grid * P.n_scen * RG_ACC * sizeof(double)));
    if (out) lo.records = static_cast<rg_path_record*>(W.device(WS_RECORDS, m * sizeof(rg_path_record)));
    if (cube) lo.cube = static_cast<float*>(W.device(WS_CUBE, m * cube_row * sizeof(float)));
    const uint64_t path0 = req->config.first_path + first + done;
    if (fp32) {
      sh = phoenix32_tune(P, S.tb, S.scen, S.scen32, path0, m, sh, lo, false, engine_sm_count(e),
                          e->stream);  // cached shape only
      launch_phoenix32(P, S.tb, S.scen, S.scen32, path0, m, sh, lo, e->stream);
    }
    else
      launch_phoenix64(P, S.tb, S.scen, path0, m, lo, e->stream);
    if (out)
      cuda_check(cudaMemcpyAsync(out + done, lo.records, m * sizeof(rg_path_record), cudaMemcpyDeviceToHost,
                                 e->stream), "D2H records");
    if (cube)
      cuda_check(cudaMemcpyAsync(cube + done * cube_row, lo.cube, m * cube_row * sizeof(float),
                                 cudaMemcpyDeviceToHost, e->stream), "D2H cube");
    cuda_check(cudaStreamSynchronize(e->stream), "run_paths");
    e->surfaces.commit();
    done += m;
  }
}

extern "C" int32_t rg_run_paths(rg_engine* e, const rg_price_request* req, uint64_t first, uint64_t count,
                                rg_path_record* out) {
  RG_TRY({
    if (!e || !req || (count && !out)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    run_path_range(e, req, first, count, out, nullptr);
  })
}

extern "C" int32_t rg_materialize_paths(rg_engine* e, const rg_price_request* req, uint64_t first,
                                        uint64_t count, float* cube, rg_path_record* records) {
  RG_TRY({
    if (!e || !req || (count && !cube)) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    validate_request(req);
    run_path_range(e, req, first, count, records, cube);
  })
}

extern "C" int32_t rg_set_autotune(int32_t enabled) {
  RG_TRY({ p32_set_autotune(enabled != 0); })
}

extern "C" int32_t rg_set_tiled_shape(int32_t paths_per_thread, int32_t tile_steps, int32_t paths_per_block) {
  RG_TRY({ p32_force_shape(paths_per_thread, tile_steps, paths_per_block); })
}

extern "C" int32_t rg_phase_clocks(uint64_t out[4], int32_t reset) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    unsigned long long v[4];
    if (!p32_phase_clocks(v, reset != 0))
      raise(RG_ERR_UNSUPPORTED, "the library was built without phase clocks (build it with RG_PHASE_CLOCKS=1)");
    for (int k = 0; k < 4; ++k) out[k] = v[k];
  })
}

extern "C" int32_t rg_sobol_directions(int64_t dim, uint32_t* out) {
  RG_TRY({
    if (dim < 1 || dim > (int64_t(1) << 22) || !out) raise(RG_ERR_INVALID_ARGUMENT, "dim must be 1..2^22 and out non-null");
    const std::vector<uint32_t>& v = sobol_table(dim);
    memcpy(out, v.data(), v.size() * sizeof(uint32_t));
  })
}

extern "C" int32_t rg_bridge_schedule(int64_t steps, double dt, int32_t* node_off, int32_t* node_k,
                                      double* node_c, int32_t* stack_depth) {
  RG_TRY({
    if (steps < 1 || steps > (int64_t(1) << 22) || !(dt > 0.0) || !node_off || !node_k || !node_c)
      raise(RG_ERR_INVALID_ARGUMENT, "steps must be 1..2^22, dt positive, buffers non-null");
    Prepared P;
    bridge_schedule_into(steps, dt, P);
    memcpy(node_off, P.node_off.data(), P.node_off.size() * sizeof(int32_t));
    memcpy(node_k, P.node_k.data(), P.node_k.size() * sizeof(int32_t));
    memcpy(node_c, P.node_c.data(), P.node_c.size() * sizeof(double));
    if (stack_depth) *stack_depth = P.stack_max;
  })
}

extern "C" int32_t rg_merge_results(const rg_price_result* parts, int32_t n, uint64_t paths,
                                    rg_price_result* out) {
  RG_TRY({
    if (!parts || !out || n < 1) raise(RG_ERR_INVALID_ARGUMENT, "at least one part is required");
    if (paths == 0) raise(RG_ERR_INVALID_PATHS, "paths must be positive");
    double acc[RG_ACC] = {0};
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < RG_ACC; ++k) acc[k] += parts[i].path_sums[k];
    rg_price_result r;
    finish(acc, paths, parts[0].seed, &r);
    for (int i = 0; i < n && r.n_trace_events < RG_TRACE_EVENT_CAP; ++i)
      for (int j = 0; j < parts[i].n_trace_events && r.n_trace_events < RG_TRACE_EVENT_CAP; ++j)
        r.trace_events[r.n_trace_events++] = parts[i].trace_events[j];
    *out = r;
  })
}

extern "C" int32_t rg_engine_last_timing(rg_engine* e, rg_timing* out) {
  RG_TRY({
    if (!e || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lock(e->mu);
    *out = e->timing;
  })
}
