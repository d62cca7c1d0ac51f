// host_prep.cu — request validation and the host-built tables of one pricing request.
//
// Everything here is integer or FP64 work done once per request: the Sobol direction table,
// the Brownian-bridge node schedule, the Phoenix step schedule, the local-vol tenor schedule,
// discount factors and the per-scenario constants.  The heavy per-path work runs on the device.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rg_internal.h"

namespace rg {

static std::string fmt(const char* f, ...) __attribute__((format(printf, 1, 2)));
static std::string fmt(const char* f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}

// ------------------------------------------------------------------ validation ----------------
// crates/riga-engine/src/lib.rs:209-321 with the two-asset gate (:234-245) widened to
// 1..RG_MAX_ASSETS assets; error codes and messages follow the reference.
void validate_request(const rg_price_request* r) {
  if (!r) raise(RG_ERR_INVALID_ARGUMENT, "request is null");
  const rg_phoenix_trade& t = r->trade;
  const rg_market_snapshot& m = r->market;
  const rg_simulation_config& c = r->config;
  if (!r->as_of || !r->as_of[0]) raise(RG_ERR_MISSING_AS_OF, "as_of is required");
  if (!m.as_of || strcmp(r->as_of, m.as_of) != 0)
    raise(RG_ERR_AS_OF_MISMATCH, "request as_of must match the market snapshot as_of");
  if (c.paths == 0 || c.path_block_size == 0)
    raise(RG_ERR_INVALID_PATHS, "paths and path_block_size must be positive");
  if (t.steps <= 0 || !std::isfinite(t.maturity_years) || t.maturity_years <= 0.0)
    raise(RG_ERR_INVALID_SCHEDULE, "steps and maturity_years must be positive and finite");
  const int n = m.n_assets;
  if (n < 1 || n > RG_NMAX || t.n_assets != n || !m.spots || !m.vols || !m.dividend_yields ||
      !m.correlation || !t.initial_spots)
    raise(RG_ERR_INVALID_MARKET_SHAPE,
          fmt("the engine requires 1..%d assets with aligned trade and market arrays", RG_NMAX));
  for (int f = 0; f < n; ++f) {
    if (!std::isfinite(m.spots[f])) raise(RG_ERR_INVALID_MARKET, fmt("spot[%d] must be finite", f));
    if (!std::isfinite(m.vols[f])) raise(RG_ERR_INVALID_MARKET, fmt("vol[%d] must be finite", f));
  }
  if (!std::isfinite(m.risk_free_rate)) raise(RG_ERR_INVALID_MARKET, "risk_free_rate must be finite");
  for (int f = 0; f < n; ++f) {
    if (!std::isfinite(m.dividend_yields[f]))
      raise(RG_ERR_INVALID_MARKET, fmt("dividend_yield[%d] must be finite", f));
    if (!std::isfinite(t.initial_spots[f]))
      raise(RG_ERR_INVALID_MARKET, fmt("initial_spot[%d] must be finite", f));
  }
  for (int i = 0; i < n * n; ++i)
    if (!std::isfinite(m.correlation[i])) raise(RG_ERR_INVALID_MARKET, "rho must be finite");
  if (!std::isfinite(t.strike)) raise(RG_ERR_INVALID_MARKET, "strike must be finite");
  if (!std::isfinite(t.knock_in_barrier)) raise(RG_ERR_INVALID_MARKET, "KI barrier must be finite");
  bool bad = false;
  for (int f = 0; f < n; ++f)
    if (m.spots[f] <= 0.0 || t.initial_spots[f] <= 0.0 || m.vols[f] < 0.0) bad = true;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = m.correlation[i * n + j];
      if (i == j) {
        if (std::fabs(v - 1.0) > 1.0e-12) bad = true;
      } else if (std::fabs(v) > 1.0 || std::fabs(v - m.correlation[j * n + i]) > 1.0e-12) {
        bad = true;
      }
    }
  if (bad)
    raise(RG_ERR_INVALID_MARKET,
          "spots must be positive, vols non-negative, and correlation in [-1,1]");
  if (t.has_knock_out_barrier && (!std::isfinite(t.knock_out_barrier) || t.knock_out_barrier <= 0.0))
    raise(RG_ERR_INVALID_TRADE, "knock_out_barrier must be finite and positive when present");
  if (t.has_coupon_barrier && (!std::isfinite(t.coupon_barrier) || t.coupon_barrier <= 0.0))
    raise(RG_ERR_INVALID_TRADE, "coupon_barrier must be finite and positive when present");
  if (t.has_coupon_rate && (!std::isfinite(t.coupon_rate) || t.coupon_rate < 0.0))
    raise(RG_ERR_INVALID_TRADE, "coupon_rate must be finite and non-negative when present");
  if (t.strike <= 0.0 || t.knock_in_barrier <= 0.0)
    raise(RG_ERR_INVALID_TRADE, "strike must be positive and barriers finite");
  if (r->n_local_vol != 0 && (r->n_local_vol != n || !r->local_vol))
    raise(RG_ERR_INVALID_LOCAL_VOL, "local_vol.grids must be aligned with market.spots");
  if (c.variance_reduction < RG_VR_NONE || c.variance_reduction > RG_VR_SOBOL)
    raise(RG_ERR_INVALID_ARGUMENT, fmt("unknown variance_reduction %d", c.variance_reduction));
  if (c.scrambler < RG_SCRAMBLE_OWEN || c.scrambler > RG_SCRAMBLE_DIGITAL_SHIFT)
    raise(RG_ERR_INVALID_ARGUMENT, fmt("unknown scrambler %d", c.scrambler));
  if (c.precision < RG_PRECISION_FP64_PARITY || c.precision > RG_PRECISION_FP32)
    raise(RG_ERR_INVALID_ARGUMENT, fmt("unknown precision %d", c.precision));
  if (c.dim_mode < RG_DIM_WRAP_REFERENCE || c.dim_mode > RG_DIM_FULL)
    raise(RG_ERR_INVALID_ARGUMENT, fmt("unknown dim_mode %d", c.dim_mode));
  if (c.lv_grid_x < 0 || c.lv_grid_x == 1 || c.lv_grid_x > 4096)
    raise(RG_ERR_INVALID_ARGUMENT, "lv_grid_x must be 0 or 2..4096");
  if (t.steps > (int64_t(1) << 22)) raise(RG_ERR_INVALID_SCHEDULE, "at most 2^22 steps are supported");
  // Sobol points are 32-bit: every point index first_path + i + 1 (and the up to 7 extra points a
  // generation run computes past the last path) must stay below 2^32.
  if (c.paths >= (uint64_t(1) << 32) - 16 || c.first_path >= (uint64_t(1) << 32) - 16 - c.paths)
    raise(RG_ERR_INVALID_PATHS, "first_path + paths must stay below 2^32 - 16 (32-bit Sobol points)");
  // implied-vol grid shape (ImpliedVolGrid::validate, riga-market/src/lib.rs:94-111)
  for (int f = 0; f < r->n_local_vol; ++f) {
    const rg_implied_vol_grid& g = r->local_vol[f];
    if (g.n_maturities <= 0 || g.n_strikes <= 0 || !g.maturities_years || !g.strikes || !g.vols)
      raise(RG_ERR_INVALID_LOCAL_VOL, "implied vol grid has an empty axis");
    for (int i = 0; i + 1 < g.n_maturities; ++i)
      if (!(g.maturities_years[i] < g.maturities_years[i + 1]))
        raise(RG_ERR_INVALID_LOCAL_VOL, "implied vol maturities must be strictly increasing");
    for (int i = 0; i + 1 < g.n_strikes; ++i)
      if (!(g.strikes[i] < g.strikes[i + 1]))
        raise(RG_ERR_INVALID_LOCAL_VOL, "implied vol strikes must be strictly increasing");
  }
  // CorrelationMatrix::validate (riga-market/src/correlation.rs:74-93) is implied by the checks
  // above (they are tighter: 1e-12 against its 1e-9).
}

// ------------------------------------------------------------------ Sobol tables -------------
// Primitive GF(2) polynomials of degree >= 2 in (degree, value) order and the Joe–Kuo
// recurrence with unit initial direction numbers (crates/riga-engine/src/qmc.rs:247-262,
// 316-430).
static int top_bit(uint32_t v) { return 31 - __builtin_clz(v); }

static uint32_t gf2_mulmod(uint32_t a, uint32_t b, uint32_t poly) {
  const int deg = top_bit(poly);
  uint64_t r = 0, x = a;
  for (uint32_t y = b; y; y >>= 1, x <<= 1)
    if (y & 1u) r ^= x;
  for (int bit = 63; bit >= deg; --bit)
    if ((r >> bit) & 1u) r ^= uint64_t(poly) << (bit - deg);
  return uint32_t(r);
}

static uint32_t gf2_pow_x(uint64_t e, uint32_t poly) {
  uint32_t acc = 1, base = 2;
  for (; e; e >>= 1) {
    if (e & 1u) acc = gf2_mulmod(acc, base, poly);
    base = gf2_mulmod(base, base, poly);
  }
  return acc;
}

// x has multiplicative order exactly 2^deg - 1 modulo `poly`.
static bool primitive(uint32_t poly, int deg) {
  const uint64_t order = (uint64_t(1) << deg) - 1;
  if (gf2_pow_x(order, poly) != 1) return false;
  uint64_t rest = order;
  for (uint64_t p = 2; p * p <= rest; ++p) {
    if (rest % p) continue;
    if (gf2_pow_x(order / p, poly) == 1) return false;
    while (rest % p == 0) rest /= p;
  }
  return rest == 1 || gf2_pow_x(order / rest, poly) != 1;
}

static void directions(uint32_t poly, uint32_t* out32) {
  const int s = top_bit(poly);
  uint32_t m[33] = {0};
  for (int i = 1; i <= s; ++i) m[i] = 1;
  for (int k = s + 1; k <= 32; ++k) {
    uint32_t v = (m[k - s] << s) ^ m[k - s];
    for (int i = 1; i < s; ++i)
      if ((poly >> (s - i)) & 1u) v ^= m[k - i] << i;
    m[k] = v;
  }
  for (int k = 0; k < 32; ++k) out32[k] = m[k + 1] << (31 - k);
}

const std::vector<uint32_t>& sobol_table(int64_t dim) {
  static std::mutex mu;
  static std::vector<uint32_t> polys;     // primitive polynomials found so far
  static int next_degree = 2;
  static uint32_t next_poly = 0;
  static std::map<int64_t, std::vector<uint32_t>> cache;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(dim);
  if (it != cache.end()) return it->second;
  while ((int64_t)polys.size() < dim - 1) {
    if (next_poly == 0) next_poly = (1u << next_degree) | 1u;
    if (next_poly >= (1u << (next_degree + 1))) {
      ++next_degree;
      if (next_degree > 30) raise(RG_ERR_INVALID_ARGUMENT, "Sobol dimension too large");
      next_poly = (1u << next_degree) | 1u;
      continue;
    }
    if (primitive(next_poly, next_degree)) polys.push_back(next_poly);
    next_poly += 2;
  }
  std::vector<uint32_t> v(size_t(32) * size_t(dim));
  for (int k = 0; k < 32; ++k) v[k] = 1u << (31 - k);
  for (int64_t d = 1; d < dim; ++d) directions(polys[d - 1], &v[32 * d]);
  return cache.emplace(dim, std::move(v)).first->second;
}

// The FP32 kernels' Sobol tables (phoenix32.cu, phoenix32d.cu), in consumption order
// q = node·n + factor with row(q) = nf_row[q]: st[k][q] = v[row(q)][k], and lut[q][j] for the lane
// j whose point is n1 + j, n1 = a + o with a a multiple of 32.  Gray codes are linear over XOR, so
// for o + j < 32 x(n1 + j) = X(gray(a)) ^ X(gray(o + j)), and otherwise
// x = X(gray(a + 32)) ^ X(gray(o + j - 32)) with X(gray(a + 32)) = X(gray(a)) ^ v[4] ^
// v[ctz(a/32 + 1) + 5]; lut holds the lane's low-bit term X(gray((o + j) mod 32)) — with v[4] for
// the upper lanes and the digital shift folded in — and the kernels add the 32-path group's
// high-bit terms.
std::shared_ptr<const SobolLut> sobol_lut_tables(const Prepared& P, int64_t sob_dim, uint32_t o, bool shift) {
  // nf_row depends on (directions, assets, steps) and nf_shift on the seed as well
  const std::vector<int64_t> key{sob_dim, P.n, P.T, (int64_t)P.trade.seed, shift ? 1 : 0, (int64_t)o};
  static std::mutex mu;
  static std::map<std::vector<int64_t>, std::shared_ptr<const SobolLut>> cache;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  const std::vector<uint32_t>& v = sobol_table(sob_dim);
  auto out = std::make_shared<SobolLut>();
  const size_t nq = (size_t)P.T * (size_t)P.n;
  out->st.assign(32 * nq, 0u);
  out->lut.assign(nq * 32, 0u);
  for (size_t q = 0; q < nq; ++q) {
    const uint32_t* row = v.data() + 32 * (size_t)P.nf_row[q];
    for (int k = 0; k < 32; ++k) out->st[(size_t)k * nq + q] = row[k];
    for (uint32_t j = 0; j < 32; ++j) {
      const uint32_t jj = (o + j) & 31u, g = jj ^ (jj >> 1);
      uint32_t x = 0;
      for (int k = 0; k < 5; ++k)
        if ((g >> k) & 1u) x ^= row[k];
      if (o + j >= 32u) x ^= row[4];
      if (shift) x ^= P.nf_shift[q];
      out->lut[q * 32 + j] = x;
    }
  }
  std::lock_guard<std::mutex> lock(mu);
  if (cache.size() >= 32) cache.clear();  // bounded: one entry per launch shape in use
  cache[key] = out;
  return out;
}

// ------------------------------------------------------------------ Halton tables ------------
// First primes and their seeded Fisher–Yates digit permutations (qmc.rs:12-22, 128-140).
std::vector<uint32_t> first_primes(int count) {
  static std::mutex mu;
  static std::vector<uint32_t> primes;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)primes.size() < count) {
    // sieve of Eratosthenes past the count-th prime (p_n < n (ln n + ln ln n) for n >= 6)
    const double x = std::max(count, 6);
    const size_t lim = (size_t)(x * (std::log(x) + std::log(std::log(x)))) + 16;
    std::vector<char> comp(lim + 1, 0);
    primes.clear();
    for (size_t i = 2; i <= lim && (int)primes.size() < count; ++i) {
      if (comp[i]) continue;
      primes.push_back((uint32_t)i);
      for (size_t k = i * i; k <= lim; k += i) comp[k] = 1;
    }
  }
  return primes;
}

void halton_tables(int dim, uint64_t seed, std::vector<uint32_t>& base, std::vector<uint32_t>& off,
                   std::vector<uint32_t>& perm) {
  base.clear();
  off.clear();
  perm.clear();
  for (uint32_t c = 2; (int)base.size() < dim; ++c) {
    bool is_prime = true;
    for (uint32_t p : base)
      if (c % p == 0) { is_prime = false; break; }
    if (is_prime) base.push_back(c);
  }
  for (uint32_t b : base) {
    off.push_back((uint32_t)perm.size());
    size_t o = perm.size();
    for (uint32_t i = 0; i < b; ++i) perm.push_back(i);
    uint64_t state = seed ^ (uint64_t(b) * 0x9E3779B97F4A7C15ULL);
    for (uint32_t i = b - 1; i >= 1; --i) {
      state = state * 6364136223846793005ULL + 1442695040888963407ULL;
      uint64_t j = (state >> 33) % (uint64_t(i) + 1);
      std::swap(perm[o + i], perm[o + j]);
    }
  }
}

// ------------------------------------------------------------------ request preparation ------
// The in-order traversal of the reference's depth-first bridge (qmc.rs:155-191): the node
// consumed at each step, its preorder index (the QMC step whose normals it reads) and its
// conditional standard deviation.  Node 0 is the terminal point.
// The logarithms and exponentials of DupireLocalVol::calibrate (riga-market/src/lib.rs:217-245),
// in its order of operations, with the platform libm (the functions f64::ln / f64::exp call):
// [log-strike axis, gx][log(K_j / F_k), n_t * n_k][log(S_i / F_k) before clamping, n_t * gx] for
// F_k = spot * exp(rate * T_k) and S_i = exp(axis_i).  The device calibration reads them
// (CalibJob::ax); they do not depend on the implied vols or their bump.
std::vector<double> calib_axes(const rg_implied_vol_grid& g, double spot, double rate, int gx) {
  const int nt = g.n_maturities, nk = g.n_strikes;
  std::vector<double> ax((size_t)gx + (size_t)nt * nk + (size_t)nt * gx);
  double* logs = ax.data();
  double* xj = logs + gx;
  double* xd = xj + (size_t)nt * nk;
  const double s_min = g.strikes[0] * 0.55, s_max = g.strikes[nk - 1] * 1.05;
  const double log_lo = std::log(std::max(s_min, 1e-6)), log_hi = std::log(std::max(s_max, 1e-6));
  std::vector<double> s_axis(gx);
  for (int i = 0; i < gx; ++i) {
    logs[i] = log_lo + (log_hi - log_lo) * (double)i / (double)(gx - 1);
    s_axis[i] = std::exp(logs[i]);
  }
  for (int k = 0; k < nt; ++k) {
    const double forward = spot * std::exp(rate * g.maturities_years[k]);
    for (int j = 0; j < nk; ++j) xj[(size_t)k * nk + j] = std::log(g.strikes[j] / forward);
    for (int i = 0; i < gx; ++i) xd[(size_t)k * gx + i] = std::log(s_axis[i] / forward);
  }
  return ax;
}

void bridge_schedule_into(int64_t T, double dt, Prepared& P) {
  std::vector<int32_t> pre(size_t(T) + 1, -1);
  // preorder numbering of the bisection midpoints (index 0 is the terminal point)
  struct Frame { int64_t lo, hi; };
  std::vector<Frame> st;
  st.push_back({0, T});
  int32_t idx = 1;
  while (!st.empty()) {
    Frame fr = st.back();
    st.pop_back();
    if (fr.hi <= fr.lo + 1) continue;
    int64_t mid = (fr.lo + fr.hi) / 2;
    pre[mid] = idx++;
    st.push_back({mid, fr.hi});  // right after left (stack order)
    st.push_back({fr.lo, mid});
  }
  P.node_off.assign(size_t(T) + 1, 0);
  P.node_k.clear();
  P.node_c.clear();
  P.node_k.push_back(0);
  P.node_c.push_back(std::sqrt((double)T * dt));
  std::vector<int64_t> anchors{T};
  int64_t cur = 0;
  int depth_max = 1;
  for (int64_t t = 0; t < T; ++t) {
    P.node_off[t] = t == 0 ? 0 : (int32_t)P.node_k.size();
    while (anchors.back() > cur + 1) {
      int64_t hi = anchors.back(), m = (cur + hi) / 2;
      double variance = (double)(hi - m) * (double)(m - cur) / (double)(hi - cur) * dt;
      P.node_k.push_back(pre[m]);
      P.node_c.push_back(std::sqrt(variance));
      anchors.push_back(m);
      depth_max = std::max(depth_max, (int)anchors.size());
    }
    anchors.pop_back();
    cur += 1;
  }
  P.node_off[T] = (int32_t)P.node_k.size();
  P.stack_max = depth_max;
  if (depth_max > RG_STACK_MAX) raise(RG_ERR_INVALID_SCHEDULE, "Brownian-bridge depth too large");
  P.node_cf.assign(P.node_c.begin(), P.node_c.end());
}

void prepare(const rg_price_request* r, const rg_scenario* sc, int n_scen, Prepared& P) {
  const rg_phoenix_trade& t = r->trade;
  const rg_simulation_config& c = r->config;
  const int n = r->market.n_assets;
  const int64_t T = t.steps;
  P = Prepared();
  P.n = n;
  P.T = T;
  DevTrade& tr = P.trade;
  tr.n = n;
  tr.vr = c.variance_reduction;
  tr.scrambler = c.scrambler;
  tr.has_lv = r->n_local_vol ? 1 : 0;
  tr.steps = T;
  tr.periods = t.has_coupon_periods ? t.coupon_periods : 9;  // note.rs:43
  if (tr.periods < 1) tr.periods = 1;
  const int64_t call_start = t.has_call_start_step ? t.call_start_step : 0;  // note.rs:44
  tr.seed = c.seed;
  tr.dt = t.maturity_years / (double)T;  // note.rs:45
  tr.sqrt_dt = std::sqrt(tr.dt);
  tr.inv_sqrt_dt = 1.0 / std::sqrt(tr.dt);
  tr.maturity = t.maturity_years;
  for (int f = 0; f < n; ++f) tr.init[f] = t.initial_spots[f];
  tr.call_barrier = t.has_knock_out_barrier ? t.knock_out_barrier : INFINITY;  // note.rs:51-53
  tr.coupon_barrier = t.has_coupon_barrier ? t.coupon_barrier : INFINITY;
  tr.coupon_rate = t.has_coupon_rate ? t.coupon_rate : 0.0;
  tr.strike = t.strike;
  tr.ki = t.knock_in_barrier;
  tr.coupon_f = (float)tr.coupon_rate;
  tr.strike_f = (float)tr.strike;
  tr.neg_half_dt_f = (float)(-0.5 * tr.dt);
  tr.memory = t.memory_coupon ? 1 : 0;
  tr.gx = c.lv_grid_x > 0 ? c.lv_grid_x : 96;  // riga-market/src/lib.rs:28
  P.ln_ko = std::log(tr.call_barrier);
  P.ln_cb = std::log(tr.coupon_barrier);
  P.ln_ki = std::log(tr.ki);

  // QMC dimension: the reference clamps to [1, 512] and wraps (qmc.rs:9, 249, 271)
  if (tr.vr == RG_VR_SOBOL) {
    int64_t d = (int64_t)c.qmc_dimension;
    if (c.dim_mode == RG_DIM_FULL) {
      d = std::max<int64_t>(d, (int64_t)n * T);
    } else {
      d = std::min<int64_t>(std::max<int64_t>(d, 1), 512);
    }
    tr.sob_dim = d;
  } else if (tr.vr == RG_VR_HALTON) {
    if (c.dim_mode == RG_DIM_FULL) {
      // the production Halton lane: one prime per dimension, no wrap
      const int64_t d = std::max<int64_t>((int64_t)c.qmc_dimension, (int64_t)n * T);
      if (d > (int64_t(1) << 20)) raise(RG_ERR_UNSUPPORTED, "the full-dimension Halton lane holds at most 2^20 dimensions");
      tr.hal_dim = (int32_t)d;
      tr.hal_hash = 1;
    } else {
      tr.hal_dim = (int32_t)std::min<int64_t>(std::max<int64_t>((int64_t)c.qmc_dimension, 1), 512);
    }
  }

  // Phoenix step schedule (note.rs:150-218)
  const int64_t PER = tr.periods;
  const bool fixed_first = t.fixed_first_coupon != 0;
  P.step_flags.resize(T);
  P.step_period.resize(T);
  for (int64_t s = 0; s < T; ++s) {
    int64_t period = std::min((s * PER) / T, PER - 1);
    int64_t next = s + 1 == T ? PER : std::min(((s + 1) * PER) / T, PER - 1);
    uint32_t fl = 0;
    if (s + 1 == T || next != period) fl |= STEP_PERIOD_END;
    if (s >= call_start) fl |= STEP_CALL_ACTIVE;
    if (period == 0 && fixed_first) fl |= STEP_FIXED_DUE;
    else fl |= STEP_ACCRUE;
    if (s > 0 && period != std::min(((s - 1) * PER) / T, PER - 1)) fl |= STEP_PERIOD_RESET;
    P.step_flags[s] = fl;
    P.step_period[s] = (int32_t)period;
  }
  P.accr_inc.resize(PER);
  for (int64_t p = 0; p < PER; ++p) {
    int64_t a = T * (p + 1) / PER, b = T * p / PER;
    int64_t ps = std::max<int64_t>(a > b ? a - b : 0, 1);
    P.accr_inc[p] = tr.coupon_rate / (double)ps;
  }
  P.accr_f.assign(P.accr_inc.begin(), P.accr_inc.end());

  bridge_schedule_into(T, tr.dt, P);
  // per (node, factor): the QMC dimension n·k + f reduced to its table row, and its shift mask
  P.nf_row.resize(size_t(T) * n);
  P.nf_shift.resize(size_t(T) * n);
  for (int64_t nd = 0; nd < T; ++nd)
    for (int f = 0; f < n; ++f) {
      const uint64_t dim = (uint64_t)P.node_k[nd] * (uint64_t)n + (uint64_t)f;
      int32_t row = 0;
      if (tr.vr == RG_VR_SOBOL) row = (int32_t)(dim % (uint64_t)tr.sob_dim);
      else if (tr.vr == RG_VR_HALTON) row = (int32_t)(dim % (uint64_t)tr.hal_dim);  // = dim when hashed
      P.nf_row[size_t(nd) * n + f] = row;
      P.nf_shift[size_t(nd) * n + f] = rg_digital_shift(dim, tr.seed);
    }

  // Scenarios: the request's own market when none are given.
  std::vector<rg_scenario> own;
  if (n_scen == 0) {
    own.push_back(rg_scenario{r->market, nullptr});
    sc = own.data();
    n_scen = 1;
  }
  P.n_scen = n_scen;
  P.scen.resize(n_scen);
  P.scen32.resize(n_scen);
  P.df.resize(size_t(n_scen) * T);
  P.df_mat.resize(n_scen);

  // Local-vol: per-asset tenor schedule of sigma(step*dt, ·) (riga-market/src/lib.rs:324-339)
  const int gx = tr.gx;
  if (tr.has_lv) {
    P.lv_ti.resize(size_t(n) * T * 2);
    P.lv_tw.resize(size_t(n) * T);
    P.lv_twf.resize(size_t(n) * T);
    P.asset_log_lo.resize(n);
    P.asset_log_hi.resize(n);
    P.grids.resize(n);
    for (int f = 0; f < n; ++f) {
      const rg_implied_vol_grid& g = r->local_vol[f];
      P.grids[f] = &g;
      const int nt = g.n_maturities;
      P.lv_nt_max = std::max(P.lv_nt_max, nt);
      const double* ta = g.maturities_years;
      for (int64_t s = 0; s < T; ++s) {
        int ii = 0, i1 = 0;
        double wt = 0.0;
        if (nt > 1) {
          double tt = (double)s * tr.dt;
          double tc = tt < ta[0] ? ta[0] : (tt > ta[nt - 1] ? ta[nt - 1] : tt);
          while (ii + 1 < nt - 1 && tc > ta[ii + 1]) ++ii;
          double span = ta[ii + 1] - ta[ii];
          wt = span > 0.0 ? (tc - ta[ii]) / span : 0.0;
          i1 = ii + 1;
        }
        P.lv_ti[(size_t(f) * T + s) * 2] = ii;
        P.lv_ti[(size_t(f) * T + s) * 2 + 1] = i1;
        P.lv_tw[size_t(f) * T + s] = wt;
        P.lv_twf[size_t(f) * T + s] = (float)wt;
      }
      // Dupire log-strike axis [0.55 K_min, 1.05 K_max] (riga-market/src/lib.rs:217-224)
      double s_min = g.strikes[0] * 0.55, s_max = g.strikes[g.n_strikes - 1] * 1.05;
      P.asset_log_lo[f] = std::log(std::max(s_min, 1e-6));
      P.asset_log_hi[f] = std::log(std::max(s_max, 1e-6));
    }
  }

  for (int i = 0; i < n_scen; ++i) {
    const rg_market_snapshot& m = sc[i].market;
    DevScenario& d = P.scen[i];
    memset(&d, 0, sizeof d);
    DevScen32& d32 = P.scen32[i];
    memset(&d32, 0, sizeof d32);
    d.rate = m.risk_free_rate;
    for (int f = 0; f < n; ++f) {
      d.spots[f] = m.spots[f];
      d.vols[f] = m.vols[f];
      d.q[f] = m.dividend_yields[f];
      d.surf[f] = -1;
      d32.x0[f] = (float)std::log(m.spots[f] / t.initial_spots[f]);
      d32.mu_dt[f] = (float)((m.risk_free_rate - m.dividend_yields[f]) * tr.dt);
      d32.sig[f] = (float)m.vols[f];
    }
    for (int k = 0; k < n * n; ++k) d.L[k] = m.correlation[k];  // factorised on the device
    if (tr.has_lv) {
      for (int f = 0; f < n; ++f) {
        SurfaceKey key{f, m.spots[f], m.risk_free_rate,
                       sc[i].implied_vol_shift ? sc[i].implied_vol_shift[f] : 0.0};
        int found = -1;
        for (size_t j = 0; j < P.surfaces.size(); ++j)
          if (P.surfaces[j] == key) { found = (int)j; break; }
        if (found < 0) {
          found = (int)P.surfaces.size();
          P.surfaces.push_back(key);
          P.surf_nt.push_back(r->local_vol[f].n_maturities);
        }
        d.surf[f] = found;
        double h = (P.asset_log_hi[f] - P.asset_log_lo[f]) / (double)(gx - 1);
        d32.inv_h[f] = (float)(1.0 / h);
        d32.a_u[f] = (float)((std::log(t.initial_spots[f]) - P.asset_log_lo[f]) / h);
      }
    }
    // discount factors exp(-r * (step + 1) dt) and exp(-r * T) (note.rs:189, 210, 221, 238), with
    // the platform libm's exp, as the reference's f64::exp
    for (int64_t s = 0; s < T; ++s) {
      double time = (double)(s + 1) * tr.dt;
      P.df[size_t(i) * T + s] = std::exp(-m.risk_free_rate * time);
    }
    P.df_mat[i] = std::exp(-m.risk_free_rate * t.maturity_years);
  }
  P.df_f.assign(P.df.begin(), P.df.end());
  P.df_mat_f.assign(P.df_mat.begin(), P.df_mat.end());
  P.n_surf = (int)P.surfaces.size();
  // surface row offsets in the packed local-vol tables
  if (tr.has_lv) {
    std::vector<int32_t> surf_off(P.n_surf, 0);
    int32_t acc = 0;
    for (int j = 0; j < P.n_surf; ++j) {
      surf_off[j] = acc;
      acc += P.surf_nt[j] * gx;
    }
    for (int i = 0; i < n_scen; ++i)
      for (int f = 0; f < n; ++f) {
        P.scen32[i].surf_off[f] = P.scen[i].surf[f] * (int32_t)T * gx;
        P.scen[i].surf_off[f] = surf_off[P.scen[i].surf[f]];
      }
    if ((double)P.n_surf * (double)T * (double)gx >= 2147483647.0)
      raise(RG_ERR_INVALID_ARGUMENT, "too many local-vol surfaces x steps x grid points for one request");
  }
}

}  // namespace rg
