// book.cu — host side of book pricing: validation, tables, the chunked two-stream pipeline and
// the C entry points rg_price_book / rg_book_run_paths.
//
// Pipeline of one book call (engine stream S0, generation stream S1):
//   validate (each trade with the reference's request checks on its slice of the universe) →
//   host tables (QMC, bridge schedule over the universe grid, per-trade constants, per-scenario
//   discount factors) → one packed H2D copy → universe Cholesky (FP64, device) →
//   for each chunk of paths: generation of the chunk's universe increments on S1 into one of two
//   buffers, then the scan of every (trade, scenario) on S0; chunk k+1 generates while chunk k is
//   scanned → fixed-order reduce over path blocks → one D2H copy → PriceResults.
// FP64 parity mode runs the same pipeline with the FP64 kernels and no overlap.
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <map>

#include "rg_book.h"

namespace rg {
namespace bk {

void validate_book(const rg_book_request* r, const BookScenarios& sc) {
  if (!r) raise(RG_ERR_INVALID_ARGUMENT, "request is null");
  const rg_market_snapshot& u = r->universe;
  const int U = u.n_assets;
  if (!u.as_of || !u.as_of[0]) raise(RG_ERR_MISSING_AS_OF, "as_of is required");
  if (U < 1 || U > RG_BOOK_MAX_UNIVERSE || !u.spots || !u.vols || !u.dividend_yields || !u.correlation)
    raise(RG_ERR_INVALID_MARKET_SHAPE, "the universe needs 1..32 assets with aligned arrays");
  const rg_simulation_config& c = r->config;
  if (c.paths == 0 || c.path_block_size == 0) raise(RG_ERR_INVALID_PATHS, "paths and path_block_size must be positive");
  if (r->universe_steps <= 0 || !std::isfinite(r->universe_maturity_years) || r->universe_maturity_years <= 0.0)
    raise(RG_ERR_INVALID_SCHEDULE, "universe steps and maturity must be positive and finite");
  if (r->universe_steps > (int64_t(1) << 22)) raise(RG_ERR_INVALID_SCHEDULE, "at most 2^22 steps are supported");
  if (r->n_trades < 1 || !r->trades) raise(RG_ERR_INVALID_ARGUMENT, "a book needs at least one trade");
  if (c.variance_reduction != RG_VR_SOBOL && c.variance_reduction != RG_VR_HALTON)
    raise(RG_ERR_UNSUPPORTED, "books run the Sobol or Halton lane");
  if (c.trace_level != RG_TRACE_OFF)
    raise(RG_ERR_INVALID_ARGUMENT, "books record no trace events (trace_level must be off)");
  const double dt = r->universe_maturity_years / (double)r->universe_steps;
  double sub_spots[RG_NMAX], sub_vols[RG_NMAX], sub_q[RG_NMAX], sub_rho[RG_NMAX * RG_NMAX];
  for (int j = 0; j < r->n_trades; ++j) {
    const rg_book_trade& bt = r->trades[j];
    const rg_phoenix_trade& t = bt.terms;
    const int n = t.n_assets;
    const std::string tag = "trade " + std::to_string(j);
    if (n < 1 || n > RG_NMAX || !bt.underlyings)
      raise(RG_ERR_INVALID_MARKET_SHAPE, tag + " needs 1..5 underlyings");
    for (int f = 0; f < n; ++f) {
      const int a = bt.underlyings[f];
      if (a < 0 || a >= U) raise(RG_ERR_INVALID_MARKET_SHAPE, tag + " has an underlying outside the universe");
      for (int g = 0; g < f; ++g)
        if (bt.underlyings[g] == a) raise(RG_ERR_INVALID_MARKET_SHAPE, tag + " repeats an underlying");
    }
    if (t.steps < 1 || t.steps > r->universe_steps)
      raise(RG_ERR_INVALID_SCHEDULE, tag + " steps must be in 1..universe_steps");
    if (!(std::fabs(t.maturity_years - (double)t.steps * dt) <= 1e-12 * t.maturity_years))
      raise(RG_ERR_INVALID_SCHEDULE, tag + " maturity must be steps x the universe dt");
    // the reference's request checks on the trade and its slice of the base market
    for (int f = 0; f < n; ++f) {
      const int a = bt.underlyings[f];
      sub_spots[f] = u.spots[a];
      sub_vols[f] = u.vols[a];
      sub_q[f] = u.dividend_yields[a];
      for (int g = 0; g < n; ++g) sub_rho[f * n + g] = u.correlation[a * U + bt.underlyings[g]];
    }
    rg_price_request q;
    memset(&q, 0, sizeof q);
    q.trade = t;
    q.market = u;
    q.market.n_assets = n;
    q.market.spots = sub_spots;
    q.market.vols = sub_vols;
    q.market.dividend_yields = sub_q;
    q.market.correlation = sub_rho;
    q.config = c;
    q.as_of = u.as_of;
    validate_request(&q);
  }
  // the universe correlation itself (CorrelationMatrix::validate, correlation.rs:74-93)
  for (int i = 0; i < U; ++i)
    for (int k = 0; k < U; ++k) {
      const double v = u.correlation[i * U + k];
      if (!std::isfinite(v) || (i == k ? std::fabs(v - 1.0) > 1e-12
                                       : (std::fabs(v) > 1.0 || std::fabs(v - u.correlation[k * U + i]) > 1e-12)))
        raise(RG_ERR_INVALID_MARKET, "universe correlation must be symmetric with unit diagonal and entries in [-1,1]");
    }
  for (int a = 0; a < U; ++a)
    if (!(u.spots[a] > 0.0) || !(u.vols[a] >= 0.0) || !std::isfinite(u.vols[a]) || !std::isfinite(u.dividend_yields[a]))
      raise(RG_ERR_INVALID_MARKET, "universe spots must be positive and vols non-negative");
  validate_book_scenarios(u, sc);
}

void validate_book_scenarios(const rg_market_snapshot& u, const BookScenarios& spec) {
  const int U = u.n_assets;
  if (spec.per_trade) {
    const rg_book_bumps* b = spec.bumps;
    if (b && (!std::isfinite(b->spot_relative) || !std::isfinite(b->vol_absolute) || !std::isfinite(b->rate_absolute) ||
              b->spot_relative < 0.0 || b->spot_relative >= 0.1 || b->vol_absolute < 0.0 || b->rate_absolute < 0.0))
      raise(RG_ERR_INVALID_ARGUMENT, "bump sizes must be finite and non-negative, the spot move below 10%");
    return;
  }
  const rg_market_snapshot* sc = spec.sc;
  const int n_scen = spec.n;
  if (n_scen < 0 || (n_scen > 0 && !sc)) raise(RG_ERR_INVALID_ARGUMENT, "bad scenario list");
  for (int s = 0; s < n_scen; ++s) {
    if (sc[s].n_assets != U || !sc[s].spots || !sc[s].vols || !sc[s].dividend_yields)
      raise(RG_ERR_INVALID_MARKET_SHAPE, "scenario " + std::to_string(s) + " is not a market of the universe");
    if (sc[s].correlation &&
        memcmp(sc[s].correlation, u.correlation, sizeof(double) * (size_t)U * (size_t)U) != 0)
      raise(RG_ERR_INVALID_ARGUMENT,
            "scenario " + std::to_string(s) + " changes the correlation; book scenarios share the base paths");
    if (!std::isfinite(sc[s].risk_free_rate)) raise(RG_ERR_INVALID_MARKET, "scenario rate must be finite");
    for (int a = 0; a < U; ++a)
      if (!(sc[s].spots[a] > 0.0) || !std::isfinite(sc[s].spots[a]) || !(sc[s].vols[a] >= 0.0) ||
          !std::isfinite(sc[s].vols[a]) || !std::isfinite(sc[s].dividend_yields[a]))
        raise(RG_ERR_INVALID_MARKET, "scenario spots must be positive and finite, vols non-negative");
  }
}

void plan_book(const rg_book_request* r, const BookScenarios& sc, BookPlan& B) {
  const rg_market_snapshot& u = r->universe;
  const rg_simulation_config& c = r->config;
  B.U = u.n_assets;
  B.TU = r->universe_steps;
  B.dt = r->universe_maturity_years / (double)r->universe_steps;
  B.n_trades = r->n_trades;
  DevTrade& g = B.gen;
  g.n = B.U;
  g.vr = c.variance_reduction;
  g.scrambler = c.scrambler;
  g.steps = B.TU;
  g.seed = c.seed;
  g.dt = B.dt;
  g.sqrt_dt = std::sqrt(B.dt);
  g.inv_sqrt_dt = 1.0 / std::sqrt(B.dt);
  const int64_t need = (int64_t)B.U * B.TU;
  if (g.vr == RG_VR_SOBOL) {
    int64_t d = (int64_t)c.qmc_dimension;
    g.sob_dim = c.dim_mode == RG_DIM_FULL ? std::max<int64_t>(d, need) : std::min<int64_t>(std::max<int64_t>(d, 1), 512);
  } else if (c.dim_mode == RG_DIM_FULL) {
    // the production Halton lane: one prime per dimension, hashed affine digit scrambling, no wrap
    const int64_t d = std::max<int64_t>((int64_t)c.qmc_dimension, need);
    if (d > (int64_t(1) << 20)) raise(RG_ERR_UNSUPPORTED, "the full-dimension Halton lane holds at most 2^20 dimensions");
    g.hal_dim = (int32_t)d;
    g.hal_hash = 1;
  } else {
    g.hal_dim = (int32_t)std::min<int64_t>(std::max<int64_t>((int64_t)c.qmc_dimension, 1), 512);
  }
  bridge_schedule_into(B.TU, B.dt, B.br);
  B.trades.resize(B.n_trades);
  for (int j = 0; j < B.n_trades; ++j) {
    const rg_phoenix_trade& t = r->trades[j].terms;
    BookTradeDev& d = B.trades[j];
    memset(&d, 0, sizeof d);
    d.n = t.n_assets;
    d.T = (int32_t)t.steps;
    int64_t per = t.has_coupon_periods ? t.coupon_periods : 9;  // note.rs:43
    d.periods = (int32_t)std::max<int64_t>(std::min<int64_t>(per, INT32_MAX), 1);
    const int64_t cs = t.has_call_start_step ? t.call_start_step : 0;
    d.call_start = (int32_t)std::max<int64_t>(std::min<int64_t>(cs, INT32_MAX), INT32_MIN);
    for (int f = 0; f < d.n; ++f) {
      d.idx[f] = r->trades[j].underlyings[f];
      d.init[f] = t.initial_spots[f];
    }
    d.fixed_first = t.fixed_first_coupon ? 1 : 0;
    d.memory = t.memory_coupon ? 1 : 0;
    d.maturity = t.maturity_years;
    d.call_barrier = t.has_knock_out_barrier ? t.knock_out_barrier : INFINITY;
    d.coupon_barrier = t.has_coupon_barrier ? t.coupon_barrier : INFINITY;
    d.coupon_rate = t.has_coupon_rate ? t.coupon_rate : 0.0;
    d.strike = t.strike;
    d.ki = t.knock_in_barrier;
    d.ln_ko = (float)std::log(d.call_barrier);
    d.ln_cb = (float)std::log(d.coupon_barrier);
    d.ln_ki = (float)std::log(d.ki);
    d.coupon_f = (float)d.coupon_rate;
    d.strike_f = (float)d.strike;
    d.ps_a = std::max<int32_t>(1, d.T / std::max<int32_t>(d.periods, 1));
    d.inc_a = (float)(d.coupon_rate / (double)d.ps_a);
    d.inc_b = (float)(d.coupon_rate / (double)(d.ps_a + 1));
  }
  // work order: grouped by underlying count (one launch each), longest trades first in a group
  B.order.resize(B.n_trades);
  for (int j = 0; j < B.n_trades; ++j) B.order[j] = j;
  std::stable_sort(B.order.begin(), B.order.end(), [&](int a, int b) {
    if (B.trades[a].n != B.trades[b].n) return B.trades[a].n < B.trades[b].n;
    return B.trades[a].T > B.trades[b].T;
  });
  for (int n = 0; n < RG_NMAX; ++n) B.group_lo[n] = B.group_n[n] = 0;
  for (int i = 0; i < B.n_trades; ++i) {
    const int n = B.trades[B.order[i]].n;
    if (B.group_n[n - 1]++ == 0) B.group_lo[n - 1] = i;
  }
  plan_book_scenarios(r, sc, B);
}

rg_book_bump_spec trade_bump(int n, int k, const rg_book_bumps* sizes) {
  const double h = sizes && sizes->spot_relative > 0.0 ? sizes->spot_relative : 0.01;
  const double v = sizes && sizes->vol_absolute > 0.0 ? sizes->vol_absolute : 0.01;
  const double rr = sizes && sizes->rate_absolute > 0.0 ? sizes->rate_absolute : 1e-4;
  rg_book_bump_spec b{RG_BUMP_BASE, -1, -1, 0.0};
  if (k == 0) return b;
  int left = k - 1;  // position in the bump order
  auto take = [&left](int count) {
    if (left < count) return true;
    left -= count;
    return false;
  };
  const int npairs = n * (n - 1) / 2;
  auto pair_of = [](int idx, int& a, int& c) {  // (0,1), (0,2), (1,2), (0,3), ...
    for (c = 1;; ++c) {
      if (idx < c) {
        a = idx;
        return;
      }
      idx -= c;
    }
  };
  if (take(2 * n)) return {RG_BUMP_SPOT, left / 2, -1, left % 2 ? -h : h};
  if (take(n)) return {RG_BUMP_VOL, left, -1, v};
  if (take(1)) return {RG_BUMP_RATE, -1, -1, rr};
  if (take(npairs)) {
    int a, c;
    pair_of(left, a, c);
    return {RG_BUMP_SPOT_PAIR, a, c, h};
  }
  if (take(n)) return {RG_BUMP_VOL, left, -1, -v};
  if (take(1)) return {RG_BUMP_RATE, -1, -1, -rr};
  if (take(npairs)) {
    int a, c;
    pair_of(left, a, c);
    return {RG_BUMP_SPOT_PAIR, a, c, -h};
  }
  for (double m : {2.0, 5.0, 10.0})
    if (take(2 * n)) return {RG_BUMP_SPOT, left / 2, -1, left % 2 ? -m * h : m * h};
  if (take(2 * n)) return {RG_BUMP_VOL, left / 2, -1, left % 2 ? -2.0 * v : 2.0 * v};
  if (take(2)) return {RG_BUMP_RATE, -1, -1, left ? -2.0 * rr : 2.0 * rr};
  raise(RG_ERR_INVALID_ARGUMENT, "no such bump scenario");
}

// The scenario-dependent tables: the markets the (trade, scenario) pairs price under, discount
// factors per distinct rate, per-pair FP32 constants.  Common scenarios are markets 0..S-1 in
// order; per-trade bump markets are the base market with one trade's bump applied, each distinct
// market kept once.
void plan_book_scenarios(const rg_book_request* r, const BookScenarios& spec, BookPlan& B) {
  const rg_market_snapshot& u = r->universe;
  const int U = B.U;
  B.scen.clear();
  std::vector<int32_t> pair_mkt;
  auto market_of = [&](const rg_market_snapshot& m) {
    BookScenDev d;
    memset(&d, 0, sizeof d);
    d.rate = m.risk_free_rate;
    for (int a = 0; a < U; ++a) {
      d.spots[a] = m.spots[a];
      d.vols[a] = m.vols[a];
      d.q[a] = m.dividend_yields[a];
    }
    return d;
  };
  if (!spec.per_trade) {
    const rg_market_snapshot* sc = spec.sc;
    int n_scen = spec.n;
    if (n_scen == 0) {
      sc = &u;
      n_scen = 1;
    }
    B.S = n_scen;
    for (int s = 0; s < B.S; ++s) B.scen.push_back(market_of(sc[s]));
    pair_mkt.resize((size_t)B.n_trades * B.S);
    for (int j = 0; j < B.n_trades; ++j)
      for (int s = 0; s < B.S; ++s) pair_mkt[(size_t)j * B.S + s] = s;
  } else {
    B.S = RG_BOOK_TRADE_SCENARIOS;
    const BookScenDev base = market_of(u);
    std::map<std::vector<uint8_t>, int32_t> seen;
    pair_mkt.resize((size_t)B.n_trades * B.S);
    for (int j = 0; j < B.n_trades; ++j) {
      const BookTradeDev& t = B.trades[j];
      for (int k = 0; k < B.S; ++k) {
        const rg_book_bump_spec b = trade_bump(t.n, k, spec.bumps);
        BookScenDev d = base;
        switch (b.kind) {
          case RG_BUMP_SPOT: d.spots[t.idx[b.first]] *= 1.0 + b.size; break;
          case RG_BUMP_SPOT_PAIR:
            d.spots[t.idx[b.first]] *= 1.0 + b.size;
            d.spots[t.idx[b.second]] *= 1.0 + b.size;
            break;
          case RG_BUMP_VOL: d.vols[t.idx[b.first]] = std::max(0.0, d.vols[t.idx[b.first]] + b.size); break;
          case RG_BUMP_RATE: d.rate += b.size; break;
          default: break;
        }
        std::vector<uint8_t> key(reinterpret_cast<const uint8_t*>(&d), reinterpret_cast<const uint8_t*>(&d) + sizeof d);
        auto it = seen.find(key);
        int32_t m;
        if (it == seen.end()) {
          m = (int32_t)B.scen.size();
          seen.emplace(std::move(key), m);
          B.scen.push_back(d);
        } else {
          m = it->second;
        }
        pair_mkt[(size_t)j * B.S + k] = m;
      }
    }
  }
  // discount factors exp(-r (t+1) dt) on the universe grid (note.rs:189, 210), one row per
  // distinct rate, with the platform libm's exp
  std::vector<double> rates;
  for (BookScenDev& d : B.scen) {
    int row = -1;
    for (size_t i = 0; i < rates.size(); ++i)
      if (rates[i] == d.rate) row = (int)i;
    if (row < 0) {
      row = (int)rates.size();
      rates.push_back(d.rate);
    }
    d.dfrow = row;
  }
  B.df.resize(rates.size() * (size_t)B.TU);
  for (size_t i = 0; i < rates.size(); ++i)
    for (int64_t t = 0; t < B.TU; ++t) B.df[i * B.TU + t] = std::exp(-rates[i] * ((double)(t + 1) * B.dt));
  B.dfm.resize((size_t)B.n_trades * B.S);
  B.pair32.resize((size_t)B.n_trades * B.S);
  for (int j = 0; j < B.n_trades; ++j)
    for (int s = 0; s < B.S; ++s) {
      const BookTradeDev& t = B.trades[j];
      const int32_t mi = pair_mkt[(size_t)j * B.S + s];
      const BookScenDev& m = B.scen[mi];
      B.dfm[(size_t)j * B.S + s] = std::exp(-m.rate * t.maturity);  // note.rs:221, 238 (libm)
      BookPair32& p = B.pair32[(size_t)j * B.S + s];
      memset(&p, 0, sizeof p);
      p.mkt = mi;
      p.dfrow = m.dfrow;
      for (int f = 0; f < t.n; ++f) {
        const int a = t.idx[f];
        const double v = m.vols[a];
        p.x0[f] = (float)std::log(m.spots[a] / t.init[f]);
        p.drift[f] = (float)((m.rate - m.q[a] - 0.5 * v * v) * B.dt);
        p.sig[f] = (float)v;
      }
    }
}

void* book_buf(rg_engine* E, int slot, size_t bytes) {
  E->book_bufs[slot].ensure(bytes);
  return E->book_bufs[slot].ptr;
}

BookStaged stage_book_static(DevBuf& tables, cudaStream_t st, const rg_book_request* r, const BookPlan& B) {
  Pack pk;
  const int U = B.U;
  size_t o_sobol = 0, o_hb = 0, o_ho = 0, o_hp = 0;
  std::vector<uint32_t> hb, ho, hp;
  if (B.gen.vr == RG_VR_SOBOL) {
    o_sobol = pk.add(sobol_table(B.gen.sob_dim));
  } else if (B.gen.hal_hash) {
    o_hb = pk.add(first_primes(B.gen.hal_dim).data(), (size_t)B.gen.hal_dim);  // no permutation tables
    o_ho = o_hp = o_hb;
  } else {
    halton_tables(B.gen.hal_dim, B.gen.seed, hb, ho, hp);
    o_hb = pk.add(hb);
    o_ho = pk.add(ho);
    o_hp = pk.add(hp);
  }
  const size_t o_noff = pk.add(B.br.node_off), o_nk = pk.add(B.br.node_k), o_nc = pk.add(B.br.node_c),
               o_ncf = pk.add(B.br.node_cf);
  const size_t o_tr = pk.add(B.trades), o_ord = pk.add(B.order);
  const size_t o_corr = pk.add(r->universe.correlation, (size_t)U * U);
  const size_t o_L = pk.reserve(sizeof(double) * U * U), o_L32 = pk.reserve(sizeof(float) * U * U);
  const size_t o_work = pk.reserve(sizeof(double) * 2 * U * U);
  tables.ensure(pk.host.size());
  uint8_t* dev = static_cast<uint8_t*>(tables.ptr);
  cuda_check(cudaMemcpyAsync(dev, pk.host.data(), pk.host.size(), cudaMemcpyHostToDevice, st), "book H2D");
  BookStaged out;
  DevTables& tb = out.tb;
  tb.sobol = B.gen.vr == RG_VR_SOBOL ? reinterpret_cast<const uint32_t*>(dev + o_sobol) : nullptr;
  tb.hal_base = B.gen.vr == RG_VR_HALTON ? reinterpret_cast<const uint32_t*>(dev + o_hb) : nullptr;
  tb.hal_off = B.gen.vr == RG_VR_HALTON ? reinterpret_cast<const uint32_t*>(dev + o_ho) : nullptr;
  tb.hal_perm = B.gen.vr == RG_VR_HALTON ? reinterpret_cast<const uint32_t*>(dev + o_hp) : nullptr;
  tb.node_off = reinterpret_cast<const int32_t*>(dev + o_noff);
  tb.node_k = reinterpret_cast<const int32_t*>(dev + o_nk);
  tb.node_c = reinterpret_cast<const double*>(dev + o_nc);
  tb.node_cf = reinterpret_cast<const float*>(dev + o_ncf);
  BookDev& bk = out.bk;
  bk.U = U;
  bk.S = B.S;
  bk.n_trades = B.n_trades;
  bk.TU = B.TU;
  bk.trades = reinterpret_cast<const BookTradeDev*>(dev + o_tr);
  bk.order = reinterpret_cast<const int32_t*>(dev + o_ord);
  out.L = reinterpret_cast<double*>(dev + o_L);
  out.L32 = reinterpret_cast<float*>(dev + o_L32);
  bk.L = out.L;
  bk.L32 = out.L32;
  launch_cholesky_big(reinterpret_cast<const double*>(dev + o_corr), U, out.L,
                      reinterpret_cast<double*>(dev + o_work), st);
  launch_book_l32(out.L, U, out.L32, st);
  return out;
}

ScenarioPack pack_book_scenarios(const BookPlan& B) {
  ScenarioPack sp;
  sp.o_scen = sp.pk.add(B.scen);
  sp.o_p32 = sp.pk.add(B.pair32);
  sp.o_df = sp.pk.add(B.df);
  sp.o_dfm = sp.pk.add(B.dfm);
  sp.o_df_f = sp.pk.add(std::vector<float>(B.df.begin(), B.df.end()));
  sp.o_dfm_f = sp.pk.add(std::vector<float>(B.dfm.begin(), B.dfm.end()));
  return sp;
}

void point_scenarios(const ScenarioPack& sp, const uint8_t* dev, int S, BookDev& bk) {
  bk.S = S;
  bk.scen = reinterpret_cast<const BookScenDev*>(dev + sp.o_scen);
  bk.pair32 = reinterpret_cast<const BookPair32*>(dev + sp.o_p32);
  bk.df = reinterpret_cast<const double*>(dev + sp.o_df);
  bk.dfm = reinterpret_cast<const double*>(dev + sp.o_dfm);
  bk.df_f = reinterpret_cast<const float*>(dev + sp.o_df_f);
  bk.dfm_f = reinterpret_cast<const float*>(dev + sp.o_dfm_f);
}

// The tensor map of one chunk's FP32 increments, viewed as [TU][U][npaths] with rows of `rowlen`
// floats: boxes of Pb paths × 1 asset × TT steps (zero-filled past npaths and TU).
CUtensorMap increments_map(const float* incr, uint64_t npaths, uint64_t rowlen, int U, int64_t TU, int Pb, int TT) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cuda_check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
               "cuTensorMapEncodeTiled entry point");
    if (!fn || q != cudaDriverEntryPointSuccess) raise(RG_ERR_GPU_ERROR, "cuTensorMapEncodeTiled unavailable");
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  CUtensorMap map;
  const cuuint64_t dims[3] = {npaths, (cuuint64_t)U, (cuuint64_t)TU};
  const cuuint64_t strides[2] = {rowlen * 4, (cuuint64_t)U * rowlen * 4};
  const cuuint32_t box[3] = {(cuuint32_t)Pb, 1, (cuuint32_t)TT};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(incr), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) raise(RG_ERR_GPU_ERROR, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return map;
}

void increments_maps(const float* incr, uint64_t npaths, uint64_t rowlen, int U, int64_t TU, const Book32Shape& sh,
                     CUtensorMap* maps) {
  for (int n = 1; n <= RG_NMAX; ++n)
    maps[n - 1] = increments_map(incr, npaths, rowlen, U, TU, sh.Pb, book_stage_steps(n, sh.TT));
}

// Paths per generation chunk: a multiple of `unit` whose increments fit the budget.
uint64_t chunk_paths(uint64_t paths, int U, int64_t TU, size_t elem, uint64_t unit) {
  const uint64_t per_path = (uint64_t)U * (uint64_t)TU * elem;
  uint64_t cap = kIncrBudget / per_path;
  cap = cap / unit * unit;
  if (cap < unit) cap = unit;
  return paths < cap ? paths : cap;
}

}  // namespace bk

size_t estimate_book_bytes(const rg_book_request* r, int n_scen) {
  using namespace bk;
  const size_t S = n_scen > 0 ? (size_t)n_scen : 1;
  const size_t U = (size_t)(r->universe.n_assets > 0 ? r->universe.n_assets : 1);
  const size_t TU = (size_t)(r->universe_steps > 0 ? r->universe_steps : 1);
  const size_t pairs = (size_t)(r->n_trades > 0 ? r->n_trades : 1) * S;
  const uint64_t P = r->config.paths;
  const bool fp32 = r->config.precision == RG_PRECISION_FP32;
  const size_t elem = fp32 ? sizeof(float) : sizeof(double);
  int group[RG_NMAX] = {0};
  for (int32_t j = 0; j < r->n_trades; ++j) {
    const int n = r->trades[j].terms.n_assets;
    if (n >= 1 && n <= RG_NMAX) ++group[n - 1];
  }
  int gmin = 0;
  for (int n = 0; n < RG_NMAX; ++n)
    if (group[n] > 0 && (gmin == 0 || group[n] < gmin)) gmin = group[n];
  const uint64_t unit =
      fp32 ? (uint64_t)book32_shape((int)std::min<size_t>(S, 32), device_sm_count(), P, gmin).blk_paths : 128;
  const uint64_t PC = chunk_paths(P, (int)U, (int64_t)TU, elem, unit);
  const uint64_t chunks = (P + PC - 1) / PC;
  size_t b = (size_t)PC * U * TU * elem * (fp32 && chunks > 1 ? 2 : 1);
  const uint64_t blocks = fp32 ? (P + unit - 1) / unit : ((PC + 127) / 128) * chunks;
  b += (size_t)blocks * pairs * RG_ACC * 8 + pairs * RG_ACC * 8;
  size_t sob_rows = r->config.dim_mode == RG_DIM_FULL ? U * TU : 512;
  b += sob_rows * 128 + TU * 32 + S * TU * 12 + pairs * 100 + (size_t)r->n_trades * 256 + (size_t(64) << 10);
  return b + b / 8 + (size_t(1) << 20);
}

// Under per-trade bump sets a book prices 16 (trade, scenario) pairs per trade, as under 16 common
// scenarios, and plans one market per distinct bumped universe market (at most 16 per trade), each
// with its per-step tables.
size_t estimate_book_trade_bumps_bytes(const rg_book_request* r) {
  const size_t TU = (size_t)(r->universe_steps > 0 ? r->universe_steps : 1);
  const size_t markets = std::min<size_t>((size_t)(r->n_trades > 0 ? r->n_trades : 1) * RG_BOOK_TRADE_SCENARIOS, 4096);
  return estimate_book_bytes(r, RG_BOOK_TRADE_SCENARIOS) + markets * (TU * 16 + 256);
}

namespace {

using namespace bk;

// Prices (records == nullptr) or replays [first, first + count) of the book.
// Every input of the FP32 universe increments of paths [path_base, path_base + P): the universe
// correlation and grid, the QMC settings and the path range (spots, vols, rates and the trades
// enter only the scans).
static std::vector<uint8_t> universe_key_bytes(const rg_book_request* r, uint64_t path_base, uint64_t P) {
  std::vector<uint8_t> b;
  auto put = [&b](const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  };
  const int64_t U = r->universe.n_assets;
  const int64_t ints[8] = {U, r->universe_steps, (int64_t)r->config.seed, r->config.variance_reduction,
                           (int64_t)r->config.qmc_dimension, r->config.scrambler, r->config.dim_mode,
                           (int64_t)r->config.precision};
  const uint64_t range[2] = {path_base, P};
  put(ints, sizeof ints);
  put(range, sizeof range);
  put(&r->universe_maturity_years, sizeof(double));
  put(r->universe.correlation, sizeof(double) * (size_t)(U * U));
  return b;
}

void run_book(rg_engine* E, const rg_book_request* r, const BookScenarios& sc, rg_price_result* out,
              uint64_t first, uint64_t count, rg_path_record* records) {
  validate_book(r, sc);
  BookPlan B;
  plan_book(r, sc, B);
  const int pairs = B.n_trades * B.S;
  const bool fp32 = r->config.precision == RG_PRECISION_FP32 && !records;
  BookStaged st = stage_book_static(E->book_bufs[BK_TABLES], E->stream, r, B);
  {
    const ScenarioPack sp = pack_book_scenarios(B);
    uint8_t* dev = static_cast<uint8_t*>(book_buf(E, BK_SCEN, sp.pk.host.size()));
    cuda_check(cudaMemcpyAsync(dev, sp.pk.host.data(), sp.pk.host.size(), cudaMemcpyHostToDevice, E->stream),
               "book scenarios H2D");
    point_scenarios(sp, dev, B.S, st.bk);
  }
  const uint64_t path_base = r->config.first_path + first;
  const uint64_t P = records ? count : r->config.paths;
  cudaStream_t s0 = E->stream, s1 = E->gen_stream;
  if (fp32) {
    // the path blocks (hence the sums) follow the device's SM count; the persistent scans' grid
    // follows the engine's SM cap
    Book32Shape sh = book32_shape(B.S, device_sm_count(), P, B.min_group());
    sh.grid = std::min(sh.grid, book32_shape(B.S, engine_sm_count(E), P, B.min_group()).grid);
    const uint64_t PC = chunk_paths(P, B.U, B.TU, sizeof(float), (uint64_t)sh.blk_paths);
    const uint64_t n_chunks = (P + PC - 1) / PC;
    const uint64_t blocks_per_chunk = (PC + sh.blk_paths - 1) / sh.blk_paths;
    const uint64_t total_blocks = (P + sh.blk_paths - 1) / sh.blk_paths;
    const uint64_t rowlen_max = (PC + 63) / 64 * 64;  // rows padded for 16-byte tensor-map strides
    const size_t incr_bytes = sizeof(float) * (size_t)B.U * (size_t)B.TU * (size_t)rowlen_max;
    float* incr[2] = {static_cast<float*>(book_buf(E, BK_INCR0, incr_bytes)),
                      static_cast<float*>(book_buf(E, BK_INCR1, n_chunks > 1 ? incr_bytes : 256))};
    double* partial = static_cast<double*>(book_buf(E, BK_PARTIAL, sizeof(double) * total_blocks * pairs * RG_ACC));
    int32_t* scratch = static_cast<int32_t*>(book_buf(E, BK_SCRATCH, 256));
    int* status = scratch + 1;
    cuda_check(cudaMemsetAsync(scratch, 0, 256, s0), "book status reset");
    // a book of one path chunk whose universe increments this engine generated last time (same
    // universe correlation, grid, QMC settings and paths) scans them again without regenerating
    std::vector<uint8_t> ukey;
    bool resident = false;
    if (n_chunks == 1) {
      ukey = universe_key_bytes(r, path_base, P);
      resident = E->universe_ptr == incr[0] && E->universe_key == ukey;
    }
    E->universe_key.clear();  // set again only when this call completes
    E->universe_ptr = nullptr;
    // the generation stream waits for the tables and the Cholesky factor
    cuda_check(cudaEventRecord(E->book_ev[0], s0), "event");
    cuda_check(cudaStreamWaitEvent(s1, E->book_ev[0], 0), "stream wait");
    for (uint64_t c = 0; c < n_chunks; ++c) {
      const uint64_t p0 = c * PC, np = std::min<uint64_t>(PC, P - p0);
      float* buf = incr[c & 1];
      if (c >= 2) {
        // buffer reuse: the scan of chunk c-2 must be done with it
        cuda_check(cudaStreamWaitEvent(s1, E->book_ev[2 + (c & 1)], 0), "stream wait");
      }
      const uint64_t rowlen = (np + 63) / 64 * 64;
      if (!resident) {
        launch_book_gen32(B.gen, st.tb, st.L32, B.U, path_base + p0, np, rowlen, buf, s1);
        cuda_check(cudaEventRecord(E->book_ev[1], s1), "event");
        cuda_check(cudaStreamWaitEvent(s0, E->book_ev[1], 0), "stream wait");
      }
      CUtensorMap maps[RG_NMAX];
      increments_maps(buf, np, rowlen, B.U, B.TU, sh, maps);
      launch_book_trade32(st.bk, sh, maps, np, c * blocks_per_chunk, B.group_lo, B.group_n, partial, scratch, status, s0);
      cuda_check(cudaEventRecord(E->book_ev[2 + (c & 1)], s0), "event");
    }
    double* dsums = static_cast<double*>(book_buf(E, BK_SUMS, sizeof(double) * pairs * RG_ACC));
    launch_book_reduce_strided(partial, (int64_t)total_blocks, (int64_t)pairs * RG_ACC, RG_ACC, pairs, dsums, s0);
    std::vector<double> hs((size_t)pairs * RG_ACC);
    int hstat = 0;
    cuda_check(cudaMemcpyAsync(hs.data(), dsums, sizeof(double) * hs.size(), cudaMemcpyDeviceToHost, s0), "D2H");
    cuda_check(cudaMemcpyAsync(&hstat, status, sizeof(int), cudaMemcpyDeviceToHost, s0), "D2H");
    cuda_check(cudaStreamSynchronize(s0), "book pricing");
    if (hstat == KSTAT_TIMEOUT) raise(RG_ERR_TIMEOUT, "book_trade32_kernel: a bounded stage wait ran out");
    if (hstat) raise(RG_ERR_GPU_ERROR, "book_trade32_kernel reported a bad work item");
    for (size_t k = 0; k < hs.size(); ++k)
      if (!std::isfinite(hs[k])) raise(RG_ERR_GPU_ERROR, "book: non-finite path sums");
    for (int p = 0; p < pairs; ++p) finish(hs.data() + (size_t)p * RG_ACC, P, r->config.seed, &out[p]);
    if (n_chunks == 1) {
      E->universe_key.swap(ukey);
      E->universe_ptr = incr[0];
    }
    return;
  }
  E->universe_key.clear();  // the FP64 path writes its own increments into the same buffer
  E->universe_ptr = nullptr;
  // FP64 parity: generation then scan per chunk on the engine stream
  const uint64_t PC = chunk_paths(P, B.U, B.TU, sizeof(double), 128);
  const uint64_t n_chunks = (P + PC - 1) / PC;
  const int blocks_per_chunk = (int)((PC + 127) / 128);
  const uint64_t total_blocks = n_chunks * (uint64_t)blocks_per_chunk;
  double* incr = static_cast<double*>(book_buf(E, BK_INCR0, sizeof(double) * (size_t)B.U * (size_t)B.TU * (size_t)PC));
  double* partial = static_cast<double*>(book_buf(E, BK_PARTIAL, sizeof(double) * total_blocks * pairs * RG_ACC));
  rg_path_record* drec = records ? static_cast<rg_path_record*>(book_buf(E, BK_RECORDS, sizeof(rg_path_record) * (size_t)PC * pairs)) : nullptr;
  std::vector<double> hs((size_t)pairs * RG_ACC, 0.0);
  for (uint64_t c = 0; c < n_chunks; ++c) {
    const uint64_t p0 = c * PC, np = std::min<uint64_t>(PC, P - p0);
    launch_book_gen64(B.gen, st.tb, st.L, B.U, path_base + p0, np, incr, s0);
    const int blocks = (int)((np + 127) / 128);
    launch_book_trade64(B.gen, st.bk, incr, path_base + p0, np, partial, blocks, drec, s0);
    if (records) {
      cuda_check(cudaMemcpyAsync(records + (size_t)p0 * pairs, drec, sizeof(rg_path_record) * (size_t)np * pairs,
                                 cudaMemcpyDeviceToHost, s0), "D2H records");
      cuda_check(cudaStreamSynchronize(s0), "book replay");
      continue;
    }
    // sum this chunk's blocks into the running FP64 totals, pair by pair, in block order
    double* dsums = static_cast<double*>(book_buf(E, BK_SUMS, sizeof(double) * pairs * RG_ACC));
    launch_book_reduce_strided(partial, blocks, RG_ACC, (int64_t)blocks * RG_ACC, pairs, dsums, s0);
    std::vector<double> part((size_t)pairs * RG_ACC);
    cuda_check(cudaMemcpyAsync(part.data(), dsums, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s0), "D2H");
    cuda_check(cudaStreamSynchronize(s0), "book pricing");
    for (size_t k = 0; k < part.size(); ++k) hs[k] += part[k];
  }
  if (records) return;
  for (int p = 0; p < pairs; ++p) finish(hs.data() + (size_t)p * RG_ACC, P, r->config.seed, &out[p]);
}

}  // namespace

}  // namespace rg

using namespace rg;

extern "C" int32_t rg_price_book(rg_engine* e, const rg_book_request* request, const rg_market_snapshot* scenarios,
                                 int32_t n_scenarios, rg_price_result* out) {
  RG_TRY({
    if (!e || !request || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    int32_t g = rg_guard_device();
    if (g) return g;
    std::lock_guard<std::mutex> lock(e->mu);
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    BookScenarios sc;
    sc.sc = scenarios;
    sc.n = n_scenarios;
    run_book(e, request, sc, out, 0, 0, nullptr);
  })
}

extern "C" int32_t rg_price_book_trade_bumps(rg_engine* e, const rg_book_request* request, const rg_book_bumps* sizes,
                                             rg_price_result* out) {
  RG_TRY({
    if (!e || !request || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    int32_t g = rg_guard_device();
    if (g) return g;
    std::lock_guard<std::mutex> lock(e->mu);
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    BookScenarios sc;
    sc.bumps = sizes;
    sc.per_trade = true;
    run_book(e, request, sc, out, 0, 0, nullptr);
  })
}

extern "C" int32_t rg_book_trade_bump(int32_t n_underlyings, int32_t scenario, const rg_book_bumps* sizes,
                                      rg_book_bump_spec* out) {
  RG_TRY({
    if (!out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    if (n_underlyings < 1 || n_underlyings > RG_NMAX || scenario < 0 || scenario >= RG_BOOK_TRADE_SCENARIOS)
      raise(RG_ERR_INVALID_ARGUMENT, "1..5 underlyings and scenarios 0..15");
    *out = bk::trade_bump(n_underlyings, scenario, sizes);
  })
}

extern "C" int32_t rg_book_run_paths(rg_engine* e, const rg_book_request* request, const rg_market_snapshot* scenarios,
                                     int32_t n_scenarios, uint64_t first_path, uint64_t count, rg_path_record* out) {
  RG_TRY({
    if (!e || !request || !out) raise(RG_ERR_INVALID_ARGUMENT, "null argument");
    int32_t g = rg_guard_device();
    if (g) return g;
    if (count == 0) raise(RG_ERR_INVALID_ARGUMENT, "count must be positive");
    if (first_path > request->config.paths || count > request->config.paths - first_path)
      raise(RG_ERR_PATH_OUT_OF_RANGE, "path range is outside the configured path count");
    std::lock_guard<std::mutex> lock(e->mu);
    cuda_check(cudaSetDevice(e->device), "cudaSetDevice");
    BookScenarios sc;
    sc.sc = scenarios;
    sc.n = n_scenarios;
    run_book(e, request, sc, nullptr, first_path, count, out);
  })
}
