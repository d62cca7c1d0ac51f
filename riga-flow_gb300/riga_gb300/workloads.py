"""Seeded synthetic workloads of the benchmark configurations.

* ``plain3`` — 3-asset worst-of Phoenix under flat-vol correlated GBM: spots 100, vols
  0.20/0.25/0.30, uniform correlation 0.5, r = 0.03, q = 0.01, 3y, 756 daily steps, daily KO at
  100% from step 63, 12 quarterly 2% coupons with memory at a 70% barrier, final EKI at 60%,
  put strike 100%, Sobol points digitally shifted from seed 1.
* ``lv3_greeks`` — the same Phoenix terms on 3 assets under Dupire local vol: each asset's raw
  SVI smile (a, b, rho, m, sigma) is drawn from a SplitMix64 stream seeded 1 within
  a∈[0.01,0.04], b∈[0.05,0.2], rho∈[-0.7,-0.2], m∈[-0.1,0.1], sigma∈[0.1,0.3]; total variance
  w(k, T) = T·w_SVI(k), so the implied vol is sqrt(w_SVI(k)) on 40 log-moneyness × 24 expiries;
  the Dupire grid has 40 log-strike points; correlation 0.4; 15 CRN bumps (±1% spot per asset,
  +1 vol point per asset, +1bp rate, two cross-gamma corners (+1%, +1%) on pairs (0,1) and (0,2),
  −1 vol point per asset).

* ``lv5_large`` — the large fused run: a 5-asset worst-of Phoenix (same terms, 5y, 1260 daily
  steps, 20 quarterly coupons) under Dupire local vol, seeded SVI smiles (SplitMix64 seed 5) on
  64 log-moneyness × 32 expiries with a 64-point Dupire grid, correlation from a seeded 2-factor
  model (the book's loading rule), 2^24 Sobol or Halton points.

There is no public dataset or evaluation suite for this path; these seeded inputs stand in for
the configurations' shapes, sizes and value distributions.
"""
from __future__ import annotations

import copy
import math

from . import abi
from .types import (EngineOptions, ImpliedVolGrid, MarketSnapshot, PhoenixTrade, PriceRequest,
                    SimulationConfig, VarianceReduction)

MASK64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014): state += golden gamma, output = mix64(state)."""

    def __init__(self, seed: int):
        self.state = seed & MASK64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def phoenix_trade(n: int, steps: int = 756, years: float = 3.0, trade_id: str = "plain3") -> PhoenixTrade:
    return PhoenixTrade(trade_id=trade_id, initial_spots=[100.0] * n, maturity_years=years,
                        steps=steps, strike=1.00, knock_in_barrier=0.60, knock_out_barrier=1.00,
                        coupon_barrier=0.70, coupon_rate=0.02, memory_coupon=True,
                        coupon_periods=12 if steps == 756 else max(1, round(12 * steps / 756)),
                        fixed_first_coupon=False, call_start_step=63 if steps >= 63 else 0)


def production_options(lv_grid_x: int = 0) -> EngineOptions:
    return EngineOptions(scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, precision=abi.PRECISION_FP32,
                         dim_mode=abi.DIM_FULL, lv_grid_x=lv_grid_x)


def plain3(paths: int = 1 << 16, steps: int = 756, fp32: bool = False) -> PriceRequest:
    n = 3
    as_of = "2026-01-02"
    req = PriceRequest(
        trade=phoenix_trade(n, steps, 3.0 * steps / 756),
        market=MarketSnapshot(as_of, [100.0] * n, [0.20, 0.25, 0.30], 0.03, [0.01] * n,
                              [[1.0 if i == j else 0.5 for j in range(n)] for i in range(n)]),
        config=SimulationConfig(paths, 4096, 1, "off", VarianceReduction("sobol", n * steps)),
        as_of=as_of)
    req.options = production_options() if fp32 else EngineOptions(
        scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, precision=abi.PRECISION_FP64_PARITY,
        dim_mode=abi.DIM_FULL)
    return req


def svi_grids(n: int, seed: int = 1, n_k: int = 40, n_t: int = 24, years: float = 3.0,
              spot: float = 100.0):
    rng = SplitMix64(seed)
    ks = [-1.0 + 1.5 * i / (n_k - 1) for i in range(n_k)]           # log-moneyness in [-1, 0.5]
    mats = [years * (j + 1) / n_t for j in range(n_t)]
    grids, params = [], []
    for _ in range(n):
        a = rng.uniform(0.01, 0.04)
        b = rng.uniform(0.05, 0.2)
        rho = rng.uniform(-0.7, -0.2)
        m = rng.uniform(-0.1, 0.1)
        sig = rng.uniform(0.1, 0.3)
        params.append((a, b, rho, m, sig))
        w = [a + b * (rho * (k - m) + math.sqrt((k - m) ** 2 + sig * sig)) for k in ks]
        vols_row = [math.sqrt(x) for x in w]
        grids.append(ImpliedVolGrid(mats, [spot * math.exp(k) for k in ks], [list(vols_row) for _ in mats]))
    return grids, params


def lv3(paths: int = 1 << 20, steps: int = 756, fp32: bool = True) -> PriceRequest:
    n = 3
    as_of = "2026-01-02"
    grids, _ = svi_grids(n, years=3.0 * steps / 756)
    req = PriceRequest(
        trade=phoenix_trade(n, steps, 3.0 * steps / 756, "lv3"),
        market=MarketSnapshot(as_of, [100.0] * n, [0.25] * n, 0.03, [0.01] * n,
                              [[1.0 if i == j else 0.4 for j in range(n)] for i in range(n)]),
        config=SimulationConfig(paths, 4096, 1, "off", VarianceReduction("sobol", n * steps)),
        as_of=as_of, local_vol=grids)
    req.options = production_options(40) if fp32 else EngineOptions(
        scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, precision=abi.PRECISION_FP64_PARITY,
        dim_mode=abi.DIM_FULL, lv_grid_x=40)
    return req


def lv5_large(paths: int = 1 << 24, steps: int = 1260, fp32: bool = True, kind: str = "sobol") -> PriceRequest:
    n = 5
    as_of = "2026-01-02"
    years = 5.0 * steps / 1260
    grids, _ = svi_grids(n, seed=5, n_k=64, n_t=32, years=years)
    corr = book_universe(n_assets=n, n_factors=2, seed=4, as_of=as_of).correlation
    req = PriceRequest(
        trade=phoenix_trade(n, steps, years, "lv5_large"),
        market=MarketSnapshot(as_of, [100.0] * n, [0.25] * n, 0.03, [0.01] * n, corr),
        config=SimulationConfig(paths, 4096, 1, "off", VarianceReduction(kind, n * steps)),
        as_of=as_of, local_vol=grids)
    req.options = production_options(64) if fp32 else EngineOptions(
        scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, precision=abi.PRECISION_FP64_PARITY,
        dim_mode=abi.DIM_FULL, lv_grid_x=64)
    return req


def crn15_scenarios(req: PriceRequest):
    """Base + the 15 CRN bumps, as (label, MarketSnapshot, implied-vol shift) triples."""
    n = len(req.market.spots)
    base = req.market
    out = [("base", copy.deepcopy(base), [0.0] * n)]

    def spot_bump(mult):
        m = copy.deepcopy(base)
        m.spots = [s * k for s, k in zip(m.spots, mult)]
        return m

    for f in range(n):
        for sgn, lab in ((1, "+"), (-1, "-")):
            mult = [1.0] * n
            mult[f] = 1.0 + sgn * 0.01
            out.append((f"spot[{f}]{lab}", spot_bump(mult), [0.0] * n))
    for f in range(n):
        m = copy.deepcopy(base)
        m.vols = [v + (0.01 if i == f else 0.0) for i, v in enumerate(m.vols)]
        out.append((f"vol[{f}]+", m, [0.01 if i == f else 0.0 for i in range(n)]))
    m = copy.deepcopy(base)
    m.risk_free_rate += 1e-4
    out.append(("rate+", m, [0.0] * n))
    for (i, j) in ((0, 1), (0, 2)):
        mult = [1.0] * n
        mult[i] = mult[j] = 1.01
        out.append((f"cross[{i},{j}]++", spot_bump(mult), [0.0] * n))
    for f in range(n):
        m = copy.deepcopy(base)
        m.vols = [v - (0.01 if i == f else 0.0) for i, v in enumerate(m.vols)]
        out.append((f"vol[{f}]-", m, [-0.01 if i == f else 0.0 for i in range(n)]))
    return out


# ---------------------------------------------------------------------- books ----------------
# The book configuration: a 20-asset universe with a 4-factor correlation C = B·Bᵀ + diag(1 -
# Σ_k B_ik²), loadings B_ik ∈ U[0.2, 0.7] with every row rescaled so that Σ_k B_ik² <= 0.95 (an
# unscaled row could exceed 1, which is not a correlation), vols U[0.15, 0.45], spots 100,
# r = 0.03, q = 0.01, on a 5-year grid of 1260 daily steps.  Trades draw 1..5 distinct
# underlyings, a maturity of 1..5 years (252 steps a year, truncating the universe grid), a
# daily KO barrier U[0.95, 1.10] from step 63, a coupon barrier U[0.60, 0.80], an EKI barrier
# U[0.50, 0.70], and a quarterly coupon U[1%, 3%] with memory; put strike 100%.

BOOK_STEPS_PER_YEAR = 252


def book_universe(n_assets: int = 20, n_factors: int = 4, seed: int = 1, as_of: str = "2026-01-02") -> MarketSnapshot:
    rng = SplitMix64(seed)
    B = [[rng.uniform(0.2, 0.7) for _ in range(n_factors)] for _ in range(n_assets)]
    for row in B:
        ss = sum(b * b for b in row)
        if ss > 0.95:
            scale = math.sqrt(0.95 / ss)
            for k in range(n_factors):
                row[k] *= scale
    corr = [[1.0 if i == j else sum(B[i][k] * B[j][k] for k in range(n_factors))
             for j in range(n_assets)] for i in range(n_assets)]
    vols = [rng.uniform(0.15, 0.45) for _ in range(n_assets)]
    return MarketSnapshot(as_of, [100.0] * n_assets, vols, 0.03, [0.01] * n_assets, corr)


def book_trades(n_trades: int, universe_assets: int, seed: int = 2, max_years: int = 5,
                steps_per_year: int = BOOK_STEPS_PER_YEAR):
    from .types import BookTrade

    rng = SplitMix64(seed)
    dt = 1.0 / steps_per_year
    out = []
    for j in range(n_trades):
        n = 1 + rng.next_u64() % 5
        n = min(n, universe_assets)
        pool = list(range(universe_assets))
        under = []
        for _ in range(n):
            under.append(pool.pop(rng.next_u64() % len(pool)))
        years = 1 + rng.next_u64() % max_years
        steps = years * steps_per_year
        terms = PhoenixTrade(
            trade_id=f"book-{j}", initial_spots=[100.0] * n, maturity_years=steps * dt, steps=steps,
            strike=1.00, knock_in_barrier=rng.uniform(0.50, 0.70),
            knock_out_barrier=rng.uniform(0.95, 1.10), coupon_barrier=rng.uniform(0.60, 0.80),
            coupon_rate=rng.uniform(0.01, 0.03), memory_coupon=True, coupon_periods=4 * years,
            fixed_first_coupon=False, call_start_step=63)
        out.append(BookTrade(terms, under))
    return out


def book(paths: int = 1 << 18, n_trades: int = 4096, fp32: bool = True, n_assets: int = 20,
         max_years: int = 5, steps_per_year: int = BOOK_STEPS_PER_YEAR, seed: int = 1):
    """The book configuration (defaults: 4,096 trades, 2^18 Sobol paths, digital shift, seed 1)."""
    from .types import BookRequest

    universe = book_universe(n_assets, seed=seed)
    steps = max_years * steps_per_year
    config = SimulationConfig(paths, paths, 1, "off", VarianceReduction("sobol", n_assets * steps))
    options = production_options() if fp32 else EngineOptions(
        scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, dim_mode=abi.DIM_FULL)
    return BookRequest(universe, steps, steps / steps_per_year,
                       book_trades(n_trades, n_assets, seed + 1, max_years, steps_per_year), config, options)


def book_scenarios(universe: MarketSnapshot, groups: int = 4):
    """The book's common CRN set: the base and 15 bumps — every spot ±1%, every vol ±1 point, the
    rate ±1bp, spot +1% and -1% on each of `groups` contiguous asset groups, and every spot +1%
    together with every vol +1 point."""
    def bump(spot=None, vol=0.0, rate=0.0, members=None):
        m = copy.deepcopy(universe)
        idx = range(len(m.spots)) if members is None else members
        for a in idx:
            if spot is not None:
                m.spots[a] *= spot
            m.vols[a] += vol
        m.risk_free_rate += rate
        return m

    n = len(universe.spots)
    size = (n + groups - 1) // groups
    grp = [list(range(g * size, min(n, (g + 1) * size))) for g in range(groups)]
    out = [("base", copy.deepcopy(universe)), ("spot_up", bump(1.01)), ("spot_down", bump(0.99)),
           ("vol_up", bump(vol=0.01)), ("vol_down", bump(vol=-0.01)), ("rate_up", bump(rate=1e-4)),
           ("rate_down", bump(rate=-1e-4))]
    out += [(f"group{g}_spot_up", bump(1.01, members=grp[g])) for g in range(groups)]
    out += [(f"group{g}_spot_down", bump(0.99, members=grp[g])) for g in range(groups)]
    out.append(("spot_up_vol_up", bump(1.01, vol=0.01)))
    return out


def small_book(paths: int = 512, n_assets: int = 6, n_trades: int = 8, steps_per_year: int = 12,
               max_years: int = 3, fp32: bool = False, seed: int = 5):
    """A book small enough for the oracle: the book configuration's shapes at toy sizes."""
    b = book(paths, n_trades, fp32, n_assets, max_years, steps_per_year, seed)
    for bt in b.trades:
        bt.terms.call_start_step = min(bt.terms.call_start_step, bt.terms.steps // 4)
    return b
