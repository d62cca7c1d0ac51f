"""GPU tests of book pricing (rg_price_book / rg_book_run_paths) through the C ABI.

Bars, each written in its assertion:
* FP64 parity mode against the oracle on the same scrambled points: per (path, trade, scenario)
  record the KO step, the qualifying-coupon count and the paid periods exactly, payoffs within
  1e-12 relative; aggregated results within 1e-12 relative (the oracle runs the portable exp/log
  the parity kernels use).
* A one-trade book on every universe asset over the whole grid is bit-identical to that trade
  priced alone by rg_price_put_leg (FP64).
* FP32 production mode: every (trade, scenario) price within min(0.1 × MC standard error, 1bp of
  notional) of the FP64 book on the same points.
* Continuous batching precondition: a trade's FP32 result is bit-identical alone and in the mix.
"""
from __future__ import annotations

import copy

import pytest

import oracle as O
from riga_gb300 import abi, workloads
from riga_gb300.build import build_library
from riga_gb300.engine import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    build_library()
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(autouse=True)
def portable_oracle():
    O.set_portable_math(True)
    yield
    O.set_portable_math(False)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_fp64_book_records_match_the_oracle(engine):
    b = workloads.small_book(paths=256, n_trades=6)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:3]
    got = engine.book_run_paths_raw(b, sc, 0, 64)
    want = O.book_run_paths(b, sc, 0, 64)
    assert len(got) == len(want) == 64 * 6 * 3
    for g, w in zip(got, want):
        assert (g.path_id, g.knocked_out, g.ko_step, g.ki_hit, g.qualified_steps, g.paid_periods) == \
            (w.path_id, w.knocked_out, w.ko_step, w.ki_hit, w.qualified_steps, w.paid_periods)
        for f in ("pv", "put_payoff", "coupon_pv", "memory_coupon_pv", "funding", "worst_final"):
            assert _rel(getattr(g, f), getattr(w, f)) <= 1e-12, f


def test_fp64_book_prices_match_the_oracle(engine):
    b = workloads.small_book(paths=1024, n_trades=5)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:4]
    got = engine.price_book_raw(b, sc)
    want = O.price_book(b, sc, threads=8)
    for g, w in zip(got, want):
        assert (g.ko_count, g.ki_count, g.put_eligible_count, g.coupon_path_count) == \
            (w.ko_count, w.ki_count, w.put_eligible_count, w.coupon_path_count)
        assert _rel(g.pv, w.pv) <= 1e-12
        assert _rel(g.mc_error, w.mc_error) <= 1e-9


def _halton(b):
    b.config.variance_reduction = workloads.VarianceReduction("halton", b.config.variance_reduction.dimension)
    return b


def test_fp64_halton_book_matches_the_oracle(engine):
    """The book lanes on scrambled Halton points (the universe's normals by the FP64 permuted
    radical inverse, qmc.rs:93-153): per-path records against the oracle."""
    b = _halton(workloads.small_book(paths=256, n_trades=5))
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:2]
    got = engine.book_run_paths_raw(b, sc, 0, 64)
    want = O.book_run_paths(b, sc, 0, 64)
    for g, w in zip(got, want):
        assert (g.ko_step, g.qualified_steps, g.paid_periods) == (w.ko_step, w.qualified_steps, w.paid_periods)
        for f in ("pv", "worst_final"):
            assert _rel(getattr(g, f), getattr(w, f)) <= 1e-12, f


def test_fp32_halton_book_within_a_tenth_of_the_standard_error(engine):
    """FP32 Halton books take the integer radical inverse; every price stays within min(0.1 SE,
    1bp) of the FP64 book on the same points."""
    b64 = _halton(workloads.small_book(paths=1 << 14, n_trades=6, steps_per_year=52, max_years=2))
    b32 = copy.deepcopy(b64)
    b32.options = workloads.production_options()
    sc = [m for _, m in workloads.book_scenarios(b64.universe)][:4]
    r64 = engine.price_book_raw(b64, sc)
    r32 = engine.price_book_raw(b32, sc)
    for a, w in zip(r32, r64):
        assert abs(a.pv - w.pv) <= min(0.1 * w.mc_error, 1e-4)


def test_one_trade_book_is_bit_identical_to_price_put_leg(engine):
    req = workloads.plain3(paths=2048, steps=126)
    n = len(req.market.spots)
    from riga_gb300.types import BookRequest, BookTrade
    b = BookRequest(copy.deepcopy(req.market), req.trade.steps, req.trade.maturity_years,
                    [BookTrade(copy.deepcopy(req.trade), list(range(n)))], copy.deepcopy(req.config),
                    copy.deepcopy(req.options))
    booked = engine.book_run_paths_raw(b, None, 0, 512)
    single = engine.run_paths_raw(req, 0, 512)
    for g, w in zip(booked, single):
        assert (g.ko_step, g.qualified_steps, g.paid_periods, g.pv, g.worst_final) == \
            (w.ko_step, w.qualified_steps, w.paid_periods, w.pv, w.worst_final)


def test_fp32_book_within_a_tenth_of_the_standard_error(engine):
    b64 = workloads.small_book(paths=1 << 14, n_trades=8, steps_per_year=52, max_years=2)
    b32 = copy.deepcopy(b64)
    b32.options = workloads.production_options()
    sc = [m for _, m in workloads.book_scenarios(b64.universe)]
    r64 = engine.price_book_raw(b64, sc)
    r32 = engine.price_book_raw(b32, sc)
    for a, w in zip(r32, r64):
        bound = min(0.1 * w.mc_error, 1e-4)  # min(0.1 SE, 1bp of notional)
        assert abs(a.pv - w.pv) <= bound


def test_fp32_trade_is_bit_identical_alone_and_in_the_mix(engine):
    b = workloads.small_book(paths=1 << 13, n_trades=7, steps_per_year=52, max_years=2, fp32=True)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:5]
    mixed = engine.price_book_raw(b, sc)
    for j in (0, 4, 6):
        alone = copy.deepcopy(b)
        alone.trades = [b.trades[j]]
        res = engine.price_book_raw(alone, sc)
        for s in range(len(sc)):
            assert bytes(res[s]) == bytes(mixed[j * len(sc) + s])


def test_fp32_book_is_deterministic_across_calls(engine):
    b = workloads.small_book(paths=1 << 12, n_trades=5, steps_per_year=52, fp32=True)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:3]
    a = engine.price_book_raw(b, sc)
    c = engine.price_book_raw(b, sc)
    assert [bytes(x) for x in a] == [bytes(x) for x in c]


def test_book_errors_keep_the_reference_codes(engine):
    b = workloads.small_book(paths=64, n_trades=2)
    b.trades[1].underlyings[0] = 77
    with pytest.raises(abi.RigaError) as e:
        engine.price_book_raw(b)
    assert e.value.code == "invalid_market_shape"


def test_resident_book_replays_equal_the_one_shot_price(engine):
    """rg_book_create / rg_book_price: the graph-replayed price equals rg_price_book bit for bit,
    for several scenario sets and counts, whatever stage depth the autotuner picked."""
    b = workloads.small_book(paths=1 << 13, n_trades=9, steps_per_year=52, max_years=3, fp32=True)
    sc = [m for _, m in workloads.book_scenarios(b.universe)]
    with engine.resident_book(b) as rb:
        for subset in (sc, sc[:5], sc, sc[3:11], None):
            got = rb.price_raw(subset)
            want = engine.price_book_raw(b, subset)
            assert [bytes(x) for x in got] == [bytes(x) for x in want]
        assert rb.tuned_stage(16) in (8, 16, 32, 64)
        assert rb.tuned_stage(5) in (8, 16, 32)
        assert rb.tuned_stage(7) == 0


def test_resident_book_keeps_the_reference_error_codes(engine):
    b = workloads.small_book(paths=1 << 10, n_trades=2, steps_per_year=12, fp32=True)
    with engine.resident_book(b) as rb:
        sc = copy.deepcopy(b.universe)
        sc.spots = sc.spots[:-1]
        with pytest.raises(abi.RigaError) as e:
            rb.price_raw([sc])
        assert e.value.code == "invalid_market_shape"
    b64 = workloads.small_book(paths=64, n_trades=1)
    with pytest.raises(abi.RigaError) as e:
        engine.resident_book(b64)
    assert e.value.code == "unsupported"


def test_resident_universe_increments_equal_a_fresh_generation(engine):
    """An engine keeps the universe increments of its last one-chunk FP32 book; a book on the same
    universe, grid and path set scans them again without regenerating, and prices exactly as a
    fresh engine that generates them.  A changed correlation is generated afresh."""
    b = workloads.small_book(paths=1 << 13, n_trades=7, steps_per_year=52, max_years=2, fp32=True)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:4]
    engine.price_book_raw(b, sc)
    sub = copy.deepcopy(b)
    sub.trades = b.trades[2:5]
    fresh = Engine(0)
    try:
        reused = engine.price_book_raw(sub, sc)
        assert [bytes(x) for x in reused] == [bytes(x) for x in fresh.price_book_raw(sub, sc)]
        b2 = copy.deepcopy(sub)
        n = len(b2.universe.correlation)
        b2.universe.correlation = [[1.0 if i == j else 0.98 * b2.universe.correlation[i][j] for j in range(n)]
                                   for i in range(n)]
        sc2 = [m for _, m in workloads.book_scenarios(b2.universe)][:4]
        r2 = engine.price_book_raw(b2, sc2)
        assert [bytes(x) for x in r2] == [bytes(x) for x in fresh.price_book_raw(b2, sc2)]
        assert r2[0].pv != reused[0].pv
    finally:
        fresh.close()


# ------------------------------------------------------------------ per-trade bump sets -------
def _bumped_markets(universe, underlyings, n):
    """The 16 universe markets of one trade's bump set, built here from the published rule
    (rg_book_trade_bump) — the check that the library applied each bump to the right asset."""
    from riga_gb300.engine import trade_bump

    out = []
    for k in range(abi.BOOK_TRADE_SCENARIOS):
        kind, first, second, size = trade_bump(n, k)
        m = copy.deepcopy(universe)
        if kind == abi.BUMP_SPOT:
            m.spots[underlyings[first]] *= 1.0 + size
        elif kind == abi.BUMP_SPOT_PAIR:
            m.spots[underlyings[first]] *= 1.0 + size
            m.spots[underlyings[second]] *= 1.0 + size
        elif kind == abi.BUMP_VOL:
            m.vols[underlyings[first]] = max(0.0, m.vols[underlyings[first]] + size)
        elif kind == abi.BUMP_RATE:
            m.risk_free_rate += size
        out.append(m)
    return out


@pytest.mark.parametrize("fp32", [False, True])
def test_per_trade_bumps_equal_the_bumped_markets(engine, fp32):
    """rg_price_book_trade_bumps prices trade j under its own 16 scenarios.  For trades of every
    underlying count, the same 16 bumped universe markets given as a common scenario list price that
    trade to the same bytes: the bump set is exactly the published rule, applied to the trade's own
    underlyings, on the same paths and arithmetic."""
    b = workloads.small_book(paths=1024 if not fp32 else 8192, n_trades=10, fp32=fp32)
    per = engine.price_book_trade_bumps_raw(b)
    S = abi.BOOK_TRADE_SCENARIOS
    assert len(per) == len(b.trades) * S
    seen = set()
    for j, bt in enumerate(b.trades):
        n = len(bt.underlyings)
        if n in seen:
            continue
        seen.add(n)
        common = engine.price_book_raw(b, _bumped_markets(b.universe, bt.underlyings, n))
        for k in range(S):
            assert bytes(per[j * S + k]) == bytes(common[j * S + k]), (j, n, k)
    assert len(seen) >= 3


def test_resident_per_trade_bumps_replay_the_one_shot_price(engine):
    b = workloads.small_book(paths=8192, n_trades=10, fp32=True)
    one = engine.price_book_trade_bumps_raw(b)
    with engine.resident_book(b) as rb:
        first = rb.price_trade_bumps_raw()
        again = rb.price_trade_bumps_raw()
        half = rb.price_trade_bumps_raw((0.005, 0.0, 0.0))  # other sizes: recaptured tables
        back = rb.price_trade_bumps_raw()
    assert [bytes(x) for x in first] == [bytes(x) for x in one] == [bytes(x) for x in again] == \
        [bytes(x) for x in back]
    assert [bytes(x) for x in half] != [bytes(x) for x in one]
