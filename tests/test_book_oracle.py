"""CPU checks of the book restatement (oracle) and the book request types.

A book is many Phoenix trades on one universe path set under one common scenario set.  Its
restatement is pinned to the single-trade restatement (itself pinned to the reference's golden and
known answers): a book holding one trade on every universe asset, in order, over the whole grid
must reproduce that trade's own price path by path.  The other properties here are exact: trades
do not interact (a trade's result is the same alone and in the mix), scenarios do not interact,
and invalid books fail with the reference's error codes."""
from __future__ import annotations

import copy

import pytest

import oracle as O
from riga_gb300 import abi, workloads
from riga_gb300.types import BookRequest, BookTrade, MarketSnapshot


def _single_trade_book(req, paths):
    """A book whose universe is `req`'s market and whose one trade is `req`'s trade."""
    n = len(req.market.spots)
    b = BookRequest(copy.deepcopy(req.market), req.trade.steps, req.trade.maturity_years,
                    [BookTrade(copy.deepcopy(req.trade), list(range(n)))], copy.deepcopy(req.config),
                    copy.deepcopy(req.options))
    b.config.paths = paths
    b.config.trace_level = "off"
    return b


def _rec(r):
    return (r.path_id, r.knocked_out, r.ko_step, r.ki_hit, r.qualified_steps, r.paid_periods,
            r.pv, r.put_payoff, r.coupon_pv, r.memory_coupon_pv, r.funding, r.worst_final)


@pytest.mark.parametrize("scrambler", [abi.SCRAMBLE_DIGITAL_SHIFT, abi.SCRAMBLE_OWEN])
def test_one_trade_book_is_that_trades_price(scrambler):
    req = workloads.plain3(paths=256, steps=63)
    req.options.scrambler = scrambler
    book = _single_trade_book(req, 256)
    single = O.run_paths(req, 0, 64)
    booked = O.book_run_paths(book, None, 0, 64)
    assert [_rec(r) for r in booked] == [_rec(r) for r in single]
    a = O.price_put_leg(req, threads=4)
    b = O.price_book(book, None, threads=4)[0]
    assert (b.ko_count, b.ki_count, b.put_eligible_count, b.coupon_path_count) == \
        (a.ko_count, a.ki_count, a.put_eligible_count, a.coupon_path_count)
    assert b.pv == pytest.approx(a.pv, rel=1e-12)
    assert b.mc_error == pytest.approx(a.mc_error, rel=1e-10)


def test_one_trade_book_matches_the_halton_lane():
    req = workloads.plain3(paths=128, steps=40)
    req.config.variance_reduction.kind = "halton"
    book = _single_trade_book(req, 128)
    assert [_rec(r) for r in O.book_run_paths(book, None, 0, 32)] == [_rec(r) for r in O.run_paths(req, 0, 32)]


def test_trades_price_the_same_alone_and_in_the_mix():
    b = workloads.small_book(paths=256, n_trades=6)
    sc = [m for _, m in workloads.book_scenarios(b.universe)][:3]
    mixed = O.price_book(b, sc, threads=4)
    S = len(sc)
    for j in (0, 3, 5):
        alone = copy.deepcopy(b)
        alone.trades = [b.trades[j]]
        res = O.price_book(alone, sc, threads=4)
        for s in range(S):
            assert bytes(res[s]) == bytes(mixed[j * S + s])


def test_scenarios_do_not_interact():
    b = workloads.small_book(paths=128, n_trades=3)
    sc = [m for _, m in workloads.book_scenarios(b.universe)]
    full = O.price_book(b, sc[:5], threads=2)
    sub = O.price_book(b, [sc[4], sc[2]], threads=2)
    for j in range(3):
        assert bytes(sub[j * 2 + 0]) == bytes(full[j * 5 + 4])
        assert bytes(sub[j * 2 + 1]) == bytes(full[j * 5 + 2])


def test_a_truncated_trade_reads_the_head_of_the_universe_paths():
    """A trade shorter than the grid reads the first T_j steps of paths bridged over the whole
    grid, not a bridge over its own T_j steps: cutting the universe grid to T_j steps changes the
    trade's paths."""
    b = workloads.small_book(paths=64, n_trades=1, steps_per_year=12, max_years=3)
    t = b.trades[0]
    t.terms.steps = 12
    t.terms.maturity_years = 12 * b.dt
    t.terms.call_start_step = 0
    long_rec = O.book_run_paths(b, None, 0, 16)
    cut = copy.deepcopy(b)
    cut.universe_steps = 12
    cut.universe_maturity_years = 12 * b.dt
    cut.config.variance_reduction.dimension = len(cut.universe.spots) * 12
    short_rec = O.book_run_paths(cut, None, 0, 16)
    assert any(a.worst_final != c.worst_final for a, c in zip(long_rec, short_rec))


@pytest.mark.parametrize("mutate,code", [
    (lambda b: b.trades[0].underlyings.__setitem__(0, 99), "invalid_market_shape"),
    (lambda b: setattr(b.trades[0].terms, "steps", b.universe_steps + 1), "invalid_schedule"),
    (lambda b: setattr(b.config, "trace_level", "full"), "invalid_argument"),
    (lambda b: setattr(b.config.variance_reduction, "kind", "none"), "unsupported"),
    (lambda b: setattr(b.trades[0].terms, "strike", -1.0), "invalid_trade"),
    (lambda b: b.universe.spots.__setitem__(0, -5.0), "invalid_market"),
    (lambda b: setattr(b.config, "paths", 0), "invalid_paths"),
    (lambda b: setattr(b.universe, "as_of", ""), "missing_as_of"),
])
def test_invalid_books_keep_the_reference_error_codes(mutate, code):
    b = workloads.small_book(paths=32, n_trades=2)
    mutate(b)
    with pytest.raises(abi.RigaError) as e:
        O.price_book(b, None, threads=1)
    assert e.value.code == code


def test_scenarios_must_keep_the_base_correlation():
    b = workloads.small_book(paths=32, n_trades=2)
    sc = copy.deepcopy(b.universe)
    sc.correlation[0][1] = sc.correlation[1][0] = 0.1
    with pytest.raises(abi.RigaError) as e:
        O.price_book(b, [sc], threads=1)
    assert e.value.code == "invalid_argument"


def test_book_configuration_shapes():
    b = workloads.book(paths=1 << 18, n_trades=4096)
    assert len(b.trades) == 4096 and b.universe_steps == 1260 and len(b.universe.spots) == 20
    ns = {len(t.underlyings) for t in b.trades}
    years = {t.terms.steps // 252 for t in b.trades}
    assert ns == {1, 2, 3, 4, 5} and years == {1, 2, 3, 4, 5}
    for t in b.trades:
        assert len(set(t.underlyings)) == len(t.underlyings)
        assert 0.95 <= t.terms.knock_out_barrier <= 1.10 and 0.60 <= t.terms.coupon_barrier <= 0.80
        assert 0.50 <= t.terms.knock_in_barrier <= 0.70 and 0.01 <= t.terms.coupon_rate <= 0.03
    import numpy as np
    C = np.array(b.universe.correlation)
    assert np.allclose(C, C.T) and np.allclose(np.diag(C), 1.0) and np.linalg.eigvalsh(C).min() > 0
    assert len(workloads.book_scenarios(b.universe)) == 16
