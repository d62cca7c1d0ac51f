"""Pins the CPU oracle against the reference's own known answers and golden vector.

Every test cites the reference test it restates.  The oracle is test infrastructure: it is the
checker the CUDA engine is compared against in test_engine_gpu.py.
"""
from __future__ import annotations

import copy
import ctypes as C
import math

import pytest

import oracle as O
from conftest import json_close
from riga_gb300 import abi
from riga_gb300.types import (ImpliedVolGrid, MarketSnapshot, PhoenixTrade, PriceRequest,
                              SimulationConfig, VarianceReduction, result_to_json)


def lib():
    return O.lib()


# ----------------------------------------------------------------------- qmc.rs ----------------
def test_probit_matches_known_quantiles(known_answers):
    """qmc.rs:512-517"""
    ka = known_answers["probit"]
    for p, v, tol in zip(ka["p"], ka["value"], ka["tol"]):
        assert abs(lib().or_probit(p) - v) < tol


def test_radical_inverse_matches_van_der_corput(known_answers):
    """qmc.rs:502-510"""
    ka = known_answers["van_der_corput_base2"]
    assert [lib().or_radical_inverse(i, 2) for i in ka["index"]] == ka["value"]
    k3 = known_answers["radical_inverse_base3"]
    for i, v in zip(k3["index"], k3["value"]):
        assert abs(lib().or_radical_inverse(i, 3) - v) < k3["tol"]


def test_brownian_bridge_increments_have_the_right_variance():
    """qmc.rs:436-477 — same deterministic LCG uniforms, n = 64, dt = 1/252, 20,000 reps."""
    n, dt, reps = 64, 1.0 / 252.0, 20_000
    state = 12345
    mask = (1 << 64) - 1
    inc_m2 = term_m2 = 0.0
    probit = lib().or_probit
    for _ in range(reps):
        normals = []
        for _ in range(n):
            state = (state * 6364136223846793005 + 1) & mask
            normals.append(probit(0.5 + ((state >> 11) / float(1 << 53) - 0.5)))
        inc = O.bridge_increments(normals, dt)
        inc_m2 += sum(v * v for v in inc)
        term_m2 += sum(inc) ** 2
    inc_var = inc_m2 / (reps * n)
    term_var = term_m2 / reps
    assert abs(inc_var - dt) < 0.05 * dt
    assert abs(term_var - n * dt) < 0.1 * n * dt


def _sobol_uniform(v, dim_count, point, dim, seed):
    x = lib().or_sobol_int(v, dim_count, point, dim)
    x = lib().or_owen_scramble(x, dim, seed)
    return (x + 0.5) / 4294967296.0


def test_sobol_is_reproducible_and_well_distributed():
    """qmc.rs:479-500 — Sobol::new(8, 42): per-dimension means within 0.01 over 4096 points and
    seed 43 decorrelates the Owen scramble."""
    v = O.sobol_table(8)
    for dim in range(8):
        mean = sum(_sobol_uniform(v, 8, p, dim, 42) for p in range(1, 4097)) / 4096
        assert abs(mean - 0.5) < 0.01, (dim, mean)
    a = [lib().or_owen_scramble(lib().or_sobol_int(v, 8, 2, d), d, 42) for d in range(8)]
    b = [lib().or_owen_scramble(lib().or_sobol_int(v, 8, 2, d), d, 43) for d in range(8)]
    assert a != b


def test_sobol_direction_table_is_the_unit_initial_joe_kuo_table():
    """qmc.rs:247-262, 316-363: dim 0 is van der Corput; dim 1 uses x^2+x+1 with the unit initial
    values m1 = m2 = 1, so the recurrence m_k = 4m_{k-2} ^ m_{k-2} ^ 2m_{k-1} gives 1, 1, 7, 11, 13, 61."""
    v = O.sobol_table(3)
    assert [v[k] for k in range(32)] == [1 << (31 - k) for k in range(32)]
    masks = (C.c_uint32 * 6)()
    lib().or_primitive_polynomials(6, masks)
    assert list(masks) == [0b111, 0b1011, 0b1101, 0b10011, 0b11001, 0b100101]
    m = [v[32 + k] >> (31 - k) for k in range(6)]
    assert m == [1, 1, 7, 11, 13, 61]
    # the first Sobol points in dim 1 (unscrambled): 1/2, 3/4, 1/4
    assert [lib().or_sobol_int(v, 3, n, 1) / 2 ** 32 for n in (1, 2, 3)] == [0.5, 0.75, 0.25]


def test_primitive_polynomial_counts_by_degree():
    """qmc.rs:345-430: the count of primitive polynomials of degree d is phi(2^d - 1) / d."""
    masks = (C.c_uint32 * 1108)()
    lib().or_primitive_polynomials(1108, masks)
    by_degree = {}
    for mk in masks:
        d = mk.bit_length() - 1
        by_degree[d] = by_degree.get(d, 0) + 1
    assert [by_degree[d] for d in range(2, 13)] == [1, 2, 2, 6, 6, 18, 16, 48, 60, 176, 144]
    assert list(masks) == sorted(masks)


def test_halton_permutation_is_a_seeded_permutation():
    """qmc.rs:93-153: digit permutations are permutations, reproducible, seed dependent."""
    primes = (C.c_uint32 * 16)()
    lib().or_first_primes(16, primes)
    assert list(primes) == [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53]
    for base in (2, 3, 53):
        p42 = (C.c_uint32 * base)()
        p43 = (C.c_uint32 * base)()
        lib().or_halton_permutation(base, 42, p42)
        lib().or_halton_permutation(base, 43, p43)
        assert sorted(p42) == list(range(base))
        again = (C.c_uint32 * base)()
        lib().or_halton_permutation(base, 42, again)
        assert list(again) == list(p42)
    assert list(p42) != list(p43)


def test_owen_scramble_is_a_bijection_on_prefixes():
    """qmc.rs:292-308: nested scrambling maps distinct 8-bit prefixes to distinct prefixes."""
    outs = {lib().or_owen_scramble(x << 24, 5, 99) >> 24 for x in range(256)}
    assert len(outs) == 256


# ----------------------------------------------------------------------- correlation.rs -------
def test_two_factor_cholesky_reproduces_the_closed_form(known_answers):
    """correlation.rs:266-279"""
    rho = known_answers["cholesky_2x2"]["rho"]
    L = O.cholesky([[1.0, rho], [rho, 1.0]])
    assert abs(L[0][0] - 1.0) < 1e-15
    assert abs(L[1][0] - rho) < 1e-15
    assert abs(L[1][1] - math.sqrt(1.0 - rho * rho)) < 1e-15
    z = known_answers["cholesky_2x2"]["z"]
    y1 = L[1][0] * z[0] + L[1][1] * z[1]
    assert abs(y1 - (rho * z[0] + math.sqrt(1 - rho * rho) * z[1])) < 1e-15


def test_cholesky_reconstructs_and_is_lower_triangular(known_answers):
    """correlation.rs:281-305"""
    rows = known_answers["cholesky_3x3"]["rows"]
    L = O.cholesky(rows)
    for i in range(3):
        for j in range(i + 1, 3):
            assert L[i][j] == 0.0
        for j in range(3):
            assert abs(sum(L[i][k] * L[j][k] for k in range(3)) - rows[i][j]) < 1e-12


def test_non_psd_matrix_is_clamped(known_answers):
    """correlation.rs:307-330"""
    rows = known_answers["psd_clamp"]["rows"]
    assert O.min_eigenvalue(rows) < 0.0
    rep = O.psd_clamp(rows, 1e-8)
    assert O.min_eigenvalue(rep) >= -1e-9
    for i in range(3):
        assert abs(rep[i][i] - 1.0) < 1e-12
    L = O.cholesky(rep)
    for i in range(3):
        for j in range(3):
            assert abs(sum(L[i][k] * L[j][k] for k in range(3)) - rep[i][j]) < 1e-10


def test_cholesky_validation_rejects_malformed_matrices():
    """correlation.rs:332-337"""
    with pytest.raises(abi.RigaError):
        O.cholesky([[0.5, 0.0], [0.0, 1.0]])
    with pytest.raises(abi.RigaError):
        O.cholesky([[1.0, 2.0], [2.0, 1.0]])


# ----------------------------------------------------------------------- riga-market ----------
def test_flat_smile_collapses_to_the_constant_implied_vol(known_answers):
    """crates/riga-market/src/lib.rs:400-412"""
    ka = known_answers["flat_smile"]
    grid = ImpliedVolGrid(ka["maturities"], ka["strikes"],
                          [[ka["vol"]] * len(ka["strikes"]) for _ in ka["maturities"]])
    *_, surf = O.lv_calibrate(grid, ka["spot"], ka["rate"])
    for t in ka["t"]:
        for s in ka["s"]:
            assert abs(O.lv_sigma(surf, t, s) - ka["vol"]) < ka["tol"]


def test_calibrated_local_vol_matches_the_reference_grid(termsheet1, known_answers):
    """crates/riga-engine/src/fixture.rs:507-527"""
    ka = known_answers["termsheet1_lv_nodes"]
    req = termsheet1.request
    for f, s, expected in ka["cases"]:
        *_, surf = O.lv_calibrate(req.local_vol[f], req.market.spots[f], req.market.risk_free_rate)
        assert abs(O.lv_sigma(surf, ka["t"], s) - expected) < ka["tol"]


def test_fixture_market_inputs_and_trade_economics_are_mapped(termsheet1, known_answers):
    """crates/riga-engine/src/fixture.rs:471-505"""
    ka = known_answers["termsheet1_mapping"]
    r = termsheet1.request
    assert r.market.spots == ka["spots"]
    for v, e in zip(r.market.vols, ka["vols_approx"]):
        assert abs(v - e) < ka["vols_tol"]
    assert abs(r.market.risk_free_rate - ka["rate_approx"]) < ka["rate_tol"]
    assert r.market.dividend_yields == ka["dividends"]
    assert r.market.correlation[0][1] == ka["rho"]
    assert r.trade.initial_spots == ka["initial_spots"]
    assert (r.trade.strike, r.trade.knock_in_barrier, r.trade.knock_out_barrier) == (
        ka["strike"], ka["ki"], ka["ko"])
    assert (r.trade.coupon_barrier, r.trade.coupon_rate) == (ka["coupon_barrier"], ka["coupon_rate"])
    assert r.trade.memory_coupon
    assert r.trade.coupon_periods == ka["coupon_periods"]
    assert r.trade.fixed_first_coupon == ka["fixed_first_coupon"]
    assert r.trade.call_start_step == ka["call_start_step"]
    assert termsheet1.market_is_pinned
    assert len(r.local_vol) == 2
    assert [len(r.local_vol[0].maturities_years), len(r.local_vol[0].strikes)] == ka["grid_shape"]


def test_date_conversion_counts_actual_days_and_weekdays(known_answers):
    """crates/riga-engine/src/fixture.rs:531-538"""
    from riga_gb300.fixture import civil_day_number, remaining_business_steps

    ka = known_answers["termsheet1_dates"]
    years, weekdays = remaining_business_steps(ka["as_of"], ka["final"])
    assert abs(years - ka["days"] / 365.0) < 2.3e-16
    assert ka["weekdays_range"][0] < weekdays < ka["weekdays_range"][1]
    assert civil_day_number(ka["final"]) - civil_day_number(ka["as_of"]) == ka["days"]


# ----------------------------------------------------------------------- the pricer -----------
def test_termsheet1_golden_matches_structured_result(termsheet1, golden_result):
    """crates/riga-engine/src/lib.rs:489-498: the full PriceResult JSON within 1e-12 — the oracle
    reproduces the reference's golden vector (pseudo-random lane, Dupire LV, 30,000 paths)."""
    res = O.price_put_leg(termsheet1.request, threads=1)
    got = result_to_json(res, termsheet1.request)
    assert json_close(got, golden_result) == []


def test_termsheet1_put_is_inside_documented_relative_tolerance(termsheet1, golden_result):
    """crates/riga-engine/src/lib.rs:459-487"""
    res = O.price_put_leg(termsheet1.request, threads=1)
    e = termsheet1.expected
    assert abs(res.legs.down_and_in_put - e["put_pv"]) / e["put_pv"] <= e["relative_tolerance"]
    assert abs(res.ki_probability - e["ki_probability"]) <= e["ki_probability_tolerance"]


def _small(termsheet1, paths=512, lane="none"):
    r = copy.deepcopy(termsheet1.request)
    r.config.paths = paths
    r.config.path_block_size = 128
    if lane != "none":
        r.config.variance_reduction = VarianceReduction(lane, r.trade.steps * 2)
    return r


@pytest.mark.parametrize("lane", ["none", "sobol", "halton"])
def test_ko_gates_the_put_but_not_ki(termsheet1, lane):
    """note.rs:381-401 and explain.rs:405-424"""
    no_call = _small(termsheet1, lane=lane)
    no_call.trade.knock_out_barrier = None
    early = copy.deepcopy(no_call)
    early.trade.knock_out_barrier = 1.0e-6
    a = O.price_put_leg(no_call, threads=1)
    b = O.price_put_leg(early, threads=1)
    assert a.ki_probability == b.ki_probability
    assert a.legs.down_and_in_put > 0.0
    assert b.legs.down_and_in_put == 0.0
    ra, rb = O.run_paths(no_call, 0, 512), O.run_paths(early, 0, 512)
    for x, y in zip(ra, rb):
        assert x.worst_final == y.worst_final and x.ki_hit == y.ki_hit
        assert y.knocked_out and y.put_payoff == 0.0


@pytest.mark.parametrize("lane", ["none", "sobol"])
def test_replayed_paths_aggregate_to_the_pricing_result(termsheet1, lane):
    """explain.rs:389-403 and note.rs:403-479: per-path records reproduce the aggregate legs,
    counts and transition moments."""
    r = _small(termsheet1, paths=2000, lane=lane)
    res = O.price_put_leg(r, threads=1)
    recs = list(O.run_paths(r, 0, 2000))
    n = len(recs)
    assert abs(sum(x.put_payoff for x in recs) / n - res.legs.down_and_in_put) < 1e-12
    assert abs(sum(x.ki_hit for x in recs) / n - res.ki_probability) < 1e-12

    def moments(vals):
        m = sum(vals) / len(vals)
        return m, (sum((v - m) ** 2 for v in vals) / (len(vals) - 1) if len(vals) > 1 else 0.0)

    cases = [(0, [x.funding for x in recs if x.knocked_out]),
             (1, [x.put_payoff for x in recs if x.ki_hit]),
             (2, [x.coupon_pv for x in recs if x.coupon_pv > 0.0])]
    for k, vals in cases:
        m, v = moments(vals)
        assert res.stats[k].output_count == len(vals)
        assert abs(res.stats[k].mean_payoff - m) < 1e-12
        assert abs(res.stats[k].variance_payoff - v) < 1e-12
    surviving = sum(1 for x in recs if not x.knocked_out)
    assert res.ledger[1].population_before == surviving
    assert res.ledger[1].population_after == sum(1 for x in recs if x.ki_hit and not x.knocked_out)


def test_same_request_gives_identical_results(termsheet1):
    """crates/riga-engine/src/lib.rs:500-506; and the chunked multi-threaded QMC run equals the
    sequential one within the reference's 1e-12 (only the summation order differs)."""
    r = _small(termsheet1, paths=8192, lane="sobol")
    a = result_to_json(O.price_put_leg(r, threads=1), r)
    b = result_to_json(O.price_put_leg(r, threads=1), r)
    assert a == b
    c = result_to_json(O.price_put_leg(r, threads=4), r)
    assert json_close(c, a, tol=1e-12) == []


def test_invalid_inputs_have_uniform_error_shape(termsheet1):
    """crates/riga-engine/src/lib.rs:595-607 plus the other validate() branches (lib.rs:209-321)."""
    def code(mut):
        r = copy.deepcopy(termsheet1.request)
        mut(r)
        with pytest.raises(abi.RigaError) as e:
            O.price_put_leg(r, threads=1)
        return e.value.code

    def corr(r):
        r.market.correlation = [[1.0, 2.0], [2.0, 1.0]]
    assert code(corr) == "invalid_market"
    assert code(lambda r: setattr(r, "as_of", "")) == "missing_as_of"
    assert code(lambda r: setattr(r, "as_of", "2026-09-08")) == "as_of_mismatch"
    assert code(lambda r: setattr(r.config, "paths", 0)) == "invalid_paths"
    assert code(lambda r: setattr(r.trade, "steps", 0)) == "invalid_schedule"
    assert code(lambda r: setattr(r.trade, "knock_out_barrier", -1.0)) == "invalid_trade"
    assert code(lambda r: setattr(r.trade, "coupon_rate", -0.1)) == "invalid_trade"
    assert code(lambda r: setattr(r.market, "spots", [1.0])) == "invalid_market_shape"
    assert code(lambda r: setattr(r, "local_vol", r.local_vol[:1])) == "invalid_local_vol"


@pytest.mark.slow
def test_qmc_reduces_the_put_estimator_variance(termsheet1):
    """crates/riga-engine/src/lib.rs:653-688: over 12 seeds at 4096 paths the Sobol+Owen estimator
    of the PUT leg has lower variance than the pseudo-random one."""
    def measure(kind):
        vals = []
        for seed in range(1, 13):
            r = _small(termsheet1, paths=4096, lane=kind)
            r.config.seed = seed
            vals.append(O.price_put_leg(r, threads=4).legs.down_and_in_put)
        m = sum(vals) / len(vals)
        return sum((v - m) ** 2 for v in vals) / (len(vals) - 1)

    mc, sobol = measure("none"), measure("sobol")
    assert sobol > 0.0 and mc / sobol > 1.0


def _three_asset_request(paths=1024, steps=63):
    """A 3-asset flat-vol worst-of Phoenix (the 3-asset plain configuration, shortened)."""
    n = 3
    return PriceRequest(
        trade=PhoenixTrade("plain3", [100.0] * n, 0.25, steps, 1.0, 0.60, 1.00, 0.70, 0.02, True,
                           4, False, 5),
        market=MarketSnapshot("2026-01-02", [100.0] * n, [0.20, 0.25, 0.30], 0.03, [0.01] * n,
                              [[1.0 if i == j else 0.5 for j in range(n)] for i in range(n)]),
        config=SimulationConfig(paths, 4096, 1, "off", VarianceReduction("sobol", n * steps)),
        as_of="2026-01-02")


def test_n_asset_generalisation_orders_qmc_dimensions_by_step_then_factor():
    """note.rs:89-98 generalised: dim(step, factor) = N·step + factor; an asset whose vol is zero
    and whose correlation row is the identity leaves the other assets' paths unchanged."""
    r3 = _three_asset_request()
    res3 = O.price_put_leg(r3, threads=1)
    assert 0.0 < res3.ki_probability < 1.0
    assert abs(res3.pv - res3.legs.total) == 0.0
    recs = O.run_paths(r3, 0, 64)
    assert all(rec.sobol_index == rec.path_id + 1 for rec in recs)


def test_risk_batch_follows_the_reference_scenario_set(termsheet1):
    """crates/riga-risk/src/lib.rs:222-241 (scenario_count 1+4n+4) and :53-92 (central formulas
    recomputed from the scenario prices)."""
    r = _small(termsheet1, paths=256, lane="sobol")
    cfg = abi.CentralDifferenceConfig(0.01, 0.01, 1e-4, 0.01, abi.CRN)
    rep = O.price_risk_batch(r, cfg, threads=2)
    assert rep.scenario_count == 1 + 4 * 2 + 4
    base = O.price_put_leg(r, threads=1)
    assert abs(rep.base.pv - base.pv) < 1e-14
    a = rep.assets[0]
    h = r.market.spots[0] * 0.01
    assert abs(a.delta.value - (a.spot_up_pv - a.spot_down_pv) / (2 * h)) < 1e-12
    assert abs(a.gamma.value - (a.spot_up_pv - 2 * rep.base.pv + a.spot_down_pv) / (h * h)) < 1e-9
    up = copy.deepcopy(r)
    up.market.spots[0] += h
    assert abs(O.price_put_leg(up, threads=1).pv - a.spot_up_pv) < 1e-14
    cfg_bad = abi.CentralDifferenceConfig(0.01, 0.01, 1e-4, 0.01, abi.NO_CRN)
    with pytest.raises(abi.RigaError) as e:
        O.price_risk_batch(r, cfg_bad)
    assert e.value.code == "no_crn_rejected"
    cfg_vol = abi.CentralDifferenceConfig(0.01, 0.9, 1e-4, 0.01, abi.CRN)
    with pytest.raises(abi.RigaError) as e:
        O.price_risk_batch(r, cfg_vol)
    assert e.value.code == "invalid_volatility_bump"


# ----------------------------------------------------------------------- portable exp/log -----
def _ulp_diff(a: float, b: float) -> int:
    import struct

    ia = struct.unpack("<q", struct.pack("<d", a))[0]
    ib = struct.unpack("<q", struct.pack("<d", b))[0]
    return abs(ia - ib)


def test_portable_exp_log_are_within_two_ulp_of_libm():
    """The deterministic exp/log shared with the GPU parity kernel (Cody–Waite + Taylor; artanh
    series) stay within 2 ulp of the platform libm over the ranges the path uses."""
    import random

    rng = random.Random(7)
    L = lib()
    worst_e = worst_l = 0
    for _ in range(100_000):
        x = rng.uniform(-40.0, 10.0)
        worst_e = max(worst_e, _ulp_diff(L.or_pexp(x), math.exp(x)))
        y = math.exp(rng.uniform(-40.0, 12.0))
        worst_l = max(worst_l, _ulp_diff(L.or_plog(y), math.log(y)) if abs(math.log(y)) > 1e-3 else 0)
    assert worst_e <= 2 and worst_l <= 2, (worst_e, worst_l)
    assert L.or_pexp(0.0) == 1.0 and L.or_plog(1.0) == 0.0
    assert L.or_pexp(-800.0) == 0.0 and L.or_pexp(800.0) == math.inf
    assert L.or_plog(0.0) == -math.inf and math.isnan(L.or_plog(-1.0))
    for x in (1e-300, 5e-324, 2.0 ** -1030, 0.1, 0.5, 2.0, 1e300):
        assert _ulp_diff(L.or_plog(x), math.log(x)) <= 2, x


def test_portable_math_oracle_stays_close_to_the_libm_oracle(termsheet1, golden_result):
    """Replacing libm's per-path exp/log by the portable ones (the calibration and the discount
    factors stay libm's in both modes) keeps the golden PriceResult within the reference's own
    1e-12 (crates/riga-engine/src/lib.rs:489-498)."""
    with O.portable_math():
        res = O.price_put_leg(termsheet1.request, threads=1)
    got = result_to_json(res, termsheet1.request)
    assert json_close(got, golden_result, tol=1e-12) == []


def test_production_halton_lane_is_a_scrambled_radical_inverse():
    """The engine's full-dimension Halton lane (no counterpart in the reference): each digit goes
    through an invertible affine map mod the prime base, so points 1..b-1 of base b take b-1
    distinct first digits — one per stratum of width 1/b — and every value lies in [0, 1)."""
    L = lib()
    for dim, b in ((0, 2), (7, 19), (6299, 62989)):
        us = [L.or_halton_hashed_u(n, b, 1, dim) for n in range(1, min(b, 4000))]
        assert all(0.0 <= u < 1.0 for u in us)
        strata = {int(u * b) for u in us}
        assert len(strata) == len(us)
    # two dimensions of neighbouring large primes are not in lockstep (the unscrambled radical
    # inverse n/b would give a correlation near 1 over the first points)
    import statistics
    a = [L.or_halton_hashed_u(n, 62983, 1, 6298) for n in range(1, 4001)]
    c = [L.or_halton_hashed_u(n, 62989, 1, 6299) for n in range(1, 4001)]
    assert abs(statistics.correlation(a, c)) < 0.1
