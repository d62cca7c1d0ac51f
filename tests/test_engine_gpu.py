"""GPU parity tests: the CUDA engine, called through the C ABI, against the CPU oracle.

Bars (each written into the assertion that checks it):
* FP64 parity mode — per path, the knock-out step, the qualifying-coupon count and the number of
  paid periods equal the oracle's exactly; discounted payoffs agree within 1e-12 relative; the
  aggregate PriceResult within the reference's own 1e-12 (crates/riga-engine/src/lib.rs:453).
  The oracle runs with the portable deterministic exp/log the parity kernel uses: the Dupire
  calibration amplifies last-ulp differences between elementary-function libraries about a
  million-fold, so both sides must share one exp/log (the oracle's libm mode is pinned to the
  reference golden separately, in test_oracle.py).
* FP32 production mode — every price within min(0.1 × MC standard error, 1bp of notional) of the
  FP64 oracle on the same scrambled points; the same bound for the CRN bump differences.
"""
from __future__ import annotations

import copy
import math

import numpy as np
import pytest

import oracle as O
from conftest import json_close
from riga_gb300 import abi, gpu, workloads
from riga_gb300.build import build_library
from riga_gb300.engine import Engine
from riga_gb300.types import EngineOptions, VarianceReduction, result_to_json

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


def _lane(req, kind, dim=None, **opts):
    r = copy.deepcopy(req)
    r.config.variance_reduction = VarianceReduction(kind, dim if dim is not None else r.trade.steps * len(r.market.spots))
    r.options = EngineOptions(**opts)
    return r


def _termsheet(termsheet1, paths=2048, kind="sobol", **opts):
    r = _lane(termsheet1.request, kind, **opts)
    r.config.paths = paths
    return r


def max_rel_dev(gpu_recs, cpu_recs):
    worst = 0.0
    for g, c in zip(gpu_recs, cpu_recs):
        for f in ("pv", "put_payoff", "coupon_pv", "memory_coupon_pv", "funding", "worst_final"):
            a, b = getattr(g, f), getattr(c, f)
            if a != b:
                worst = max(worst, abs(a - b) / max(abs(b), 1e-300))
    return worst


def assert_records_match(gpu_recs, cpu_recs, rel=1e-12):
    mism = []
    for g, c in zip(gpu_recs, cpu_recs):
        assert g.path_id == c.path_id
        if (g.ko_step, g.qualified_steps, g.paid_periods, g.ki_hit) != (c.ko_step, c.qualified_steps, c.paid_periods, c.ki_hit):
            mism.append((g.path_id, (g.ko_step, c.ko_step), (g.qualified_steps, c.qualified_steps),
                         (g.paid_periods, c.paid_periods), g.worst_final))
            continue
        for f in ("pv", "put_payoff", "coupon_pv", "memory_coupon_pv", "funding", "worst_final"):
            a, b = getattr(g, f), getattr(c, f)
            assert abs(a - b) <= rel * max(abs(b), 1e-300) or a == b, (g.path_id, f, a, b)
    assert mism == [], f"event mismatches (path, ko, qualified, paid, worst): {mism[:5]}"


# ------------------------------------------------------------------ device ---------------------
def test_device_is_a_gb300(engine):
    """gpu.rs:500-512 and lib.rs:618-629"""
    gpu.ensure_available()
    assert gpu.arch() == "sm_103"
    assert gpu.device_name()


# ------------------------------------------------------------------ FP64 parity ---------------
@pytest.mark.parametrize("kind,extra", [("sobol", {}), ("halton", {}),
                                        ("sobol", {"scrambler": abi.SCRAMBLE_DIGITAL_SHIFT,
                                                   "dim_mode": abi.DIM_FULL})])
def test_fp64_parity_termsheet1_per_path(engine, termsheet1, kind, extra):
    """Reference two-asset Dupire-LV trade on the QMC lanes: per-path events exact, payoffs to
    1e-12 relative (note.rs:81-259, explain.rs:90-316)."""
    r = _termsheet(termsheet1, 2048, kind, **extra)
    g = engine.run_paths_raw(r, 0, 2048)
    c = O.run_paths(r, 0, 2048)
    assert_records_match(g, c)


@pytest.mark.parametrize("kind", ["sobol", "halton"])
def test_fp64_parity_termsheet1_price_result(engine, termsheet1, kind):
    """The whole PriceResult within the reference's 1e-12 (lib.rs:430-457)."""
    r = _termsheet(termsheet1, 4096, kind)
    r.config.trace_level = "aggregated"
    got = result_to_json(engine.price_raw(r), r)
    exp = result_to_json(O.price_put_leg(r, threads=1), r)
    assert json_close(got, exp, tol=1e-12) == []


def test_fp64_parity_three_asset_flat_vol(engine):
    """The 3-asset plain configuration (756 steps, digital shift) at 2048 paths."""
    r = workloads.plain3(2048)
    assert_records_match(engine.run_paths_raw(r, 0, 2048), O.run_paths(r, 0, 2048))
    got = result_to_json(engine.price_raw(r), r)
    exp = result_to_json(O.price_put_leg(r, threads=8), r)
    assert json_close(got, exp, tol=1e-12) == []


def test_fp64_parity_three_asset_local_vol(engine):
    """The 3-asset Dupire configuration (SVI smiles, 40-point grid) at 512 paths."""
    r = workloads.lv3(512, fp32=False)
    assert_records_match(engine.run_paths_raw(r, 0, 512), O.run_paths(r, 0, 512))


@pytest.mark.parametrize("case", ["plain3", "lv3", "termsheet1"])
def test_fp64_parity_is_bit_level(engine, termsheet1, case):
    """Same algorithm, operation order and exp/log on both sides: per-path outputs agree to the
    last bit (reported as the largest relative deviation, required to be 0)."""
    if case == "plain3":
        r = workloads.plain3(1024)
    elif case == "lv3":
        r = workloads.lv3(256, fp32=False)
    else:
        r = _termsheet(termsheet1, 1024)
    dev = max_rel_dev(engine.run_paths_raw(r, 0, r.config.paths), O.run_paths(r, 0, r.config.paths))
    assert dev == 0.0, dev


@pytest.mark.parametrize("n", [1, 4, 5])
def test_fp64_parity_other_asset_counts(engine, n):
    r = workloads.plain3(512, steps=126)
    r.trade.initial_spots = [100.0] * n
    r.market.spots = [100.0 + 3 * i for i in range(n)]
    r.market.vols = [0.2 + 0.03 * i for i in range(n)]
    r.market.dividend_yields = [0.01] * n
    r.market.correlation = [[1.0 if i == j else 0.3 for j in range(n)] for i in range(n)]
    r.config.variance_reduction = VarianceReduction("sobol", n * 126)
    assert_records_match(engine.run_paths_raw(r, 0, 512), O.run_paths(r, 0, 512))


def test_path_ranges_shard_exactly(engine):
    """Points come from the path index alone (qmc.rs:269-290): records of [a, b) ∪ [b, c) equal
    the records of [a, c) — the sharding property of the multi-rank path."""
    r = workloads.plain3(4096, steps=63)
    whole = engine.run_paths_raw(r, 0, 4096)
    lo = engine.run_paths_raw(r, 0, 1500)
    hi = engine.run_paths_raw(r, 1500, 2596)
    for a, b in zip(list(lo) + list(hi), whole):
        assert (a.path_id, a.pv, a.ko_step) == (b.path_id, b.pv, b.ko_step)


@pytest.mark.parametrize("fp32", [False, True])
def test_sharded_fused_launches_merge_to_one_launch(engine, fp32):
    """Two ranks' shards (first_path = rank × paths) of a CRN batch, merged by rg_merge_results,
    against one launch over both ranges: event counts exact, every price within 1e-12 relative
    (the shards only reorder FP64 additions)."""
    from riga_gb300 import sharding

    req = workloads.lv3(paths=1 << 14, steps=126, fp32=fp32)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(req)]
    parts = [engine.price_scenarios_raw(sharding.shard_request(req, r, 2), scen) for r in range(2)]
    whole_req = copy.deepcopy(req)
    whole_req.config.paths *= 2
    whole = engine.price_scenarios_raw(whole_req, scen)
    for s in range(len(scen)):
        m = sharding.merge(engine.lib, [parts[0][s], parts[1][s]], whole_req.config.paths)
        w = whole[s]
        assert (m.ko_count, m.ki_count, m.put_eligible_count, m.coupon_path_count) == \
            (w.ko_count, w.ki_count, w.put_eligible_count, w.coupon_path_count)
        assert m.pv == pytest.approx(w.pv, rel=1e-12)
        assert m.mc_error == pytest.approx(w.mc_error, rel=1e-9)


def test_repeated_launches_are_bit_identical(engine):
    r = workloads.plain3(1 << 14, steps=126)
    a = engine.price_raw(r)
    b = engine.price_raw(r)
    assert bytes(a) == bytes(b)
    r.options = workloads.production_options()
    assert bytes(engine.price_raw(r)) == bytes(engine.price_raw(r))


def test_ko_gates_the_put_but_not_ki(engine, termsheet1):
    """note.rs:381-401"""
    r = _termsheet(termsheet1, 1024)
    r.trade.knock_out_barrier = None
    e = copy.deepcopy(r)
    e.trade.knock_out_barrier = 1.0e-6
    a, b = engine.price_raw(r), engine.price_raw(e)
    assert a.ki_probability == b.ki_probability
    assert a.legs.down_and_in_put > 0.0 and b.legs.down_and_in_put == 0.0


# ------------------------------------------------------------------ FP32 production ------------
def _fp32_bound(res64: abi.PriceResult) -> float:
    return min(0.1 * res64.mc_error, 1e-4)


def test_fp32_matches_fp64_within_a_tenth_of_the_standard_error(engine):
    r = workloads.plain3(1 << 14)
    r64 = copy.deepcopy(r)
    r.options = workloads.production_options()
    res32 = engine.price_raw(r)
    res64 = O.price_put_leg(r64, threads=8)
    bound = _fp32_bound(res64)
    assert abs(res32.pv - res64.pv) <= bound, (res32.pv, res64.pv, bound)
    assert abs(res32.legs.down_and_in_put - res64.legs.down_and_in_put) <= bound
    assert abs(res32.ki_probability - res64.ki_probability) <= 2.0 / r.config.paths


def test_fp32_crn_batch_matches_fp64_scenarios(engine):
    """16 scenarios (base + 15 CRN bumps) of the 3-asset Dupire configuration in one fused FP32
    launch against the FP64 oracle priced scenario by scenario."""
    r = workloads.lv3(2048, steps=126, fp32=True)
    scen = workloads.crn15_scenarios(r)
    got = engine.price_scenarios_raw(r, [(m, s) for _, m, s in scen])
    r64 = workloads.lv3(2048, steps=126, fp32=False)
    exp = O.price_scenarios(r64, [(m, s) for _, m, s in scen], threads=8)
    for (label, _, _), g, e in zip(scen, got, exp):
        bound = _fp32_bound(e)
        assert abs(g.pv - e.pv) <= bound, (label, g.pv, e.pv, bound)
    # the CRN differences (delta numerators) keep the same bound
    for i in (1, 3, 5):
        dg, de = got[i].pv - got[i + 1].pv, exp[i].pv - exp[i + 1].pv
        assert abs(dg - de) <= _fp32_bound(exp[0]), (i, dg, de)


@pytest.mark.parametrize("steps,n_scen", [(1, 1), (2, 16), (5, 1), (63, 16), (64, 3), (65, 16),
                                          (129, 32), (300, 1), (1000, 16)])
def test_fp32_time_tiles_at_awkward_step_counts(engine, steps, n_scen):
    """The FP32 kernel walks time in subtrees of the bridge's bisection tree; step counts around
    and between the tile sizes, and 1-32 scenarios (256- and 1024-thread blocks, 32-256 paths per
    CTA), all price within the FP32 bound of the FP64 oracle.  One step makes every path pay the
    same (standard error 0), so the bound has a floor of 1e-7 of notional, about FP32's
    resolution at 1."""
    r = workloads.plain3(2048, steps=steps, fp32=True)
    r.trade.coupon_periods = max(1, min(12, steps // 3))
    r.trade.call_start_step = min(63, steps // 2)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(r)]
    scen = (scen * 2)[:n_scen]
    got = engine.price_scenarios_raw(r, scen)
    r64 = copy.deepcopy(r)
    r64.options.precision = abi.PRECISION_FP64_PARITY
    exp = O.price_scenarios(r64, scen, threads=8)
    for i, (g, e) in enumerate(zip(got, exp)):
        bound = max(_fp32_bound(e), 1e-7)
        assert abs(g.pv - e.pv) <= bound, (i, g.pv, e.pv, bound)


@pytest.mark.parametrize("n,lv,owen", [(1, False, False), (3, False, False), (3, True, False), (5, True, False),
                                        (3, True, True)])
def test_direct_and_tiled_fp32_kernels_agree(engine, n, lv, owen):
    """A single scenario at 2^18 paths runs on the direct kernel (one path per thread); the same
    scenario twice runs on the tiled kernel.  Both compute every path's FP32 payoff with the same
    operations in the same order, sum each 32-path chunk by the same butterfly and reduce the chunks
    in chunk order, so the prices are identical to the last bit."""
    if lv:
        r = workloads.lv5_large(paths=1 << 18, steps=252) if n == 5 else workloads.lv3(paths=1 << 18, steps=252)
    else:
        r = workloads.plain3(1 << 18, steps=252, fp32=True)
        if n != 3:
            r.trade.initial_spots = [100.0] * n
            r.market.spots = [100.0 + 3 * i for i in range(n)]
            r.market.vols = [0.2 + 0.03 * i for i in range(n)]
            r.market.dividend_yields = [0.01] * n
            r.market.correlation = [[1.0 if i == j else 0.3 for j in range(n)] for i in range(n)]
            r.config.variance_reduction = VarianceReduction("sobol", n * 252)
    if owen:
        r.options.scrambler = abi.SCRAMBLE_OWEN
    one = engine.price_raw(r)
    assert engine.last_timing().smem_bytes < 64 * 1024 and engine.last_timing().block == 256
    base = (copy.deepcopy(r.market), [0.0] * n)
    two = engine.price_scenarios_raw(r, [base, base])
    assert engine.last_timing().tile_steps > 0  # the tiled kernel
    for t in two:
        assert (t.pv, t.mc_error, t.ki_probability, t.ko_count, t.coupon_path_count) == \
            (one.pv, one.mc_error, one.ki_probability, one.ko_count, one.coupon_path_count)


def test_autotuned_tile_depth_keeps_prices(engine):
    """The tiled kernel's autotuner changes the paths per thread and the time-tile depth, never a
    path's arithmetic nor the 32-path chunks of the sums: 16 CRN scenarios priced with the
    autotuner off (the formula shape), then on (the first call tunes, the second reuses the tuned
    shape) are identical byte for byte."""
    lib = engine.lib
    r = workloads.lv3(paths=1 << 19, steps=252)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(r)]
    abi.check(lib, lib.rg_set_autotune(0))
    try:
        off = engine.price_scenarios_raw(r, scen)
        t_off = engine.last_timing().tile_steps
    finally:
        abi.check(lib, lib.rg_set_autotune(1))
    first = engine.price_scenarios_raw(r, scen)
    second = engine.price_scenarios_raw(r, scen)
    t_on = engine.last_timing().tile_steps
    assert t_off > 0 and t_on in (t_off, 24, 32, 48, 64, 80, 96, 128)
    assert engine.last_timing().paths_per_thread in (1, 2)
    for a, b, c in zip(off, first, second):
        assert bytes(a) == bytes(b) == bytes(c)


@pytest.mark.parametrize("n,lv", [(3, True), (5, True), (2, False)])
def test_every_tiled_shape_prices_identically(engine, n, lv):
    """Paths per thread (one, or two in packed FP32x2 arithmetic), tile depth and the paths per CTA
    tile (the block) are schedule only: every forced shape gives the same bytes, on a ragged path
    count."""
    lib = engine.lib
    paths = (1 << 15) + 77
    if lv:
        r = workloads.lv5_large(paths=paths, steps=252) if n == 5 else workloads.lv3(paths=paths, steps=252)
    else:
        r = workloads.plain3(paths, steps=252, fp32=True)
        r.trade.initial_spots = [100.0] * n
        r.market.spots = [100.0 + 3 * i for i in range(n)]
        r.market.vols = [0.2 + 0.03 * i for i in range(n)]
        r.market.dividend_yields = [0.01] * n
        r.market.correlation = [[1.0 if i == j else 0.3 for j in range(n)] for i in range(n)]
        r.config.variance_reduction = VarianceReduction("sobol", n * 252)
    scen = []
    for k in range(16):  # base, spot and vol bumps of each asset in turn, a rate bump
        m = copy.deepcopy(r.market)
        f = k % n
        if k % 4 == 1:
            m.spots[f] *= 1.01
        elif k % 4 == 2:
            m.vols[f] += 0.01
        elif k % 4 == 3:
            m.risk_free_rate += 1e-4
        scen.append((m, [0.01 if (lv and k % 4 == 2 and i == f) else 0.0 for i in range(n)]))
    got = []
    try:
        for ppt, tt, pb in ((1, 24, 0), (2, 24, 0), (2, 48, 0), (1, 32, 0), (1, 48, 32), (2, 32, 64)):
            abi.check(lib, lib.rg_set_tiled_shape(ppt, tt, pb))
            got.append(engine.price_scenarios_raw(r, scen))
            tm = engine.last_timing()
            assert (tm.paths_per_thread, tm.tile_steps) == (ppt, tt)
            assert tm.block * ppt == 16 * (pb or 64)  # 16 scenario slots x paths per CTA tile
    finally:
        abi.check(lib, lib.rg_set_tiled_shape(0, 0, 0))
    for g in got[1:]:
        assert [bytes(a) for a in g] == [bytes(a) for a in got[0]]


def test_resident_surfaces_reproduce_the_calibration():
    """Calibrated Dupire surfaces stay resident on the engine: a repeated request copies them
    instead of recalibrating (shorter prologue) and prices byte for byte the same; a request whose
    implied grid differs is calibrated afresh and matches a new engine's price of it."""
    r = workloads.lv3(paths=1 << 14, steps=252)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(r)]
    e1, e2 = Engine(0), Engine(0)
    try:
        a = e1.price_scenarios_raw(r, scen)
        t_cal = e1.last_timing().prologue_ms
        b = e1.price_scenarios_raw(r, scen)
        t_res = e1.last_timing().prologue_ms
        assert [bytes(x) for x in a] == [bytes(x) for x in b]
        assert t_res < t_cal, (t_res, t_cal)
        r2 = copy.deepcopy(r)
        r2.local_vol[0].vols = [[v + 0.001 for v in row] for row in r2.local_vol[0].vols]
        c = e1.price_scenarios_raw(r2, scen)
        assert c[0].pv != a[0].pv
        d = e2.price_scenarios_raw(r2, scen)
        assert [bytes(x) for x in c] == [bytes(x) for x in d]
        # the FP64 parity kernel reads the same resident surfaces
        r64 = workloads.lv3(256, steps=126, fp32=False)
        assert_records_match(e1.run_paths_raw(r64, 0, 256), e2.run_paths_raw(r64, 0, 256), rel=0.0)
        assert_records_match(e1.run_paths_raw(r64, 0, 256), O.run_paths(r64, 0, 256))
    finally:
        e1.close()
        e2.close()


def test_more_surfaces_than_resident_entries():
    """32 scenarios on 5 assets, every spot shifted per scenario: 160 surfaces in one launch, more
    than the engine keeps.  Priced twice on one engine (the second call mixes resident copies,
    fresh calibrations and evictions inside one calibration launch) and once on a fresh engine:
    all three identical byte for byte."""
    r = workloads.lv5_large(paths=1 << 12, steps=63)
    scen = []
    for k in range(32):
        m = copy.deepcopy(r.market)
        m.spots = [sp * (1.0 + 0.001 * (k + 1) * (i + 1)) for i, sp in enumerate(m.spots)]
        scen.append((m, [0.0] * 5))
    e1, e2 = Engine(0), Engine(0)
    try:
        a = e1.price_scenarios_raw(r, scen)
        b = e1.price_scenarios_raw(r, scen[::-1])[::-1]
        c = e2.price_scenarios_raw(r, scen)
        assert [bytes(x) for x in a] == [bytes(x) for x in c]
        assert [x.pv for x in b] == [x.pv for x in c]
    finally:
        e1.close()
        e2.close()


def test_uploaded_surfaces_are_resident():
    """rg_surfaces_upload calibrates the 16-scenario batch's surfaces ahead of pricing: the first
    priced call then copies them (prologue as short as a repeat's) and prices byte for byte what a
    fresh engine computes."""
    r = workloads.lv3(paths=1 << 14, steps=252)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(r)]
    e1, e2 = Engine(0), Engine(0)
    try:
        n = e1.upload_surfaces(r, scen)
        assert n >= 3
        a = e1.price_scenarios_raw(r, scen)
        t_first = e1.last_timing().prologue_ms
        b = e2.price_scenarios_raw(r, scen)
        t_cal = e2.last_timing().prologue_ms
        assert [bytes(x) for x in a] == [bytes(x) for x in b]
        assert t_first < t_cal, (t_first, t_cal)
    finally:
        e1.close()
        e2.close()


def test_large_fused_config_fp64_parity():
    """The large fused configuration's shape (5 assets, 64x32 SVI smiles, 64-point Dupire grid,
    2-factor correlation, 1260 steps) in the FP64 parity kernel, per path against the oracle."""
    eng = Engine(0)
    try:
        r = workloads.lv5_large(paths=128, fp32=False)
        assert_records_match(eng.run_paths_raw(r, 0, 128), O.run_paths(r, 0, 128))
    finally:
        eng.close()


@pytest.mark.parametrize("kind", ["sobol", "halton"])
def test_large_fused_config_fp32_within_bound(engine, kind):
    """FP32 production kernel on the large configuration (Sobol, and the Halton cross-check
    points) within min(0.1 SE, 1bp) of FP64 on the same 2^16 points.  The FP64 side is the parity
    kernel, whose per-path equality with the oracle on this shape is the test above: at a few
    thousand paths one knock-out event flipped by FP32 rounding moves the price by more than 1bp,
    so the bound needs a path count the CPU oracle cannot price within a test."""
    r = workloads.lv5_large(paths=1 << 16, kind=kind)
    r64 = workloads.lv5_large(paths=1 << 16, fp32=False, kind=kind)
    got = engine.price_raw(r)
    exp = engine.price_raw(r64)
    bound = _fp32_bound(exp)
    assert abs(got.pv - exp.pv) <= bound, (got.pv, exp.pv, bound)


def test_fp64_risk_batch_matches_the_oracle(engine, termsheet1):
    """crates/riga-risk/src/lib.rs:573-626 on the device: every scenario price within 1e-12."""
    r = _termsheet(termsheet1, 512)
    cfg = abi.CentralDifferenceConfig(0.01, 0.01, 1e-4, 0.01, abi.CRN)
    g = engine.price_risk_batch_raw(r, cfg)
    c = O.price_risk_batch(r, cfg, threads=8)
    assert g.scenario_count == c.scenario_count == 13
    for f in ("rate_up_pv", "rate_down_pv", "correlation_up_pv", "correlation_down_pv"):
        assert abs(getattr(g, f) - getattr(c, f)) <= 1e-12, f
    for i in range(2):
        for f in ("spot_up_pv", "spot_down_pv", "vol_up_pv", "vol_down_pv"):
            assert abs(getattr(g.assets[i], f) - getattr(c.assets[i], f)) <= 1e-12, (i, f)
    assert abs(g.base.pv - c.base.pv) <= 1e-12


# ------------------------------------------------------------------ errors --------------------
def test_invalid_requests_keep_the_reference_error_codes(engine, termsheet1):
    """lib.rs:595-607 and the validate() branches (lib.rs:209-321) through the C ABI."""
    def code(mut, kind="sobol"):
        r = _termsheet(termsheet1, 64, kind)
        mut(r)
        with pytest.raises(abi.RigaError) as e:
            engine.price_raw(r)
        return e.value.code

    def corr(r):
        r.market.correlation = [[1.0, 2.0], [2.0, 1.0]]
    assert code(corr) == "invalid_market"
    assert code(lambda r: setattr(r, "as_of", "")) == "missing_as_of"
    assert code(lambda r: setattr(r.config, "paths", 0)) == "invalid_paths"
    assert code(lambda r: setattr(r.trade, "steps", 0)) == "invalid_schedule"
    assert code(lambda r: setattr(r.market, "spots", [1.0])) == "invalid_market_shape"
    with pytest.raises(abi.RigaError) as e:
        engine.run_paths_raw(_termsheet(termsheet1, 64), 60, 10)
    assert e.value.code == "path_out_of_range"


# ------------------------------------------------------------------ gpu backend drop-ins --------
def test_gpu_worst_of_is_bit_identical_to_scalar():
    """gpu.rs:595-621: the same LCG inputs, compared bit for bit with the scalar minimum."""
    n = 4096
    seed = 0x12345678
    a = np.empty(n, np.float32)
    b = np.empty(n, np.float32)
    for i in range(n):
        seed = (seed * 1664525 + 1013904223) & 0xFFFFFFFF
        a[i] = np.float32(seed >> 8) / np.float32(1 << 24) * np.float32(1.8) + np.float32(0.2)
        seed = (seed * 1664525 + 1013904223) & 0xFFFFFFFF
        b[i] = np.float32(seed >> 8) / np.float32(1 << 24) * np.float32(1.8) + np.float32(0.2)
    out = gpu.worst_of(a, b)
    assert np.array_equal(out.view(np.uint32), np.minimum(a, b).view(np.uint32))
    w = gpu.resident_worst_of(a, b)
    w.reduce()
    assert np.array_equal(w.download(), out)



def test_production_halton_lane_matches_the_oracle(engine):
    """The full-dimension Halton lane (one prime per dimension, hashed affine digit scrambling):
    FP64 per-path records equal the oracle's, and the FP32 lane stays within min(0.1 SE, 1bp) of
    FP64 on the same points, through the tiled and the direct kernels."""
    r = workloads.plain3(512, steps=126)
    r.config.variance_reduction = VarianceReduction("halton", 3 * 126)
    r.options = EngineOptions(scrambler=abi.SCRAMBLE_DIGITAL_SHIFT, precision=abi.PRECISION_FP64_PARITY,
                              dim_mode=abi.DIM_FULL)
    assert_records_match(engine.run_paths_raw(r, 0, 512), O.run_paths(r, 0, 512))
    for paths in (1 << 14, 1 << 18):
        r64 = workloads.lv3(paths, steps=126, fp32=False)
        r64.config.variance_reduction = VarianceReduction("halton", 3 * 126)
        r32 = copy.deepcopy(r64)
        r32.options = workloads.production_options(40)
        want = engine.price_raw(r64)
        got = engine.price_raw(r32)
        assert abs(got.pv - want.pv) <= min(0.1 * want.mc_error, 1e-4), (paths, got.pv, want.pv)
