"""Replay materialisation: the f32 spot cube of a priced trade's path range.

The cube is the PathCube layout of crates/riga-engine/src/pathcube.rs:19-35 ([path][time][factor])
filled with the spots explain::run_paths holds after each multiplicative step
(crates/riga-engine/src/explain.rs:183-193).  CPU tests pin the oracle's cube against its own
records and, in the pseudo-random lane, against PathCube's gbm_evolve of the same ChaCha8 block;
the GPU test checks the device cube against the oracle's bit for bit.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

import oracle as O
from riga_gb300 import abi, workloads
from riga_gb300.types import VarianceReduction


def _records_equal(a, b):
    fields = ("path_id", "ko_step", "qualified_steps", "paid_periods", "ki_hit", "pv", "put_payoff",
              "coupon_pv", "memory_coupon_pv", "funding", "worst_final")
    for x, y in zip(a, b):
        for f in fields:
            assert getattr(x, f) == getattr(y, f), (x.path_id, f)


def test_oracle_cube_records_equal_run_paths():
    r = workloads.plain3(64, steps=126)
    cube, recs = O.materialize_paths(r, 5, 40)
    _records_equal(recs, O.run_paths(r, 5, 40))
    assert cube.shape == (40 * 126 * 3,)


def test_oracle_cube_last_step_gives_the_worst_final():
    """worst_final = min_f S_f(T)/S0_f (note.rs:145-148): the cube's last row, in f32."""
    r = workloads.plain3(64, steps=126)
    cube, recs = O.materialize_paths(r, 0, 64)
    c = cube.reshape(64, 126, 3)
    init = np.asarray(r.trade.initial_spots)
    worst = (c[:, -1, :].astype(np.float64) / init).min(axis=1)
    ref = np.array([x.worst_final for x in recs])
    np.testing.assert_allclose(worst, ref, rtol=2e-7)


def test_oracle_cube_knock_out_step_is_visible_in_the_cube():
    """The first step at or after the call start where every S_f/S0_f >= the KO barrier is the
    record's ko_step (note.rs:192-218), read off the cube (f32 rounding margin allowed)."""
    r = workloads.plain3(256, steps=126)
    cube, recs = O.materialize_paths(r, 0, 256)
    c = cube.reshape(256, 126, 3).astype(np.float64) / np.asarray(r.trade.initial_spots)
    barrier = r.trade.knock_out_barrier
    checked = 0
    for i, rec in enumerate(recs):
        if rec.ko_step < 0:
            continue
        up = c[i].min(axis=1)
        assert up[rec.ko_step] >= barrier * (1 - 1e-6)
        assert np.all(up[r.trade.call_start_step:rec.ko_step] < barrier * (1 + 1e-6))
        checked += 1
    assert checked > 0


def test_oracle_mc_lane_cube_matches_pathcube_gbm_evolve():
    """Pseudo-random lane: the trade's normals are ChaCha8 StandardNormal draws in
    [path][step][factor] order (note.rs:123-127), the same stream generate_correlated_block
    lays out (pathcube.rs:37-66); evolving that block with gbm_evolve (log space, f32 shocks)
    reproduces the trade's multiplicative FP64 spot path to f32 accuracy."""
    r = workloads.plain3(8, steps=63)
    r.config.variance_reduction = VarianceReduction("none", 0)
    T, P = 63, 8
    cube, _ = O.materialize_paths(r, 0, P)
    L = np.linalg.cholesky(np.asarray(r.market.correlation, dtype=np.float64))
    block = O.generate_correlated_block(r.config.seed, P, T, L.tolist())
    dt = r.trade.maturity_years / T
    ev = O.gbm_evolve(r.market.spots, r.market.vols, r.market.risk_free_rate, r.market.dividend_yields, dt,
                      block, P, T)
    np.testing.assert_allclose(cube, np.ctypeslib.as_array(ev), rtol=2e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["plain3", "lv3", "mc"])
def test_device_cube_is_bit_identical_to_the_oracle(case):
    from riga_gb300.build import build_library
    from riga_gb300.engine import Engine

    O.set_portable_math(True)
    try:
        if case == "plain3":
            r = workloads.plain3(512, steps=252)
        elif case == "lv3":
            r = workloads.lv3(128, steps=252, fp32=False)
        else:
            r = workloads.plain3(256, steps=126)
            r.config.variance_reduction = VarianceReduction("none", 0)
        build_library()
        e = Engine(0)
        try:
            first, count = (0, r.config.paths) if case == "mc" else (17, r.config.paths - 40)
            pc, recs = e.materialize_paths(r, first, count)
            cube, orecs = O.materialize_paths(r, first, count)
            assert pc.data.shape == cube.shape
            assert np.array_equal(pc.data.view(np.uint32), cube.view(np.uint32))
            assert [x["ko_step"] for x in recs] == [x.ko_step for x in orecs]
            assert [x["pv"] for x in recs] == [x.pv for x in orecs]
            # without records, and with the FP32 production setting (ignored: always FP64)
            r32 = copy.deepcopy(r)
            r32.options.precision = abi.PRECISION_FP32
            pc2, none = e.materialize_paths(r32, first, count, with_records=False)
            assert none is None and np.array_equal(pc2.data, pc.data)
        finally:
            e.close()
    finally:
        O.set_portable_math(False)
