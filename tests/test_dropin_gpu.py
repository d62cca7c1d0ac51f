"""The `gpu`-backend drop-ins against the reference's own kernels, bit for bit.

The reference's `gpu` backend (crates/riga-engine/src/gpu.rs) runs two CUDA kernels held as source
in a Rust string: ``worst_of`` and ``lv_propagate`` (gpu.rs:27-76).  ``oracle/ref_gpu.py`` extracts
that source verbatim and compiles it with NVRTC's default arithmetic; these tests run it on the
same inputs as the engine's ``rg_worst_of``, ``rg_lv_terminal_spots`` and ``rg_resident_lv_*``
and require identical bits: every terminal spot and every knock-out step index equal.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle as O
import ref_gpu
from riga_gb300 import gpu
from riga_gb300.build import build_library

pytestmark = pytest.mark.gpu

_f = C.POINTER(C.c_float)


@pytest.fixture(scope="module")
def ref():
    build_library()
    lib = ref_gpu.lib()
    if lib is None:
        pytest.skip("the reference's gpu.rs kernel source has not been extracted into oracle/_ref")
    return lib


def _fp(a):
    return a.ctypes.data_as(_f)


def ref_lv(lib, normals, rows, axes, s0, refs, bar, paths, steps, dt, rate, divs):
    gx = axes.size // 2
    out = np.empty(paths * 2, np.float32)
    ko = np.empty(paths, np.int32)
    rc = lib.ref_lv_propagate(_fp(normals), _fp(rows), _fp(axes), gx, _fp(s0), float(refs[0]),
                              float(refs[1]), float(bar), paths, steps, float(dt), float(rate),
                              float(divs[0]), float(divs[1]), _fp(out), ko.ctypes.data_as(C.POINTER(C.c_int)))
    assert rc == 0, f"reference kernel: CUDA error {rc}"
    return out, ko


def lv_inputs(termsheet1, paths, steps=None, seed=7):
    """Per-step local-vol rows from the termsheet1 surfaces calibrated by the oracle (FP64, rounded
    to f32 as the reference's callers do), on the fixture's grid or a finer one of ``steps``
    steps over the same maturity; seeded standard normals [path, step, 2]."""
    req = termsheet1.request
    steps = steps or req.trade.steps
    dt = np.float32(req.trade.maturity_years / steps)
    gx = 96
    rows = np.zeros(2 * steps * gx, np.float32)
    axes = []
    for f in range(2):
        t_axis, log_s, v, _ = O.lv_calibrate(req.local_vol[f], req.market.spots[f], req.market.risk_free_rate)
        t_axis = np.asarray(t_axis)
        v = np.asarray(v).reshape(len(t_axis), gx)
        for s in range(steps):
            tc = min(max(s * float(dt), t_axis[0]), t_axis[-1])
            i = int(np.clip(np.searchsorted(t_axis, tc, side="left") - 1, 0, len(t_axis) - 2))
            w = (tc - t_axis[i]) / (t_axis[i + 1] - t_axis[i])
            rows[(f * steps + s) * gx:(f * steps + s + 1) * gx] = (1 - w) * v[i] + w * v[i + 1]
        axes += list(log_s)
    normals = np.random.default_rng(seed).standard_normal(paths * steps * 2).astype(np.float32)
    return normals, rows, np.asarray(axes, np.float32), steps, dt


def _market(termsheet1):
    req = termsheet1.request
    s0 = np.asarray(req.market.spots, np.float32)
    refs = np.asarray(req.trade.initial_spots, np.float32)
    divs = np.asarray(req.market.dividend_yields, np.float32)
    return s0, refs, divs, np.float32(req.market.risk_free_rate)


@pytest.mark.parametrize("paths,steps,bar", [(1024, None, 1.1), (1000, None, 1.02), (2048, 1260, 1.05)])
def test_lv_terminal_spots_equal_the_reference_kernel(ref, termsheet1, paths, steps, bar):
    """gpu.rs:209-277 on the fixture's grid, on a ragged path count, and on a 1,260-step grid."""
    normals, rows, axes, steps, dt = lv_inputs(termsheet1, paths, steps)
    s0, refs, divs, rate = _market(termsheet1)
    out, ko = gpu.lv_terminal_spots(normals, rows, axes, s0, refs, bar, paths, steps, dt, rate, divs)
    r_out, r_ko = ref_lv(ref, normals, rows, axes, s0, refs, bar, paths, steps, dt, rate, divs)
    assert np.array_equal(out.view(np.uint32), r_out.view(np.uint32))
    assert np.array_equal(ko, r_ko)
    assert (ko >= 0).any() and (ko < 0).any()  # both branches of the knock-out test are exercised


def test_resident_lv_runs_equal_the_reference_kernel(ref, termsheet1):
    """gpu.rs:409-488: each resident run under a spot bump equals the reference kernel's launch."""
    paths = 2048
    normals, rows, axes, steps, dt = lv_inputs(termsheet1, paths)
    base, refs, divs, rate = _market(termsheet1)
    res = gpu.resident_lv(normals, rows, axes, paths, steps, dt)
    for bump in (np.float32(1.0), np.float32(1.005), np.float32(0.99)):
        s0 = base * bump
        res.run(s0, refs, 1.1, rate, divs)
        rt, rk = res.download()
        t, k = ref_lv(ref, normals, rows, axes, s0, refs, 1.1, paths, steps, dt, rate, divs)
        assert np.array_equal(rt.view(np.uint32), t.view(np.uint32))
        assert np.array_equal(rk, k)


def test_worst_of_equals_the_reference_kernel(ref):
    """gpu.rs:28-31 ``a < b ? a : b`` including its edge cases: signed zeros, infinities and NaN
    in either operand (a NaN in ``a`` yields ``b``), on a ragged length."""
    rng = np.random.default_rng(3)
    n = 10007
    a = rng.uniform(0.2, 2.0, n).astype(np.float32)
    b = rng.uniform(0.2, 2.0, n).astype(np.float32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0], np.float32)
    a[:36] = np.repeat(special, 6)
    b[:36] = np.tile(special, 6)
    out = gpu.worst_of(a, b)
    r = np.empty(n, np.float32)
    assert ref.ref_worst_of(_fp(a), _fp(b), _fp(r), n) == 0
    assert np.array_equal(out.view(np.uint32), r.view(np.uint32))
    w = gpu.resident_worst_of(a, b)
    w.reduce()
    assert np.array_equal(w.download().view(np.uint32), r.view(np.uint32))
