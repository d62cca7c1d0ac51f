"""rg_price_put_leg_static: pricing for callers that cannot allocate device memory.

Such callers (hosts whose memory pool owns the device, processes under a hard device-memory
budget, plugins that must not call cudaMalloc/cudaFree behind their host's back) get the same
pipeline with every device buffer in the library's static 16 MiB region.  Its results must equal rg_price_put_leg's for the same
request, within the parity tolerance of the other GPU tests (1e-12), on two calls in a row — the
region keeps the previous call's contents, so the second call checks that nothing stale leaks.
This file is collected last so a failure here cannot stop the rest of the GPU suite.
"""
from __future__ import annotations

import ctypes as C

import pytest

from conftest import json_close
from riga_gb300 import abi, workloads
from riga_gb300.build import build_library
from riga_gb300.engine import Engine
from riga_gb300.types import result_to_json

pytestmark = pytest.mark.gpu


def _static(lib, req):
    a = req.to_abi()
    out = abi.PriceResult()
    abi.check(lib, lib.rg_price_put_leg_static(a.ptr, C.byref(out)))
    return out


@pytest.mark.parametrize("case", ["fp64_flat", "fp32_local_vol"])
def test_static_entry_point_matches_the_allocating_one(case):
    build_library()
    lib = abi.load_library()
    if case == "fp64_flat":
        req = workloads.plain3(4096, steps=252)
        req.config.trace_level = "aggregated"
    else:
        req = workloads.lv3(1 << 15, steps=252, fp32=True)
    eng = Engine(0)
    try:
        expected = result_to_json(eng.price_raw(req), req)
    finally:
        eng.close()
    for _ in range(2):
        got = result_to_json(_static(lib, req), req)
        assert json_close(got, expected, tol=1e-12) == []


def test_static_entry_point_rejects_requests_beyond_its_region():
    build_library()
    lib = abi.load_library()
    req = workloads.plain3(1 << 23, steps=63)
    req.config.trace_level = "aggregated"  # 4 bytes of KO step per path: 32 MiB > 16 MiB
    a = req.to_abi()
    out = abi.PriceResult()
    status = lib.rg_price_put_leg_static(a.ptr, C.byref(out))
    assert abi.STATUS_CODES[status] == "invalid_argument"
    assert "16 MiB" in abi.last_error(lib)


def test_static_entry_point_recovers_after_overflowing_while_staging():
    """A long local-vol request fits its tables but not its FP32 local-vol rows (3 surfaces x 12,000
    steps x 40 points x 8 bytes = 11.5 MB beside about 7 MB of tables), so the region overflows
    inside staging, after the calibration kernel is already queued.  The error must be
    invalid_argument, and the next call must still equal rg_price_put_leg."""
    build_library()
    lib = abi.load_library()
    big = workloads.lv3(2048, steps=12000, fp32=True)
    a = big.to_abi()
    out = abi.PriceResult()
    status = lib.rg_price_put_leg_static(a.ptr, C.byref(out))
    assert abi.STATUS_CODES[status] == "invalid_argument"
    assert "16 MiB" in abi.last_error(lib)
    req = workloads.lv3(1 << 15, steps=252, fp32=True)
    eng = Engine(0)
    try:
        expected = result_to_json(eng.price_raw(req), req)
    finally:
        eng.close()
    got = result_to_json(_static(lib, req), req)
    assert json_close(got, expected, tol=1e-12) == []


def test_static_entry_point_declines_the_pseudo_random_lane(termsheet1):
    """The ChaCha8 lane's normal stream lives in engine buffers, not in the static region."""
    build_library()
    lib = abi.load_library()
    req = termsheet1.request
    a = req.to_abi()
    out = abi.PriceResult()
    status = lib.rg_price_put_leg_static(a.ptr, C.byref(out))
    assert lib.rg_status_code(status).decode() == "unsupported"
