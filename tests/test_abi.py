"""CPU checks of the C-ABI library: it loads, exports every symbol the header declares, maps
status codes to the reference's RigaError codes, fails loudly without a GPU, and its host-built
tables (Sobol directions, streamed bridge schedule) agree with the oracle."""
from __future__ import annotations

import ctypes as C
import math
import random
import re

import pytest

import oracle as O
from conftest import ROOT
from riga_gb300 import abi
from riga_gb300.build import build_library

HEADER = ROOT / "include" / "riga_gb300.h"


@pytest.fixture(scope="module")
def lib():
    build_library()
    return abi.load_library()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    assert set(names) == set(abi.SIGNATURES), "ctypes signatures must cover the header exactly"


def test_status_codes_match_the_reference_error_codes(lib):
    for code, name in abi.STATUS_CODES.items():
        assert lib.rg_status_code(code).decode() == name
    assert lib.rg_status_code(999).decode() == "unknown"
    assert lib.rg_abi_version() == 1


def test_no_gpu_fails_loudly_without_fallback(lib):
    """crates/riga-engine/src/lib.rs:188-202, gpu.rs:573-589: no silent CPU fallback."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert abi.STATUS_CODES[lib.rg_ensure_available()] == "gpu_unavailable"
    h = C.c_void_p()
    assert abi.STATUS_CODES[lib.rg_engine_create(0, C.byref(h))] == "gpu_unavailable"
    assert "CUDA device 0" in abi.last_error(lib)
    buf = C.create_string_buffer(64)
    assert abi.STATUS_CODES[lib.rg_device_name(buf, 64)] == "gpu_unavailable"
    a = (C.c_float * 4)(1, 2, 3, 4)
    assert abi.STATUS_CODES[lib.rg_worst_of(a, a, a, 4)] == "gpu_unavailable"


def test_sobol_directions_equal_the_oracle_table(lib):
    """qmc.rs:247-262, 316-430: the engine's host-built table is the reference's."""
    for dim in (1, 8, 512, 2268):
        buf = (C.c_uint32 * (32 * dim))()
        assert lib.rg_sobol_directions(dim, buf) == 0
        assert list(buf) == list(O.sobol_table(dim)), dim


@pytest.mark.parametrize("steps", [1, 2, 3, 7, 64, 105, 756])
def test_streamed_bridge_schedule_reproduces_the_depth_first_bridge(lib, steps):
    """qmc.rs:155-191: walking the schedule's in-order traversal over the same normals gives the
    reference bridge's increments (to FP64 rounding)."""
    dt = 3.0 / 756.0
    off = (C.c_int32 * (steps + 1))()
    k = (C.c_int32 * steps)()
    c = (C.c_double * steps)()
    depth = C.c_int32()
    assert lib.rg_bridge_schedule(steps, dt, off, k, c, C.byref(depth)) == 0
    assert sorted(k) == list(range(steps)) and k[0] == 0
    assert off[0] == 0 and off[steps] == steps
    assert depth.value <= math.ceil(math.log2(steps)) + 2 if steps > 1 else depth.value == 1
    rng = random.Random(steps)
    normals = [rng.gauss(0.0, 1.0) for _ in range(steps)]
    ref = O.bridge_increments(normals, dt)
    # the device traversal, restated
    stack, cur, out = [], 0.0, []
    for t in range(steps):
        for nd in range(off[t], off[t + 1]):
            z = normals[k[nd]]
            stack.append(z * c[nd] if nd == 0 else 0.5 * (cur + stack[-1]) + z * c[nd])
        nxt = stack.pop()
        out.append(nxt - cur)
        cur = nxt
    assert max(abs(a - b) for a, b in zip(out, ref)) == 0.0


def test_per_trade_bump_rule(lib):
    """rg_book_trade_bump (host only): scenario 0 is the base; every trade gets 15 distinct bumps
    on its own underlyings in the documented order — spot up and down and vol up of each
    underlying first, then the rate and the cross-gamma corners."""
    from riga_gb300.engine import trade_bump

    for n in range(1, 6):
        specs = [trade_bump(n, k) for k in range(abi.BOOK_TRADE_SCENARIOS)]
        assert specs[0][0] == abi.BUMP_BASE
        assert len(set(specs[1:])) == 15
        for i in range(n):
            assert specs[1 + 2 * i] == (abi.BUMP_SPOT, i, -1, 0.01)
            assert specs[2 + 2 * i] == (abi.BUMP_SPOT, i, -1, -0.01)
        vols = [s for s in specs if s[0] == abi.BUMP_VOL and s[3] == 0.01]
        assert [s[1] for s in vols] == list(range(n))
        for s in specs[1:]:
            assert 0 <= s[1] < n or s[0] == abi.BUMP_RATE
    three = [trade_bump(3, k) for k in range(16)]
    assert three[10] == (abi.BUMP_RATE, -1, -1, 1e-4)
    assert three[11:14] == [(abi.BUMP_SPOT_PAIR, 0, 1, 0.01), (abi.BUMP_SPOT_PAIR, 0, 2, 0.01),
                            (abi.BUMP_SPOT_PAIR, 1, 2, 0.01)]
    assert trade_bump(2, 1, (0.02, 0.0, 0.0))[3] == 0.02
