"""The reference's public pricing API over the engine's C ABI.

* ``price_put_leg`` — ``riga_engine::price_put_leg`` (crates/riga-engine/src/lib.rs:183-186)
* ``price_scenarios`` — a CRN scenario batch in one fused launch (crates/riga-risk/src/lib.rs:253-258)
* ``price_risk_batch`` — ``riga_risk::price_risk_batch`` (crates/riga-risk/src/lib.rs:573-626)
* ``run_paths`` / ``reconstruct_path`` / ``query_worst_percentile`` —
  crates/riga-engine/src/explain.rs:90-372
* ``price_book_raw`` / ``book_run_paths_raw`` — many trades on one universe under one common CRN
  scenario set (``rg_price_book``; the reference prices one trade per request)
"""
from __future__ import annotations

import ctypes as C
import math
import threading
from typing import Optional

from . import abi
from .abi import RigaError, check, load_library
from .types import (BookRequest, PriceRequest, market_to_abi, markets_to_abi, record_to_dict,
                    result_to_json)


class Engine:
    """One engine handle: a CUDA stream plus its resident device workspace."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        check(self.lib, self.lib.rg_engine_create(device, C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.rg_engine_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- pricing ---------------
    def price_raw(self, request: PriceRequest) -> abi.PriceResult:
        a = request.to_abi()
        out = abi.PriceResult()
        check(self.lib, self.lib.rg_price_put_leg(self.handle, a.ptr, C.byref(out)))
        return out

    def last_timing(self) -> abi.Timing:
        """Device-time breakdown of this engine's last call (rg_engine_last_timing)."""
        tm = abi.Timing()
        check(self.lib, self.lib.rg_engine_last_timing(self.handle, C.byref(tm)))
        return tm

    def price_put_leg(self, request: PriceRequest) -> dict:
        return result_to_json(self.price_raw(request), request)

    # -------------------------------------------------------------- books -----------------
    def price_book_raw(self, book: BookRequest, scenarios=None) -> list:
        """Results of every (trade, scenario), trade-major: ``out[j * S + s]``.  ``scenarios`` is
        a list of universe ``MarketSnapshot``s (None: the base market alone)."""
        a = book.to_abi()
        keep = []
        arr, n = markets_to_abi(scenarios, keep.append)
        S = max(1, n)
        out = (abi.PriceResult * (len(book.trades) * S))()
        check(self.lib, self.lib.rg_price_book(self.handle, a.ptr, arr, n, out))
        return list(out)

    def price_book_trade_bumps_raw(self, book: BookRequest, sizes=None) -> list:
        """Every trade under its own 16 scenarios (rg_price_book_trade_bumps): ``out[j * 16 + k]`` is
        trade j under its bump k (``trade_bump``).  ``sizes``: (spot relative, vol absolute, rate
        absolute) or None for (1%, 1 vol point, 1bp)."""
        a = book.to_abi()
        b = abi.BookBumps(*(sizes or (0.0, 0.0, 0.0)))
        out = (abi.PriceResult * (len(book.trades) * abi.BOOK_TRADE_SCENARIOS))()
        check(self.lib, self.lib.rg_price_book_trade_bumps(self.handle, a.ptr, C.byref(b), out))
        return list(out)

    def resident_book(self, book: BookRequest) -> "ResidentBook":
        """Upload `book` once (rg_book_create); price it under many scenario sets."""
        return ResidentBook(self, book)

    def book_run_paths_raw(self, book: BookRequest, scenarios, first: int, count: int) -> list:
        """Per-path records ``out[(p * n_trades + j) * S + s]`` of paths [first, first + count)."""
        a = book.to_abi()
        keep = []
        arr, n = markets_to_abi(scenarios, keep.append)
        S = max(1, n)
        out = (abi.PathRecord * (count * len(book.trades) * S))()
        check(self.lib, self.lib.rg_book_run_paths(self.handle, a.ptr, arr, n, first, count, out))
        return list(out)

    def price_scenarios_raw(self, request: PriceRequest, scenarios) -> list:
        """``scenarios``: list of (MarketSnapshot, implied-vol shift list or None)."""
        a = request.to_abi()
        keep = []
        arr = (abi.Scenario * len(scenarios))()
        for i, (mk, shift) in enumerate(scenarios):
            arr[i].market = market_to_abi(mk, lambda x: (keep.append(x), x)[1])
            if shift is not None:
                buf = (C.c_double * len(shift))(*shift)
                keep.append(buf)
                arr[i].implied_vol_shift = C.cast(buf, C.POINTER(C.c_double))
        out = (abi.PriceResult * len(scenarios))()
        check(self.lib, self.lib.rg_price_scenarios(self.handle, a.ptr, arr, len(scenarios), out))
        return list(out)

    def upload_surfaces(self, request: PriceRequest, scenarios=None) -> int:
        """Calibrates the request's (and its scenarios') Dupire surfaces on the device and keeps
        them resident on this engine (rg_surfaces_upload); returns the number of surfaces."""
        a = request.to_abi()
        keep = []
        scenarios = scenarios or []
        arr = (abi.Scenario * max(1, len(scenarios)))()
        for i, (mk, shift) in enumerate(scenarios):
            arr[i].market = market_to_abi(mk, lambda x: (keep.append(x), x)[1])
            if shift is not None:
                buf = (C.c_double * len(shift))(*shift)
                keep.append(buf)
                arr[i].implied_vol_shift = C.cast(buf, C.POINTER(C.c_double))
        n = C.c_int32(0)
        check(self.lib, self.lib.rg_surfaces_upload(self.handle, a.ptr, arr, len(scenarios), C.byref(n)))
        return n.value

    def price_risk_batch_raw(self, request: PriceRequest, config: Optional[abi.CentralDifferenceConfig] = None):
        cfg = config or abi.CentralDifferenceConfig(0.01, 0.01, 1e-4, 0.01, abi.CRN)
        a = request.to_abi()
        out = abi.BatchRiskReport()
        check(self.lib, self.lib.rg_price_risk_batch(self.handle, a.ptr, C.byref(cfg), C.byref(out)))
        return out

    def run_paths_raw(self, request: PriceRequest, first: int = 0, count: Optional[int] = None):
        count = request.config.paths - first if count is None else count
        a = request.to_abi()
        out = (abi.PathRecord * max(1, count))()
        check(self.lib, self.lib.rg_run_paths(self.handle, a.ptr, first, count, out))
        return out

    def run_paths(self, request: PriceRequest, first: int = 0, count: Optional[int] = None) -> list:
        n = request.config.paths - first if count is None else count
        return [record_to_dict(r) for r in self.run_paths_raw(request, first, n)][:n]

    def materialize_paths(self, request: PriceRequest, first: int = 0, count: Optional[int] = None,
                          with_records: bool = True):
        """PathCube slice of a priced trade (``rg_materialize_paths``): the f32 spots
        ``[count][steps][n]`` of paths [first, first + count) under the base scenario, and the
        same paths' PathRecord dicts (or None)."""
        import numpy as np
        from .pathcube import PathCube

        count = request.config.paths - first if count is None else count
        n = len(request.market.spots)
        steps = request.trade.steps
        a = request.to_abi()
        cube = np.empty(max(1, count * steps * n), dtype=np.float32)
        recs = (abi.PathRecord * max(1, count))() if with_records else None
        check(self.lib, self.lib.rg_materialize_paths(self.handle, a.ptr, first, count,
                                                      cube.ctypes.data_as(C.POINTER(C.c_float)), recs))
        out = PathCube(count, steps, n, cube[: count * steps * n])
        return out, ([record_to_dict(r) for r in recs][:count] if with_records else None)

    def reconstruct_path(self, request: PriceRequest, path_id: int) -> dict:
        """explain.rs:319-333: one path re-simulated from its identity alone."""
        if path_id >= request.config.paths:
            raise RigaError("path_out_of_range",
                            f"path_id {path_id} is outside the configured path count {request.config.paths}")
        return record_to_dict(self.run_paths_raw(request, path_id, 1)[0])

    def query_worst_percentile(self, request: PriceRequest, percentile: float, max_sample: int) -> dict:
        """explain.rs:336-372"""
        if not (0.0 <= percentile <= 1.0):
            raise RigaError("invalid_percentile", "percentile must be within [0, 1]")
        recs = [record_to_dict(r) for r in self.run_paths_raw(request)]
        recs.sort(key=lambda r: r["worst_final"])
        total = len(recs)
        selected = math.ceil(total * percentile)
        return {"percentile": percentile,
                "threshold_worst_final": recs[selected - 1]["worst_final"] if selected else 0.0,
                "selected": selected, "total": total, "sample": recs[: min(selected, max_sample)]}


_default: Optional[Engine] = None
_lock = threading.Lock()


def default_engine() -> Engine:
    global _default
    with _lock:
        if _default is None:
            _default = Engine(0)
        return _default


def price_put_leg(request: PriceRequest) -> dict:
    return default_engine().price_put_leg(request)


def price_risk_batch(request: PriceRequest, config=None):
    return default_engine().price_risk_batch_raw(request, config)


class ResidentBook:
    """A book resident on the engine's device (rg_book_*): priced by CUDA-graph replay."""

    def __init__(self, engine: Engine, book: BookRequest):
        self.engine = engine
        self.lib = engine.lib
        self.n_trades = len(book.trades)
        a = book.to_abi()
        h = C.c_void_p()
        check(self.lib, self.lib.rg_book_create(engine.handle, a.ptr, C.byref(h)))
        self.handle = h

    def price_raw(self, scenarios=None) -> list:
        keep = []
        arr, n = markets_to_abi(scenarios, keep.append)
        out = (abi.PriceResult * (self.n_trades * max(1, n)))()
        check(self.lib, self.lib.rg_book_price(self.handle, arr, n, out))
        return list(out)

    def price_trade_bumps_raw(self, sizes=None) -> list:
        """rg_book_price_trade_bumps: ``out[j * 16 + k]``, trade j under its bump k."""
        b = abi.BookBumps(*(sizes or (0.0, 0.0, 0.0)))
        out = (abi.PriceResult * (self.n_trades * abi.BOOK_TRADE_SCENARIOS))()
        check(self.lib, self.lib.rg_book_price_trade_bumps(self.handle, C.byref(b), out))
        return list(out)

    def tuned_stage(self, n_scenarios: int) -> int:
        v = C.c_int32()
        check(self.lib, self.lib.rg_book_tuned_stage(self.handle, n_scenarios, C.byref(v)))
        return v.value

    def close(self):
        if self.handle:
            self.lib.rg_book_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def trade_bump(n_underlyings: int, scenario: int, sizes=None):
    """The bump of scenario ``scenario`` (0..15) of a book trade on ``n_underlyings`` underlyings
    (rg_book_trade_bump): (kind, first, second, size) with kind one of abi.BUMP_*."""
    lib = load_library()
    b = abi.BookBumps(*(sizes or (0.0, 0.0, 0.0)))
    out = abi.BookBumpSpec()
    check(lib, lib.rg_book_trade_bump(n_underlyings, scenario, C.byref(b), C.byref(out)))
    return out.kind, out.first, out.second, out.size
