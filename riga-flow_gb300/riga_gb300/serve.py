"""The serving front: the engine's continuous-batching server behind an MCP-shaped request loop.

``Server`` wraps ``rg_server_*`` (include/riga_gb300.h): requests are submitted without blocking,
admitted by the native server as slots and device memory free up, run concurrently on their own
CUDA streams, and collected by ticket.

``McpLoop`` is the request loop of crates/riga-mcp/src/main.rs reduced to the pricing tools: a
JSON-RPC 2.0 ``tools/call`` for ``price_trade`` ({"request": PriceRequest JSON, "options"?: engine
knobs}), ``risk_batch`` ({"request": ..., "options"?}), ``price_book`` ({"book": BookRequest JSON, "scenarios": [...]}) and
``price_book_async`` (returns a task, as the reference's SEP-2663 task path does, main.rs:1000-
1042), plus ``tasks/get``, ``tasks/result`` and ``tasks/cancel``.  Synchronous tools also go
through the server, so concurrent clients share its continuous batching.  The replay tools
``reconstruct_path`` ({"request", "path_id"}), ``query_path_cube`` / ``query_pathcube``
({"request", "percentile", "max_sample"}, main.rs:319-360) and ``materialize_paths`` ({"request",
"first_path"?, "count"?}: at most 4096 paths, the reference's PathCube cap, main.rs:2134-2160)
run synchronously on a replay engine of the loop's own.  ``python -m riga_gb300.serve`` runs the
loop over stdin/stdout, one JSON message per line.
"""
from __future__ import annotations

import ctypes as C
import json
import sys
import threading
from typing import Optional

from . import abi
from .abi import RigaError, check, load_library
from .types import (BookRequest, BookTrade, EngineOptions, MarketSnapshot, PhoenixTrade, PriceRequest,
                    SimulationConfig, VarianceReduction, market_to_abi, markets_to_abi, result_to_json)

STATES = ("working", "working", "completed", "failed", "cancelled")  # SEP-2663 task status per RG_JOB_*


class Server:
    """One ``rg_server``: `slots` engines on `device`, admission within `memory_budget` bytes; requests
    of at least `large_work` path-steps × scenarios hold at most `max_large_slots` slots and size
    their kernels for `large_max_sms` SMs (0: the library's defaults, half the slots, 2^31 and two
    thirds of the SMs; -1: every SM)."""

    def __init__(self, device: int = 0, slots: int = 4, memory_budget: int = 0, lib=None,
                 max_large_slots: int = 0, large_work: int = 0, large_max_sms: int = 0):
        self.lib = lib or load_library()
        self.device = device
        cfg = abi.ServerConfig(device, slots, memory_budget, max_large_slots, large_work, large_max_sms)
        h = C.c_void_p()
        check(self.lib, self.lib.rg_server_create(C.byref(cfg), C.byref(h)))
        self.handle = h
        self._kinds = {}

    def close(self):
        if self.handle:
            self.lib.rg_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- submission --------------
    def submit_price(self, request: PriceRequest, scenarios=None) -> int:
        """``scenarios``: list of (MarketSnapshot, implied-vol shift or None), or None."""
        a = request.to_abi()
        keep = []
        arr, n = None, 0
        if scenarios:
            arr = (abi.Scenario * len(scenarios))()
            for i, (mk, shift) in enumerate(scenarios):
                arr[i].market = market_to_abi(mk, lambda x: (keep.append(x), x)[1])
                if shift is not None:
                    buf = (C.c_double * len(shift))(*shift)
                    keep.append(buf)
                    arr[i].implied_vol_shift = C.cast(buf, C.POINTER(C.c_double))
            n = len(scenarios)
        t = C.c_uint64()
        check(self.lib, self.lib.rg_server_submit_price(self.handle, a.ptr, arr, n, C.byref(t)))
        self._kinds[t.value] = abi.JOB_PRICE
        return t.value

    def submit_risk(self, request: PriceRequest, config: Optional[abi.CentralDifferenceConfig] = None) -> int:
        a = request.to_abi()
        cfg = config or default_risk_config()
        t = C.c_uint64()
        check(self.lib, self.lib.rg_server_submit_risk(self.handle, a.ptr, C.byref(cfg), C.byref(t)))
        self._kinds[t.value] = abi.JOB_RISK
        return t.value

    def submit_book(self, book: BookRequest, scenarios=None) -> int:
        a = book.to_abi()
        keep = []
        arr, n = markets_to_abi(scenarios, keep.append)
        t = C.c_uint64()
        check(self.lib, self.lib.rg_server_submit_book(self.handle, a.ptr, arr, n, C.byref(t)))
        self._kinds[t.value] = abi.JOB_BOOK
        return t.value

    def submit_book_trade_bumps(self, book: BookRequest, sizes: Optional[abi.BookBumps] = None) -> int:
        """Every trade of `book` under its own 16 scenarios (base + 15 bumps on its own underlyings);
        results[j * 16 + k] is trade j under its scenario k."""
        a = book.to_abi()
        t = C.c_uint64()
        check(self.lib, self.lib.rg_server_submit_book_trade_bumps(self.handle, a.ptr,
                                                                   C.byref(sizes) if sizes else None, C.byref(t)))
        self._kinds[t.value] = abi.JOB_BOOK_BUMPS
        return t.value

    # -------------------------------------------------------------- collection --------------
    def poll(self, ticket: int) -> abi.JobInfo:
        info = abi.JobInfo()
        check(self.lib, self.lib.rg_server_poll(self.handle, ticket, C.byref(info)))
        return info

    def wait(self, ticket: int, timeout_ms: int = -1) -> abi.JobInfo:
        info = abi.JobInfo()
        check(self.lib, self.lib.rg_server_wait(self.handle, ticket, timeout_ms, C.byref(info)))
        if info.state == abi.JOB_FAILED:
            raise RigaError(self.lib.rg_status_code(info.status).decode(), abi.last_error(self.lib))
        return info

    def results(self, ticket: int) -> list:
        info = self.wait(ticket)
        out = (abi.PriceResult * max(1, info.n_results))()
        check(self.lib, self.lib.rg_server_results(self.handle, ticket, out, info.n_results))
        return list(out)[: info.n_results]

    def risk_report(self, ticket: int) -> abi.BatchRiskReport:
        self.wait(ticket)
        out = abi.BatchRiskReport()
        check(self.lib, self.lib.rg_server_risk_report(self.handle, ticket, C.byref(out)))
        return out

    def cancel(self, ticket: int):
        check(self.lib, self.lib.rg_server_cancel(self.handle, ticket))

    def release(self, ticket: int):
        check(self.lib, self.lib.rg_server_release(self.handle, ticket))
        self._kinds.pop(ticket, None)

    def stats(self) -> abi.ServerStats:
        s = abi.ServerStats()
        check(self.lib, self.lib.rg_server_get_stats(self.handle, C.byref(s)))
        return s


def default_risk_config() -> abi.CentralDifferenceConfig:
    """CentralDifferenceConfig::default (crates/riga-risk/src/lib.rs:24-49)."""
    c = abi.CentralDifferenceConfig()
    c.spot_relative_bump, c.volatility_absolute_bump = 0.01, 0.01
    c.rate_absolute_bump, c.correlation_absolute_bump = 1e-4, 0.01
    c.random_number_policy = abi.CRN
    return c


# ---------------------------------------------------------------------- JSON shapes ------------
def book_from_json(d: dict) -> BookRequest:
    """``{"universe": MarketSnapshot, "universe_steps", "universe_maturity_years", "trades":
    [{"terms": PhoenixTrade, "underlyings": [...]}], "config": SimulationConfig, "options"?}``"""
    u = d["universe"]
    universe = MarketSnapshot(u["as_of"], list(u["spots"]), list(u["vols"]), float(u["risk_free_rate"]),
                              list(u["dividend_yields"]), [list(r) for r in u["correlation"]])
    trades = []
    for t in d["trades"]:
        tt = t["terms"]
        trades.append(BookTrade(PhoenixTrade(
            trade_id=tt["trade_id"], initial_spots=list(tt["initial_spots"]),
            maturity_years=float(tt["maturity_years"]), steps=int(tt["steps"]), strike=float(tt["strike"]),
            knock_in_barrier=float(tt["knock_in_barrier"]), knock_out_barrier=tt.get("knock_out_barrier"),
            coupon_barrier=tt.get("coupon_barrier"), coupon_rate=tt.get("coupon_rate"),
            memory_coupon=bool(tt.get("memory_coupon", False)), coupon_periods=tt.get("coupon_periods"),
            fixed_first_coupon=bool(tt.get("fixed_first_coupon", False)),
            call_start_step=tt.get("call_start_step")), list(t["underlyings"])))
    c = d["config"]
    config = SimulationConfig(int(c["paths"]), int(c.get("path_block_size", c["paths"])), int(c["seed"]),
                              c.get("trace_level", "off"),
                              VarianceReduction.from_json(c.get("variance_reduction", {})))
    o = d.get("options", {})
    options = EngineOptions(**{k: int(v) for k, v in o.items()})
    return BookRequest(universe, int(d["universe_steps"]), float(d["universe_maturity_years"]), trades,
                       config, options)


def market_from_json(m: dict) -> MarketSnapshot:
    return MarketSnapshot(m["as_of"], list(m["spots"]), list(m["vols"]), float(m["risk_free_rate"]),
                          list(m["dividend_yields"]), [list(r) for r in m["correlation"]])


def _result_numbers(r: abi.PriceResult) -> dict:
    return {"pv": r.pv, "mc_error": r.mc_error, "ki_probability": r.ki_probability,
            "ko_count": r.ko_count, "ki_count": r.ki_count, "coupon_path_count": r.coupon_path_count}


def _risk_json(rep: abi.BatchRiskReport) -> dict:
    assets = []
    for i in range(rep.n_assets):
        a = rep.assets[i]
        assets.append({"asset_index": a.asset_index, "delta": a.delta.value, "gamma": a.gamma.value,
                       "vega": a.vega.value, "delta_mc_error_upper_bound": a.delta.mc_error_upper_bound})
    return {"pv": rep.base.pv, "pv_mc_error": rep.pv_mc_error, "scenario_count": rep.scenario_count,
            "assets": assets, "rate_up_pv": rep.rate_up_pv, "rate_down_pv": rep.rate_down_pv,
            "correlation_up_pv": rep.correlation_up_pv, "correlation_down_pv": rep.correlation_down_pv}


# ---------------------------------------------------------------------- the request loop -------
def cube_checksum(data) -> int:
    """The PathCube checksum of the reference's generate_paths tool (main.rs:2145-2148): fold of
    rotate_left(acc, 1) ^ f32 bits over the cube in order."""
    import numpy as np

    acc = 0
    mask = (1 << 64) - 1
    for b in np.ascontiguousarray(data, dtype=np.float32).view(np.uint32).tolist():
        acc = (((acc << 1) | (acc >> 63)) & mask) ^ b
    return acc


class McpLoop:
    """JSON-RPC 2.0 dispatch of the pricing tools and the task methods onto a ``Server``."""

    REPLAY_TOOLS = ("reconstruct_path", "query_path_cube", "query_pathcube", "materialize_paths")
    CUBE_CAP = 4096

    def __init__(self, server: Server):
        self.server = server
        self._tasks = {}  # task id -> (ticket, tool, request object)
        self._lock = threading.Lock()
        self._next = 1
        self._replay = None  # Engine for the replay tools, created on first use
        self._replay_lock = threading.Lock()

    def close(self):
        if self._replay is not None:
            self._replay.close()
            self._replay = None

    def _replay_tool(self, name, args):
        from .engine import Engine

        opts = EngineOptions(**{k: int(v) for k, v in (args.get("options") or {}).items()})
        req = PriceRequest.from_json(args["request"], opts)
        first = int(args.get("first_path", 0))
        count = int(args.get("count", min(self.CUBE_CAP, max(0, req.config.paths - first))))
        if name == "materialize_paths" and count > self.CUBE_CAP:
            raise RigaError("invalid_paths", f"at most {self.CUBE_CAP} paths per materialisation")
        with self._replay_lock:
            if self._replay is None:
                self._replay = Engine(self.server.device)
            e = self._replay
            if name == "reconstruct_path":
                return {"structuredContent": e.reconstruct_path(req, int(args["path_id"]))}
            if name in ("query_path_cube", "query_pathcube"):
                return {"structuredContent": e.query_worst_percentile(req, float(args["percentile"]),
                                                                      int(args["max_sample"]))}
            cube, recs = e.materialize_paths(req, first, count)
            return {"structuredContent": {"first_path": first, "paths": cube.paths, "times": cube.times,
                                          "factors": cube.factors, "checksum": cube_checksum(cube.data),
                                          "data": [float(v) for v in cube.data], "records": recs}}

    def handle(self, msg: dict) -> dict:
        mid = msg.get("id")
        try:
            result = self._dispatch(msg.get("method"), msg.get("params") or {})
            return {"jsonrpc": "2.0", "id": mid, "result": result}
        except RigaError as e:
            return {"jsonrpc": "2.0", "id": mid, "error": {"code": -32000, "message": e.message,
                                                           "data": {"code": e.code}}}
        except (KeyError, TypeError, ValueError) as e:
            return {"jsonrpc": "2.0", "id": mid, "error": {"code": -32602, "message": f"invalid params: {e}"}}

    def _dispatch(self, method, params):
        if method == "tools/call":
            name, args = params["name"], params.get("arguments") or {}
            if name in self.REPLAY_TOOLS:
                return self._replay_tool(name, args)
            if name == "health":
                st = self.server.stats()
                return {"status": "ok", "queued": st.queued, "running": st.running,
                        "completed": st.completed, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms}
            ticket, tool, obj = self._submit(name, args)
            if name.endswith("_async"):
                with self._lock:
                    tid = f"task-{self._next}"
                    self._next += 1
                    self._tasks[tid] = (ticket, tool, obj)
                return {"task": {"taskId": tid, "status": "working"}}
            return self._collect(ticket, tool, obj)
        if method in ("tasks/get", "tasks/result", "tasks/cancel"):
            tid = params["taskId"]
            with self._lock:
                if tid not in self._tasks:
                    raise KeyError(f"unknown task {tid}")
                ticket, tool, obj = self._tasks[tid]
            if method == "tasks/cancel":
                self.server.cancel(ticket)
                return {"taskId": tid, "status": STATES[self.server.poll(ticket).state]}
            if method == "tasks/get":
                return {"taskId": tid, "status": STATES[self.server.poll(ticket).state]}
            return self._collect(ticket, tool, obj)
        raise ValueError(f"unknown method {method}")

    def _submit(self, name, args):
        # engine knobs the reference's request JSON does not carry; absent = the reference's arithmetic
        opts = EngineOptions(**{k: int(v) for k, v in (args.get("options") or {}).items()})
        if name == "price_trade":
            req = PriceRequest.from_json(args["request"], opts)
            return self.server.submit_price(req), name, req
        if name == "risk_batch":
            req = PriceRequest.from_json(args["request"], opts)
            return self.server.submit_risk(req), name, req
        if name in ("price_book", "price_book_async"):
            book = book_from_json(args["book"])
            sc = [market_from_json(m) for m in args.get("scenarios", [])] or None
            return self.server.submit_book(book, sc), "price_book", (book, sc)
        raise ValueError(f"unknown tool {name}")

    def _collect(self, ticket, tool, obj):
        if tool == "price_trade":
            res = self.server.results(ticket)[0]
            return {"structuredContent": result_to_json(res, obj)}
        if tool == "risk_batch":
            return {"structuredContent": _risk_json(self.server.risk_report(ticket))}
        book, sc = obj
        res = self.server.results(ticket)
        S = len(sc) if sc else 1
        rows = [{"trade_id": book.trades[j].terms.trade_id, "scenario": s, **_result_numbers(res[j * S + s])}
                for j in range(len(book.trades)) for s in range(S)]
        return {"structuredContent": {"results": rows}}


def main(argv=None):
    server = Server()
    loop = McpLoop(server)
    for line in sys.stdin:
        line = line.strip()
        if not line:
            continue
        try:
            msg = json.loads(line)
        except json.JSONDecodeError as e:
            print(json.dumps({"jsonrpc": "2.0", "id": None, "error": {"code": -32700, "message": str(e)}}), flush=True)
            continue
        print(json.dumps(loop.handle(msg)), flush=True)
    loop.close()
    server.close()


if __name__ == "__main__":
    main()
