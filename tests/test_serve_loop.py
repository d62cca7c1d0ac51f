"""CPU tests of the MCP-shaped request loop (riga_gb300.serve.McpLoop) against a fake server:
tool dispatch, the task lifecycle (tasks/get, tasks/result, tasks/cancel) and error mapping.  The
native server behind it is tested on the GPU (test_server_gpu.py); the server refuses to start
without a GPU, which is checked here too."""
from __future__ import annotations

import pytest

from riga_gb300 import abi, workloads
from riga_gb300.abi import RigaError
from riga_gb300.serve import McpLoop, Server


class FakeServer:
    def __init__(self):
        self.jobs = {}
        self.next = 1

    def _add(self, kind, obj):
        t = self.next
        self.next += 1
        self.jobs[t] = {"kind": kind, "obj": obj, "state": abi.JOB_QUEUED}
        return t

    def submit_price(self, req, scenarios=None):
        return self._add("price", req)

    def submit_risk(self, req, config=None):
        return self._add("risk", req)

    def submit_book(self, book, scenarios=None):
        if len(book.trades) == 0:
            raise RigaError("invalid_argument", "a book needs at least one trade")
        return self._add("book", (book, scenarios))

    def poll(self, t):
        info = abi.JobInfo()
        info.state = self.jobs[t]["state"]
        return info

    def cancel(self, t):
        if self.jobs[t]["state"] == abi.JOB_QUEUED:
            self.jobs[t]["state"] = abi.JOB_CANCELLED

    def results(self, t):
        j = self.jobs[t]
        if j["state"] == abi.JOB_CANCELLED:
            raise RigaError("cancelled", "request was cancelled")
        j["state"] = abi.JOB_DONE
        n = 1
        if j["kind"] == "book":
            book, sc = j["obj"]
            n = len(book.trades) * (len(sc) if sc else 1)
        out = []
        for i in range(n):
            r = abi.PriceResult()
            r.pv = 1.0 + i
            r.seed = 1
            out.append(r)
        return out

    def risk_report(self, t):
        self.jobs[t]["state"] = abi.JOB_DONE
        rep = abi.BatchRiskReport()
        rep.base.pv = 0.97
        rep.n_assets = 1
        rep.assets[0].delta.value = 0.5
        return rep

    def stats(self):
        return abi.ServerStats()


def _book_json(b):
    return {"universe": b.universe.to_json(), "universe_steps": b.universe_steps,
            "universe_maturity_years": b.universe_maturity_years,
            "trades": [{"terms": t.terms.to_json(), "underlyings": t.underlyings} for t in b.trades],
            "config": {**b.config.to_json(), "trace_level": "off"},
            "options": {"scrambler": b.options.scrambler, "precision": b.options.precision,
                        "dim_mode": b.options.dim_mode}}


def test_price_trade_returns_the_reference_result_json():
    loop = McpLoop(FakeServer())
    req = workloads.plain3(paths=64, steps=12)
    out = loop.handle({"jsonrpc": "2.0", "id": 7, "method": "tools/call",
                       "params": {"name": "price_trade", "arguments": {"request": req.to_json()}}})
    assert out["id"] == 7 and "result" in out
    res = out["result"]["structuredContent"]
    assert res["pv"] == 1.0 and len(res["stats"]) == 3 and len(res["ledger"]) == 3


def test_book_async_task_lifecycle():
    loop = McpLoop(FakeServer())
    b = workloads.small_book(paths=32, n_trades=3)
    sc = [m.to_json() for _, m in workloads.book_scenarios(b.universe)][:2]
    out = loop.handle({"id": 1, "method": "tools/call",
                       "params": {"name": "price_book_async", "arguments": {"book": _book_json(b), "scenarios": sc}}})
    tid = out["result"]["task"]["taskId"]
    assert out["result"]["task"]["status"] == "working"
    assert loop.handle({"id": 2, "method": "tasks/get", "params": {"taskId": tid}})["result"]["status"] == "working"
    rows = loop.handle({"id": 3, "method": "tasks/result", "params": {"taskId": tid}})["result"]["structuredContent"]["results"]
    assert len(rows) == 3 * 2 and rows[0]["trade_id"] == b.trades[0].terms.trade_id
    assert loop.handle({"id": 4, "method": "tasks/get", "params": {"taskId": tid}})["result"]["status"] == "completed"


def test_cancelled_task_reports_cancelled():
    loop = McpLoop(FakeServer())
    b = workloads.small_book(paths=32, n_trades=1)
    tid = loop.handle({"id": 1, "method": "tools/call", "params": {"name": "price_book_async",
                                                                   "arguments": {"book": _book_json(b)}}})["result"]["task"]["taskId"]
    assert loop.handle({"id": 2, "method": "tasks/cancel", "params": {"taskId": tid}})["result"]["status"] == "cancelled"
    err = loop.handle({"id": 3, "method": "tasks/result", "params": {"taskId": tid}})["error"]
    assert err["data"]["code"] == "cancelled"


def test_risk_batch_and_errors():
    loop = McpLoop(FakeServer())
    req = workloads.plain3(paths=64, steps=12)
    out = loop.handle({"id": 1, "method": "tools/call", "params": {"name": "risk_batch", "arguments": {"request": req.to_json()}}})
    assert out["result"]["structuredContent"]["assets"][0]["delta"] == 0.5
    assert loop.handle({"id": 2, "method": "tools/call", "params": {"name": "nope"}})["error"]["code"] == -32602
    assert loop.handle({"id": 3, "method": "tasks/get", "params": {"taskId": "task-99"}})["error"]["code"] == -32602
    b = workloads.small_book(paths=32, n_trades=1)
    bj = _book_json(b)
    bj["trades"] = []
    err = loop.handle({"id": 4, "method": "tools/call", "params": {"name": "price_book", "arguments": {"book": bj}}})["error"]
    assert err["data"]["code"] == "invalid_argument"


def test_server_needs_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RigaError) as e:
        Server()
    assert e.value.code == "gpu_unavailable"


def test_cube_checksum_is_the_rotate_xor_fold():
    """main.rs:2145-2148: acc = rotate_left(acc, 1) ^ bits over the f32 cube."""
    import numpy as np

    from riga_gb300.serve import cube_checksum
    assert cube_checksum(np.zeros(0, dtype=np.float32)) == 0
    assert cube_checksum(np.array([1.0], dtype=np.float32)) == 0x3F800000
    assert cube_checksum(np.array([1.0, 2.0], dtype=np.float32)) == (0x3F800000 << 1) ^ 0x40000000
    top = np.array([-0.0] + [0.0] * 33, dtype=np.float32)  # sign bit rotated 33 times wraps past bit 63
    assert cube_checksum(top) == 1


def test_materialize_paths_is_capped_before_any_device_work():
    req = workloads.plain3(1 << 13, steps=63)
    loop = McpLoop(FakeServer())
    out = loop.handle({"jsonrpc": "2.0", "id": 9, "method": "tools/call",
                       "params": {"name": "materialize_paths",
                                  "arguments": {"request": req.to_json(), "count": 5000}}})
    assert out["error"]["data"]["code"] == "invalid_paths"
