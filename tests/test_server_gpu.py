"""GPU tests of the continuous-batching server (rg_server_*) and the MCP-shaped loop over it.

* Every request's result is bit-identical in the mix and alone: a mix of price, CRN-batch, risk
  and book requests submitted from several threads at once, against the same requests priced one
  at a time through a plain engine.
* Work overlaps: with several slots, requests that were queued together run at the same time.
* Admission by device memory: with a budget that holds one request at a time, requests never
  overlap and all complete; single trades pass a book that waits for memory, and the server
  counts the wait; a request larger than the whole budget is rejected at submission.
* Books under per-trade bump sets through the server equal the direct call.
* Tasks: a queued request can be cancelled, a wait can time out, and stats report p50/p99.
"""
from __future__ import annotations

import copy
import json
import threading

import pytest

from riga_gb300 import abi, workloads
from riga_gb300.abi import RigaError
from riga_gb300.build import build_library
from riga_gb300.engine import Engine
from riga_gb300.serve import McpLoop, Server, default_risk_config
from riga_gb300.types import result_to_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    build_library()
    e = Engine(0)
    yield e
    e.close()


def _mix():
    """(kind, request, scenarios) of a varied request mix."""
    mix = []
    mix.append(("price", workloads.plain3(paths=1 << 12, steps=126), None))
    p32 = workloads.plain3(paths=1 << 14, steps=252, fp32=True)
    mix.append(("price", p32, [(m, s) for _, m, s in workloads.crn15_scenarios(p32)][:8]))
    lv = workloads.lv3(paths=1 << 13, steps=126)
    mix.append(("price", lv, [(m, s) for _, m, s in workloads.crn15_scenarios(lv)]))
    mix.append(("risk", workloads.plain3(paths=1 << 11, steps=63), None))
    b = workloads.small_book(paths=1 << 12, n_trades=6, steps_per_year=52, fp32=True)
    mix.append(("book", b, [m for _, m in workloads.book_scenarios(b.universe)]))
    b64 = workloads.small_book(paths=512, n_trades=3)
    mix.append(("book", b64, [m for _, m in workloads.book_scenarios(b64.universe)][:2]))
    return mix


def _alone(engine, kind, req, sc):
    if kind == "price":
        return [engine.price_raw(req)] if sc is None else engine.price_scenarios_raw(req, sc)
    if kind == "risk":
        return engine.price_risk_batch_raw(req, default_risk_config())
    return engine.price_book_raw(req, sc)


def _submit(server, kind, req, sc):
    if kind == "price":
        return server.submit_price(req, sc)
    if kind == "risk":
        return server.submit_risk(req)
    return server.submit_book(req, sc)


def _collect(server, kind, t):
    return server.risk_report(t) if kind == "risk" else server.results(t)


def test_results_are_identical_alone_and_in_the_mix(engine):
    mix = _mix() * 2
    alone = [_alone(engine, k, r, s) for k, r, s in mix]
    with Server(slots=4) as srv:
        tickets = [None] * len(mix)

        def submit(i):
            tickets[i] = _submit(srv, *mix[i])

        threads = [threading.Thread(target=submit, args=(i,)) for i in range(len(mix))]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        got = [_collect(srv, mix[i][0], tickets[i]) for i in range(len(mix))]
        st = srv.stats()
    assert st.completed == len(mix) and st.failed == 0
    assert st.p50_ms > 0 and st.p99_ms >= st.p50_ms
    for (kind, _, _), a, g in zip(mix, alone, got):
        if kind == "risk":
            assert bytes(a) == bytes(g)
        else:
            assert [bytes(x) for x in a] == [bytes(x) for x in g]


def test_queued_requests_overlap_on_the_device():
    reqs = [workloads.lv3(paths=1 << 17, steps=252) for _ in range(4)]
    for r in reqs:
        r.options = workloads.production_options()
    with Server(slots=4) as srv:
        ts = [srv.submit_price(r, [(m, s) for _, m, s in workloads.crn15_scenarios(r)]) for r in reqs]
        infos = [srv.wait(t) for t in ts]
    spans = sorted((i.start_s, i.end_s) for i in infos)
    assert any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    assert len({i.slot for i in infos}) > 1


def test_memory_budget_admits_one_request_at_a_time():
    books = [workloads.small_book(paths=1 << 13, n_trades=4, steps_per_year=52, fp32=True, seed=s) for s in range(4)]
    with Server(slots=4, memory_budget=1 << 62) as probe:
        t = probe.submit_book(books[0])
        est = probe.wait(t).device_bytes
    with Server(slots=4, memory_budget=int(est * 1.5)) as srv:
        ts = [srv.submit_book(b) for b in books]
        infos = [srv.wait(t) for t in ts]
        results = [srv.results(t) for t in ts]
    spans = sorted((i.start_s, i.end_s) for i in infos)
    assert all(spans[k + 1][0] >= spans[k][1] for k in range(len(spans) - 1))
    assert all(len(r) == 4 for r in results)


def test_small_requests_pass_a_book_waiting_for_memory():
    books = [workloads.small_book(paths=1 << 13, n_trades=4, steps_per_year=52, fp32=True, seed=s) for s in range(2)]
    single = workloads.lv3(paths=1 << 12, steps=63, fp32=True)
    with Server(slots=4, memory_budget=1 << 62) as probe:
        est = probe.wait(probe.submit_book(books[0])).device_bytes
        small = probe.wait(probe.submit_price(single)).device_bytes
    budget = int(est * 1.5)
    assert small <= budget // 16
    with Server(slots=4, memory_budget=budget) as srv:
        tb = [srv.submit_book(b) for b in books]
        ts = [srv.submit_price(single) for _ in range(6)]
        books_info = [srv.wait(t) for t in tb]
        singles_info = [srv.wait(t) for t in ts]
        st = srv.stats()
    assert books_info[1].start_s >= books_info[0].end_s  # the books never overlap
    assert st.memory_waits >= 1 and st.peak_reserved_bytes <= budget
    assert any(i.start_s < books_info[1].start_s for i in singles_info)  # singles passed the waiting book
    assert st.completed == 8 and st.failed == 0


def test_book_trade_bumps_through_the_server_equal_the_direct_call(engine):
    b = workloads.small_book(paths=1 << 12, n_trades=6, steps_per_year=52, fp32=True)
    direct = engine.price_book_trade_bumps_raw(b)
    with Server(slots=2) as srv:
        got = srv.results(srv.submit_book_trade_bumps(b))
    assert len(got) == len(direct) == 6 * abi.BOOK_TRADE_SCENARIOS
    for a, d in zip(got, direct):
        assert bytes(a) == bytes(d)


def test_a_request_larger_than_the_budget_is_rejected():
    with Server(slots=2, memory_budget=1 << 20) as srv:
        with pytest.raises(RigaError) as e:
            srv.submit_book(workloads.small_book(paths=1 << 14, n_trades=4, steps_per_year=52, fp32=True))
        assert e.value.code == "invalid_argument"


def test_cancel_a_queued_request_and_wait_timeouts():
    big = workloads.lv3(paths=1 << 17, steps=756)
    big.options = workloads.production_options()
    sc = [(m, s) for _, m, s in workloads.crn15_scenarios(big)]
    with Server(slots=1) as srv:
        a = srv.submit_price(big, sc)
        b = srv.submit_price(big, sc)
        srv.cancel(b)
        assert srv.poll(b).state == abi.JOB_CANCELLED
        with pytest.raises(RigaError) as e:
            srv.wait(a, timeout_ms=0)
        assert e.value.code == "device_timeout"
        assert srv.wait(a).state == abi.JOB_DONE
        with pytest.raises(RigaError) as e:
            srv.results(b)
        assert e.value.code == "cancelled"
        st = srv.stats()
        assert st.completed == 1 and st.cancelled == 1


def test_failed_request_reports_the_reference_code():
    with Server(slots=2) as srv:
        b = workloads.small_book(paths=64, n_trades=2)
        b.trades[1].underlyings[0] = 40
        t = srv.submit_book(b)
        with pytest.raises(RigaError) as e:
            srv.wait(t)
        assert e.value.code == "invalid_market_shape"
        assert srv.stats().failed == 1


def test_mcp_loop_over_the_gpu_server(engine):
    """The reference's request JSON alone prices with the reference's arithmetic (Owen scrambling,
    FP64, 512-dimension wrap); the engine knobs ride in "options"."""
    from riga_gb300.types import EngineOptions, PriceRequest
    req = workloads.plain3(paths=1 << 12, steps=126)
    plain = PriceRequest.from_json(req.to_json())
    with Server(slots=2) as srv:
        loop = McpLoop(srv)
        out = loop.handle({"jsonrpc": "2.0", "id": 1, "method": "tools/call",
                           "params": {"name": "price_trade", "arguments": {"request": req.to_json()}}})
        knobs = {"scrambler": req.options.scrambler, "precision": req.options.precision,
                 "dim_mode": req.options.dim_mode}
        out2 = loop.handle({"jsonrpc": "2.0", "id": 2, "method": "tools/call",
                            "params": {"name": "price_trade", "arguments": {"request": req.to_json(), "options": knobs}}})
    assert out["result"]["structuredContent"] == result_to_json(engine.price_raw(plain), plain)
    assert out2["result"]["structuredContent"] == result_to_json(engine.price_raw(req), req)


def test_concurrent_requests_of_different_launch_shapes(engine):
    """FP32 requests with 1..16 scenarios (shared-memory footprints from ~60 to ~160 KB) priced
    concurrently on four slots all succeed and equal the same requests priced alone: a kernel's
    launch attributes are process-wide, so no request may narrow them for another."""
    base = workloads.lv3(paths=1 << 14, steps=252)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(base)]
    reqs = [(base, scen[:k]) for k in (1, 2, 3, 5, 8, 11, 16)] * 3
    alone = [engine.price_scenarios_raw(r, sc) for r, sc in reqs]
    with Server(slots=4) as srv:
        ts = [srv.submit_price(r, sc) for r, sc in reqs]
        got = [srv.results(t) for t in ts]
    for a, g in zip(alone, got):
        assert [bytes(x) for x in a] == [bytes(x) for x in g]


def test_mcp_replay_tools(engine):
    """reconstruct_path / query_path_cube / materialize_paths over the loop's replay engine equal
    the engine's own answers; the cube's records are the run_paths records of its range."""
    from riga_gb300.serve import cube_checksum
    req = workloads.plain3(paths=1 << 10, steps=126)
    args = {"request": req.to_json(), "options": {"scrambler": req.options.scrambler,
                                                  "precision": req.options.precision,
                                                  "dim_mode": req.options.dim_mode}}
    with Server(slots=1) as srv:
        loop = McpLoop(srv)
        try:
            call = lambda name, **kw: loop.handle({"jsonrpc": "2.0", "id": 1, "method": "tools/call",
                                                   "params": {"name": name, "arguments": {**args, **kw}}})
            rec = call("reconstruct_path", path_id=77)["result"]["structuredContent"]
            q = call("query_path_cube", percentile=0.05, max_sample=4)["result"]["structuredContent"]
            q2 = call("query_pathcube", percentile=0.05, max_sample=4)["result"]["structuredContent"]
            cube = call("materialize_paths", first_path=70, count=16)["result"]["structuredContent"]
        finally:
            loop.close()
    same = lambda a, b: json.dumps(a, sort_keys=True) == json.dumps(b, sort_keys=True)  # ko_time NaN
    assert same(rec, engine.reconstruct_path(req, 77))
    assert same(q, q2) and same(q, engine.query_worst_percentile(req, 0.05, 4))
    pc, recs = engine.materialize_paths(req, 70, 16)
    assert same(cube["records"], recs) and same(cube["records"][7], rec)
    assert cube["data"] == [float(v) for v in pc.data]
    assert cube["checksum"] == cube_checksum(pc.data)
    assert (cube["paths"], cube["times"], cube["factors"]) == (16, 126, 3)


def test_small_requests_pass_large_ones_waiting_for_a_large_slot():
    """Two slots, one of which large requests may hold: two large CRN batches and then a small
    request are submitted; the small one runs beside the first large one and finishes before the
    second large one starts, and the two large ones never overlap."""
    big = workloads.lv3(paths=1 << 20, steps=756)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(big)]
    small = workloads.lv3(paths=1 << 12, steps=126)
    with Server(slots=2, max_large_slots=1, large_work=1 << 28) as srv:
        t1 = srv.submit_price(big, scen)
        t2 = srv.submit_price(big, scen)
        t3 = srv.submit_price(small)
        i3 = srv.wait(t3)
        i2 = srv.wait(t2)
        i1 = srv.wait(t1)
    assert i3.end_s <= i2.start_s, (i3.end_s, i2.start_s)
    assert i2.start_s >= i1.end_s, (i2.start_s, i1.end_s)
