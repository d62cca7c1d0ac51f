"""The multi-rank path on host cores: path-range shards priced on two ``gloo`` ranks, their FP64
path sums gathered with one ``all_gather`` and merged on rank 0 by the library's
``rg_merge_results``, against one single-range price of all paths.

Each rank prices its shard with the oracle (the GPU kernels match it bit for bit on these
sizes, which the GPU tests check); what is under test here is the sharding arithmetic, the
collective and the merge."""
from __future__ import annotations

import os
import socket
import sys

import pytest

import oracle as O
from conftest import ROOT
from riga_gb300 import abi, sharding, workloads
from riga_gb300.build import build_library

PATHS_PER_RANK = 384
STEPS = 63


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _summary(r):
    return {"pv": r.pv, "mc_error": r.mc_error, "ki_probability": r.ki_probability,
            "counts": (r.ko_count, r.ki_count, r.put_eligible_count, r.coupon_path_count),
            "stats": [(s.output_count, s.probability, s.mean_payoff, s.variance_payoff) for s in r.stats],
            "legs": (r.legs.coupon, r.legs.memory_coupon, r.legs.down_and_in_put, r.legs.funding)}


def _requests():
    req = workloads.plain3(paths=PATHS_PER_RANK, steps=STEPS)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(req)][:4]
    return req, scen


def _rank_main(rank, world, port, lib_path, q):
    sys.path.insert(0, str(ROOT / "riga-flow_gb300"))
    sys.path.insert(0, str(ROOT / "oracle"))
    import torch.distributed as dist

    import oracle as O_
    from riga_gb300 import abi as abi_, sharding as sh_

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        req, scen = _requests()
        shard = sh_.shard_request(req, rank, world)
        res = list(O_.price_scenarios(shard, scen, threads=2))
        gathered = sh_.gather_path_sums(res)
        if rank == 0:
            lib = abi_.load_library(lib_path)
            merged = sh_.merge_gathered(lib, gathered, PATHS_PER_RANK, req.config.seed)
            q.put(("ok", [_summary(m) for m in merged]))
        dist.barrier()
    except Exception as e:  # reported to the test through the queue
        q.put(("error", f"rank {rank}: {type(e).__name__}: {e}"))
        raise
    finally:
        dist.destroy_process_group()


@pytest.fixture(scope="module")
def lib_path():
    return str(build_library())


def test_shard_request_offsets_path_ranges():
    req, _ = _requests()
    req.options.first_path = 7
    got = [sharding.shard_request(req, r, 4).options.first_path for r in range(4)]
    assert got == [7 + r * PATHS_PER_RANK for r in range(4)]
    assert req.options.first_path == 7  # the caller's request is not modified
    with pytest.raises(ValueError):
        sharding.shard_request(req, 4, 4)


def test_oracle_path_sums_rebuild_its_result(lib_path):
    """The oracle's path sums, run through the library's merge alone, give the oracle's result."""
    lib = abi.load_library(lib_path)
    req, _ = _requests()
    ref = O.price_put_leg(req, threads=2)
    one = sharding.merge(lib, [ref], req.config.paths)
    a, b = _summary(one), _summary(ref)
    assert a["counts"] == b["counts"]
    assert a["pv"] == pytest.approx(b["pv"], rel=1e-13, abs=1e-15)
    assert a["mc_error"] == pytest.approx(b["mc_error"], rel=1e-9)


def test_two_gloo_ranks_merge_to_the_single_range_result(lib_path):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, lib_path, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a rank did not finish"
    status, payload = q.get(timeout=5)
    assert status == "ok", payload
    assert all(p.exitcode == 0 for p in procs)

    req, scen = _requests()
    req.config.paths = 2 * PATHS_PER_RANK
    single = [_summary(r) for r in O.price_scenarios(req, scen, threads=2)]
    assert len(payload) == len(single) == len(scen)
    for got, want in zip(payload, single):
        assert got["counts"] == want["counts"]
        assert got["pv"] == pytest.approx(want["pv"], rel=1e-12, abs=1e-14)
        assert got["ki_probability"] == want["ki_probability"]
        assert got["mc_error"] == pytest.approx(want["mc_error"], rel=1e-9)
        for gs, ws in zip(got["stats"], want["stats"]):
            assert gs[0] == ws[0] and gs[1] == ws[1]
            assert gs[2] == pytest.approx(ws[2], rel=1e-12, abs=1e-14)
            assert gs[3] == pytest.approx(ws[3], rel=1e-8, abs=1e-14)
        for gl, wl in zip(got["legs"], want["legs"]):
            assert gl == pytest.approx(wl, rel=1e-12, abs=1e-14)
