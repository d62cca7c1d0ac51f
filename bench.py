#!/usr/bin/env python3
"""Benchmark of the fused CRN Phoenix engine on the 3-asset Dupire local-vol configuration.

Workload (one "step"): price one trade under base + 15 common-random-number bumps — 16 scenarios —
over 2^20 Sobol paths (digital shift from seed 1) and 756 daily steps, 3 assets under seeded SVI
smiles calibrated to a 40-point Dupire grid, FP32 path state with FP64 sums.  A path-step is one
time step of one path for one (trade, scenario), all assets included.

* ``value`` — path-steps/s with inputs resident: path-steps ÷ device time of the prologue
  kernels + the fused kernel + the final reduction (CUDA events on the engine's stream).
* ``e2e`` — the same metric through the C ABI call a user makes (``rg_price_scenarios``) with host
  inputs: host table build, H2D, all kernels, D2H and result assembly, wall-clock.
* ``--impl reference`` times the reference algorithm's CPU restatement (the oracle) on every host
  core on a bounded sample of the same workload.

Multi-GPU: one process per GPU (torchrun); rank r prices paths [r·P, (r+1)·P) of the same Sobol
sequence (weak scaling), and rank 0 merges the ranks' FP64 path sums in rank order.
"""
from __future__ import annotations

import argparse
import copy
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "riga-flow_gb300"))

METRIC = "path-steps/sec and trades·bumps/sec at ≤1bp error vs FP64; p50/p99 latency"
UNIT = "path-steps/s"


def workload_request(paths: int, steps: int, fp32: bool = True, rank: int = 0, world: int = 1):
    from riga_gb300 import sharding, workloads

    req = sharding.shard_request(workloads.lv3(paths=paths, steps=steps, fp32=fp32), rank, world)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(req)]
    return req, scen


def config_block(paths, steps, n_scen, world):
    return {"workload": f"lv3_crn16: 3-asset worst-of Phoenix under Dupire local vol (seeded SVI, "
                        f"40-point grid), {paths} Sobol paths per GPU (digital shift, seed 1), "
                        f"{steps} steps, base + {n_scen - 1} CRN bumps in one fused launch",
            "paths_per_gpu": paths, "steps": steps, "scenarios": n_scen, "assets": 3,
            "precision": "fp32 path state, fp64 sums", "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": f"path-range shards x{world}" if world > 1 else "single GPU"}


# ----------------------------------------------------------------------------- flops model ---
# Algorithmic FP32 work per unit (FMA = 2 flops), fixed in code:
#   per (path, factor, step) generation: inverse normal 30, bridge 5               -> 35
#   per (path, scenario, step): correlate N(N+1) + payoff 3
#   per (path, scenario, factor, step): local-vol lookup 12, Euler step 6, min 1   -> 19
GEN_FLOPS, ASSET_FLOPS, PAY_FLOPS = 35, 19, 3


def flops_per_launch(paths, steps, n_assets, n_scen):
    per_path_step = GEN_FLOPS * n_assets + n_scen * (n_assets * (n_assets + 1) + PAY_FLOPS + ASSET_FLOPS * n_assets)
    return float(paths) * steps * per_path_step


def n_scen_slots(n_scen):
    """Scenario slots of the tiled FP32 kernel's CTA: the scenario count rounded up to a power of two,
    at least 4."""
    sb = 4
    while sb < n_scen:
        sb <<= 1
    return sb


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


# ----------------------------------------------------------------------------- clocks ---------
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        self.file.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or not f[0].isdigit() or int(f[0]) != self.index:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------- CPU baseline ---
def cpu_rate(paths_hint: int, steps: int, target_s: float):
    """Oracle path-steps/s on every host core for a bounded sample of the workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    req, scen = workload_request(64, steps, fp32=False)
    t0 = time.perf_counter()
    O.price_scenarios(req, scen, threads=threads)
    dt = time.perf_counter() - t0
    per_path = dt / 64.0
    paths = int(max(256, min(paths_hint, target_s / max(per_path, 1e-9))))
    paths = max(threads * 64, (paths // (threads * 64)) * threads * 64)
    req, scen = workload_request(paths, steps, fp32=False)
    t0 = time.perf_counter()
    O.price_scenarios(req, scen, threads=threads)
    dt = time.perf_counter() - t0
    units = float(paths) * steps * len(scen)
    return units / dt, threads, paths, dt


def cpu_rows(steps: int, target_s: float):
    """The CPU rows beside the headline baseline: the oracle on one thread (the shape of the
    reference's own single-threaded loop) on a sample of the bench workload, and the plain
    configuration (3-asset flat-vol Phoenix, FP64, 2^16 Sobol paths x 756 steps, price only) at its
    full size on every host thread, with the time a full-size bench workload would take."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from riga_gb300 import workloads

    O.build()
    threads = os.cpu_count() or 1
    req, scen = workload_request(16, steps, fp32=False)
    t0 = time.perf_counter()
    O.price_scenarios(req, scen, threads=1)
    per_path = (time.perf_counter() - t0) / 16.0
    paths = int(max(16, min(1 << 20, target_s / max(per_path, 1e-9)))) // 16 * 16
    req, scen = workload_request(paths, steps, fp32=False)
    t0 = time.perf_counter()
    O.price_scenarios(req, scen, threads=1)
    dt1 = time.perf_counter() - t0
    one = float(paths) * steps * len(scen) / dt1
    plain = workloads.plain3(paths=1 << 16, steps=756)
    t0 = time.perf_counter()
    O.price_put_leg(plain, threads=threads)
    dtp = time.perf_counter() - t0
    return {"one_thread": {"value": one, "unit": UNIT, "cores": 1, "kind": "port",
                           "sample": f"oracle FP64 on 1 thread, {paths} paths x {steps} steps x {len(scen)} "
                                     f"scenarios ({dt1:.1f} s)"},
            "plain_full_size": {"value": float(1 << 16) * 756 / dtp, "unit": UNIT, "cores": threads, "kind": "port",
                                "wall_s": dtp,
                                "sample": "the plain configuration at full size: 3-asset flat-vol Phoenix, FP64, "
                                          "2^16 Sobol paths x 756 steps, price only, every host thread"}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    rates = []
    for i in range(args.warmup + args.steps):
        rate, cores, paths, dt = cpu_rate(args.paths, args.timesteps, args.cpu_seconds)
        if i >= args.warmup:
            rates.append(rate)
    value = statistics.median(rates)
    sample = (f"oracle FP64 restatement of the reference path (scenario by scenario, as the "
              f"reference re-prices each bump), {paths} paths x {args.timesteps} steps x 16 scenarios per step")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded SVI smiles, CRN bump set)",
            "config": config_block(args.paths, args.timesteps, 16, 1),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- book (cfg 2) --
def book_measure(eng, n_trades: int, paths: int):
    """The book configuration in one call: `n_trades` trades of the 20-asset universe at `paths`
    Sobol paths, every trade under its own 16 scenarios (base + 15 bumps on its own underlyings),
    FP32, host inputs (rg_price_book_trade_bumps); then the same book resident (graph replay)."""
    import torch
    from riga_gb300 import abi, workloads

    S = abi.BOOK_TRADE_SCENARIOS
    b = workloads.book(paths=paths, n_trades=n_trades, fp32=True)
    warm = copy.deepcopy(b)
    warm.config.paths = 1 << 12
    eng.price_book_trade_bumps_raw(warm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.price_book_trade_bumps_raw(b)
    wall = time.perf_counter() - t0
    units = float(sum(t.terms.steps for t in b.trades)) * paths * S
    # accuracy at the book's path count: FP32 against the FP64 book on the same points, a seeded
    # sample of 64 trades of the book distribution (1-5 underlyings), every price and every bump
    # difference (bumped minus base) within min(0.1 SE, 1bp)
    t_acc = time.perf_counter()
    sample = workloads.book(paths=paths, n_trades=64, fp32=True, seed=11)
    r32 = eng.price_book_trade_bumps_raw(sample)
    r64 = eng.price_book_trade_bumps_raw(workloads.book(paths=paths, n_trades=64, fp32=False, seed=11))
    acc_s = time.perf_counter() - t_acc
    err_p = err_d = 0.0
    within = True
    for j in range(64):
        b32, b64 = r32[j * S], r64[j * S]
        for k in range(S):
            a, w = r32[j * S + k], r64[j * S + k]
            bound = min(0.1 * w.mc_error, 1e-4)
            e = abs(a.pv - w.pv)
            d = abs((a.pv - b32.pv) - (w.pv - b64.pv))
            err_p, err_d = max(err_p, e), max(err_d, d)
            within = within and e <= bound and d <= bound
    counts = [0] * 5
    for t in sample.trades:
        counts[len(t.underlyings) - 1] += 1
    # the same book resident on the device: created once (increments generated), the first price
    # tunes and captures, the second replays the graph
    t0 = time.perf_counter()
    rb = eng.resident_book(b)
    create_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    rb.price_trade_bumps_raw()
    first_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    rb.price_trade_bumps_raw()
    replay_s = time.perf_counter() - t0
    stage = rb.tuned_stage(1000 + S)
    rb.close()
    return {"workload": f"book: {n_trades} Phoenix trades (1-5 underlyings, 1-5y) on a 20-asset 4-factor "
                        f"universe, one universe path set on 1260 daily steps, {paths} Sobol paths, every "
                        f"trade under {S} scenarios of its own (base + 15 bumps on its own underlyings: spot "
                        f"+-1%, vol +1pt, rate +1bp, cross-gamma corners, ...), one rg_price_book_trade_bumps "
                        f"call with host inputs",
            "trades": n_trades, "paths": paths, "scenarios_per_trade": S, "wall_s": wall,
            "path_steps_per_s": units / wall, "trades_bumps_per_s": n_trades * S / wall,
            "accuracy": {"max_abs_err_price": err_p, "max_abs_err_bump_difference": err_d,
                         "within_min_0.1se_1bp": within, "fp64_and_fp32_s": acc_s,
                         "sample": f"64 trades (seed 11; by underlying count 1-5: {counts}), {paths} paths, "
                                   f"{S} per-trade scenarios, every price and every bump difference"},
            "resident": {"create_s": create_s, "first_price_s": first_s, "replay_s": replay_s,
                         "path_steps_per_s": units / replay_s, "trades_bumps_per_s": n_trades * S / replay_s,
                         "tuned_steps_per_stage": stage,
                         "note": "rg_book_create once, then rg_book_price_trade_bumps: CUDA-graph replay, "
                                 "increments resident"}}


def fp64_plain_rate(eng):
    """The plain FP64 GPU path: the FP64 parity kernel pricing one trade per call (3-asset
    flat-vol Phoenix, 2^16 paths, 756 steps), path-steps/s through rg_price_put_leg."""
    from riga_gb300 import workloads

    req = workloads.plain3(paths=1 << 16, steps=756)
    eng.price_raw(req)
    t0 = time.perf_counter()
    eng.price_raw(req)
    wall = time.perf_counter() - t0
    return float(1 << 16) * 756 / wall


# ----------------------------------------------------------------------------- large (cfg 4) ---
def large_measure(eng, paths: int = 1 << 24, sample_paths: int = 1 << 16):
    """The large fused configuration: 5-asset worst-of Phoenix under Dupire local vol (64x32 SVI
    grid, 64-point Dupire grid), 2-factor correlation, 1260 steps, `paths` Sobol paths in one FP32
    launch with host inputs (rg_price_put_leg), cross-checked by the same run on scrambled Halton
    points; FP32 against the FP64 parity kernel on the first `sample_paths` points."""
    from riga_gb300 import workloads

    out = {"workload": f"large fused: 5-asset worst-of Phoenix, Dupire local vol (seeded SVI 64x32, "
                       f"64-point grid), 2-factor correlation, 5y x 1260 daily steps, {paths} paths, "
                       f"one scenario, FP32 path state, FP64 sums, no path cube",
           "paths": paths, "steps": 1260, "assets": 5}
    res = {}
    for kind in ("sobol", "halton"):
        req = workloads.lv5_large(paths=paths, kind=kind)
        warm = workloads.lv5_large(paths=1 << 12, kind=kind)
        eng.price_raw(warm)
        t0 = time.perf_counter()
        r = eng.price_raw(req)
        wall = time.perf_counter() - t0
        tm = eng.last_timing()
        res[kind] = r
        out[kind] = {"pv": r.pv, "mc_error": r.mc_error, "wall_s": wall, "kernel_ms": tm.kernel_ms,
                     "path_steps_per_s": float(paths) * 1260 / wall,
                     "kernel_path_steps_per_s": float(paths) * 1260 / (tm.kernel_ms / 1e3)}
    s, h = res["sobol"], res["halton"]
    out["halton_vs_sobol_in_se"] = abs(s.pv - h.pv) / math.sqrt(s.mc_error ** 2 + h.mc_error ** 2)
    # the cross-check by randomized QMC: independent scramblings (seeds 1-4) of each lane, the
    # lanes' means compared in units of the replicates' own standard error (the MC standard error
    # of one run does not measure a QMC estimate's error)
    reps = {"sobol": [], "halton": []}
    for kind in reps:
        for seed in (1, 2, 3, 4):
            req = workloads.lv5_large(paths=paths, kind=kind)
            req.config.seed = seed
            reps[kind].append(eng.price_raw(req).pv)
    rq = {}
    for kind, v in reps.items():
        m = statistics.mean(v)
        rq[kind] = {"seeds": [1, 2, 3, 4], "pv": v, "mean": m, "rqmc_se": statistics.stdev(v) / math.sqrt(len(v))}
    se = math.sqrt(rq["sobol"]["rqmc_se"] ** 2 + rq["halton"]["rqmc_se"] ** 2)
    out["rqmc_cross_check"] = dict(rq, halton_vs_sobol_in_rqmc_se=abs(rq["sobol"]["mean"] - rq["halton"]["mean"]) / se)
    r32 = eng.price_raw(workloads.lv5_large(paths=sample_paths))
    r64 = eng.price_raw(workloads.lv5_large(paths=sample_paths, fp32=False))
    out["accuracy"] = {"abs_err_vs_fp64": abs(r32.pv - r64.pv), "bound_min_0.1se_1bp": min(0.1 * r64.mc_error, 1e-4),
                       "within_bound": abs(r32.pv - r64.pv) <= min(0.1 * r64.mc_error, 1e-4),
                       "sample": f"first {sample_paths} Sobol points, FP32 kernel vs FP64 parity kernel"}
    return out


# ----------------------------------------------------------------------------- serving (cfg 3) -
def serving_measure(duration_s: float = 60.0, rate_per_s: float = 200.0, book_rate_per_s: float = 1.0,
                    budget_gib: float = 24.0, seed: int = 7):
    """Seeded Poisson arrivals at `rate_per_s` into the continuous-batching server (4 slots) for
    `duration_s` seconds: single 3-asset local-vol trades at 2^14 paths (756 steps, FP32) and, at
    `book_rate_per_s` of the arrivals, books of 16-256 trades of the book distribution at 2^18 paths;
    every request takes 0, 7 or 15 CRN bumps (a book's 15 are per-trade bumps on its own underlyings,
    its 7 the first 8 scenarios of the universe-wide common set).  The server admits requests within
    a device-memory budget of `budget_gib` GiB, which holds one 2^18-path book (its double-buffered
    universe increments) beside the singles, so overlapping books wait for memory.  Latency is
    submit to completion per request; throughput counts every finished request's path-steps."""
    from riga_gb300 import workloads
    from riga_gb300.serve import Server

    rng = workloads.SplitMix64(seed)
    single = workloads.lv3(paths=1 << 14, steps=756, fp32=True)
    scen = [(m, s) for _, m, s in workloads.crn15_scenarios(single)]
    book_paths = 1 << 18
    bk = workloads.book(paths=book_paths, n_trades=256, fp32=True)
    bsc = [m for _, m in workloads.book_scenarios(bk.universe)][:8]
    plan, t = [], 0.0
    while True:
        t += -math.log(1.0 - rng.uniform(0.0, 1.0)) / rate_per_s
        if t >= duration_s:
            break
        k = (0, 7, 15)[rng.next_u64() % 3]
        if rng.uniform(0.0, 1.0) < book_rate_per_s / rate_per_s:
            plan.append((t, "book", k, 16 + rng.next_u64() % 241))
        else:
            plan.append((t, "price", k, 1))

    def submit(srv, kind, k, n_trades):
        if kind == "price":
            return srv.submit_price(single, scen[: k + 1] if k else None), float(1 << 14) * 756 * (k + 1)
        b = copy.copy(bk)
        b.trades = bk.trades[:n_trades]
        steps = float(sum(tr.terms.steps for tr in b.trades)) * book_paths
        if k == 15:
            return srv.submit_book_trade_bumps(b), steps * 16
        return srv.submit_book(b, bsc if k == 7 else None), steps * (k + 1)

    budget = int(budget_gib * (1 << 30))
    lat, split = {}, {}
    units = 0.0
    with Server(slots=4, memory_budget=budget) as srv:
        # warm-up outside the timed window: every request shape once per slot, books at their
        # largest (256 trades, 15 per-trade bumps) so that engines hold their largest buffers (the
        # first book on an engine pays the one-time cost of its tables and kernel loading)
        tickets = []
        for _ in range(4):
            for k in (0, 7, 15):
                tickets += [submit(srv, "book", k, 256 if k == 15 else 16)[0], submit(srv, "price", k, 1)[0]]
        for tk in tickets:
            srv.wait(tk)
            srv.release(tk)
        st0 = srv.stats()
        t0 = time.perf_counter()
        live = []
        for at, kind, k, n_trades in plan:
            delay = at - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tk, u = submit(srv, kind, k, n_trades)
            live.append((tk, kind, k, n_trades))
            units += u
        for tk, kind, k, n_trades in live:
            info = srv.wait(tk)
            srv.release(tk)
            lat.setdefault((kind, k), []).append(1e3 * (info.end_s - info.submit_s))
            split.setdefault(kind, []).append((1e3 * (info.start_s - info.submit_s), 1e3 * (info.end_s - info.start_s)))
        wall = time.perf_counter() - t0
        st = srv.stats()

    def pct(v, q):
        v = sorted(v)
        return v[min(len(v) - 1, max(0, math.ceil(q * len(v)) - 1))]

    every = [x for v in lat.values() for x in v]
    classes = {}
    for (kind, k), v in sorted(lat.items()):
        name = ("single_2^14_paths" if kind == "price" else "book_16-256_trades_2^18_paths") + f"_{k}_bumps"
        classes[name] = {"requests": len(v), "p50_ms": pct(v, 0.50), "p99_ms": pct(v, 0.99), "max_ms": max(v)}
    # where the time goes, per kind: waiting in the queue (submit -> start) and running (start -> end)
    phases = {kind: {"queue_p50_ms": pct([a for a, _ in v], 0.5), "queue_p99_ms": pct([a for a, _ in v], 0.99),
                     "run_p50_ms": pct([b for _, b in v], 0.5), "run_p99_ms": pct([b for _, b in v], 0.99)}
              for kind, v in split.items()}
    n_books = sum(1 for p in plan if p[1] == "book")
    return {"workload": f"Poisson arrivals at {rate_per_s:g}/s for {duration_s:g} s (seed {seed}): single 3-asset "
                        f"local-vol trades at 2^14 paths x 756 steps and, at {book_rate_per_s:g}/s, books of "
                        f"16-256 trades of the book distribution at 2^18 paths; 0, 7 or 15 CRN bumps per request "
                        f"(books: 15 per-trade bumps, or the first 8 common scenarios); 4 slots, device-memory "
                        f"budget {budget_gib:g} GiB",
            "requests": len(plan), "books": n_books, "completed": st.completed - st0.completed,
            "failed": st.failed - st0.failed, "p50_ms": pct(every, 0.50), "p99_ms": pct(every, 0.99),
            "max_ms": max(every), "classes": classes, "phases": phases, "wall_s": wall,
            "path_steps_per_s": units / wall,
            "busy_s": st.busy_s - st0.busy_s,
            "admission": {"device_memory_budget_bytes": budget, "memory_waits": st.memory_waits - st0.memory_waits,
                          "peak_reserved_bytes": st.peak_reserved_bytes,
                          "note": "memory_waits: requests that waited at the head of the queue because their "
                                  "device-memory estimate did not fit beside the running requests"},
            "sustained_rate": f"{rate_per_s:g} requests/s, of which {book_rate_per_s:g}/s books (the book rate "
                              f"the GPU sustains beside the singles)",
            "warm_up": "24 requests before the timed window (each slot: a single with 0, 7 and 15 bumps, 16-trade "
                       "books with 0 and 7 bumps and a 256-trade book with 15 per-trade bumps)"}


# ----------------------------------------------------------------------------- GPU arm --------
def run_gpu(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from riga_gb300 import abi, sharding
    from riga_gb300.build import build_library
    from riga_gb300.engine import Engine
    import ctypes as C

    build_library()
    eng = Engine(local)
    if args.shape:
        knobs = [int(x) for x in args.shape.split(",")] + [0]
        abi.check(eng.lib, eng.lib.rg_set_tiled_shape(knobs[0], knobs[1], knobs[2]))
    P, T = args.paths, args.timesteps
    req, scen = workload_request(P, T, fp32=True, rank=rank, world=world)
    n_scen = len(scen)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def one_step():
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = eng.price_scenarios_raw(req, scen)
        wall = time.perf_counter() - t0
        tm = abi.Timing()
        abi.check(eng.lib, eng.lib.rg_engine_last_timing(eng.handle, C.byref(tm)))
        return res, wall, tm

    for _ in range(args.warmup):
        one_step()
    if args.phase_clocks:
        # the tiled kernel's per-phase CTA clock cycles over the timed steps (a library built with
        # RG_PHASE_CLOCKS=1 only; the counters add a few instructions per phase)
        clk4 = (C.c_uint64 * 4)()
        abi.check(eng.lib, eng.lib.rg_phase_clocks(clk4, 1))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    walls, dev_ms, ker_ms, timings = [], [], [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            res, wall, tm = one_step()
            walls.append(wall)
            dev_ms.append(tm.prologue_ms + tm.kernel_ms + tm.reduce_ms)
            ker_ms.append(tm.kernel_ms)
            timings.append(tm)
    torch.cuda.synchronize()
    tot = torch.tensor([sum(dev_ms), sum(walls)], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(tot, op=torch.distributed.ReduceOp.MAX)
        # the one gather: every rank's FP64 path sums, merged in rank order on rank 0
        gathered = sharding.gather_path_sums(res, device=torch.device("cuda", local))
    dev_total_s, wall_total_s = tot[0].item() / 1e3, tot[1].item()
    units = float(P) * T * n_scen * world * args.steps
    value = units / dev_total_s
    e2e = units / wall_total_s
    if rank != 0:
        return
    merged_pv = None
    if world > 1:
        merged_pv = sharding.merge_gathered(eng.lib, gathered, P, req.config.seed)[0].pv
    # accuracy: FP32 against the FP64 parity kernel on the same points (outside the timed region)
    req64, _ = workload_request(P, T, fp32=False, rank=rank, world=world)
    t_acc = time.perf_counter()
    res64 = eng.price_scenarios_raw(req64, scen)
    acc_s = time.perf_counter() - t_acc
    errs = [abs(a.pv - b.pv) for a, b in zip(res, res64)]
    bounds = [min(0.1 * b.mc_error, 1e-4) for b in res64]
    peaks = measured_peaks()
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * sm_max * 1e6 / 1e12
    kern_avg_s = statistics.mean(ker_ms) / 1e3
    achieved = flops_per_launch(P, T, 3, n_scen) / kern_avg_s / 1e12
    # DRAM bytes per launch of the fused kernel, from the committed ncu capture at this size
    traffic = None
    tfile = ROOT / "profiles" / "phoenix32_lv3_crn16_dram.md"
    if tfile.exists() and P == 1 << 20 and T == 756 and n_scen == 16:
        for ln in tfile.read_text().splitlines():
            if ln.startswith("traffic_bytes_per_launch:"):
                traffic = float(ln.split(":", 1)[1])
    clocks = clk.summary()
    tm = timings[-1]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded SVI smiles, CRN bump set; no public dataset exists for this path)",
        "config": config_block(P, T, n_scen, world),
        "trades_bumps_per_s": n_scen * world * args.steps / dev_total_s,
        "latency_ms": {"p50": 1e3 * statistics.median(walls),
                       "p99": 1e3 * sorted(walls)[max(0, int(round(0.99 * len(walls))) - 1)]},
        "accuracy": {"max_abs_err_vs_fp64": max(errs), "bound_min_0.1se_1bp": min(bounds),
                     "within_bound": all(e <= b for e, b in zip(errs, bounds)),
                     "fp64_parity_kernel_s": acc_s},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "peak_source": f"nominal FP32: {sms} SMs x 128 lanes x 2 x sm_max_mhz {sm_max} "
                                    f"(MEASURED_PEAKS.json has no FP32 figure)",
                     "kernel_ms": 1e3 * kern_avg_s,
                     "flops_per_launch": flops_per_launch(P, T, 3, n_scen)},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(tm.h2d_bytes),
                "d2h_bytes_per_step": int(tm.d2h_bytes)},
        "gpu_launches": int(tm.kernel_launches) * args.steps,
        "launch": {"grid": tm.grid, "block": tm.block, "smem_bytes": tm.smem_bytes,
                   "tile_steps": tm.tile_steps, "paths_per_thread": tm.paths_per_thread,
                   "paths_per_cta_tile": tm.block * tm.paths_per_thread // n_scen_slots(n_scen),
                   "tuned_by": (f"forced by --shape {args.shape} (rg_set_tiled_shape)" if args.shape else
                                "autotuner (rg_set_autotune): paths per CTA tile, paths per thread and tile depth, "
                                "timed during warm-up")},
        "clocks": clocks,
    }
    if merged_pv is not None:
        line["merged_base_pv"] = merged_pv
    if args.phase_clocks:
        abi.check(eng.lib, eng.lib.rg_phase_clocks(clk4, 0))
        tot = float(sum(clk4)) or 1.0
        line["phase_clocks"] = {"cycles": list(clk4), "share": {k: v / tot for k, v in zip(
            ("generation", "bridge", "stepping", "path_close"), clk4)},
            "note": "CTA wall clock cycles per phase of the tiled kernel over the timed steps (RG_PHASE_CLOCKS=1 build)"}
    if world == 1 and not args.no_book:
        book = book_measure(eng, args.book_trades, args.book_paths)
        plain = fp64_plain_rate(eng)
        book["fp64_plain_path_steps_per_s"] = plain
        book["fp64_plain_workload"] = ("FP64 parity kernel, one trade per call: 3-asset flat-vol Phoenix, "
                                       "2^16 paths x 756 steps, rg_price_put_leg")
        book["throughput_vs_fp64_plain"] = book["path_steps_per_s"] / plain
        line["book"] = book
    if world == 1 and not args.no_large:
        line["large"] = large_measure(eng, paths=args.large_paths, sample_paths=min(1 << 16, args.large_paths))
    if world == 1 and not args.no_serving:
        line["serving"] = serving_measure(duration_s=args.serving_seconds)
    if world == 1 and not args.no_cpu_baseline:
        rate, cores, paths, dt = cpu_rate(P, T, args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"oracle FP64 on {cores} host threads, {paths} paths x {T} steps "
                                          f"x {n_scen} scenarios ({dt:.1f} s)"}
        rows = cpu_rows(T, args.cpu_seconds)
        rows["bench_workload_at_full_size_s"] = {
            "value": float(P) * T * n_scen / rate, "cores": cores,
            "note": "the bench workload (all its paths and scenarios) on every host thread at the sampled rate: "
                    "too long to run inside the bench"}
        line["cpu_baseline_rows"] = rows
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--paths", type=int, default=1 << 20)
    ap.add_argument("--timesteps", type=int, default=756)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-book", action="store_true", help="skip the book (cfg 2) measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving (cfg 3) measurement")
    ap.add_argument("--no-large", action="store_true", help="skip the large fused (cfg 4) measurement")
    ap.add_argument("--only", choices=["book", "serving", "large"], default=None,
                    help="run one secondary measurement alone (for profiling) and print its JSON")
    ap.add_argument("--large-paths", type=int, default=1 << 24, help="paths of the large fused (cfg 4) run")
    ap.add_argument("--book-trades", type=int, default=4096)
    ap.add_argument("--book-paths", type=int, default=1 << 18)
    ap.add_argument("--serving-seconds", type=float, default=60.0, help="window of the serving (cfg 3) run")
    ap.add_argument("--phase-clocks", action="store_true",
                    help="report the tiled kernel's per-phase clock cycles (needs a library built with RG_PHASE_CLOCKS=1)")
    ap.add_argument("--shape", default=None, metavar="PPT,TT[,PB]",
                    help="force the tiled FP32 kernel's paths per thread, tile depth and paths per CTA tile "
                         "(rg_set_tiled_shape) instead of autotuning them, e.g. for a profiler capture with no "
                         "tuning launches")
    args = ap.parse_args()
    if args.only:
        import torch

        torch.cuda.set_device(0)
        from riga_gb300.build import build_library
        from riga_gb300.engine import Engine

        build_library()
        if args.only == "book":
            print(json.dumps(book_measure(Engine(0), args.book_trades, args.book_paths)), flush=True)
        elif args.only == "large":
            print(json.dumps(large_measure(Engine(0), paths=args.large_paths,
                                           sample_paths=min(1 << 16, args.large_paths))), flush=True)
        else:
            print(json.dumps(serving_measure(duration_s=args.serving_seconds)), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
