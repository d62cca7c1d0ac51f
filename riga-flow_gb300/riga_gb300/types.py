"""Request and result types mirroring the reference's serde types, with their JSON forms.

* ``PhoenixTrade``, ``MarketSnapshot``, ``SimulationConfig``, ``VarianceReduction``, ``TraceLevel``,
  ``PriceResult`` and friends: crates/riga-core/src/lib.rs:21-255.
* ``ImpliedVolGrid``: crates/riga-market/src/lib.rs:83-91; ``LocalVolSpec`` / ``PriceRequest``:
  crates/riga-engine/src/lib.rs:31-46.

``to_json``/``from_json`` use the reference's serde field names and shapes, so a request or a
result round-trips through the same JSON a riga-flow client sends and receives.  The engine's own
knobs (scrambler, precision, dimension mode, Dupire grid width) live in ``EngineOptions`` and are
not part of the reference's JSON.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
from dataclasses import dataclass, field
from typing import Any, Optional

from . import abi

TRACE_LEVELS = ("off", "aggregated", "sampled", "full")


def _f64_json(x: float) -> str:
    """Format an f64 the way serde_json (ryu) does: shortest round-trip digits, ``1.0`` for
    integral values, ``1e-7`` style exponents outside [1e-5, 1e16)."""
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    if math.isnan(x) or math.isinf(x):
        return "null"
    sign = "-" if x < 0 else ""
    r = repr(abs(x))
    mant, _, exp = r.partition("e")
    e = int(exp) if exp else 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    # position of the decimal point relative to the start of `digits`
    point = len(ip) + e - (len(ip + fp) - len((ip + fp).lstrip("0")))
    digits = digits.rstrip("0") or "0"
    length, kk = len(digits), point
    k = kk - length
    if 0 <= k and kk <= 16:
        return sign + digits + "0" * k + ".0"
    if 0 < kk <= 16:
        return sign + digits[:kk] + "." + digits[kk:]
    if -5 < kk <= 0:
        return sign + "0." + "0" * (-kk) + digits
    if length == 1:
        return f"{sign}{digits}e{kk - 1}"
    return f"{sign}{digits[0]}.{digits[1:]}e{kk - 1}"


def dumps_serde(value: Any) -> str:
    """Compact JSON with serde_json's float formatting (keys in insertion order)."""
    if isinstance(value, bool):
        return "true" if value else "false"
    if value is None:
        return "null"
    if isinstance(value, int):
        return str(value)
    if isinstance(value, float):
        return _f64_json(value)
    if isinstance(value, str):
        return json.dumps(value, ensure_ascii=False)
    if isinstance(value, (list, tuple)):
        return "[" + ",".join(dumps_serde(v) for v in value) + "]"
    if isinstance(value, dict):
        return "{" + ",".join(json.dumps(k) + ":" + dumps_serde(v) for k, v in value.items()) + "}"
    raise TypeError(type(value))


@dataclass
class VarianceReduction:
    """``VarianceReduction {None | Halton{dimension} | Sobol{dimension}}`` (riga-core lib.rs:88-106)."""

    kind: str = "none"
    dimension: int = 0

    def to_json(self) -> dict:
        return {"kind": self.kind} if self.kind == "none" else {"kind": self.kind, "dimension": self.dimension}

    @staticmethod
    def from_json(d: dict) -> "VarianceReduction":
        return VarianceReduction(d.get("kind", "none"), int(d.get("dimension", 0)))

    @property
    def code(self) -> int:
        return {"none": abi.VR_NONE, "halton": abi.VR_HALTON, "sobol": abi.VR_SOBOL}[self.kind]


@dataclass
class PhoenixTrade:
    trade_id: str
    initial_spots: list
    maturity_years: float
    steps: int
    strike: float
    knock_in_barrier: float
    knock_out_barrier: Optional[float] = None
    coupon_barrier: Optional[float] = None
    coupon_rate: Optional[float] = None
    memory_coupon: bool = False
    coupon_periods: Optional[int] = None
    fixed_first_coupon: bool = False
    call_start_step: Optional[int] = None

    def to_json(self) -> dict:
        return dict(self.__dict__)


@dataclass
class MarketSnapshot:
    as_of: str
    spots: list
    vols: list
    risk_free_rate: float
    dividend_yields: list
    correlation: list  # nested rows

    def to_json(self) -> dict:
        return {"as_of": self.as_of, "spots": [float(x) for x in self.spots],
                "vols": [float(x) for x in self.vols], "risk_free_rate": float(self.risk_free_rate),
                "dividend_yields": [float(x) for x in self.dividend_yields],
                "correlation": [[float(x) for x in row] for row in self.correlation]}

    def snapshot_id(self) -> str:
        """SHA-256 of the serde_json bytes, riga-core lib.rs:47-55."""
        return "sha256:" + hashlib.sha256(dumps_serde(self.to_json()).encode()).hexdigest()


@dataclass
class SimulationConfig:
    paths: int = 30_000
    path_block_size: int = 4_096
    seed: int = 1_729
    trace_level: str = "aggregated"
    variance_reduction: VarianceReduction = field(default_factory=VarianceReduction)

    def to_json(self) -> dict:
        return {"paths": self.paths, "path_block_size": self.path_block_size, "seed": self.seed,
                "trace_level": self.trace_level,
                "variance_reduction": self.variance_reduction.to_json()}


@dataclass
class ImpliedVolGrid:
    maturities_years: list
    strikes: list
    vols: list  # [n_maturity][n_strike]

    def to_json(self) -> dict:
        return {"maturities_years": list(self.maturities_years), "strikes": list(self.strikes),
                "vols": [list(r) for r in self.vols]}


@dataclass
class EngineOptions:
    """This engine's knobs; all-default reproduces the reference's arithmetic."""

    scrambler: int = abi.SCRAMBLE_OWEN
    precision: int = abi.PRECISION_FP64_PARITY
    dim_mode: int = abi.DIM_WRAP_REFERENCE
    lv_grid_x: int = 0
    first_path: int = 0


@dataclass
class PriceRequest:
    trade: PhoenixTrade
    market: MarketSnapshot
    config: SimulationConfig
    as_of: str
    local_vol: Optional[list] = None  # list[ImpliedVolGrid] (LocalVolSpec.grids)
    options: EngineOptions = field(default_factory=EngineOptions)

    def to_json(self) -> dict:
        d = {"trade": self.trade.to_json(), "market": self.market.to_json(),
             "config": self.config.to_json(), "as_of": self.as_of}
        if self.local_vol is not None:
            d["local_vol"] = {"grids": [g.to_json() for g in self.local_vol]}
        return d

    @staticmethod
    def from_json(d: dict, options: Optional[EngineOptions] = None) -> "PriceRequest":
        t, m, c = d["trade"], d["market"], d["config"]
        trade = PhoenixTrade(
            trade_id=t["trade_id"], initial_spots=list(t["initial_spots"]),
            maturity_years=float(t["maturity_years"]), steps=int(t["steps"]),
            strike=float(t["strike"]), knock_in_barrier=float(t["knock_in_barrier"]),
            knock_out_barrier=t.get("knock_out_barrier"), coupon_barrier=t.get("coupon_barrier"),
            coupon_rate=t.get("coupon_rate"), memory_coupon=bool(t.get("memory_coupon", False)),
            coupon_periods=t.get("coupon_periods"),
            fixed_first_coupon=bool(t.get("fixed_first_coupon", False)),
            call_start_step=t.get("call_start_step"))
        market = MarketSnapshot(m["as_of"], list(m["spots"]), list(m["vols"]),
                                float(m["risk_free_rate"]), list(m["dividend_yields"]),
                                [list(r) for r in m["correlation"]])
        config = SimulationConfig(int(c["paths"]), int(c["path_block_size"]), int(c["seed"]),
                                  c.get("trace_level", "aggregated"),
                                  VarianceReduction.from_json(c.get("variance_reduction", {})))
        lv = None
        if d.get("local_vol") is not None:
            lv = [ImpliedVolGrid(list(g["maturities_years"]), list(g["strikes"]),
                                 [list(r) for r in g["vols"]]) for g in d["local_vol"]["grids"]]
        return PriceRequest(trade, market, config, d["as_of"], lv, options or EngineOptions())

    # ------------------------------------------------------------------ ABI conversion ------
    def to_abi(self) -> "AbiRequest":
        return AbiRequest(self)


def _darr(values) -> C.Array:
    vals = [float(v) for v in values]
    return (C.c_double * max(1, len(vals)))(*vals)


class AbiRequest:
    """Owns the ctypes buffers behind one ``rg_price_request``."""

    def __init__(self, req: PriceRequest):
        t, m, c, o = req.trade, req.market, req.config, req.options
        self._keep = []
        n = len(m.spots)
        self.n = n

        def keep(x):
            self._keep.append(x)
            return x

        tr = trade_to_abi(t, keep)

        self.market = market_to_abi(m, keep)
        cfg = config_to_abi(c, o)

        r = abi.PriceRequest()
        r.trade = tr
        r.market = self.market
        r.config = cfg
        r.as_of = keep(req.as_of.encode())
        if req.local_vol is not None:
            grids = (abi.ImpliedVolGrid * max(1, len(req.local_vol)))()
            for i, g in enumerate(req.local_vol):
                grids[i].n_maturities = len(g.maturities_years)
                grids[i].n_strikes = len(g.strikes)
                grids[i].maturities_years = C.cast(keep(_darr(g.maturities_years)), C.POINTER(C.c_double))
                grids[i].strikes = C.cast(keep(_darr(g.strikes)), C.POINTER(C.c_double))
                flat = [v for row in g.vols for v in row]
                grids[i].vols = C.cast(keep(_darr(flat)), C.POINTER(C.c_double))
            keep(grids)
            r.n_local_vol = len(req.local_vol)
            r.local_vol = C.cast(grids, C.POINTER(abi.ImpliedVolGrid))
        else:
            r.n_local_vol = 0
            r.local_vol = None
        self.req = r
        self.ptr = C.pointer(r)


def trade_to_abi(t: PhoenixTrade, keep) -> abi.Trade:
    tr = abi.Trade()
    tr.trade_id = keep(t.trade_id.encode())
    tr.n_assets = len(t.initial_spots)
    tr.initial_spots = C.cast(keep(_darr(t.initial_spots)), C.POINTER(C.c_double))
    tr.maturity_years = t.maturity_years
    tr.steps = t.steps
    tr.strike = t.strike
    tr.knock_in_barrier = t.knock_in_barrier
    for name in ("knock_out_barrier", "coupon_barrier", "coupon_rate"):
        v = getattr(t, name)
        setattr(tr, "has_" + name, 0 if v is None else 1)
        setattr(tr, name, 0.0 if v is None else float(v))
    tr.memory_coupon = int(bool(t.memory_coupon))
    tr.has_coupon_periods = 0 if t.coupon_periods is None else 1
    tr.coupon_periods = 0 if t.coupon_periods is None else int(t.coupon_periods)
    tr.fixed_first_coupon = int(bool(t.fixed_first_coupon))
    tr.has_call_start_step = 0 if t.call_start_step is None else 1
    tr.call_start_step = 0 if t.call_start_step is None else int(t.call_start_step)
    return tr


def config_to_abi(c: SimulationConfig, o: EngineOptions) -> abi.SimConfig:
    cfg = abi.SimConfig()
    cfg.paths, cfg.path_block_size, cfg.seed = c.paths, c.path_block_size, c.seed
    cfg.trace_level = TRACE_LEVELS.index(c.trace_level)
    cfg.variance_reduction = c.variance_reduction.code
    cfg.qmc_dimension = c.variance_reduction.dimension
    cfg.scrambler, cfg.precision, cfg.dim_mode, cfg.lv_grid_x = (
        o.scrambler, o.precision, o.dim_mode, o.lv_grid_x)
    cfg.first_path = o.first_path
    return cfg


# ---------------------------------------------------------------------- books ----------------
@dataclass
class BookTrade:
    """One trade of a book: Phoenix terms on `underlyings` (indices into the book's universe)."""

    terms: PhoenixTrade
    underlyings: list


@dataclass
class BookRequest:
    """Many trades on one asset universe over one common grid (``rg_book_request``)."""

    universe: MarketSnapshot
    universe_steps: int
    universe_maturity_years: float
    trades: list  # list[BookTrade]
    config: SimulationConfig
    options: EngineOptions = field(default_factory=EngineOptions)

    @property
    def dt(self) -> float:
        return self.universe_maturity_years / self.universe_steps

    def to_abi(self) -> "AbiBookRequest":
        return AbiBookRequest(self)


class AbiBookRequest:
    """Owns the ctypes buffers behind one ``rg_book_request``."""

    def __init__(self, book: BookRequest):
        self._keep = []

        def keep(x):
            self._keep.append(x)
            return x

        arr = (abi.BookTrade * len(book.trades))()
        for i, bt in enumerate(book.trades):
            arr[i].terms = trade_to_abi(bt.terms, keep)
            idx = (C.c_int32 * max(1, len(bt.underlyings)))(*[int(a) for a in bt.underlyings])
            arr[i].underlyings = C.cast(keep(idx), C.POINTER(C.c_int32))
        keep(arr)
        r = abi.BookRequest()
        r.universe = market_to_abi(book.universe, keep)
        r.universe_steps = int(book.universe_steps)
        r.universe_maturity_years = float(book.universe_maturity_years)
        r.n_trades = len(book.trades)
        r.trades = C.cast(arr, C.POINTER(abi.BookTrade))
        cfg = config_to_abi(book.config, book.options)
        r.config = cfg
        self.req = r
        self.ptr = C.pointer(r)


def markets_to_abi(markets, keep):
    """A C array of ``rg_market_snapshot`` (or (None, 0) for an empty list); `keep` is called with
    every ctypes buffer the array points into, so the caller can hold them alive."""
    if not markets:
        return None, 0

    def hold(x):
        keep(x)
        return x

    arr = (abi.Market * len(markets))()
    for i, m in enumerate(markets):
        arr[i] = market_to_abi(m, hold)
    hold(arr)
    return arr, len(markets)


def market_to_abi(m: MarketSnapshot, keep) -> abi.Market:
    mk = abi.Market()
    mk.as_of = keep(m.as_of.encode())
    mk.n_assets = len(m.spots)
    mk.spots = C.cast(keep(_darr(m.spots)), C.POINTER(C.c_double))
    mk.vols = C.cast(keep(_darr(m.vols)), C.POINTER(C.c_double))
    mk.risk_free_rate = m.risk_free_rate
    mk.dividend_yields = C.cast(keep(_darr(m.dividend_yields)), C.POINTER(C.c_double))
    mk.correlation = C.cast(keep(_darr([v for row in m.correlation for v in row])), C.POINTER(C.c_double))
    return mk


# ---------------------------------------------------------------------- results --------------
TRANSITION_IDS = ("daily_global_ko", "final_fixing_eki", "memory_coupon")


def _fmt6(x: float) -> str:
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    return f"{x:.6f}"


def result_to_json(res: abi.PriceResult, request: PriceRequest) -> dict:
    """Assemble the reference's ``PriceResult`` JSON (note.rs:262-372) from the ABI result."""
    t = request.trade
    snapshot = request.market.snapshot_id()
    call_barrier = t.knock_out_barrier if t.knock_out_barrier is not None else math.inf
    coupon_barrier = t.coupon_barrier if t.coupon_barrier is not None else math.inf
    evidence = [f"trade:{t.trade_id}", f"market:{snapshot}", f"seed:{request.config.seed}"]
    conditions = (
        f"all names >= {_fmt6(call_barrier)} during callable observations",
        f"terminal worst <= {_fmt6(t.knock_in_barrier)} and no prior autocall; put strike {_fmt6(t.strike)}",
        f"daily worst-of >= coupon barrier {_fmt6(coupon_barrier)}; memory carry enabled="
        f"{'true' if t.memory_coupon else 'false'}",
    )
    legs = res.legs
    out = {
        "pv": res.pv,
        "mc_error": res.mc_error,
        "ki_probability": res.ki_probability,
        "legs": {k: getattr(legs, k) for k in ("par_redemption", "coupon", "memory_coupon",
                                                 "down_and_in_put", "funding", "discounting",
                                                 "total")},
        "stats": [{"transition_id": TRANSITION_IDS[i], "input_count": res.stats[i].input_count,
                   "output_count": res.stats[i].output_count,
                   "probability": res.stats[i].probability,
                   "mean_payoff": res.stats[i].mean_payoff,
                   "variance_payoff": res.stats[i].variance_payoff,
                   "mean_delta": res.stats[i].mean_delta, "mean_vega": res.stats[i].mean_vega}
                  for i in range(abi.RG_N_TRANSITIONS)],
        "ledger": [{"transition_id": TRANSITION_IDS[i], "condition": conditions[i],
                    "population_before": res.ledger[i].population_before,
                    "population_after": res.ledger[i].population_after,
                    "pv_impact": res.ledger[i].pv_impact,
                    "delta_impact": res.ledger[i].delta_impact,
                    "vega_impact": res.ledger[i].vega_impact,
                    "evidence_refs": list(evidence)}
                   for i in range(abi.RG_N_TRANSITIONS)],
    }
    events = [f"daily_global_ko:path={res.trace_events[i].path_id}:t={res.trace_events[i].time:.6f}"
              for i in range(res.n_trace_events)]
    if events:
        out["trace_events"] = events
    out["determinism"] = {"seed": request.config.seed, "as_of": request.as_of,
                          "market_snapshot_id": snapshot}
    return out


def record_to_dict(r: abi.PathRecord) -> dict:
    return {"path_id": r.path_id, "rng_seed": r.rng_seed, "sobol_index": r.sobol_index,
            "worst_final": r.worst_final, "knocked_out": bool(r.knocked_out),
            "ko_step": r.ko_step, "ko_time": r.ko_time, "ki_hit": bool(r.ki_hit),
            "qualified_steps": r.qualified_steps, "paid_periods": r.paid_periods,
            "put_payoff": r.put_payoff, "coupon_pv": r.coupon_pv,
            "memory_coupon_pv": r.memory_coupon_pv, "funding": r.funding, "pv": r.pv}
