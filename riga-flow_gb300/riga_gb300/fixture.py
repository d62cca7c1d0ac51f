"""Loader for the reference's ``termsheet1`` fixture document.

Restates ``load_termsheet1_fixture`` (crates/riga-engine/src/fixture.rs:150-460): dates become
weekday step counts (:64-123), the ATM term structures and the discount curve are interpolated at
the remaining maturity (:125-148), and the captured implied grids become ``LocalVolSpec`` grids
(:299-357).
"""
from __future__ import annotations

import json
from dataclasses import dataclass
from pathlib import Path

from .types import (ImpliedVolGrid, MarketSnapshot, PhoenixTrade, PriceRequest,
                    SimulationConfig, VarianceReduction)


def tenor_years(tenor: str):
    """fixture.rs:54-62"""
    if tenor.endswith("M"):
        return float(tenor[:-1]) / 12.0
    if tenor.endswith("Y"):
        return float(tenor[:-1])
    return None


def civil_day_number(date: str) -> int:
    """Days-from-civil, fixture.rs:64-94."""
    year, month, day = (int(x) for x in date.split("-"))
    if not (1 <= month <= 12 and 1 <= day <= 31):
        raise ValueError(f"invalid ISO date {date}")
    year -= 1 if month <= 2 else 0
    era = year // 400
    yoe = year - era * 400
    mp = month + (-3 if month > 2 else 9)
    doy = (153 * mp + 2) // 5 + day - 1
    doe = yoe * 365 + yoe // 4 - yoe // 100 + doy
    return era * 146_097 + doe


def weekday_steps(start: str, end: str) -> int:
    """fixture.rs:96-108: weekdays in (start, end]."""
    a, b = civil_day_number(start), civil_day_number(end)
    if b < a:
        raise ValueError("end date must not precede start date")
    return sum(1 for d in range(a + 1, b + 1) if (d + 3) % 7 < 5)


def remaining_business_steps(as_of: str, maturity: str):
    """fixture.rs:110-123"""
    a, b = civil_day_number(as_of), civil_day_number(maturity)
    if b <= a:
        raise ValueError("maturity must be after as_of")
    return (b - a) / 365.0, weekday_steps(as_of, maturity)


def interpolate_curve(points, time: float) -> float:
    """fixture.rs:125-148"""
    if time <= points[0][0]:
        return points[0][1]
    for (x0, y0), (x1, y1) in zip(points, points[1:]):
        if time <= x1:
            w = (time - x0) / (x1 - x0)
            return y0 + w * (y1 - y0)
    return points[-1][1]


@dataclass
class LoadedFixture:
    name: str
    request: PriceRequest
    expected: dict
    market_is_pinned: bool


def load_termsheet1_fixture(path) -> LoadedFixture:
    root = json.loads(Path(path).read_text())
    if root.get("fixture") != "termsheet1":
        raise ValueError("expected fixture id termsheet1")
    assets = root["trade_economics"]["reference_assets"]
    names = [a["symbol"] for a in assets]
    md = root["market_data"]

    def points(asset):
        return [(tenor_years(r["tenor"]), float(r["atm_implied_vol"]))
                for r in md["vol_surfaces"][asset]]

    as_of = root["as_of"]
    t, steps = remaining_business_steps(as_of, root["trade_economics"]["final_fixing_date"])
    vols = [interpolate_curve(points(n), t) for n in names]
    disc = [(tenor_years(r["tenor"]), float(r["zero_rate"])) for r in md["discount_curve"]["points"]]
    rate = interpolate_curve(disc, t)
    te = root["trade_economics"]
    future = [r for r in te["schedule"] if r["observation"] > as_of]
    fixed_first = future[0].get("coupon_type") == "fixed"
    call_start = te["callable"]["period_start"]
    call_start_step = 0 if call_start <= as_of else weekday_steps(as_of, call_start)
    spots = [md.get("as_of_spots", {}).get(n, md["initial_fixings"]["spots"][n]) for n in names]
    local_vol = None
    lvs = md.get("local_vol_surfaces")
    if isinstance(lvs, dict) and any(n in lvs for n in names):
        local_vol = []
        for n in names:
            node = lvs[n]
            rows = []
            for k, date in enumerate(node["maturities"]):
                years = (civil_day_number(date) - civil_day_number(as_of)) / 365.0
                rows.append((years, [float(v) for v in node["vols"][k]]))
            rows.sort(key=lambda r: r[0])
            local_vol.append(ImpliedVolGrid([r[0] for r in rows],
                                            [float(k) for k in node["strikes"]],
                                            [r[1] for r in rows]))
    b = te["barriers"]
    run = root["run"]
    request = PriceRequest(
        trade=PhoenixTrade(
            trade_id=te.get("trade_id", "termsheet1"),
            initial_spots=[float(md["initial_fixings"]["spots"][n]) for n in names],
            maturity_years=t, steps=steps,
            strike=float(b["exercise"]["level_pct"]),
            knock_in_barrier=float(b["knock_in"]["level_pct"]),
            knock_out_barrier=b.get("call", {}).get("level_pct"),
            coupon_barrier=b.get("coupon", {}).get("level_pct"),
            coupon_rate=te.get("coupon", {}).get("rate_per_period"),
            memory_coupon=bool(te.get("coupon", {}).get("memory", False)),
            coupon_periods=len(future), fixed_first_coupon=fixed_first,
            call_start_step=call_start_step),
        market=MarketSnapshot(md["as_of"], [float(s) for s in spots], vols, rate,
                              [float(md["dividend_yields"]["annual_continuous"][n]) for n in names],
                              md["correlation_matrix"]["values"]),
        config=SimulationConfig(int(run.get("paths", 30_000)), int(run.get("path_block_size", 4_096)),
                                int(run.get("seed", 1_729)), "aggregated", VarianceReduction()),
        as_of=as_of, local_vol=local_vol)
    exp = root["expected"]
    pinned = (root.get("to_capture") == [] and
              all(str(v).startswith(("pinned", "captured")) for v in root["provenance"].values()))
    return LoadedFixture("termsheet1", request,
                         {"put_pv": exp["put"]["value"], "relative_tolerance": exp["put"]["tol_rel"],
                          "ki_probability": exp["ki_prob"]["value"],
                          "ki_probability_tolerance": exp["ki_prob"]["tol_abs"]}, pinned)
