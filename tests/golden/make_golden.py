"""Regenerates the committed golden fixtures under tests/golden/ from the reference checkout.

Run it where the reference is mounted:  python tests/golden/make_golden.py /path/to/riga-flow

* termsheet1.json          — the reference's fixture document (docs/fixture/termsheet1.json),
                             copied verbatim: market data, trade economics and acceptance block.
* termsheet1.golden.json   — the reference's golden PriceResult for that fixture
                             (fixtures/termsheet1.golden.json), copied verbatim.
* known_answers.json       — the numeric known answers the reference's own unit tests assert,
                             transcribed from the cited test lines (qmc.rs, correlation.rs,
                             riga-market lib.rs, fixture.rs).

Nothing at test time reads the reference checkout; only these committed files.
"""
from __future__ import annotations

import json
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

KNOWN_ANSWERS = {
    # crates/riga-engine/src/qmc.rs:512-517
    "probit": {"p": [0.5, 0.975, 0.025], "value": [0.0, 1.959963984540054, -1.959963984540054],
               "tol": [1e-9, 1e-6, 1e-6]},
    # crates/riga-engine/src/qmc.rs:502-510
    "van_der_corput_base2": {"index": [1, 2, 3, 4], "value": [0.5, 0.25, 0.75, 0.125]},
    "radical_inverse_base3": {"index": [1, 2], "value": [1.0 / 3.0, 2.0 / 3.0], "tol": 1e-15},
    # crates/riga-market/src/correlation.rs:266-279
    "cholesky_2x2": {"rho": 0.4041, "z": [0.3, -1.2], "tol": 1e-15},
    # crates/riga-market/src/correlation.rs:281-305
    "cholesky_3x3": {"rows": [[1.0, 0.5, 0.3], [0.5, 1.0, 0.2], [0.3, 0.2, 1.0]], "tol": 1e-12},
    # crates/riga-market/src/correlation.rs:307-330
    "psd_clamp": {"rows": [[1.0, 0.9, -0.9], [0.9, 1.0, 0.9], [-0.9, 0.9, 1.0]], "floor": 1e-8},
    # crates/riga-market/src/lib.rs:386-412
    "flat_smile": {"maturities": [0.1, 0.25, 0.5, 1.0], "strikes": [60.0, 80.0, 100.0, 120.0, 140.0],
                   "vol": 0.20, "spot": 100.0, "rate": 0.0, "t": [0.1, 0.2, 0.3, 0.5],
                   "s": [70.0, 90.0, 100.0, 110.0, 130.0], "tol": 1e-9},
    # crates/riga-engine/src/fixture.rs:507-527
    "termsheet1_lv_nodes": {"t": 0.40274,
                            "cases": [[0, 180.0, 0.467727], [0, 268.0, 0.430912],
                                      [1, 240.0, 0.346527], [1, 268.0, 0.352650]],
                            "tol": 3.0e-3},
    # crates/riga-engine/src/fixture.rs:471-505
    "termsheet1_mapping": {"spots": [267.885, 258.355], "vols_approx": [0.45619, 0.35599],
                           "vols_tol": 0.002, "rate_approx": 0.038825, "rate_tol": 0.0005,
                           "dividends": [0.0, 0.002979], "rho": 0.4593248180905,
                           "initial_spots": [239.97, 260.0], "strike": 0.78, "ki": 0.70,
                           "ko": 1.10, "coupon_barrier": 0.1, "coupon_rate": 0.009642,
                           "coupon_periods": 5, "fixed_first_coupon": False,
                           "call_start_step": 0, "grid_shape": [10, 21]},
    # crates/riga-engine/src/fixture.rs:531-538
    "termsheet1_dates": {"as_of": "2026-09-07", "final": "2027-02-01", "days": 147,
                         "weekdays_range": [100, 110]},
    # crates/riga-engine/src/lib.rs:459-487 (MC lane acceptance)
    "termsheet1_acceptance": {"put_pv": 0.02112, "put_tol_rel": 0.05, "ki": 0.102, "ki_tol": 0.03},
}


def main(reference: str) -> None:
    ref = Path(reference)
    shutil.copyfile(ref / "docs/fixture/termsheet1.json", HERE / "termsheet1.json")
    shutil.copyfile(ref / "fixtures/termsheet1.golden.json", HERE / "termsheet1.golden.json")
    (HERE / "known_answers.json").write_text(json.dumps(KNOWN_ANSWERS, indent=1) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the riga-flow checkout>")
    main(sys.argv[1])
