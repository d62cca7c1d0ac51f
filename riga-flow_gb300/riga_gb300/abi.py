"""ctypes mirror of ``include/riga_gb300.h`` and the loader for the in-tree engine library.

Struct layouts follow the header field by field; the header cites the reference type each one
mirrors (crates/riga-core/src/lib.rs, crates/riga-engine/src/lib.rs, crates/riga-risk/src/lib.rs).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT_DIR = PKG_DIR.parent  # riga-flow_gb300/
LIB_PATH = ROOT_DIR / "_build" / "libriga_gb300.so"

RG_MAX_ASSETS = 5
RG_TRACE_EVENT_CAP = 64
RG_N_TRANSITIONS = 3

STATUS_CODES = {
    0: "ok",
    1: "missing_as_of",
    2: "as_of_mismatch",
    3: "invalid_paths",
    4: "invalid_schedule",
    5: "invalid_market_shape",
    6: "invalid_market",
    7: "invalid_trade",
    8: "invalid_local_vol",
    9: "shape_mismatch",
    10: "gpu_unavailable",
    11: "gpu_error",
    12: "no_crn_rejected",
    13: "invalid_spot_bump",
    14: "invalid_volatility_bump",
    15: "invalid_rate_bump",
    16: "invalid_correlation_bump",
    17: "risk_input_shape",
    18: "risk_paths_required",
    19: "path_out_of_range",
    20: "invalid_argument",
    21: "unsupported",
    22: "invalid_percentile",
    23: "cancelled",
    24: "device_timeout",
}

TRACE_OFF, TRACE_AGGREGATED, TRACE_SAMPLED, TRACE_FULL = 0, 1, 2, 3
VR_NONE, VR_HALTON, VR_SOBOL = 0, 1, 2
SCRAMBLE_OWEN, SCRAMBLE_DIGITAL_SHIFT = 0, 1
PRECISION_FP64_PARITY, PRECISION_FP32 = 0, 1
DIM_WRAP_REFERENCE, DIM_FULL = 0, 1
CRN, NO_CRN = 0, 1

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


class Trade(C.Structure):
    _fields_ = [
        ("trade_id", C.c_char_p),
        ("n_assets", C.c_int32),
        ("initial_spots", _dp),
        ("maturity_years", C.c_double),
        ("steps", C.c_int64),
        ("strike", C.c_double),
        ("knock_in_barrier", C.c_double),
        ("has_knock_out_barrier", C.c_int32),
        ("knock_out_barrier", C.c_double),
        ("has_coupon_barrier", C.c_int32),
        ("coupon_barrier", C.c_double),
        ("has_coupon_rate", C.c_int32),
        ("coupon_rate", C.c_double),
        ("memory_coupon", C.c_int32),
        ("has_coupon_periods", C.c_int32),
        ("coupon_periods", C.c_int64),
        ("fixed_first_coupon", C.c_int32),
        ("has_call_start_step", C.c_int32),
        ("call_start_step", C.c_int64),
    ]


class Market(C.Structure):
    _fields_ = [
        ("as_of", C.c_char_p),
        ("n_assets", C.c_int32),
        ("spots", _dp),
        ("vols", _dp),
        ("risk_free_rate", C.c_double),
        ("dividend_yields", _dp),
        ("correlation", _dp),
    ]


class SimConfig(C.Structure):
    _fields_ = [
        ("paths", C.c_uint64),
        ("path_block_size", C.c_uint64),
        ("seed", C.c_uint64),
        ("trace_level", C.c_int32),
        ("variance_reduction", C.c_int32),
        ("qmc_dimension", C.c_uint64),
        ("scrambler", C.c_int32),
        ("precision", C.c_int32),
        ("dim_mode", C.c_int32),
        ("lv_grid_x", C.c_int32),
        ("first_path", C.c_uint64),
    ]


class ImpliedVolGrid(C.Structure):
    _fields_ = [
        ("n_maturities", C.c_int32),
        ("n_strikes", C.c_int32),
        ("maturities_years", _dp),
        ("strikes", _dp),
        ("vols", _dp),
    ]


class PriceRequest(C.Structure):
    _fields_ = [
        ("trade", Trade),
        ("market", Market),
        ("config", SimConfig),
        ("as_of", C.c_char_p),
        ("n_local_vol", C.c_int32),
        ("local_vol", C.POINTER(ImpliedVolGrid)),
    ]


class Legs(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "par_redemption", "coupon", "memory_coupon", "down_and_in_put", "funding", "discounting",
        "total")]


class TransitionStats(C.Structure):
    _fields_ = [
        ("input_count", C.c_uint64),
        ("output_count", C.c_uint64),
        ("probability", C.c_double),
        ("mean_payoff", C.c_double),
        ("variance_payoff", C.c_double),
        ("mean_delta", C.c_double),
        ("mean_vega", C.c_double),
    ]


class LedgerEntry(C.Structure):
    _fields_ = [
        ("population_before", C.c_uint64),
        ("population_after", C.c_uint64),
        ("pv_impact", C.c_double),
        ("delta_impact", C.c_double),
        ("vega_impact", C.c_double),
    ]


class TraceEvent(C.Structure):
    _fields_ = [("path_id", C.c_uint64), ("time", C.c_double)]


class PriceResult(C.Structure):
    _fields_ = [
        ("pv", C.c_double),
        ("mc_error", C.c_double),
        ("ki_probability", C.c_double),
        ("legs", Legs),
        ("stats", TransitionStats * RG_N_TRANSITIONS),
        ("ledger", LedgerEntry * RG_N_TRANSITIONS),
        ("seed", C.c_uint64),
        ("ko_count", C.c_uint64),
        ("ki_count", C.c_uint64),
        ("put_eligible_count", C.c_uint64),
        ("coupon_path_count", C.c_uint64),
        ("n_trace_events", C.c_int32),
        ("trace_events", TraceEvent * RG_TRACE_EVENT_CAP),
        ("path_sums", C.c_double * 16),
    ]


class Timing(C.Structure):
    _fields_ = [("h2d_ms", C.c_double), ("prologue_ms", C.c_double), ("kernel_ms", C.c_double),
                ("reduce_ms", C.c_double), ("d2h_ms", C.c_double), ("device_ms", C.c_double),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64),
                ("kernel_launches", C.c_int32), ("grid", C.c_int32), ("block", C.c_int32),
                ("smem_bytes", C.c_int32), ("tile_steps", C.c_int32), ("paths_per_thread", C.c_int32)]


class Scenario(C.Structure):
    _fields_ = [("market", Market), ("implied_vol_shift", _dp)]


class CentralDifferenceConfig(C.Structure):
    _fields_ = [
        ("spot_relative_bump", C.c_double),
        ("volatility_absolute_bump", C.c_double),
        ("rate_absolute_bump", C.c_double),
        ("correlation_absolute_bump", C.c_double),
        ("random_number_policy", C.c_int32),
    ]


class FdEstimate(C.Structure):
    _fields_ = [("value", C.c_double), ("mc_error_upper_bound", C.c_double)]


class AssetGreeks(C.Structure):
    _fields_ = [
        ("asset_index", C.c_int32),
        ("spot_bump", C.c_double),
        ("volatility_bump", C.c_double),
        ("delta", FdEstimate),
        ("gamma", FdEstimate),
        ("vega", FdEstimate),
        ("spot_up_pv", C.c_double),
        ("spot_down_pv", C.c_double),
        ("vol_up_pv", C.c_double),
        ("vol_down_pv", C.c_double),
        ("spot_up_mc_error", C.c_double),
        ("spot_down_mc_error", C.c_double),
        ("vol_up_mc_error", C.c_double),
        ("vol_down_mc_error", C.c_double),
    ]


class TransitionRisk(C.Structure):
    _fields_ = [("pv_impact", C.c_double), ("delta_impact", C.c_double), ("vega_impact", C.c_double)]


class BatchRiskReport(C.Structure):
    _fields_ = [
        ("base", PriceResult),
        ("scenario_count", C.c_uint64),
        ("seed", C.c_uint64),
        ("n_assets", C.c_int32),
        ("assets", AssetGreeks * RG_MAX_ASSETS),
        ("transitions", TransitionRisk * RG_N_TRANSITIONS),
        ("rate_up_pv", C.c_double),
        ("rate_down_pv", C.c_double),
        ("correlation_up_pv", C.c_double),
        ("correlation_down_pv", C.c_double),
        ("rate_bump", C.c_double),
        ("correlation_bump", C.c_double),
        ("pv_mc_error", C.c_double),
    ]


class PathRecord(C.Structure):
    _fields_ = [
        ("path_id", C.c_uint64),
        ("rng_seed", C.c_uint64),
        ("sobol_index", C.c_uint64),
        ("worst_final", C.c_double),
        ("knocked_out", C.c_int32),
        ("ko_step", C.c_int32),
        ("ko_time", C.c_double),
        ("ki_hit", C.c_int32),
        ("qualified_steps", C.c_int32),
        ("paid_periods", C.c_int32),
        ("put_payoff", C.c_double),
        ("coupon_pv", C.c_double),
        ("memory_coupon_pv", C.c_double),
        ("funding", C.c_double),
        ("pv", C.c_double),
    ]


class BookTrade(C.Structure):
    _fields_ = [("terms", Trade), ("underlyings", C.POINTER(C.c_int32))]


class BookRequest(C.Structure):
    _fields_ = [("universe", Market), ("universe_steps", C.c_int64),
                ("universe_maturity_years", C.c_double), ("n_trades", C.c_int32),
                ("trades", C.POINTER(BookTrade)), ("config", SimConfig)]


class BookBumps(C.Structure):
    _fields_ = [("spot_relative", C.c_double), ("vol_absolute", C.c_double), ("rate_absolute", C.c_double)]


class BookBumpSpec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("first", C.c_int32), ("second", C.c_int32), ("size", C.c_double)]


BOOK_TRADE_SCENARIOS = 16
BUMP_BASE, BUMP_SPOT, BUMP_VOL, BUMP_RATE, BUMP_SPOT_PAIR = 0, 1, 2, 3, 4


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("slots", C.c_int32), ("device_memory_budget", C.c_uint64),
                ("max_large_slots", C.c_int32), ("large_work", C.c_uint64), ("large_max_sms", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("kind", C.c_int32), ("slot", C.c_int32),
                ("n_results", C.c_uint64), ("device_bytes", C.c_uint64),
                ("submit_s", C.c_double), ("start_s", C.c_double), ("end_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("queued", C.c_uint64), ("running", C.c_uint64),
                ("device_bytes_held", C.c_uint64), ("device_memory_budget", C.c_uint64),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("busy_s", C.c_double), ("memory_waits", C.c_uint64), ("peak_reserved_bytes", C.c_uint64)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = range(5)
JOB_PRICE, JOB_RISK, JOB_BOOK, JOB_BOOK_BUMPS = range(4)


class RigaError(Exception):
    """Mirror of ``RigaError { code, message }`` (crates/riga-core/src/lib.rs:5-19)."""

    def __init__(self, code: str, message: str):
        super().__init__(f"{code}: {message}")
        self.code = code
        self.message = message


# Every symbol the header declares, with its ctypes signature (restype, argtypes).
_vp = C.c_void_p
_i32, _i64, _u64 = C.c_int32, C.c_int64, C.c_uint64
SIGNATURES = {
    "rg_status_code": (C.c_char_p, [_i32]),
    "rg_last_error": (_i32, [C.c_char_p, C.c_size_t]),
    "rg_abi_version": (_i32, []),
    "rg_ensure_available": (_i32, []),
    "rg_device_name": (_i32, [C.c_char_p, C.c_size_t]),
    "rg_arch": (_i32, [C.c_char_p, C.c_size_t]),
    "rg_engine_create": (_i32, [_i32, C.POINTER(_vp)]),
    "rg_engine_destroy": (None, [_vp]),
    "rg_price_put_leg": (_i32, [_vp, C.POINTER(PriceRequest), C.POINTER(PriceResult)]),
    "rg_price_put_leg_static": (_i32, [C.POINTER(PriceRequest), C.POINTER(PriceResult)]),
    "rg_price_scenarios": (_i32, [_vp, C.POINTER(PriceRequest), C.POINTER(Scenario), _i32,
                                  C.POINTER(PriceResult)]),
    "rg_price_risk_batch": (_i32, [_vp, C.POINTER(PriceRequest),
                                   C.POINTER(CentralDifferenceConfig),
                                   C.POINTER(BatchRiskReport)]),
    "rg_run_paths": (_i32, [_vp, C.POINTER(PriceRequest), _u64, _u64, C.POINTER(PathRecord)]),
    "rg_materialize_paths": (_i32, [_vp, C.POINTER(PriceRequest), _u64, _u64, C.POINTER(C.c_float),
                                    C.POINTER(PathRecord)]),
    "rg_merge_results": (_i32, [C.POINTER(PriceResult), _i32, _u64, C.POINTER(PriceResult)]),
    "rg_engine_last_timing": (_i32, [_vp, C.POINTER(Timing)]),
    "rg_set_autotune": (_i32, [_i32]),
    "rg_set_tiled_shape": (_i32, [_i32, _i32, _i32]),
    "rg_phase_clocks": (_i32, [C.POINTER(C.c_uint64), _i32]),
    "rg_surfaces_upload": (_i32, [_vp, C.POINTER(PriceRequest), C.POINTER(Scenario), _i32, C.POINTER(_i32)]),
    "rg_price_book": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(Market), _i32,
                             C.POINTER(PriceResult)]),
    "rg_book_run_paths": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(Market), _i32, _u64, _u64,
                                 C.POINTER(PathRecord)]),
    "rg_price_book_trade_bumps": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(BookBumps), C.POINTER(PriceResult)]),
    "rg_book_trade_bump": (_i32, [_i32, _i32, C.POINTER(BookBumps), C.POINTER(BookBumpSpec)]),
    "rg_book_price_trade_bumps": (_i32, [_vp, C.POINTER(BookBumps), C.POINTER(PriceResult)]),
    "rg_book_create": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(_vp)]),
    "rg_book_price": (_i32, [_vp, C.POINTER(Market), _i32, C.POINTER(PriceResult)]),
    "rg_book_tuned_stage": (_i32, [_vp, _i32, C.POINTER(_i32)]),
    "rg_book_destroy": (None, [_vp]),
    "rg_server_create": (_i32, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "rg_server_destroy": (None, [_vp]),
    "rg_server_submit_price": (_i32, [_vp, C.POINTER(PriceRequest), C.POINTER(Scenario), _i32,
                                      C.POINTER(_u64)]),
    "rg_server_submit_risk": (_i32, [_vp, C.POINTER(PriceRequest), C.POINTER(CentralDifferenceConfig),
                                     C.POINTER(_u64)]),
    "rg_server_submit_book": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(Market), _i32,
                                     C.POINTER(_u64)]),
    "rg_server_submit_book_trade_bumps": (_i32, [_vp, C.POINTER(BookRequest), C.POINTER(BookBumps),
                                                 C.POINTER(_u64)]),
    "rg_server_poll": (_i32, [_vp, _u64, C.POINTER(JobInfo)]),
    "rg_server_wait": (_i32, [_vp, _u64, _i64, C.POINTER(JobInfo)]),
    "rg_server_results": (_i32, [_vp, _u64, C.POINTER(PriceResult), _u64]),
    "rg_server_risk_report": (_i32, [_vp, _u64, C.POINTER(BatchRiskReport)]),
    "rg_server_cancel": (_i32, [_vp, _u64]),
    "rg_server_release": (_i32, [_vp, _u64]),
    "rg_server_get_stats": (_i32, [_vp, C.POINTER(ServerStats)]),
    "rg_chacha8_normals": (_i32, [_u64, _u64, _u64, C.POINTER(C.c_double)]),
    "rg_generate_correlated_block": (_i32, [_u64, _i64, _i64, _i32, C.POINTER(C.c_double), _fp]),
    "rg_gbm_evolve": (_i32, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double),
                             _i32, C.c_double, _fp, _i64, _i64, _fp]),
    "rg_sobol_directions": (_i32, [_i64, C.POINTER(C.c_uint32)]),
    "rg_bridge_schedule": (_i32, [_i64, C.c_double, C.POINTER(_i32), C.POINTER(_i32),
                                  C.POINTER(C.c_double), C.POINTER(_i32)]),
    "rg_worst_of": (_i32, [_fp, _fp, _fp, _i64]),
    "rg_lv_terminal_spots": (_i32, [_fp, _fp, _fp, _i64, _fp, _fp, C.c_float, _i64, _i64,
                                    C.c_float, C.c_float, _fp, _fp, C.POINTER(_i32)]),
    "rg_resident_lv_create": (_i32, [_fp, _fp, _fp, _i64, _i64, _i64, C.c_float,
                                     C.POINTER(_vp)]),
    "rg_resident_lv_run": (_i32, [_vp, _fp, _fp, C.c_float, C.c_float, _fp]),
    "rg_resident_lv_download": (_i32, [_vp, _fp, C.POINTER(_i32)]),
    "rg_resident_lv_synchronize": (_i32, [_vp]),
    "rg_resident_lv_destroy": (None, [_vp]),
    "rg_resident_worst_of_create": (_i32, [_fp, _fp, _i64, C.POINTER(_vp)]),
    "rg_resident_worst_of_reduce": (_i32, [_vp]),
    "rg_resident_worst_of_download": (_i32, [_vp, _fp]),
    "rg_resident_worst_of_synchronize": (_i32, [_vp]),
    "rg_resident_worst_of_destroy": (None, [_vp]),
}

_LIB = None


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load the in-tree engine library (built by ``riga_gb300.build.build_library``).

    There is no fallback: a missing library raises, so no code path silently runs elsewhere.
    """
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RigaError("gpu_unavailable",
                        f"engine library {p} is not built; run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def last_error(lib: C.CDLL) -> str:
    buf = C.create_string_buffer(1024)
    lib.rg_last_error(buf, len(buf))
    return buf.value.decode("utf-8", "replace")


def check(lib: C.CDLL, status: int) -> None:
    if status != 0:
        raise RigaError(STATUS_CODES.get(status, f"status_{status}"), last_error(lib))
