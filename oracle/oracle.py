"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle (``riga_oracle.c``) restates the reference's CPU algorithm in plain C; this module loads
it for the tests, the smoke check and the benchmark's CPU-baseline leg.  The product package never
imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libriga_oracle.so"
sys.path.insert(0, str(HERE.parent / "riga-flow_gb300"))

from riga_gb300 import abi  # noqa: E402  (ctypes struct definitions only)

_lib = None


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        d, u32, u64, i32, i64 = C.c_double, C.c_uint32, C.c_uint64, C.c_int32, C.c_int64
        P = C.POINTER
        sig = {
            "or_probit": (d, [d]),
            "or_radical_inverse": (d, [u64, u32]),
            "or_mix64": (u64, [u64]),
            "or_halton_hashed_u": (d, [u32, u32, u64, u64]),
            "or_owen_scramble": (u32, [u32, u64, u64]),
            "or_digital_shift": (u32, [u64, u64]),
            "or_primitive_polynomials": (None, [i64, P(u32)]),
            "or_direction_numbers": (None, [u32, P(u32)]),
            "or_sobol_table": (None, [i64, P(u32)]),
            "or_sobol_int": (u32, [P(u32), i64, u64, u64]),
            "or_bridge_increments": (None, [P(d), i64, d, P(d)]),
            "or_first_primes": (i32, [i32, P(u32)]),
            "or_halton_permutation": (None, [u32, u64, P(u32)]),
            "or_min_eigenvalue": (d, [P(d), i32]),
            "or_psd_clamp": (None, [P(d), i32, d, P(d)]),
            "or_cholesky": (i32, [P(d), i32, P(d)]),
            "or_lv_sigma": (d, [C.c_void_p, d, d]),
            "or_validate": (i32, [P(abi.PriceRequest)]),
            "or_price_put_leg": (i32, [P(abi.PriceRequest), i32, P(abi.PriceResult)]),
            "or_run_paths": (i32, [P(abi.PriceRequest), u64, u64, P(abi.PathRecord)]),
            "or_materialize_paths": (i32, [P(abi.PriceRequest), u64, u64, P(C.c_float), P(abi.PathRecord)]),
            "or_price_scenarios": (i32, [P(abi.PriceRequest), P(abi.Scenario), i32, i32,
                                         P(abi.PriceResult)]),
            "or_price_risk_batch": (i32, [P(abi.PriceRequest), P(abi.CentralDifferenceConfig),
                                          i32, P(abi.BatchRiskReport)]),
            "or_last_error": (C.c_char_p, []),
            "or_set_portable_math": (None, [i32]),
            "or_pexp": (d, [d]),
            "or_plog": (d, [d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def set_portable_math(on: bool) -> None:
    """Select the portable deterministic exp/log (bit-identical to the GPU parity kernel) or the
    platform libm (default; reproduces the reference golden bit for bit)."""
    lib().or_set_portable_math(1 if on else 0)


class portable_math:
    """Context manager: run the oracle with the portable exp/log."""

    def __enter__(self):
        set_portable_math(True)

    def __exit__(self, *exc):
        set_portable_math(False)


class OracleError(abi.RigaError):
    pass


def _check(st: int) -> None:
    if st:
        raise OracleError(abi.STATUS_CODES.get(st, str(st)), lib().or_last_error().decode())


class LvSurface(C.Structure):
    _fields_ = [("n_t", C.c_int32), ("gx", C.c_int32), ("t_axis", C.POINTER(C.c_double)),
                ("log_s", C.POINTER(C.c_double)), ("v", C.POINTER(C.c_double))]


def lv_calibrate(grid, spot: float, rate: float, gx: int = 96):
    """``DupireLocalVol::calibrate`` restated; returns (t_axis, log_s, v[n_t][gx], handle)."""
    L = lib()
    nt, nk = len(grid.maturities_years), len(grid.strikes)
    g = abi.ImpliedVolGrid()
    mats = (C.c_double * nt)(*grid.maturities_years)
    ks = (C.c_double * nk)(*grid.strikes)
    vs = (C.c_double * (nt * nk))(*[v for r in grid.vols for v in r])
    g.n_maturities, g.n_strikes = nt, nk
    g.maturities_years = C.cast(mats, C.POINTER(C.c_double))
    g.strikes = C.cast(ks, C.POINTER(C.c_double))
    g.vols = C.cast(vs, C.POINTER(C.c_double))
    surf = LvSurface()
    L.or_lv_calibrate.restype = C.c_int32
    L.or_lv_calibrate.argtypes = [C.POINTER(abi.ImpliedVolGrid), C.c_double, C.c_double,
                                  C.c_int32, C.POINTER(LvSurface)]
    _check(L.or_lv_calibrate(C.byref(g), spot, rate, gx, C.byref(surf)))
    t_axis = [surf.t_axis[i] for i in range(surf.n_t)]
    log_s = [surf.log_s[i] for i in range(surf.gx)]
    v = [[surf.v[k * surf.gx + i] for i in range(surf.gx)] for k in range(surf.n_t)]
    return t_axis, log_s, v, surf


def lv_sigma(surf: LvSurface, t: float, s: float) -> float:
    return lib().or_lv_sigma(C.byref(surf), t, s)


def price_put_leg(request, threads: int = 0) -> abi.PriceResult:
    """``price_put_leg`` restated on the CPU (threads 0 = all host cores)."""
    a = request.to_abi()
    out = abi.PriceResult()
    th = threads if threads > 0 else (os.cpu_count() or 1)
    _check(lib().or_price_put_leg(a.ptr, th, C.byref(out)))
    return out


def run_paths(request, first: int, count: int):
    a = request.to_abi()
    out = (abi.PathRecord * max(1, count))()
    _check(lib().or_run_paths(a.ptr, first, count, out))
    return out


def materialize_paths(request, first: int, count: int):
    """(f32 cube [count * steps * n], PathRecord array) of paths [first, first + count)."""
    import numpy as np
    a = request.to_abi()
    n = len(request.market.spots)
    cube = np.empty(max(1, count * request.trade.steps * n), dtype=np.float32)
    out = (abi.PathRecord * max(1, count))()
    _check(lib().or_materialize_paths(a.ptr, first, count, cube.ctypes.data_as(C.POINTER(C.c_float)), out))
    return cube[: count * request.trade.steps * n], out


def price_scenarios(request, scenarios, threads: int = 0):
    """``scenarios`` is a list of (MarketSnapshot, vol_shift list or None)."""
    from riga_gb300.types import market_to_abi

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
    th = threads if threads > 0 else (os.cpu_count() or 1)
    _check(lib().or_price_scenarios(a.ptr, arr, len(scenarios), th, out))
    return out


def chacha8_normals(seed: int, count: int):
    buf = (C.c_double * max(1, count))()
    L = lib()
    L.or_chacha8_normals.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_double)]
    L.or_chacha8_normals(seed, count, buf)
    return buf


def generate_correlated_block(seed: int, paths: int, times: int, chol):
    """pathcube::generate_correlated_block restated; `chol` is a factors x factors list of rows."""
    n = len(chol)
    Lm = (C.c_double * (n * n))(*[v for r in chol for v in r])
    out = (C.c_float * max(1, paths * times * n))()
    L = lib()
    L.or_generate_correlated_block.argtypes = [C.c_uint64, C.c_int64, C.c_int64, C.c_int32,
                                               C.POINTER(C.c_double), C.POINTER(C.c_float)]
    L.or_generate_correlated_block(seed, paths, times, n, Lm, out)
    return out


def gbm_evolve(s0, vols, rate, q, dt, block, paths, times):
    """pathcube::gbm_evolve restated; `block` is a flat f32 sequence [path][time][factor]."""
    n = len(s0)
    arr = lambda v: (C.c_double * n)(*v)
    blk = (C.c_float * len(block))(*block) if not isinstance(block, C.Array) else block
    out = (C.c_float * max(1, paths * times * n))()
    L = lib()
    L.or_gbm_evolve.restype = C.c_int32
    L.or_gbm_evolve.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_double),
                                C.c_int32, C.c_double, C.POINTER(C.c_float), C.c_int64, C.c_int64,
                                C.POINTER(C.c_float)]
    _check(L.or_gbm_evolve(arr(s0), arr(vols), rate, arr(q), n, dt, blk, paths, times, out))
    return out


def price_book(book, scenarios=None, threads: int = 0):
    """A book (``riga_gb300.types.BookRequest``) under a common scenario set: ``out[j * S + s]``."""
    from riga_gb300.types import markets_to_abi

    a = book.to_abi()
    keep = []
    arr, n = markets_to_abi(scenarios, keep.append)
    S = max(1, n)
    out = (abi.PriceResult * (len(book.trades) * S))()
    th = threads if threads > 0 else (os.cpu_count() or 1)
    L = lib()
    L.or_price_book.restype = C.c_int32
    L.or_price_book.argtypes = [C.POINTER(abi.BookRequest), C.POINTER(abi.Market), C.c_int32, C.c_int32,
                                C.POINTER(abi.PriceResult)]
    _check(L.or_price_book(a.ptr, arr, n, th, out))
    return list(out)


def book_run_paths(book, scenarios, first: int, count: int):
    """Per-path records ``out[(p * n_trades + j) * S + s]`` of book paths [first, first + count)."""
    from riga_gb300.types import markets_to_abi

    a = book.to_abi()
    keep = []
    arr, n = markets_to_abi(scenarios, keep.append)
    S = max(1, n)
    out = (abi.PathRecord * (count * len(book.trades) * S))()
    L = lib()
    L.or_book_run_paths.restype = C.c_int32
    L.or_book_run_paths.argtypes = [C.POINTER(abi.BookRequest), C.POINTER(abi.Market), C.c_int32, C.c_uint64,
                                    C.c_uint64, C.POINTER(abi.PathRecord)]
    _check(L.or_book_run_paths(a.ptr, arr, n, first, count, out))
    return list(out)


def price_risk_batch(request, cfg: abi.CentralDifferenceConfig, threads: int = 0):
    a = request.to_abi()
    out = abi.BatchRiskReport()
    th = threads if threads > 0 else (os.cpu_count() or 1)
    _check(lib().or_price_risk_batch(a.ptr, C.byref(cfg), th, C.byref(out)))
    return out


def sobol_table(dimension: int):
    buf = (C.c_uint32 * (32 * dimension))()
    lib().or_sobol_table(dimension, buf)
    return buf


def bridge_increments(normals, dt: float):
    n = len(normals)
    a = (C.c_double * n)(*normals)
    o = (C.c_double * n)()
    lib().or_bridge_increments(a, n, dt, o)
    return list(o)


def cholesky(rows):
    n = len(rows)
    a = (C.c_double * (n * n))(*[v for r in rows for v in r])
    l = (C.c_double * (n * n))()
    _check(lib().or_cholesky(a, n, l))
    return [[l[i * n + j] for j in range(n)] for i in range(n)]


def min_eigenvalue(rows) -> float:
    n = len(rows)
    a = (C.c_double * (n * n))(*[v for r in rows for v in r])
    return lib().or_min_eigenvalue(a, n)


def psd_clamp(rows, floor: float):
    n = len(rows)
    a = (C.c_double * (n * n))(*[v for r in rows for v in r])
    o = (C.c_double * (n * n))()
    lib().or_psd_clamp(a, n, floor, o)
    return [[o[i * n + j] for j in range(n)] for i in range(n)]
