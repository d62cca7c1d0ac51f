"""PathCube on the GPU: the reference's crates/riga-engine/src/pathcube.rs API over the C ABI.

* ``generate_correlated_block(seed, paths, times, chol)`` — ``BrownianBlock``: f32
  ``[path][time][factor]`` of L·z with z the ChaCha8 StandardNormal stream (pathcube.rs:37-66),
  generated on the device (``rg_generate_correlated_block``).
* ``gbm_evolve(s0, vols, rate, dividend_yields, dt, block)`` — ``PathCube`` of f32 spots
  (pathcube.rs:146-187, ``rg_gbm_evolve``).
* ``PathCube.terminal``, ``terminal_worst``, ``worst_percentile_threshold``, ``write_archive``,
  ``read_archive`` — the host-side queries of pathcube.rs:70-140 (serde JSON archive).
"""
from __future__ import annotations

import ctypes as C
import json
import math
from dataclasses import dataclass

import numpy as np

from . import abi
from .abi import RigaError, check, load_library


@dataclass
class BrownianBlock:
    paths: int
    times: int
    factors: int
    data: np.ndarray  # f32, flat [path][time][factor]

    def index(self, path: int, time: int, factor: int) -> int:
        return (path * self.times + time) * self.factors + factor

    def get(self, path: int, time: int, factor: int) -> float:
        return float(self.data[self.index(path, time, factor)])

    def cell(self, path: int, time: int) -> np.ndarray:
        i = self.index(path, time, 0)
        return self.data[i:i + self.factors]


@dataclass
class PathCube:
    paths: int
    times: int
    factors: int
    data: np.ndarray  # f32, flat [path][time][factor]

    def index(self, path: int, time: int, factor: int) -> int:
        return (path * self.times + time) * self.factors + factor

    def get(self, path: int, time: int, factor: int) -> float:
        return float(self.data[self.index(path, time, factor)])

    def terminal(self) -> list:
        cube = self.data.reshape(self.paths, self.times, self.factors)
        return [cube[:, -1, f].copy() for f in range(self.factors)]

    def terminal_worst(self, initial_spots) -> np.ndarray:
        cube = self.data.reshape(self.paths, self.times, self.factors)
        ratios = cube[:, -1, :] / np.asarray(initial_spots, dtype=np.float32)
        return ratios.min(axis=1)

    def worst_percentile_threshold(self, initial_spots, percentile: float) -> float:
        worst = np.sort(self.terminal_worst(initial_spots))
        index = max(0, math.ceil(len(worst) * percentile) - 1)
        return float(worst[min(index, len(worst) - 1)])

    def write_archive(self, path) -> None:
        with open(path, "w") as f:
            json.dump({"paths": self.paths, "times": self.times, "factors": self.factors,
                       "data": [float(v) for v in self.data]}, f)

    @staticmethod
    def read_archive(path) -> "PathCube":
        with open(path) as f:
            d = json.load(f)
        return PathCube(d["paths"], d["times"], d["factors"], np.asarray(d["data"], dtype=np.float32))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def generate_correlated_block(seed: int, paths: int, times: int, chol, lib=None) -> BrownianBlock:
    """`chol`: the factors × factors lower Cholesky factor (rows)."""
    lib = lib or load_library()
    L = np.ascontiguousarray(np.asarray(chol, dtype=np.float64))
    f = L.shape[0]
    out = np.empty(max(1, paths * times * f), dtype=np.float32)
    check(lib, lib.rg_generate_correlated_block(seed, paths, times, f, _dptr(L), _fptr(out)))
    return BrownianBlock(paths, times, f, out[: paths * times * f])


def gbm_evolve(s0, vols, rate: float, dividend_yields, dt: float, block: BrownianBlock, lib=None) -> PathCube:
    lib = lib or load_library()
    f = len(s0)
    if len(vols) != f or len(dividend_yields) != f:
        raise RigaError("shape_mismatch", "s0, vols and dividend_yields must have equal length")
    if block.factors != f:
        raise RigaError("shape_mismatch", "Brownian block factor count must match the spot count")
    s = np.asarray(s0, dtype=np.float64)
    v = np.asarray(vols, dtype=np.float64)
    q = np.asarray(dividend_yields, dtype=np.float64)
    data = np.ascontiguousarray(block.data, dtype=np.float32)
    out = np.empty(max(1, data.size), dtype=np.float32)
    check(lib, lib.rg_gbm_evolve(_dptr(s), _dptr(v), rate, _dptr(q), f, dt, _fptr(data), block.paths,
                                 block.times, _fptr(out)))
    return PathCube(block.paths, block.times, f, out[: data.size])


def chacha8_normals(seed: int, first: int, count: int, lib=None) -> np.ndarray:
    """Draws [first, first + count) of ChaCha8Rng::seed_from_u64(seed) → StandardNormal."""
    lib = lib or load_library()
    out = np.empty(max(1, count), dtype=np.float64)
    check(lib, lib.rg_chacha8_normals(seed, first, count, _dptr(out)))
    return out[:count]
