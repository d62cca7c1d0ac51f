"""CPU checks of the PathCube restatement (oracle) and the host side of riga_gb300.pathcube:
the reference's own pathcube.rs tests (crates/riga-engine/src/pathcube.rs:190-310) restated —
sample correlation of a 200,000-path block, byte-for-byte determinism, the shape_mismatch error,
and the archive round trip with its worst-percentile query."""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle as O
from riga_gb300.abi import RigaError
from riga_gb300.pathcube import BrownianBlock, PathCube, gbm_evolve


def test_cholesky_z_reproduces_the_target_correlation():
    rho = 0.4041
    n = 200_000
    blk = np.frombuffer(O.generate_correlated_block(1729, n, 1, O.cholesky([[1.0, rho], [rho, 1.0]])), dtype=np.float32)
    x, y = blk[0::2].astype(np.float64), blk[1::2].astype(np.float64)
    assert abs(np.corrcoef(x, y)[0, 1] - rho) < 0.01


def test_block_generation_is_deterministic_and_the_cube_reusable():
    L = O.cholesky([[1.0, 0.5], [0.5, 1.0]])
    a = bytes(O.generate_correlated_block(7, 256, 64, L))
    b = bytes(O.generate_correlated_block(7, 256, 64, L))
    assert a == b
    blk = np.frombuffer(a, dtype=np.float32)
    c1 = bytes(O.gbm_evolve([100.0, 50.0], [0.2, 0.3], 0.03, [0.0, 0.0], 1 / 252, list(blk), 256, 64))
    c2 = bytes(O.gbm_evolve([100.0, 50.0], [0.2, 0.3], 0.03, [0.0, 0.0], 1 / 252, list(blk), 256, 64))
    assert c1 == c2


def test_block_rows_are_the_stream_in_path_time_factor_order():
    L = O.cholesky([[1.0, 0.3, 0.1], [0.3, 1.0, 0.2], [0.1, 0.2, 1.0]])
    blk = np.frombuffer(O.generate_correlated_block(11, 5, 7, L), dtype=np.float32).reshape(5, 7, 3)
    z = np.frombuffer(O.chacha8_normals(11, 5 * 7 * 3), dtype=np.float64).reshape(5, 7, 3)
    Lm = np.array(L)
    for p in range(5):
        for t in range(7):
            y = [sum(Lm[i, j] * z[p, t, j] for j in range(i + 1)) for i in range(3)]
            assert list(blk[p, t]) == [np.float32(v) for v in y]


def test_factor_count_mismatch_is_rejected():
    blk = BrownianBlock(4, 4, 3, np.zeros(48, dtype=np.float32))
    with pytest.raises(RigaError) as e:
        gbm_evolve([100.0, 100.0], [0.2, 0.2], 0.01, [0.0, 0.0], 0.01, blk)
    assert e.value.code == "shape_mismatch"


def test_archive_round_trips_and_the_percentile_query(tmp_path):
    L = O.cholesky([[1.0, 0.2], [0.2, 1.0]])
    blk = list(np.frombuffer(O.generate_correlated_block(3, 8, 4, L), dtype=np.float32))
    cube = PathCube(8, 4, 2, np.frombuffer(O.gbm_evolve([100.0, 50.0], [0.2, 0.3], 0.03, [0.0, 0.0], 0.01, blk, 8, 4),
                                           dtype=np.float32).copy())
    p = tmp_path / "cube.json"
    cube.write_archive(p)
    restored = PathCube.read_archive(p)
    assert restored.paths == 8 and np.array_equal(restored.data, cube.data)
    initial = [100.0, 50.0]
    t5 = restored.worst_percentile_threshold(initial, 0.05)
    assert math.isfinite(t5) and t5 > 0 and t5 <= restored.worst_percentile_threshold(initial, 0.5)
    assert len(restored.terminal()[0]) == 8
