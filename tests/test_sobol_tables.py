"""The block decomposition behind the FP32 kernels' Sobol tables (host_prep.cu sobol_lut_tables,
phoenix32d.cu and p32_tiled.cuh): a warp's 32 points n1 .. n1 + 31 lie in at most two aligned
32-point blocks, and the Gray code is linear over XOR, so

    x(n1 + j) = X(gray(a)) ^ X(gray((o + j) mod 32))                  if o + j < 32
    x(n1 + j) = X(gray(a)) ^ v[4] ^ v[ctz(a/32 + 1) + 5] ^ X(gray(o + j - 32))   otherwise

with a = n1 rounded down to 32 and o = n1 mod 32 (X(G) = XOR of the direction numbers at the set
bits of G).  Checked here against the oracle's Gray-code Sobol integers (qmc.rs:269-282) on random
points and dimensions, including block boundaries; the GPU tests check that the kernels built on
it price bit for bit alike.
"""
from __future__ import annotations

import random

import oracle as O


def _x(row, g):
    x = 0
    for k in range(32):
        if (g >> k) & 1:
            x ^= row[k]
    return x


def _gray(n):
    return n ^ (n >> 1)


def _sobol(row, n):
    return _x(row, _gray(n))


def _ctz(x):
    return (x & -x).bit_length() - 1


def test_block_decomposition_reproduces_the_gray_code_points():
    dims = 48
    flat = O.sobol_table(dims)
    table = [list(flat[32 * d:32 * (d + 1)]) for d in range(dims)]
    rng = random.Random(5)
    cases = [(0, 0), (31, 0), (32, 3), ((1 << 20) - 1, 7)] + \
        [(rng.randrange(1 << 22), rng.randrange(1 << 8)) for _ in range(150)]
    for path0, grp in cases:
        row = table[rng.randrange(dims)]
        n1 = path0 + 32 * grp + 1  # the Sobol point of the warp's first path (point = path + 1)
        a, o = n1 & ~31, n1 & 31
        high0 = _x(row, _gray(a))
        high1 = high0 ^ row[_ctz((a >> 5) + 1) + 5]
        for j in range(32):
            low = _x(row, _gray((o + j) & 31) & 31) ^ (row[4] if o + j >= 32 else 0)
            got = (high1 if o + j >= 32 else high0) ^ low
            assert got == _sobol(row, n1 + j), (path0, grp, j)
