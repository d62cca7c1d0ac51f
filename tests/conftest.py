"""Shared test set-up: import paths, the ``gpu`` marker and common fixtures."""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "riga-flow_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session")
def known_answers():
    return json.loads((GOLDEN / "known_answers.json").read_text())


@pytest.fixture(scope="session")
def termsheet1():
    from riga_gb300.fixture import load_termsheet1_fixture

    return load_termsheet1_fixture(GOLDEN / "termsheet1.json")


@pytest.fixture(scope="session")
def golden_result():
    return json.loads((GOLDEN / "termsheet1.golden.json").read_text())


def json_close(actual, expected, path="result", tol=1e-12, out=None):
    """The reference's assert_json_close (crates/riga-engine/src/lib.rs:430-457): equal keys,
    numbers within ``tol`` absolute, everything else exactly equal.  Returns the mismatches."""
    out = [] if out is None else out
    if isinstance(expected, dict):
        if sorted(actual) != sorted(expected):
            out.append((path, "keys", sorted(actual), sorted(expected)))
        for k in expected:
            if k in actual:
                json_close(actual[k], expected[k], f"{path}.{k}", tol, out)
    elif isinstance(expected, list):
        if len(actual) != len(expected):
            out.append((path, "len", len(actual), len(expected)))
        for i, (a, e) in enumerate(zip(actual, expected)):
            json_close(a, e, f"{path}[{i}]", tol, out)
    elif isinstance(expected, (int, float)) and not isinstance(expected, bool):
        if not abs(actual - expected) <= tol:
            out.append((path, actual, expected))
    elif actual != expected:
        out.append((path, actual, expected))
    return out


def host_threads() -> int:
    return max(1, min(8, os.cpu_count() or 1))
