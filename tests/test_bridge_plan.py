"""The FP32 tiled kernel's level-ordered bridge plans against the streamed bridge, on the host.

The kernel evaluates each time tile's Brownian-bridge nodes level by level from a plan that the
host builds by running the streamed bridge (crates/riga-engine/src/qmc.rs:158-191) on node ids;
this compiles ``tests/native/bridge_plan_check.cu`` against the engine library and checks that a
plan reproduces the streamed bridge's increments bit for bit for 33 step counts and every tile
depth.  No GPU is used.
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "riga-flow_gb300" / "csrc"
LIBDIR = ROOT / "riga-flow_gb300" / "_build"


def test_bridge_plans_reproduce_the_streamed_bridge(tmp_path):
    sys.path.insert(0, str(ROOT / "riga-flow_gb300"))
    from riga_gb300.build import build_library, nvcc

    build_library()
    exe = tmp_path / "bridge_plan_check"
    cmd = [nvcc(), "-std=c++17", "-O1", "-I", str(CSRC), str(ROOT / "tests" / "native" / "bridge_plan_check.cu"),
           "-L", str(LIBDIR), "-lriga_gb300", "-Xlinker", f"-rpath={LIBDIR}", "-o", str(exe)]
    if shutil.which(cmd[0]) is None and not Path(cmd[0]).exists():
        pytest.skip("nvcc is not available")
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatching plans" in r.stdout
