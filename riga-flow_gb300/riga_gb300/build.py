"""In-tree build of the engine library (``riga-flow_gb300/_build/libriga_gb300.so``).

Every translation unit is compiled by nvcc for sm_103a only, in parallel; the FP64 prologue and
parity kernels are compiled with ``-fmad=false`` so their products and sums round separately as
in the reference.  The library links the CUDA runtime statically, so it needs only the driver.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

from .abi import LIB_PATH, ROOT_DIR

CSRC = ROOT_DIR / "csrc"
BUILD = ROOT_DIR / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-Xptxas", "-warn-spills"]
NO_FMA = {"phoenix64.cu", "prologue.cu", "book64.cu", "mclane.cu"}
# RG_PHASE_CLOCKS=1 builds the tiled FP32 kernel with per-phase clock counters (rg_phase_clocks)
PHASE_CLOCKS = os.environ.get("RG_PHASE_CLOCKS", "0") not in ("", "0")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stamp(srcs) -> str:
    parts = []
    for p in srcs + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [
            ROOT_DIR.parent / "include" / "riga_gb300.h", Path(__file__)]:
        parts.append(f"{p.name}:{p.stat().st_mtime_ns}:{p.stat().st_size}")
    parts.append(f"phase_clocks:{int(PHASE_CLOCKS)}")
    return "\n".join(parts)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    BUILD.mkdir(parents=True, exist_ok=True)
    stamp_file = BUILD / "stamp.txt"
    stamp = _stamp(srcs)
    if not force and LIB_PATH.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB_PATH
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.name + ".o")
        flags = list(COMMON)
        if src.name in NO_FMA:
            flags += ["-fmad=false"]
        if PHASE_CLOCKS:
            flags += ["-DRG_PHASE_CLOCKS"]
        cmd = [cc, *ARCH, *flags, "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    stamp_file.write_text(stamp)
    return LIB_PATH


def ptxas_report(src: str = "phoenix32.cu") -> str:
    """``-Xptxas -v`` register/spill/shared-memory report of one translation unit."""
    p = CSRC / src
    flags = list(COMMON) + (["-fmad=false"] if src in NO_FMA else [])
    cmd = [nvcc(), *ARCH, *flags, "-Xptxas", "-v", "-I", str(CSRC), "-c", str(p), "-o", os.devnull]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stderr


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
