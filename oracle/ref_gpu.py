"""Recipe for the reference's own `gpu`-backend kernels as a GPU-side oracle (test infrastructure).

The reference's `gpu` backend compiles CUDA C source held in a Rust string constant
(``KERNEL_SRC``, crates/riga-engine/src/gpu.rs:27-76) with NVRTC.  Where the reference checkout is
mounted, :func:`extract` copies that string verbatim into ``oracle/_ref/gpu_rs_kernels.cu`` (git-
ignored, never committed); :func:`build` compiles it together with ``ref_gpu_host.cu`` (host
launchers written here) into ``oracle/_ref/libref_gpu.so`` with nvcc's defaults, which are NVRTC's
(-fmad=true, IEEE division and square root).  A machine without the checkout builds from an
already extracted ``_ref/gpu_rs_kernels.cu``; without either, the drop-in exactness tests skip.

Usage:  python oracle/ref_gpu.py <path of the riga-flow checkout>
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
SRC = REF / "gpu_rs_kernels.cu"
LIB = REF / "libref_gpu.so"
GPU_RS = Path("crates/riga-engine/src/gpu.rs")
# where the reference checkout is mounted in the build container; absent on the GPU machines,
# which build from the extracted source that travels with the repository's working tree
CHECKOUT = Path("/root/reference")
OPEN = 'const KERNEL_SRC: &str = r#"'
CLOSE = '"#;'


def extract(reference_root) -> Path:
    """Copy KERNEL_SRC out of gpu.rs verbatim (the raw string literal's contents)."""
    text = (Path(reference_root) / GPU_RS).read_text()
    i = text.index(OPEN) + len(OPEN)
    j = text.index(CLOSE, i)
    REF.mkdir(parents=True, exist_ok=True)
    SRC.write_text(text[i:j])
    return SRC


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def build(reference_root=CHECKOUT) -> Path | None:
    """Extract (when the checkout is present) and compile; None without a source."""
    if reference_root is not None and (Path(reference_root) / GPU_RS).exists():
        extract(reference_root)
    if not SRC.exists():
        return None
    deps = [SRC, HERE / "ref_gpu_host.cu"]
    if LIB.exists() and all(LIB.stat().st_mtime_ns >= d.stat().st_mtime_ns for d in deps):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared",
           "-Xcompiler", "-fPIC", "-I", str(HERE), str(HERE / "ref_gpu_host.cu"), "-o", str(tmp),
           "-cudart", "static"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL | None:
    """The compiled reference kernels, or None when no extracted source exists."""
    global _lib
    if _lib is None:
        if build() is None:
            return None
        L = C.CDLL(str(LIB))
        f, i32 = C.POINTER(C.c_float), C.c_int
        L.ref_worst_of.restype = i32
        L.ref_worst_of.argtypes = [f, f, f, i32]
        L.ref_lv_propagate.restype = i32
        L.ref_lv_propagate.argtypes = [f, f, f, i32, f, C.c_float, C.c_float, C.c_float, i32, i32,
                                       C.c_float, C.c_float, C.c_float, C.c_float, f, C.POINTER(i32)]
        _lib = L
    return _lib


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: ref_gpu.py <path of the riga-flow checkout>")
    print(build(sys.argv[1]))
