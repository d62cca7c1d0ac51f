"""The reference's ``gpu`` backend API (crates/riga-engine/src/gpu.rs:500-564) over the C ABI.

Buffers are float32 numpy arrays; results come back as numpy arrays.  There is no CPU fallback:
every call raises ``RigaError('gpu_unavailable', …)`` without a usable sm_103a device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .abi import RigaError, check, load_library

_f = C.POINTER(C.c_float)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f)


def _f32(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.float32))


def ensure_available() -> None:
    lib = load_library()
    check(lib, lib.rg_ensure_available())


def device_name() -> str:
    lib = load_library()
    buf = C.create_string_buffer(256)
    check(lib, lib.rg_device_name(buf, 256))
    return buf.value.decode()


def arch() -> str:
    lib = load_library()
    buf = C.create_string_buffer(64)
    check(lib, lib.rg_arch(buf, 64))
    return buf.value.decode()


def worst_of(a, b) -> np.ndarray:
    a, b = _f32(a), _f32(b)
    if a.shape != b.shape:
        raise RigaError("shape_mismatch", "worst-of inputs must have equal length")
    out = np.empty_like(a)
    lib = load_library()
    check(lib, lib.rg_worst_of(_fp(a), _fp(b), _fp(out), a.size))
    return out


def lv_terminal_spots(normals, rows, ls_axis, s0, references, call_barrier, paths, steps, dt,
                      rate, dividends):
    normals, rows, ls_axis = _f32(normals), _f32(rows), _f32(ls_axis)
    s0, references, dividends = _f32(s0), _f32(references), _f32(dividends)
    gx = ls_axis.size // 2
    out = np.empty(paths * 2, dtype=np.float32)
    ko = np.empty(paths, dtype=np.int32)
    lib = load_library()
    check(lib, lib.rg_lv_terminal_spots(_fp(normals), _fp(rows), _fp(ls_axis), gx, _fp(s0),
                                        _fp(references), float(call_barrier), paths, steps,
                                        float(dt), float(rate), _fp(dividends), _fp(out),
                                        ko.ctypes.data_as(C.POINTER(C.c_int32))))
    return out, ko


class ResidentLv:
    """gpu.rs:409-488: upload once, ``run`` per spot bump, ``download`` blocks."""

    def __init__(self, normals, rows, ls_axis, paths, steps, dt):
        self.lib = load_library()
        self._keep = [_f32(normals), _f32(rows), _f32(ls_axis)]
        self.paths = paths
        h = C.c_void_p()
        gx = self._keep[2].size // 2
        check(self.lib, self.lib.rg_resident_lv_create(_fp(self._keep[0]), _fp(self._keep[1]),
                                                       _fp(self._keep[2]), gx, paths, steps,
                                                       float(dt), C.byref(h)))
        self.h = h

    def run(self, s0, references, call_barrier, rate, dividends):
        s0, references, dividends = _f32(s0), _f32(references), _f32(dividends)
        check(self.lib, self.lib.rg_resident_lv_run(self.h, _fp(s0), _fp(references),
                                                     float(call_barrier), float(rate),
                                                     _fp(dividends)))

    def download(self):
        out = np.empty(self.paths * 2, dtype=np.float32)
        ko = np.empty(self.paths, dtype=np.int32)
        check(self.lib, self.lib.rg_resident_lv_download(self.h, _fp(out),
                                                          ko.ctypes.data_as(C.POINTER(C.c_int32))))
        return out, ko

    def synchronize(self):
        check(self.lib, self.lib.rg_resident_lv_synchronize(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.rg_resident_lv_destroy(self.h)
            self.h = None


def resident_lv(normals, rows, ls_axis, paths, steps, dt) -> ResidentLv:
    return ResidentLv(normals, rows, ls_axis, paths, steps, dt)


class ResidentWorstOf:
    """gpu.rs:362-405"""

    def __init__(self, a, b):
        self.lib = load_library()
        a, b = _f32(a), _f32(b)
        if a.shape != b.shape:
            raise RigaError("shape_mismatch", "worst-of inputs must have equal length")
        self._keep = [a, b]
        self.n = a.size
        h = C.c_void_p()
        check(self.lib, self.lib.rg_resident_worst_of_create(_fp(a), _fp(b), a.size, C.byref(h)))
        self.h = h

    def reduce(self):
        check(self.lib, self.lib.rg_resident_worst_of_reduce(self.h))

    def download(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float32)
        check(self.lib, self.lib.rg_resident_worst_of_download(self.h, _fp(out)))
        return out

    def synchronize(self):
        check(self.lib, self.lib.rg_resident_worst_of_synchronize(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.rg_resident_worst_of_destroy(self.h)
            self.h = None


def resident_worst_of(a, b) -> ResidentWorstOf:
    return ResidentWorstOf(a, b)
