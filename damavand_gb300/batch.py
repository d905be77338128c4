"""Many independent circuits of uneven size and depth in one persistent launch.

``Batch`` wraps ``dmv_batch_*`` (include/damavand_gpu.h): all statevectors in
one device arena, all circuits planned into window passes, one persistent
kernel with per-circuit dependency counters, captured with the arena reset and
the per-circuit Pauli-Z reductions in a CUDA graph. The reference runs one
circuit per process; this has no counterpart there.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import Gate, check, dptr, lib

_PREC = {"complex128": _lib.C128, "complex64": _lib.C64}
_ARITH = {"fp64": _lib.ARITH_FP64, "fp64-direct": _lib.ARITH_FP64_DIRECT, "fp32x2": _lib.ARITH_FP32X2,
          "int64": _lib.ARITH_INT64}


class Batch:
    def __init__(self, circuits, precision: str = "complex128", arithmetic: str = "fp64"):
        """circuits: list of (num_qubits, gates), gates as (kind, target, control, is_observable, theta)
        tuples (observable gates are skipped, as by Circuit.forward)."""
        self.num_qubits = [int(n) for n, _ in circuits]
        flat = []
        offsets = [0]
        for _, gates in circuits:
            sel = [g for g in gates if not g[3]]
            flat.extend(sel)
            offsets.append(len(flat))
        arr = (Gate * max(len(flat), 1))()
        for i, (kind, target, control, _obs, theta) in enumerate(flat):
            arr[i].kind, arr[i].target, arr[i].control, arr[i].theta = kind, target, control, theta
        nq = np.ascontiguousarray(self.num_qubits, dtype=np.int32)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        h = ctypes.c_void_p()
        check(lib.dmv_batch_create(len(circuits), nq.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                   off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), arr, _PREC[precision],
                                   _ARITH[arithmetic], ctypes.byref(h)))
        self._h = h
        self.precision = precision
        self.num_gates = len(flat)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.dmv_batch_destroy(h)
            self._h = ctypes.c_void_p()

    def configure(self, tile_bits: int = 12, low_bits: int = 6, tiles_per_item: int = 4) -> None:
        check(lib.dmv_batch_configure(self._h, tile_bits, low_bits, tiles_per_item))

    def autotune(self) -> dict:
        k, low, tpi, ms = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        check(lib.dmv_batch_autotune(self._h, ctypes.byref(k), ctypes.byref(low), ctypes.byref(tpi),
                                     ctypes.byref(ms)))
        return {"tile_bits": k.value, "low_bits": low.value, "tiles_per_item": tpi.value, "ms": ms.value}

    def run(self) -> float:
        """Resets every state to |0...0>, applies every circuit, reduces every <Z_q>; returns ms."""
        ms = ctypes.c_double()
        check(lib.dmv_batch_run(self._h, ctypes.byref(ms)))
        return ms.value

    def expect_z(self) -> list:
        out = np.empty(sum(self.num_qubits), dtype=np.float64)
        check(lib.dmv_batch_expect_z(self._h, dptr(out)))
        res, pos = [], 0
        for n in self.num_qubits:
            res.append(out[pos:pos + n].copy())
            pos += n
        return res

    def state(self, index: int) -> np.ndarray:
        out = np.empty(1 << self.num_qubits[index], dtype=np.complex128)
        check(lib.dmv_batch_copy_state(self._h, index, dptr(out.view(np.float64))))
        return out

    def stats(self) -> dict:
        items, passes, ops = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        grid, ms = ctypes.c_int32(), ctypes.c_double()
        check(lib.dmv_batch_stats(self._h, ctypes.byref(items), ctypes.byref(passes), ctypes.byref(ops),
                                  ctypes.byref(grid), ctypes.byref(ms)))
        return {"items": items.value, "passes": passes.value, "ops": ops.value, "grid": abs(grid.value),
                "cuda_graph": grid.value >= 0, "last_ms": ms.value}
