"""ctypes binding of the reference-replay harness (test infrastructure only).

Runs the reference's own CUDA kernels (oracle/_ref/pdflow_ref.cubin, built
from the reference's unmodified pdflow_cudalib.cu by oracle/ref/Makefile)
through the host sequence of PD_flow_opencv (oracle/ref/refharness.c).  Used
to produce the golden vectors under tests/golden/ and to time the reference
CUDA path next to ours.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "pdflow_ref.cubin")
if not os.path.exists(CUBIN):
    CUBIN = os.path.join(HERE, "_ref", "pdflow_ref.fatbin")
LIB = os.path.join(HERE, "_build", "librefharness.so")

DUMP_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_float), ctypes.c_long)
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_lib = None


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(os.path.join(HERE, "_ref", "csf_layout.h"))


def ensure_built() -> str:
    if not os.path.exists(LIB):
        subprocess.run(["sh", os.path.join(HERE, "ref", "build_harness.sh")], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        ensure_built()
        _lib = ctypes.CDLL(LIB)
        _lib.refh_create.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.POINTER(ctypes.c_void_p)]
        _lib.refh_push.argtypes = [ctypes.c_void_p, _f32p, _f32p, DUMP_FN, ctypes.c_void_p]
        _lib.refh_solve.argtypes = [ctypes.c_void_p, _f32p, _f32p, _f32p, DUMP_FN, ctypes.c_void_p]
        _lib.refh_time_pairs.argtypes = [ctypes.c_void_p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p,
                                         ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        _lib.refh_destroy.argtypes = [ctypes.c_void_p]
        _lib.refh_error.argtypes = [ctypes.c_void_p]
        _lib.refh_error.restype = ctypes.c_char_p
        _lib.refh_set_iter_dump_mask.argtypes = [ctypes.c_void_p, ctypes.c_ulonglong]
    return _lib


class RefSolver:
    """The reference CUDA solver for one (rows, image size)."""

    def __init__(self, rows: int, width: int, height: int):
        L = lib()
        self.h = ctypes.c_void_p()
        self.rows, self.cols = rows, rows * 320 // 240
        rc = L.refh_create(CUBIN.encode(), rows, width, height, ctypes.byref(self.h))
        if rc != 0:
            msg = L.refh_error(self.h)
            raise RuntimeError(f"refh_create failed ({rc}): {msg.decode() if msg else ''}")

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed ({rc}): {lib().refh_error(self.h).decode()}")

    def solve_pair(self, I1, Z1, I2, Z2, dump: bool = False):
        store = {}

        def _cb(ctx, name, level, ptr, n):
            store[(name.decode(), level)] = np.ctypeslib.as_array(ptr, shape=(n,)).copy()

        cb = DUMP_FN(_cb) if dump else ctypes.cast(None, DUMP_FN)
        L = lib()
        f32 = lambda a: np.ascontiguousarray(a, np.float32)
        self._check(L.refh_push(self.h, f32(I1), f32(Z1), cb, None), "push 1")
        if dump:
            store = {("old_" + k[0], k[1]): v for k, v in store.items()}
        self._check(L.refh_push(self.h, f32(I2), f32(Z2), cb, None), "push 2")
        n = self.rows * self.cols
        dx, dy, dz = (np.zeros(n, np.float32) for _ in range(3))
        self._check(L.refh_solve(self.h, dx, dy, dz, cb, None), "solve")
        return (dx, dy, dz, store) if dump else (dx, dy, dz)

    def set_iter_dump_mask(self, mask: int):
        """Dump the coarsest level's state after iteration k+1 for every set bit k."""
        lib().refh_set_iter_dump_mask(self.h, mask)

    def time_pairs(self, I1, Z1, I2, Z2, reps: int) -> float:
        n = self.rows * self.cols
        dx, dy, dz = (np.zeros(n, np.float32) for _ in range(3))
        ms = ctypes.c_double()
        f32 = lambda a: np.ascontiguousarray(a, np.float32)
        self._check(lib().refh_time_pairs(self.h, f32(I1), f32(Z1), f32(I2), f32(Z2), dx, dy, dz, reps,
                                          ctypes.byref(ms)), "time")
        return ms.value

    def close(self):
        if self.h:
            lib().refh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
