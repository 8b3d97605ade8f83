"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this module, and only as the checker / the timed host-core baseline.  The
library is built from oracle/pdflow_oracle.c by oracle/Makefile (or by
`ensure_built()`, which runs the same compiler line).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_pdflow.so")

_lib = None
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")

DUMP_FN = {
    "f32": ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_float), ctypes.c_long),
    "f64": ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_double), ctypes.c_long),
}


def ensure_built(force: bool = False) -> str:
    src = os.path.join(HERE, "pdflow_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        ensure_built()
        _lib = ctypes.CDLL(LIB_PATH)
        for sfx, dump in DUMP_FN.items():
            f = getattr(_lib, f"or_solve_{sfx}")
            f.restype = ctypes.c_int
            f.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, _f32p, _f32p, _f32p, _f32p,
                          ctypes.c_void_p, _f32p, _f32p, _f32p, dump, ctypes.c_void_p]
            g = getattr(_lib, f"or_config_{sfx}")
            g.restype = ctypes.c_int
            g.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.POINTER(ctypes.c_uint)]
    return _lib


def config(rows: int, width: int, height: int) -> dict:
    out = (ctypes.c_uint * 10)()
    if lib().or_config_f64(rows, width, height, out) != 0:
        raise ValueError(f"unsupported size rows={rows} image={width}x{height}")
    v = list(out)
    return dict(cols=v[0], cam_mode=v[1], ctf_levels=v[2], pyr_levels=v[3], num_max_iter=v[4:10])


def solve(rows: int, width: int, height: int, I1, Z1, I2, Z2, precision: str = "f64",
          iters=None, dump: bool = False):
    """Run the whole coarse-to-fine solve on float column-major frames.

    Returns (dx, dy, dz) as float32 arrays of rows*cols (column-major) and, if
    `dump`, a dict {(name, level): ndarray} of intermediates."""
    L = lib()
    cols = rows * 320 // 240
    n = rows * cols
    dx, dy, dz = (np.zeros(n, np.float32) for _ in range(3))
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (I1, Z1, I2, Z2)]
    store = {}
    dt = np.float64 if precision == "f64" else np.float32

    def _cb(ctx, name, level, ptr, cnt):
        store[(name.decode(), level)] = np.ctypeslib.as_array(ptr, shape=(cnt,)).astype(dt).copy()

    cb = DUMP_FN[precision](_cb) if dump else ctypes.cast(None, DUMP_FN[precision])
    it = None
    if iters is not None:
        it = (ctypes.c_uint * 6)(*iters)
    rc = getattr(L, f"or_solve_{precision}")(rows, width, height, *arrs,
                                              ctypes.cast(it, ctypes.c_void_p) if it is not None else None,
                                              dx, dy, dz, cb, None)
    if rc != 0:
        raise ValueError(f"oracle rejected rows={rows} image={width}x{height}")
    return (dx, dy, dz, store) if dump else (dx, dy, dz)


def _stage(name: str, precision: str):
    return getattr(lib(), f"or_{name}_{precision}")


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _ptr_array(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def stage_call(name: str, precision: str, *args):
    """Call a stage function with ndarray / scalar arguments.  ndarrays are
    passed by pointer, lists of ndarrays as pointer arrays, ints as unsigned,
    floats as the stage's real type."""
    f = _stage(name, precision)
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    cargs = []
    keep = []
    for a in args:
        if isinstance(a, np.ndarray):
            cargs.append(_ptr(a))
        elif isinstance(a, (list, tuple)):
            pa = _ptr_array(a)
            keep.append(pa)
            cargs.append(ctypes.cast(pa, ctypes.c_void_p))
        elif isinstance(a, float):
            cargs.append(real(a))
        elif isinstance(a, bool):
            cargs.append(ctypes.c_int(int(a)))
        elif isinstance(a, int):
            cargs.append(ctypes.c_long(a) if a > 0xFFFFFFFF else ctypes.c_uint(a))
        elif a is None:
            cargs.append(ctypes.c_void_p(None))
        else:
            raise TypeError(type(a))
    f.restype = None
    f(*cargs)


def decode_frame(intensity: np.ndarray, depth: np.ndarray):
    """The shared host decode (oracle copy): row-major uint8/uint16 -> column-major float."""
    h, w = intensity.shape
    I = np.zeros(w * h, np.float32)
    Z = np.zeros(w * h, np.float32)
    f = lib().or_decode_frame
    f.restype = None
    f(ctypes.c_uint(w), ctypes.c_uint(h), _ptr(np.ascontiguousarray(intensity, np.uint8)),
      _ptr(np.ascontiguousarray(depth, np.uint16)), _ptr(I), _ptr(Z))
    return I, Z


def decode_frame_rgb8_mm(rgb: np.ndarray, depth_mm: np.ndarray, rotate180: bool = False):
    """The live application's conversion (oracle copy): row-major RGB888 [h, w, 3]
    and millimetre depth [h, w] -> column-major float intensity and metres."""
    h, w = depth_mm.shape
    I = np.zeros(w * h, np.float32)
    Z = np.zeros(w * h, np.float32)
    f = lib().or_decode_frame_rgb8_mm
    f.restype = None
    f(ctypes.c_uint(w), ctypes.c_uint(h), _ptr(np.ascontiguousarray(rgb, np.uint8)),
      _ptr(np.ascontiguousarray(depth_mm, np.uint16)), ctypes.c_int(int(rotate180)), _ptr(I), _ptr(Z))
    return I, Z


def energy(R: int, C: int, old: tuple, new: tuple, du, dv, dw, mu: float = 75.0, lambda_i: float = 0.04,
           lambda_d: float = 0.35, precision: str = "f64") -> float:
    """Energy of a level solution (or_energy, pdflow_oracle.c): `old`/`new` are
    the two frames' level images (colour, depth, xx, yy), column-major R*C;
    du, dv the total image-plane flow in level pixels, dw in metres."""
    dt = np.float64 if precision == "f64" else np.float32
    cv = lambda a: np.ascontiguousarray(np.asarray(a, dtype=dt).ravel())
    o = [cv(a) for a in old]
    n = [cv(a) for a in new]
    u, v, w = cv(du), cv(dv), cv(dw)
    f = _stage("energy", precision)
    real = ctypes.c_double if precision == "f64" else ctypes.c_float
    f.restype = ctypes.c_double
    keep = [_ptr_array([o[k], n[k]]) for k in range(4)]
    return float(f(ctypes.c_uint(R), ctypes.c_uint(C), real(mu), real(lambda_i), real(lambda_d),
                   *[ctypes.cast(p, ctypes.c_void_p) for p in keep], _ptr(u), _ptr(v), _ptr(w)))


def solve_seeded(rows: int, width: int, height: int, I1, Z1, I2, Z2, first: int, seed, iter_scale: float = 1.0,
                 precision: str = "f64", dump: bool = False):
    """The solve started at level `first` from `seed` ([3][N_first]: du, dv in
    level pixels, dw in metres) with zero duals, every solved level running
    ceil(num_max_iter * iter_scale) iterations (iter_scale is rounded to
    float32 first, as the GPU library receives it)."""
    L = lib()
    cols = rows * 320 // 240
    n = rows * cols
    dx, dy, dz = (np.zeros(n, np.float32) for _ in range(3))
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (I1, Z1, I2, Z2)]
    sd = np.ascontiguousarray(np.asarray(seed, dtype=np.float32).ravel())
    store = {}
    dt = np.float64 if precision == "f64" else np.float32

    def _cb(ctx, name, level, ptr, cnt):
        store[(name.decode(), level)] = np.ctypeslib.as_array(ptr, shape=(cnt,)).astype(dt).copy()

    cb = DUMP_FN[precision](_cb) if dump else ctypes.cast(None, DUMP_FN[precision])
    f = getattr(L, f"or_solve_seeded_{precision}")
    f.argtypes = [ctypes.c_uint] * 3 + [_f32p] * 4 + [ctypes.c_uint, _f32p, ctypes.c_double] + [_f32p] * 3 + \
                 [DUMP_FN[precision], ctypes.c_void_p]
    rc = f(rows, width, height, *arrs, first, sd, float(np.float32(iter_scale)), dx, dy, dz, cb, None)
    if rc != 0:
        raise ValueError(f"oracle rejected the seeded solve (rows={rows}, first={first})")
    return (dx, dy, dz, store) if dump else (dx, dy, dz)
