"""ctypes binding of libpdflow_gb300.so (the C ABI of include/pdflow.h).

The library is the only compute path: there is no CPU fallback.  Loading it
fails loudly (ExtensionMissing) when it has not been built, and a solver
cannot be created without a GB300 (sm_103) device.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

OK, ERR_ARG, ERR_OOM, ERR_CUDA, ERR_STATE, ERR_TIMEOUT, ERR_NO_DEVICE = 0, -1, -2, -3, -4, -5, -6


class ExtensionMissing(RuntimeError):
    pass


class PDFlowError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with status {code}: {last_error()}")
        self.code = code


class Params(ctypes.Structure):
    """pdflow_params (include/pdflow.h)."""
    _fields_ = [("lambda_i", ctypes.c_float), ("lambda_d", ctypes.c_float), ("mu", ctypes.c_float),
                ("fovh", ctypes.c_float), ("fovv", ctypes.c_float), ("num_max_iter", ctypes.c_uint * 6)]


TUNE_CANDIDATES = 29   # PDFLOW_TUNE_CANDIDATES: form 0, form 1, forms 2..8 x {2, 3, 4}, form 9 x {4, 6, 8},
#                        form 10 x {2, 3, 4}


class TuneLevel(ctypes.Structure):
    """pdflow_tune_level (include/pdflow.h)."""
    _fields_ = [("form", ctypes.c_int), ("iters_per_launch", ctypes.c_uint),
                ("ms_per_iter", ctypes.c_float * TUNE_CANDIDATES)]


class TuneReport(ctypes.Structure):
    """pdflow_tune_report (include/pdflow.h)."""
    _fields_ = [("levels", ctypes.c_uint), ("level", TuneLevel * 8)]


class LearnedOpts(ctypes.Structure):
    """pdflow_learned_opts (include/pdflow_net.h)."""
    _fields_ = [("iter_scale", ctypes.c_float), ("energy_margin", ctypes.c_float)]


class LearnedReport(ctypes.Structure):
    """pdflow_learned_report (include/pdflow_net.h)."""
    _fields_ = [("fallbacks", ctypes.c_uint), ("max_energy_ratio", ctypes.c_float)]


class NoiseTex(ctypes.Structure):
    """pdflow_noise_tex (include/pdflow_scene.h)."""
    _fields_ = [("perm", ctypes.c_int32 * 256), ("vals", ctypes.c_double * 256), ("cell", ctypes.c_double)]


class SceneObject(ctypes.Structure):
    """pdflow_scene_object (include/pdflow_scene.h)."""
    _fields_ = [("kind", ctypes.c_int32), ("pad_", ctypes.c_int32), ("center", ctypes.c_double * 3),
                ("rot", ctypes.c_double * 9), ("next_center", ctypes.c_double * 3), ("next_rot", ctypes.c_double * 9),
                ("size", ctypes.c_double * 3), ("albedo", ctypes.c_double), ("tex", NoiseTex)]


class SceneFrame(ctypes.Structure):
    """pdflow_scene_frame (include/pdflow_scene.h)."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("fx", ctypes.c_double),
                ("fy", ctypes.c_double), ("cx", ctypes.c_double), ("cy", ctypes.c_double),
                ("plane", ctypes.c_double * 3), ("plane_tex", NoiseTex), ("n_objects", ctypes.c_uint32),
                ("sensor_noise", ctypes.c_uint32), ("noise_seed", ctypes.c_uint64), ("objects", SceneObject * 8)]


class ServerConfig(ctypes.Structure):
    """pdflow_server_config (include/pdflow_server.h)."""
    _fields_ = [("device_budget_bytes", ctypes.c_size_t), ("slots_per_lane", ctypes.c_uint), ("learned", ctypes.c_int),
                ("iter_scale", ctypes.c_float), ("energy_margin", ctypes.c_float),
                ("net_params", ctypes.POINTER(ctypes.c_float)), ("net_param_count", ctypes.c_size_t)]


class RequestInfo(ctypes.Structure):
    """pdflow_request_info (include/pdflow_server.h)."""
    _fields_ = [("request_id", ctypes.c_ulonglong), ("stream_id", ctypes.c_uint), ("frame_index", ctypes.c_ulonglong),
                ("status", ctypes.c_int), ("has_flow", ctypes.c_int), ("batch_pairs", ctypes.c_uint),
                ("batch_fallbacks", ctypes.c_uint), ("submit_ms", ctypes.c_double), ("start_ms", ctypes.c_double),
                ("done_ms", ctypes.c_double)]


class ReplayStream(ctypes.Structure):
    """pdflow_replay_stream (include/pdflow_server.h)."""
    _fields_ = [("stream_id", ctypes.c_uint), ("frames", ctypes.c_uint),
                ("intensity", ctypes.POINTER(ctypes.c_void_p)), ("depth", ctypes.POINTER(ctypes.c_void_p))]


class ServerStats(ctypes.Structure):
    """pdflow_server_stats (include/pdflow_server.h)."""
    _fields_ = [("lanes", ctypes.c_uint), ("streams", ctypes.c_uint), ("submitted", ctypes.c_ulonglong),
                ("completed", ctypes.c_ulonglong), ("batches", ctypes.c_ulonglong),
                ("pairs_solved", ctypes.c_ulonglong), ("fallbacks", ctypes.c_ulonglong),
                ("device_bytes", ctypes.c_size_t)]


DUMP_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_float), ctypes.c_long)

_lib = None
vp = ctypes.c_void_p
u32 = ctypes.c_uint

_SIGNATURES = {
    "pdflow_default_params": (ctypes.c_int, [u32, ctypes.POINTER(Params)]),
    "pdflow_create": (ctypes.c_int, [u32, u32, u32, ctypes.POINTER(Params), ctypes.POINTER(vp)]),
    "pdflow_destroy": (ctypes.c_int, [vp]),
    "pdflow_push_frame": (ctypes.c_int, [vp, vp, vp]),
    "pdflow_push_frame_u16": (ctypes.c_int, [vp, vp, vp]),
    "pdflow_push_frame_rgb8_mm": (ctypes.c_int, [vp, vp, vp, ctypes.c_int]),
    "pdflow_push_frames_rgb8_mm": (ctypes.c_int, [vp, u32, vp, vp, ctypes.c_int]),
    "pdflow_push_frames_rgb8_mm_device": (ctypes.c_int, [vp, u32, vp, vp, ctypes.c_int]),
    "pdflow_push_frame_u16_device": (ctypes.c_int, [vp, vp, vp]),
    "pdflow_solve": (ctypes.c_int, [vp]),
    "pdflow_read_flow": (ctypes.c_int, [vp, vp, vp, vp]),
    "pdflow_flow_device": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]),
    "pdflow_copy_flow_device": (ctypes.c_int, [vp, u32, vp, vp, vp]),
    "pdflow_read_level_images": (ctypes.c_int, [vp, u32, ctypes.c_int, vp, vp, vp, vp]),
    "pdflow_synchronize": (ctypes.c_int, [vp]),
    "pdflow_set_stream": (ctypes.c_int, [vp, vp]),
    "pdflow_get_config": (ctypes.c_int, [vp] + [ctypes.POINTER(u32)] * 5),
    "pdflow_set_graph_mode": (ctypes.c_int, [vp, ctypes.c_int]),
    "pdflow_create_batch": (ctypes.c_int, [u32, u32, u32, ctypes.POINTER(Params), u32, ctypes.POINTER(vp)]),
    "pdflow_push_frames": (ctypes.c_int, [vp, u32, vp, vp]),
    "pdflow_push_frames_u16": (ctypes.c_int, [vp, u32, vp, vp]),
    "pdflow_push_frames_u16_device": (ctypes.c_int, [vp, u32, vp, vp]),
    "pdflow_solve_batch": (ctypes.c_int, [vp, u32]),
    "pdflow_read_flow_batch": (ctypes.c_int, [vp, u32, vp, vp, vp]),
    "pdflow_batch_info": (ctypes.c_int, [vp, ctypes.POINTER(u32), ctypes.POINTER(ctypes.c_size_t)]),
    "pdflow_device_bytes": (ctypes.c_size_t, [vp]),
    "pdflow_solve_pair_noalloc": (ctypes.c_int, [u32, u32, u32, ctypes.POINTER(Params), vp, vp, vp, vp, vp, vp, vp,
                                                  vp]),
    "pdflow_last_error": (ctypes.c_char_p, []),
    "pdflow_version": (ctypes.c_char_p, []),
    "pdflow_debug_solve": (ctypes.c_int, [vp, DUMP_FN, vp]),
    "pdflow_set_iteration_form": (ctypes.c_int, [vp, ctypes.c_int]),
    "pdflow_last_solve_launches": (ctypes.c_int, [vp, ctypes.POINTER(u32)]),
    "pdflow_time_level_iterations": (ctypes.c_int, [vp, u32, u32, u32, ctypes.POINTER(ctypes.c_float)]),
    "pdflow_stage_median": (ctypes.c_int, [u32, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    "pdflow_push_frames_slots_u16": (ctypes.c_int, [vp, u32, vp, vp, vp]),
    "pdflow_push_frames_slots_u16_device": (ctypes.c_int, [vp, u32, vp, vp, vp]),
    "pdflow_solve_slots": (ctypes.c_int, [vp, u32, vp]),
    "pdflow_read_flow_slots": (ctypes.c_int, [vp, u32, vp, vp, vp, vp]),
    "pdflow_energy_batch": (ctypes.c_int, [vp, u32, vp]),
    "pdflow_image_flow_device": (ctypes.c_int, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]),
    "pdflow_solve_levels": (ctypes.c_int, [vp, u32, u32, u32, vp, ctypes.c_float, ctypes.c_int, vp]),
    "pdflow_net_create": (ctypes.c_int, [u32, ctypes.c_ulonglong, ctypes.POINTER(vp)]),
    "pdflow_net_destroy": (ctypes.c_int, [vp]),
    "pdflow_net_param_count": (ctypes.c_size_t, [vp]),
    "pdflow_net_get_params": (ctypes.c_int, [vp, vp, ctypes.c_size_t]),
    "pdflow_net_set_params": (ctypes.c_int, [vp, vp, ctypes.c_size_t]),
    "pdflow_net_set_stream": (ctypes.c_int, [vp, vp]),
    "pdflow_net_forward": (ctypes.c_int, [vp, u32, vp, vp]),
    "pdflow_net_train_step": (ctypes.c_int, [vp, u32, vp, vp, ctypes.c_float, ctypes.POINTER(ctypes.c_float)]),
    "pdflow_net_gradients": (ctypes.c_int, [vp, u32, vp, vp, vp, ctypes.POINTER(ctypes.c_float)]),
    "pdflow_solve_batch_learned": (ctypes.c_int, [vp, u32, vp, ctypes.POINTER(LearnedOpts),
                                                  ctypes.POINTER(LearnedReport)]),
    "pdflow_solve_slots_learned": (ctypes.c_int, [vp, u32, vp, vp, ctypes.POINTER(LearnedOpts),
                                                  ctypes.POINTER(LearnedReport)]),
    "pdflow_learned_energies": (ctypes.c_int, [vp, u32, vp, vp]),
    "pdflow_render_frames": (ctypes.c_int, [ctypes.POINTER(SceneFrame), u32, vp, vp, vp, vp]),
    "pdflow_net_device_bytes": (ctypes.c_size_t, [vp]),
    "pdflow_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]),
    "pdflow_server_destroy": (ctypes.c_int, [vp]),
    "pdflow_server_open_stream": (ctypes.c_int, [vp, u32, u32, ctypes.POINTER(u32)]),
    "pdflow_server_close_stream": (ctypes.c_int, [vp, u32]),
    "pdflow_server_submit": (ctypes.c_int, [vp, u32, vp, vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    "pdflow_server_wait": (ctypes.c_int, [vp, ctypes.c_ulonglong, ctypes.c_int, ctypes.POINTER(RequestInfo), vp, vp,
                                          vp]),
    "pdflow_server_get_stats": (ctypes.c_int, [vp, ctypes.POINTER(ServerStats)]),
    "pdflow_server_replay": (ctypes.c_int, [vp, ctypes.POINTER(ReplayStream), u32, ctypes.c_double, ctypes.c_ulonglong,
                                            ctypes.POINTER(RequestInfo), ctypes.POINTER(ctypes.c_double), u32,
                                            ctypes.POINTER(ctypes.c_uint)]),
    "pdflow_seed_level_inputs": (ctypes.c_int, [vp, u32, vp]),
    "pdflow_seed_level_labels": (ctypes.c_int, [vp, u32, vp]),
    "pdflow_set_level_form": (ctypes.c_int, [vp, u32, ctypes.c_int, u32]),
    "pdflow_autotune": (ctypes.c_int, [vp, u32, u32, ctypes.POINTER(TuneReport)]),
    "pdflow_read_all_solutions": (ctypes.c_int, [vp] + [vp] * 11),
    "pdflow_keep_level_solutions": (ctypes.c_int, [vp, ctypes.c_int]),
    "pdflow_read_level_solutions": (ctypes.c_int, [vp, u32] + [vp] * 11),
    "pdflow_read_level_flow": (ctypes.c_int, [vp, u32, u32] + [vp] * 6),
    "pdflow_set_tile_copy_mode": (ctypes.c_int, [ctypes.c_int, ctypes.c_int]),
    "pdflow_set_quad_prefetch": (ctypes.c_int, [ctypes.c_uint]),
    "pdflow_measure_copy_gbs": (ctypes.c_int, [ctypes.c_size_t, u32, vp, ctypes.POINTER(ctypes.c_float)]),
    "pdflow_check_div_rcp": (ctypes.c_int, [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]),
    "pdflow_strip_units": (ctypes.c_int, [u32, u32, u32, u32, ctypes.POINTER(u32), ctypes.POINTER(u32),
                                          ctypes.POINTER(u32)]),
    "pdflow_debug_wait_timeout": (ctypes.c_int, [vp, u32]),
    "pdflow_trace_solve": (ctypes.c_int, [vp, u32, ctypes.POINTER(ctypes.c_float)]),
    "pdflow_create_mixed": (ctypes.c_int, [u32, ctypes.POINTER(vp)]),
    "pdflow_push_frames_mixed": (ctypes.c_int, [vp, u32, vp, vp, vp, vp, vp]),
    "pdflow_solve_mixed": (ctypes.c_int, [vp, u32]),
    "pdflow_read_flow_mixed": (ctypes.c_int, [vp, u32, vp, vp, vp]),
    "pdflow_gemm_bf16": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int,
                                        vp, ctypes.c_int, ctypes.c_int, vp]),
}


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Loads the in-tree library (building it first if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ExtensionMissing(f"{path} is not built; run __graft_entry__.build() or python -m pdflow.build")
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGNATURES)


def last_error() -> str:
    if _lib is None:
        return ""
    s = _lib.pdflow_last_error()
    return s.decode() if s else ""


def check(code: int, what: str):
    if code != OK:
        raise PDFlowError(code, what)


def default_params(rows: int) -> Params:
    p = Params()
    check(load().pdflow_default_params(rows, ctypes.byref(p)), "pdflow_default_params")
    return p


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


_cudart_lib = None


def _cudart():
    """The CUDA runtime the library links (already loaded with it)."""
    global _cudart_lib
    if _cudart_lib is None:
        load()
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                _cudart_lib = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if _cudart_lib is None:
            raise ExtensionMissing("libcudart is not loadable")
        _cudart_lib.cudaMemcpy.restype = ctypes.c_int
        _cudart_lib.cudaMemcpy.argtypes = [vp, vp, ctypes.c_size_t, ctypes.c_int]
    return _cudart_lib


def device_to_host(dptr: int, out: np.ndarray) -> np.ndarray:
    """Blocking copy of out.nbytes bytes from device address dptr into `out`."""
    rc = _cudart().cudaMemcpy(_ptr(out), ctypes.c_void_p(dptr), out.nbytes, 2)
    if rc != 0:
        raise PDFlowError(ERR_CUDA, "cudaMemcpy device->host")
    return out


class _Extras:
    """Energy, image-plane flow and level-range solves shared by both classes."""

    def energy(self, n: int = 1) -> np.ndarray:
        """Energy of the last solve's finest-level solution (pdflow_energy_batch)."""
        e = np.zeros(n, np.float32)
        check(load().pdflow_energy_batch(self.handle, n, _ptr(e)), "pdflow_energy_batch")
        return e

    def image_flow(self, n: int = 1):
        """(du, dv, dw) [n, rows*cols] of the last solve's finest level (pixels, metres)."""
        ptrs = [vp() for _ in range(3)]
        check(load().pdflow_image_flow_device(self.handle, *[ctypes.byref(q) for q in ptrs]),
              "pdflow_image_flow_device")
        self.synchronize()
        stride = self.pair_stride()
        m = self.rows * self.cols
        out = [np.zeros((n, m), np.float32) for _ in range(3)]
        for c in range(3):
            for k in range(n):
                device_to_host(ptrs[c].value + k * stride, out[c][k])
        return out

    def keep_level_solutions(self, keep: bool = True):
        """Record every solved level's flow from the next solve on
        (pdflow_keep_level_solutions; copyAllSolutions after every level)."""
        check(load().pdflow_keep_level_solutions(self.handle, int(keep)), "pdflow_keep_level_solutions")

    def level_shape(self, level: int):
        """(rows, cols) of solved level `level` (0 = coarsest 15x20)."""
        levels = (self.rows // 15).bit_length()
        return self.rows >> (levels - 1 - level), self.cols >> (levels - 1 - level)

    def level_flow(self, level: int, pair: int = 0):
        """Pair `pair`'s record at solved level `level`: du, dv, dw (image
        plane) and dx, dy, dz (motion field), each rows_l*cols_l floats."""
        r, c = self.level_shape(level)
        names = ("du", "dv", "dw", "dx", "dy", "dz")
        out = {k: np.zeros(r * c, np.float32) for k in names}
        check(load().pdflow_read_level_flow(self.handle, pair, level, *[_ptr(out[k]) for k in names]),
              "pdflow_read_level_flow")
        return out

    def trace(self, n: int):
        """Per-level phase times of an eager plain solve of pairs [0, n)
        (pdflow_trace_solve): [{setup_ms, iterations_ms, median_ms}] coarsest first."""
        rows, cols, ctf = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
        check(load().pdflow_get_config(self.handle, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(ctf), None, None),
              "pdflow_get_config")
        ms = (ctypes.c_float * (3 * ctf.value))()
        check(load().pdflow_trace_solve(self.handle, n, ms), "pdflow_trace_solve")
        return [{"setup_ms": ms[3 * i], "iterations_ms": ms[3 * i + 1], "median_ms": ms[3 * i + 2]}
                for i in range(ctf.value)]

    def autotune(self, n: int, probe_iters: int = 12):
        """Per-level launch form and iterations per launch for pairs [0, n)
        (pdflow_autotune); returns [{form, iters_per_launch, ms_per_iter}] per level."""
        rep = TuneReport()
        check(load().pdflow_autotune(self.handle, n, probe_iters, ctypes.byref(rep)), "pdflow_autotune")
        return [{"form": rep.level[i].form, "iters_per_launch": rep.level[i].iters_per_launch,
                 "ms_per_iter": [None if not np.isfinite(x) else float(x) for x in rep.level[i].ms_per_iter]}
                for i in range(rep.levels)]

    def set_level_form(self, level: int, form: int, iters_per_launch: int = 0):
        check(load().pdflow_set_level_form(self.handle, level, form, iters_per_launch), "pdflow_set_level_form")

    def pair_stride(self) -> int:
        cap, st = u32(), ctypes.c_size_t()
        check(load().pdflow_batch_info(self.handle, ctypes.byref(cap), ctypes.byref(st)), "pdflow_batch_info")
        return int(st.value)

    def solve_levels(self, n: int, first: int, last: int = 99, seed_dptr: int | None = None,
                     iter_scale: float = 1.0, energy_level: int = -1):
        """Levels [first, last] (pdflow_solve_levels); returns the energies of
        `energy_level`'s solution when energy_level >= 0."""
        e = np.zeros(n, np.float32)
        check(load().pdflow_solve_levels(self.handle, n, first, last, ctypes.c_void_p(seed_dptr or 0),
                                         float(iter_scale), energy_level, _ptr(e)), "pdflow_solve_levels")
        return e if energy_level >= 0 else None


class Solver(_Extras):
    """One PD-Flow solver (C handle).  Method names follow the reference's
    PD_flow_opencv (scene_flow_impair.h:53-115): construct, initializeCUDA,
    createImagePyramidGPU / loadRGBDFrames, solveSceneFlowGPU, dxp/dyp/dzp,
    freeGPUMemory."""

    def __init__(self, rows: int = 240, width: int = 320, height: int = 240, params: Params | None = None,
                 use_graph: bool = True, iteration_form: int = 10):
        self.rows, self.width, self.height = rows, width, height
        self.cols = rows * 320 // 240
        self.params = params
        self._h = None
        self._use_graph = use_graph
        self._iter_form = iteration_form
        self.dxp = self.dyp = self.dzp = None

    # -- reference-shaped API --------------------------------------------------
    def initializeCUDA(self):
        lib = load()
        h = ctypes.c_void_p()
        p = ctypes.byref(self.params) if self.params is not None else None
        check(lib.pdflow_create(self.rows, self.width, self.height, p, ctypes.byref(h)), "pdflow_create")
        self._h = h
        check(lib.pdflow_set_graph_mode(h, int(self._use_graph)), "pdflow_set_graph_mode")
        check(lib.pdflow_set_iteration_form(h, int(self._iter_form)), "pdflow_set_iteration_form")
        n = self.rows * self.cols
        self.dxp, self.dyp, self.dzp = (np.zeros(n, np.float32) for _ in range(3))
        return self

    def createImagePyramidGPU(self, I: np.ndarray, Z: np.ndarray):
        """Push a frame given as the reference's float staging buffers (column-major)."""
        I = np.ascontiguousarray(I, np.float32).ravel()
        Z = np.ascontiguousarray(Z, np.float32).ravel()
        if I.size != self.width * self.height or Z.size != I.size:
            raise ValueError("frame size does not match the solver")
        check(load().pdflow_push_frame(self._h, _ptr(I), _ptr(Z)), "pdflow_push_frame")

    def push_raw(self, intensity: np.ndarray, depth: np.ndarray):
        """Push a frame as row-major uint8 intensity / uint16 depth (decoded on the GPU)."""
        i8 = np.ascontiguousarray(intensity, np.uint8)
        z16 = np.ascontiguousarray(depth, np.uint16)
        if i8.shape != (self.height, self.width) or z16.shape != i8.shape:
            raise ValueError("frame size does not match the solver")
        check(load().pdflow_push_frame_u16(self._h, _ptr(i8), _ptr(z16)), "pdflow_push_frame_u16")

    def push_rgb(self, rgb: np.ndarray, depth_mm: np.ndarray, rotate180: bool = False):
        """Push an RGB-D camera frame: row-major RGB888 [h, w, 3] and uint16
        millimetre depth [h, w], converted on the GPU as the reference's live
        application does (pdflow_push_frame_rgb8_mm)."""
        c8 = np.ascontiguousarray(rgb, np.uint8)
        z16 = np.ascontiguousarray(depth_mm, np.uint16)
        if c8.shape != (self.height, self.width, 3) or z16.shape != (self.height, self.width):
            raise ValueError("frame size does not match the solver")
        check(load().pdflow_push_frame_rgb8_mm(self._h, _ptr(c8), _ptr(z16), int(rotate180)),
              "pdflow_push_frame_rgb8_mm")

    def loadRGBDFrames(self, i1, z1, i2, z2):
        """Push two raw frames (the reference loads two PNGs, scene_flow_impair.cpp:218-277)."""
        self.push_raw(i1, z1)
        self.push_raw(i2, z2)
        return True

    def solveSceneFlowGPU(self, read_back: bool = True):
        check(load().pdflow_solve(self._h), "pdflow_solve")
        if read_back:
            self.read_flow()

    def read_flow(self):
        check(load().pdflow_read_flow(self._h, _ptr(self.dxp), _ptr(self.dyp), _ptr(self.dzp)),
              "pdflow_read_flow")
        return self.dxp, self.dyp, self.dzp

    def freeGPUMemory(self):
        if self._h is not None:
            load().pdflow_destroy(self._h)
            self._h = None

    # -- extras ----------------------------------------------------------------
    @property
    def handle(self):
        return self._h

    def synchronize(self):
        check(load().pdflow_synchronize(self._h), "pdflow_synchronize")

    def config(self):
        vals = [u32() for _ in range(5)]
        check(load().pdflow_get_config(self._h, *[ctypes.byref(v) for v in vals]), "pdflow_get_config")
        return dict(zip(("rows", "cols", "ctf_levels", "pyr_levels", "cam_mode"), (v.value for v in vals)))

    def level_images(self, level: int, frame: int):
        w, h = self.width >> level, self.height >> level
        out = [np.zeros(w * h, np.float32) for _ in range(4)]
        check(load().pdflow_read_level_images(self._h, level, frame, *[_ptr(a) for a in out]),
              "pdflow_read_level_images")
        return dict(zip(("colour", "depth", "xx", "yy"), out))

    def all_solutions(self):
        """copyAllSolutions: dx, dy, dz and both frames' depth / colour / xx / yy
        at the finest solved level (pdflow_read_all_solutions)."""
        n = self.rows * self.cols
        names = ("dx", "dy", "dz", "depth", "depth_old", "colour", "colour_old", "xx", "xx_old", "yy", "yy_old")
        out = {k: np.zeros(n, np.float32) for k in names}
        check(load().pdflow_read_all_solutions(self._h, *[_ptr(out[k]) for k in names]), "pdflow_read_all_solutions")
        return out

    def level_solutions(self, level: int):
        """copyAllSolutions at solved level `level` (pdflow_read_level_solutions;
        needs keep_level_solutions before the solve)."""
        r, c = self.level_shape(level)
        names = ("dx", "dy", "dz", "depth", "depth_old", "colour", "colour_old", "xx", "xx_old", "yy", "yy_old")
        out = {k: np.zeros(r * c, np.float32) for k in names}
        check(load().pdflow_read_level_solutions(self._h, level, *[_ptr(out[k]) for k in names]),
              "pdflow_read_level_solutions")
        return out

    def debug_solve(self):
        store = {}

        def _cb(ctx, name, level, ptr, n):
            store[(name.decode(), level)] = np.ctypeslib.as_array(ptr, shape=(n,)).copy()

        cb = DUMP_FN(_cb)
        check(load().pdflow_debug_solve(self._h, cb, None), "pdflow_debug_solve")
        self.read_flow()
        return store

    def __enter__(self):
        if self._h is None:
            self.initializeCUDA()
        return self

    def __exit__(self, *exc):
        self.freeGPUMemory()

    def __del__(self):
        try:
            self.freeGPUMemory()
        except Exception:
            pass


PD_flow = Solver


class BatchSolver(_Extras):
    """Many independent pairs of one configuration solved together
    (pdflow_create_batch).  Frames are pushed as stacks [n, height, width].
    Slot calls (push_slots / solve_slots / read_flow_slots) treat each slot as
    a camera stream that keeps its previous frame on the device."""

    def __init__(self, rows: int, width: int, height: int, max_pairs: int, params: Params | None = None,
                 use_graph: bool = True, iteration_form: int = 10):
        lib = load()
        self.rows, self.width, self.height, self.max_pairs = rows, width, height, max_pairs
        self.cols = rows * 320 // 240
        h = ctypes.c_void_p()
        p = ctypes.byref(params) if params is not None else None
        check(lib.pdflow_create_batch(rows, width, height, p, max_pairs, ctypes.byref(h)), "pdflow_create_batch")
        self._h = h
        check(lib.pdflow_set_graph_mode(h, int(use_graph)), "pdflow_set_graph_mode")
        check(lib.pdflow_set_iteration_form(h, int(iteration_form)), "pdflow_set_iteration_form")

    @property
    def handle(self):
        return self._h

    def device_bytes(self) -> int:
        return int(load().pdflow_device_bytes(self._h))

    def push_raw(self, intensity: np.ndarray, depth: np.ndarray):
        i8 = np.ascontiguousarray(intensity, np.uint8)
        z16 = np.ascontiguousarray(depth, np.uint16)
        n = i8.shape[0]
        if i8.shape != (n, self.height, self.width) or z16.shape != i8.shape:
            raise ValueError("expected stacks [n, height, width]")
        check(load().pdflow_push_frames_u16(self._h, n, _ptr(i8), _ptr(z16)), "pdflow_push_frames_u16")

    def push_rgb(self, rgb: np.ndarray, depth_mm: np.ndarray, rotate180: bool = False):
        """Push stacks [n, height, width, 3] RGB888 / [n, height, width] millimetre
        depth (pdflow_push_frames_rgb8_mm)."""
        c8 = np.ascontiguousarray(rgb, np.uint8)
        z16 = np.ascontiguousarray(depth_mm, np.uint16)
        n = z16.shape[0]
        if c8.shape != (n, self.height, self.width, 3) or z16.shape != (n, self.height, self.width):
            raise ValueError("expected stacks [n, height, width, 3] and [n, height, width]")
        check(load().pdflow_push_frames_rgb8_mm(self._h, n, _ptr(c8), _ptr(z16), int(rotate180)),
              "pdflow_push_frames_rgb8_mm")

    def push_raw_device(self, n: int, d_intensity: int, d_depth: int):
        check(load().pdflow_push_frames_u16_device(self._h, n, ctypes.c_void_p(d_intensity),
                                                   ctypes.c_void_p(d_depth)), "pdflow_push_frames_u16_device")

    def solve(self, n: int):
        check(load().pdflow_solve_batch(self._h, n), "pdflow_solve_batch")

    def read_flow(self, n: int):
        m = self.rows * self.cols
        out = [np.zeros((n, m), np.float32) for _ in range(3)]
        check(load().pdflow_read_flow_batch(self._h, n, *[_ptr(a) for a in out]), "pdflow_read_flow_batch")
        return out

    def synchronize(self):
        check(load().pdflow_synchronize(self._h), "pdflow_synchronize")

    @staticmethod
    def _slots(slots) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(slots, dtype=np.uint32).ravel())

    def push_slots(self, slots, intensity: np.ndarray, depth: np.ndarray):
        sl = self._slots(slots)
        i8 = np.ascontiguousarray(intensity, np.uint8).reshape(len(sl), self.height, self.width)
        z16 = np.ascontiguousarray(depth, np.uint16).reshape(i8.shape)
        check(load().pdflow_push_frames_slots_u16(self._h, len(sl), _ptr(sl), _ptr(i8), _ptr(z16)),
              "pdflow_push_frames_slots_u16")

    def solve_slots(self, slots):
        sl = self._slots(slots)
        check(load().pdflow_solve_slots(self._h, len(sl), _ptr(sl)), "pdflow_solve_slots")

    def read_flow_slots(self, slots):
        sl = self._slots(slots)
        m = self.rows * self.cols
        out = [np.zeros((len(sl), m), np.float32) for _ in range(3)]
        check(load().pdflow_read_flow_slots(self._h, len(sl), _ptr(sl), *[_ptr(a) for a in out]),
              "pdflow_read_flow_slots")
        return out

    def solve_learned(self, n: int, net: "Net", iter_scale: float = 0.5, energy_margin: float = 0.01):
        """Learned warm-start solve of pairs [0, n) (pdflow_solve_batch_learned)."""
        o, r = LearnedOpts(iter_scale, energy_margin), LearnedReport()
        check(load().pdflow_solve_batch_learned(self._h, n, net.handle, ctypes.byref(o), ctypes.byref(r)),
              "pdflow_solve_batch_learned")
        return dict(fallbacks=r.fallbacks, max_energy_ratio=r.max_energy_ratio)

    def solve_slots_learned(self, slots, net: "Net", iter_scale: float = 0.5, energy_margin: float = 0.01):
        sl = self._slots(slots)
        o, r = LearnedOpts(iter_scale, energy_margin), LearnedReport()
        check(load().pdflow_solve_slots_learned(self._h, len(sl), _ptr(sl), net.handle, ctypes.byref(o),
                                                ctypes.byref(r)), "pdflow_solve_slots_learned")
        return dict(fallbacks=r.fallbacks, max_energy_ratio=r.max_energy_ratio)

    def seed_level_inputs(self, n: int, d_out: int):
        check(load().pdflow_seed_level_inputs(self._h, n, vp(d_out)), "pdflow_seed_level_inputs")

    def seed_level_labels(self, n: int, d_out: int):
        check(load().pdflow_seed_level_labels(self._h, n, vp(d_out)), "pdflow_seed_level_labels")

    def learned_energies(self, n: int):
        a, b = np.zeros(n, np.float32), np.zeros(n, np.float32)
        check(load().pdflow_learned_energies(self._h, n, _ptr(a), _ptr(b)), "pdflow_learned_energies")
        return a, b

    def close(self):
        if self._h is not None:
            load().pdflow_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MixedBatch:
    """Pairs of different rows (15..480) solved together (pdflow_create_mixed):
    push(rows, frames) with frames[k] = (intensity, depth) of pair k (640x480
    for rows 480, 320x240 otherwise), then solve() and flow(k)."""

    def __init__(self, max_pairs: int, use_graph: bool = True):
        h = ctypes.c_void_p()
        check(load().pdflow_create_mixed(max_pairs, ctypes.byref(h)), "pdflow_create_mixed")
        self._h = h
        self.rows = []
        check(load().pdflow_set_graph_mode(h, int(use_graph)), "pdflow_set_graph_mode")

    @property
    def handle(self):
        return self._h

    def push(self, rows, intensity, depth):
        rows = [int(r) for r in rows]
        sel = lambda big: [k for k, r in enumerate(rows) if (r == 480) == big]
        stack = lambda ks, a, dt: (np.ascontiguousarray(np.stack([a[k] for k in ks]), dt) if ks else None)
        vi, vz = stack(sel(True), intensity, np.uint8), stack(sel(True), depth, np.uint16)
        qi, qz = stack(sel(False), intensity, np.uint8), stack(sel(False), depth, np.uint16)
        r = np.ascontiguousarray(rows, np.uint32)
        p = lambda a: _ptr(a) if a is not None else None
        check(load().pdflow_push_frames_mixed(self._h, len(rows), _ptr(r), p(vi), p(vz), p(qi), p(qz)),
              "pdflow_push_frames_mixed")
        self.rows = rows

    def solve(self, n: int | None = None):
        check(load().pdflow_solve_mixed(self._h, n or len(self.rows)), "pdflow_solve_mixed")

    def autotune(self, n: int | None = None, probe_iters: int = 12):
        """Per coarse-to-fine step (15x20 .. 480x640), the tile form and
        iterations per launch over the pairs active at that step
        (pdflow_autotune on a mixed handle); returns [{step, form,
        iters_per_launch, ms_per_iter}] for the steps some pair has."""
        rep = TuneReport()
        check(load().pdflow_autotune(self._h, n or len(self.rows), probe_iters, ctypes.byref(rep)), "pdflow_autotune")
        out = []
        for i in range(rep.levels):
            if rep.level[i].form < 0:
                continue
            ms = [None if np.isnan(x) else float(x) for x in rep.level[i].ms_per_iter]
            out.append({"step": f"{15 << i}x{20 << i}", "form": rep.level[i].form,
                        "iters_per_launch": rep.level[i].iters_per_launch, "ms_per_iter": ms})
        return out

    def flow(self, k: int):
        r = self.rows[k]
        out = [np.zeros(r * (r * 4 // 3), np.float32) for _ in range(3)]
        check(load().pdflow_read_flow_mixed(self._h, k, *[_ptr(a) for a in out]), "pdflow_read_flow_mixed")
        return out

    def synchronize(self):
        check(load().pdflow_synchronize(self._h), "pdflow_synchronize")

    def close(self):
        if self._h is not None:
            load().pdflow_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Net:
    """The warm-start network (include/pdflow_net.h).  Device buffers are
    passed as integer device addresses (e.g. torch's data_ptr())."""

    def __init__(self, max_batch: int, seed: int = 1):
        h = ctypes.c_void_p()
        check(load().pdflow_net_create(max_batch, seed, ctypes.byref(h)), "pdflow_net_create")
        self._h = h
        self.max_batch = max_batch

    @property
    def handle(self):
        return self._h

    def param_count(self) -> int:
        return int(load().pdflow_net_param_count(self._h))

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        check(load().pdflow_net_get_params(self._h, _ptr(p), p.size), "pdflow_net_get_params")
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        check(load().pdflow_net_set_params(self._h, _ptr(p), p.size), "pdflow_net_set_params")

    def forward(self, n: int, d_input: int, d_output: int):
        check(load().pdflow_net_forward(self._h, n, vp(d_input), vp(d_output)), "pdflow_net_forward")

    def train_step(self, n: int, d_input: int, d_label: int, lr: float) -> float:
        loss = ctypes.c_float()
        check(load().pdflow_net_train_step(self._h, n, vp(d_input), vp(d_label), lr, ctypes.byref(loss)),
              "pdflow_net_train_step")
        return float(loss.value)

    def gradients(self, n: int, d_input: int, d_label: int):
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_float()
        check(load().pdflow_net_gradients(self._h, n, vp(d_input), vp(d_label), _ptr(g), ctypes.byref(loss)),
              "pdflow_net_gradients")
        return float(loss.value), g

    def close(self):
        if self._h is not None:
            load().pdflow_net_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_frames(frames, d_intensity: int, d_depth: int, d_flow: int | None = None, stream: int = 0):
    """Renders SceneFrame descriptors into device buffers (pdflow_render_frames)."""
    arr = (SceneFrame * len(frames))(*frames)
    check(load().pdflow_render_frames(arr, len(frames), vp(d_intensity), vp(d_depth), vp(d_flow or 0), vp(stream)),
          "pdflow_render_frames")


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "warmstart.npz")


def load_weights(path: str | None = None) -> np.ndarray:
    """Parameters of the warm-start network (default: the shipped weights,
    trained by pdflow.train_warmstart on 20 000 synthetic pairs)."""
    with np.load(path or DEFAULT_WEIGHTS) as f:
        return np.asarray(f["params"], np.float32)


def gemm_bf16(M: int, N: int, K: int, d_a: int, lda: int, d_b: int, ldb: int, d_c: int, ldc: int,
              k_per_split: int = 0, stream: int = 0):
    """C = A * B^T on the tcgen05 tensor cores (pdflow_gemm_bf16)."""
    check(load().pdflow_gemm_bf16(M, N, K, vp(d_a), lda, vp(d_b), ldb, vp(d_c), ldc, k_per_split, vp(stream)),
          "pdflow_gemm_bf16")
