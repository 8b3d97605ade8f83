"""Python view of the request loop (include/pdflow_server.h) and a simulated
multi-camera workload for it.

`Server` wraps the C server: streams are admitted against a device budget,
frames are submitted as they arrive and results are collected with their
timings.  `simulate` drives a server with camera streams whose frames arrive
as Poisson processes (default 30 Hz each) and reports latency percentiles and
aggregate throughput; for the C server the arrivals come from its native load
generator (pdflow_server_replay: a C++ thread that sleeps until each arrival),
for other servers (tests) from a Python loop.
"""
from __future__ import annotations

import ctypes
import heapq
import time

import numpy as np

from ._lib import (ReplayStream, RequestInfo, ServerConfig, ServerStats, _ptr, check, load)


class Server:
    def __init__(self, device_budget_bytes: int, slots_per_lane: int = 8, learned: bool = False,
                 iter_scale: float = 1.0, energy_margin: float = 0.01, net_params=None):
        cfg = ServerConfig()
        cfg.device_budget_bytes = int(device_budget_bytes)
        cfg.slots_per_lane = slots_per_lane
        cfg.learned = 1 if learned else 0
        cfg.iter_scale = iter_scale
        cfg.energy_margin = energy_margin
        self._params = None
        if learned:
            self._params = np.ascontiguousarray(net_params, np.float32)
            cfg.net_params = self._params.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
            cfg.net_param_count = self._params.size
        h = ctypes.c_void_p()
        check(load().pdflow_server_create(ctypes.byref(cfg), ctypes.byref(h)), "pdflow_server_create")
        self._h = h
        self._shape = {}

    def open_stream(self, width: int, height: int) -> int:
        sid = ctypes.c_uint()
        check(load().pdflow_server_open_stream(self._h, width, height, ctypes.byref(sid)), "pdflow_server_open_stream")
        self._shape[sid.value] = (height, width)
        return sid.value

    def close_stream(self, sid: int):
        check(load().pdflow_server_close_stream(self._h, sid), "pdflow_server_close_stream")

    def submit(self, sid: int, intensity: np.ndarray, depth: np.ndarray) -> int:
        i8 = np.ascontiguousarray(intensity, np.uint8)
        z16 = np.ascontiguousarray(depth, np.uint16)
        if i8.shape != self._shape[sid] or z16.shape != i8.shape:
            raise ValueError("frame size does not match the stream")
        rid = ctypes.c_ulonglong()
        check(load().pdflow_server_submit(self._h, sid, _ptr(i8), _ptr(z16), ctypes.byref(rid)),
              "pdflow_server_submit")
        return rid.value

    def wait(self, rid: int, sid: int, timeout_ms: int = -1, want_flow: bool = True):
        info = RequestInfo()
        h, w = self._shape[sid]
        n = h * (h * 4 // 3)
        flows = [np.zeros(n, np.float32) for _ in range(3)] if want_flow else None
        args = [_ptr(f) for f in flows] if want_flow else [None, None, None]
        check(load().pdflow_server_wait(self._h, rid, timeout_ms, ctypes.byref(info), *args), "pdflow_server_wait")
        d = {k: getattr(info, k) for k, _ in RequestInfo._fields_}
        return d, (flows if (want_flow and info.has_flow) else None)

    def replay(self, sids, streams, rate_hz: float, seed: int):
        """pdflow_server_replay: streams[i] = (width, height, frames) for the
        opened stream sids[i]; returns (infos in submission order, lateness ms)."""
        keep, rs = [], (ReplayStream * len(sids))()
        for i, (sid, (_, _, frames)) in enumerate(zip(sids, streams)):
            h, w = self._shape[sid]
            arrs = [(np.ascontiguousarray(a, np.uint8), np.ascontiguousarray(z, np.uint16)) for a, z in frames]
            if any(a.shape != (h, w) or z.shape != (h, w) for a, z in arrs):
                raise ValueError("frame size does not match the stream")
            ip = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a, _ in arrs])
            dp = (ctypes.c_void_p * len(arrs))(*[z.ctypes.data for _, z in arrs])
            keep += [arrs, ip, dp]
            rs[i] = ReplayStream(sid, len(arrs), ctypes.cast(ip, ctypes.POINTER(ctypes.c_void_p)),
                                 ctypes.cast(dp, ctypes.POINTER(ctypes.c_void_p)))
        total = sum(len(f) for _, _, f in streams)
        infos, late, count = (RequestInfo * total)(), (ctypes.c_double * total)(), ctypes.c_uint()
        check(load().pdflow_server_replay(self._h, rs, len(sids), rate_hz, seed, infos, late, total,
                                          ctypes.byref(count)), "pdflow_server_replay")
        out = [{k: getattr(infos[m], k) for k, _ in RequestInfo._fields_} for m in range(count.value)]
        return out, [late[m] for m in range(count.value)]

    def stats(self) -> dict:
        st = ServerStats()
        check(load().pdflow_server_get_stats(self._h, ctypes.byref(st)), "pdflow_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self._h is not None:
            load().pdflow_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate(server: Server, streams, rate_hz: float = 30.0, seed: int = 0, want_flow: bool = False):
    """streams: list of (width, height, frames) with frames a list of
    (intensity, depth) numpy pairs.  Each stream's frames arrive as a Poisson
    process of rate `rate_hz` (exponential gaps; for a `Server`, generated and
    submitted by its native load generator unless flows are wanted back).
    Returns per-request infos and a summary: p50 / p99 latency of the frames
    that produced a flow, aggregate flows per second over the run, batch
    sizes, and how late the submissions ran against their scheduled arrival
    times (a late load generator bunches arrivals into bursts)."""
    sids = [server.open_stream(w, h) for w, h, _ in streams]
    t0 = time.perf_counter()
    if isinstance(server, Server) and not want_flow:
        infos, late = server.replay(sids, streams, rate_hz, seed)
        outs = [None] * len(infos)
    else:
        rng = np.random.default_rng(seed)
        heap = []
        for j, (_, _, frames) in enumerate(streams):
            heapq.heappush(heap, (rng.exponential(1.0 / rate_hz), j, 0))
        pending, late = [], []
        while heap:
            t_arr, j, k = heapq.heappop(heap)
            now = time.perf_counter() - t0
            if t_arr > now:
                time.sleep(t_arr - now)
            late.append((time.perf_counter() - t0 - t_arr) * 1e3)
            frames = streams[j][2]
            rid = server.submit(sids[j], *frames[k])
            pending.append((rid, sids[j]))
            if k + 1 < len(frames):
                heapq.heappush(heap, (t_arr + rng.exponential(1.0 / rate_hz), j, k + 1))
        infos, outs = [], []
        for rid, sid in pending:
            info, flow = server.wait(rid, sid, want_flow=want_flow)
            infos.append(info)
            outs.append(flow)
    wall = time.perf_counter() - t0
    lat = np.array([i["done_ms"] - i["submit_ms"] for i in infos if i["has_flow"]])
    flows = int(sum(1 for i in infos if i["has_flow"]))
    span_ms = max(i["done_ms"] for i in infos) - min(i["submit_ms"] for i in infos)
    summary = dict(streams=len(streams), rate_hz=rate_hz, requests=len(infos), flows=flows,
                   p50_ms=float(np.percentile(lat, 50)) if lat.size else None,
                   p99_ms=float(np.percentile(lat, 99)) if lat.size else None,
                   mean_ms=float(lat.mean()) if lat.size else None,
                   flows_per_s=flows / (span_ms / 1e3) if span_ms > 0 else None,
                   mean_batch_pairs=float(np.mean([i["batch_pairs"] for i in infos if i["has_flow"]])) if flows else 0,
                   wall_s=wall, errors=int(sum(1 for i in infos if i["status"] != 0)),
                   arrival_lateness_p99_ms=float(np.percentile(late, 99)) if late else None,
                   submit_span_ms=max(i["submit_ms"] for i in infos) - min(i["submit_ms"] for i in infos),
                   drain_ms=max(i["done_ms"] for i in infos) - max(i["submit_ms"] for i in infos),
                   arrival_lateness_max_ms=float(max(late)) if late else None,
                   fallbacks=int(server.stats()["fallbacks"]))
    for sid in sids:
        server.close_stream(sid)
    return infos, outs, summary
