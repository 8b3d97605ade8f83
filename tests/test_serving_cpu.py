"""Host-side logic of the serving layer, without a GPU: configuration checks of
the C server and the Poisson stream simulator's scheduling and statistics."""
import ctypes

import numpy as np
import pytest

from pdflow import ERR_ARG, PDFlowError
from pdflow import serving


def test_server_rejects_bad_configurations(built_lib):
    with pytest.raises(PDFlowError) as e:
        serving.Server(1 << 30, slots_per_lane=0)
    assert e.value.code == ERR_ARG
    with pytest.raises(PDFlowError) as e:
        serving.Server(1 << 30, slots_per_lane=65)
    assert e.value.code == ERR_ARG
    cfg = serving.ServerConfig()
    cfg.device_budget_bytes, cfg.slots_per_lane, cfg.learned, cfg.iter_scale = 1 << 30, 4, 1, 0.5
    h = ctypes.c_void_p()
    assert built_lib.pdflow_server_create(ctypes.byref(cfg), ctypes.byref(h)) == ERR_ARG   # learned without weights
    srv = serving.Server(1 << 30, slots_per_lane=4)
    with pytest.raises(PDFlowError) as e:
        srv.open_stream(641, 480)
    assert e.value.code == ERR_ARG
    srv.close()


class FakeServer:
    """Completes every request after a fixed service time from its submit."""

    def __init__(self, service_ms=5.0):
        self.t0 = None
        self.service = service_ms
        self.reqs = {}
        self.next = 1
        self.frames = {}
        self.closed = []

    def open_stream(self, w, h):
        sid = len(self.frames)
        self.frames[sid] = 0
        return sid

    def close_stream(self, sid):
        self.closed.append(sid)

    def submit(self, sid, i, z):
        import time
        now = time.perf_counter() * 1e3
        self.t0 = self.t0 if self.t0 is not None else now
        rid = self.next
        self.next += 1
        k = self.frames[sid]
        self.frames[sid] += 1
        t = now - self.t0
        self.reqs[rid] = dict(request_id=rid, stream_id=sid, frame_index=k, status=0, has_flow=int(k > 0),
                              batch_pairs=1, batch_fallbacks=0, submit_ms=t, start_ms=t, done_ms=t + self.service)
        return rid

    def wait(self, rid, sid, timeout_ms=-1, want_flow=True):
        return self.reqs.pop(rid), None

    def stats(self):
        return {"fallbacks": 0}


def test_simulator_submits_every_frame_in_stream_order_and_summarises():
    frames = [(np.zeros((2, 2), np.uint8), np.zeros((2, 2), np.uint16))] * 6
    fake = FakeServer(service_ms=5.0)
    infos, _, summary = serving.simulate(fake, [(2, 2, frames)] * 3, rate_hz=400.0, seed=3)
    assert summary["requests"] == 18 and summary["flows"] == 15           # first frame of each stream: no flow
    per_stream = {}
    for i in infos:
        per_stream.setdefault(i["stream_id"], []).append(i["frame_index"])
    assert all(v == list(range(6)) for v in per_stream.values())
    assert summary["p50_ms"] == pytest.approx(5.0) and summary["p99_ms"] == pytest.approx(5.0)
    assert summary["errors"] == 0 and sorted(fake.closed) == [0, 1, 2]
    # submissions never precede their scheduled arrival; lateness is reported
    assert 0.0 <= summary["arrival_lateness_p99_ms"] <= summary["arrival_lateness_max_ms"]
