"""The request loop: admission by device budget, continuous batching across
lanes, and results that do not depend on what else is in flight."""
import numpy as np
import pytest

from oracle import net_oracle as no
from pdflow import ERR_OOM, PDFlowError, Solver, scenes
from pdflow.serving import Server

pytestmark = pytest.mark.gpu


def stream_frames(seed, vga, n, nobj=3):
    sc = scenes.make_scene(seed, vga, nobj)
    return [scenes.render(sc, k) for k in range(n)]


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def solve_alone(server_kw, frames, vga):
    srv = Server(**server_kw)
    w, h = (640, 480) if vga else (320, 240)
    sid = srv.open_stream(w, h)
    rids = [srv.submit(sid, *f) for f in frames]
    out = [srv.wait(r, sid) for r in rids]
    srv.close()
    return out


@pytest.mark.parametrize("learned", [False, True])
def test_each_result_is_the_same_alone_and_in_the_mix(built_lib, learned):
    kw = dict(device_budget_bytes=64 << 30, slots_per_lane=3)
    if learned:
        kw.update(learned=True, iter_scale=0.5, energy_margin=0.01, net_params=no.init_params(5))
    target = stream_frames(301, False, 3)
    alone = solve_alone(kw, target, False)
    assert alone[0][1] is None and alone[0][0]["has_flow"] == 0     # first frame: nothing to pair with
    # the same stream among four others (QVGA and VGA), frames interleaved
    others = [(stream_frames(310 + j, j % 2 == 1, 3, 2 + j), j % 2 == 1) for j in range(4)]
    srv = Server(**kw)
    sid = srv.open_stream(320, 240)
    osids = [srv.open_stream(*((640, 480) if v else (320, 240))) for _, v in others]
    rids = []
    for k in range(3):
        for (fr, _), os_ in zip(others, osids):
            srv.submit(os_, *fr[k])
        rids.append(srv.submit(sid, *target[k]))
    mixed = [srv.wait(r, sid) for r in rids]
    st = srv.stats()
    srv.close()
    assert st["lanes"] >= 2 and st["streams"] == 5
    for (ia, fa), (ib, fb) in zip(alone, mixed):
        assert ia["has_flow"] == ib["has_flow"] and ia["status"] == ib["status"] == 0
        if fa is not None:
            for x, y in zip(fa, fb):
                assert np.array_equal(bits(x), bits(y))
    if not learned:   # the plain path equals a direct single-pair solve
        for k in (1, 2):
            s = Solver(240, 320, 240).initializeCUDA()
            s.loadRGBDFrames(*target[k - 1], *target[k])
            s.solveSceneFlowGPU()
            for x, y in zip(mixed[k][1], (s.dxp, s.dyp, s.dzp)):
                assert np.array_equal(bits(x), bits(y))
            s.freeGPUMemory()


def test_admission_is_bounded_by_the_device_budget(built_lib):
    probe = Server(device_budget_bytes=64 << 30, slots_per_lane=2)
    probe.open_stream(320, 240)
    lane_bytes = probe.stats()["device_bytes"]
    probe.close()
    srv = Server(device_budget_bytes=int(lane_bytes * 1.5), slots_per_lane=2)
    srv.open_stream(320, 240)
    srv.open_stream(320, 240)                 # second slot of the first lane
    with pytest.raises(PDFlowError) as e:
        srv.open_stream(320, 240)             # would need a second lane
    assert e.value.code == ERR_OOM
    srv.close()


def test_native_replay_submits_every_frame_on_schedule(built_lib):
    """pdflow_server_replay: the native load generator submits each stream's
    frames in order at Poisson arrival times and returns every request."""
    from pdflow.serving import simulate
    srv = Server(device_budget_bytes=64 << 30, slots_per_lane=4)
    streams = [(320, 240, stream_frames(400 + j, False, 5)) for j in range(3)] + \
              [(640, 480, stream_frames(410, True, 4))]
    infos, _, summary = simulate(srv, streams, rate_hz=60.0, seed=7)
    srv.close()
    assert summary["requests"] == 19 and summary["flows"] == 15 and summary["errors"] == 0
    per_stream = {}
    for i in infos:
        per_stream.setdefault(i["stream_id"], []).append(i["frame_index"])
    assert sorted(len(v) for v in per_stream.values()) == [4, 5, 5, 5]
    assert all(v == list(range(len(v))) for v in per_stream.values())
    assert all(i["done_ms"] >= i["start_ms"] >= i["submit_ms"] for i in infos)
    assert summary["arrival_lateness_p99_ms"] < 50.0
