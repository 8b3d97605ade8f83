"""bench.py's timing hygiene on the host: the clock summary covers the samples
taken during the timed region, and the cyclic collector is paused inside a
timed loop and restored after it."""
import gc

import bench


def _line(sm, mx, *reasons):
    flags = ["Active" if r else "Not Active" for r in reasons]
    return ", ".join([str(sm), str(mx), "900.0"] + flags)


def test_clock_summary_uses_the_samples_of_the_timed_region():
    s = bench.ClockSampler(0)
    s.proc = None   # no nvidia-smi here: feed the lines directly
    s.lines = [_line(1200, 2070, 0, 0, 1, 0),          # warm-up: thermal slowdown, not timed
               _line(2070, 2070, 0, 0, 0, 0),
               _line(2070, 2070, 0, 0, 0, 1)]

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s.proc = Done()
    out = s.stop(since=1)
    assert out == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 2}


def test_clock_summary_falls_back_to_all_samples():
    s = bench.ClockSampler(0)

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s.proc = Done()
    s.lines = [_line(2070, 2070, 0, 0, 0, 0)]
    assert s.stop(since=5)["samples"] == 1


def test_collector_paused_inside_and_restored_after():
    assert gc.isenabled()
    with bench.paused_gc():
        assert not gc.isenabled()
    assert gc.isenabled()
    gc.disable()
    try:
        with bench.paused_gc():
            assert not gc.isenabled()
        assert not gc.isenabled()   # a collector that was off stays off
    finally:
        gc.enable()
