"""Host logic of bench.py's end-to-end measurements, on a stand-in engine (no GPU): the
processing loop steps one timestep at a time and then reads every probe's newest sample, in
openEMS's order, and leaves Python's garbage collector as it found it."""
import gc

import bench


class _FakeEngine:
    def __init__(self, vprobes, iprobes):
        self.vprobe_ids = list(vprobes)
        self.iprobe_ids = list(iprobes)
        self.calls = []
        self.ts = 0

    def IterateTS(self, n):
        self.ts += n
        self.calls.append(("iterate", n, gc.isenabled()))

    def probe_range(self, pid, first, count):
        self.calls.append(("read", pid, first, count))
        assert first == self.ts and count == 1      # the sample of the step just run


def test_processing_loop_order_and_slots():
    e = _FakeEngine([0, 1], [2])
    e.ts = 40
    secs = bench.processing_loop(e, 3, 40)
    assert secs >= 0.0
    want = []
    for k in range(41, 44):
        want += [("iterate", 1, False), ("read", 0, k, 1), ("read", 1, k, 1), ("read", 2, k, 1)]
    assert e.calls == want


def test_processing_loop_restores_the_collector():
    assert gc.isenabled()
    bench.processing_loop(_FakeEngine([0], []), 2, 0)
    assert gc.isenabled()
    gc.disable()
    try:
        bench.processing_loop(_FakeEngine([0], []), 2, 0)
        assert not gc.isenabled()                   # was off: stays off
    finally:
        gc.enable()


def test_processing_loop_reenables_after_an_error():
    class Boom(_FakeEngine):
        def probe_range(self, pid, first, count):
            raise RuntimeError("read failed")

    try:
        bench.processing_loop(Boom([0], []), 2, 0)
    except RuntimeError:
        pass
    assert gc.isenabled()
