"""Host logic of the continuous-batching request loop (openpiv_gpu.serving) on
CPU: the device, its memory and the plan runs are faked, so the policy itself
is checked. Requests of one frame size are batched up to max_batch per slot
and dispatched while other batches are in flight; results reach the request
they belong to; a lane is created only when free memory less the reserve
holds it; an idle lane is released (oldest first) to make room, a busy one
never is; requests held for memory go through once room is made."""

import itertools
import types

import numpy as np
import pytest

from openpiv_gpu import serving


class _Device:
    """Fake clock, memory and streams: every event query advances the clock
    by one tick; a plan run occupies its stream for `latency` ticks after
    the stream's previous work, and an event recorded on a stream completes
    when the stream's work before it has."""

    def __init__(self, free, latency=3):
        self.tick = 0
        self.free = free
        self.latency = latency
        self.streams = {}

    def stream(self):
        st = types.SimpleNamespace(cuda_stream=len(self.streams) + 1, end=0)
        self.streams[st.cuda_stream] = st
        return st


class _Event:
    def __init__(self, dev):
        self.dev = dev
        self.at = None

    def record(self, stream=None):
        self.at = self.dev.tick if stream is None else max(self.dev.tick, stream.end)

    def query(self):
        self.dev.tick += 1
        return self.at is not None and self.dev.tick >= self.at

    def elapsed_time(self, end):
        return float(end.at - self.at)


class _Tensor:
    """A host buffer with the two torch methods the loop uses."""

    def __init__(self, array, registry):
        self.array = array
        registry[array.ctypes.data] = array

    def numpy(self):
        return self.array

    def data_ptr(self):
        return self.array.ctypes.data

    def __getitem__(self, k):
        return _Tensor(self.array[k], {})


def _fake_torch(dev):
    cuda = types.SimpleNamespace(
        Event=lambda enable_timing=False: _Event(dev),
        Stream=dev.stream,
        mem_get_info=lambda: (dev.free, 1 << 40),
    )
    return types.SimpleNamespace(cuda=cuda)


class _Plan:
    def __init__(self, lane):
        self.lane = lane


def _lane_estimate(shape, slots=1, max_batch=2):
    """The loop's device-memory estimate of a lane: 8-bit frames, float32
    deformed frames and spline coefficients (two frames each) per pair and
    slot, with a 25% margin."""
    return int(1.25 * slots * max_batch * shape[0] * shape[1] * (2 + 8 + 8))


def _install(monkeypatch, dev, lane_bytes=_lane_estimate):
    buffers = {}
    runs = []
    lanes = []

    class Lane:
        def __init__(self, shape, settings, max_batch, slots, dft):
            self.shape = shape
            self.max_batch = max_batch
            self.slots = [serving._Slot(self, k) for k in range(slots)]
            self.queue = serving.collections.deque()
            self.last_used = len(lanes)
            self.released = False
            for s in self.slots:
                s.inputs = tuple(_Tensor(np.zeros((max_batch,) + shape, np.uint8), buffers) for _ in range(2))
                s.outputs = tuple(_Tensor(np.zeros((max_batch, 2, 2), dt), buffers)
                                  for dt in (np.float64, np.float64, np.uint8, np.uint8))
            self.proc = types.SimpleNamespace(_plan=lambda pixel, n, slot=0: _Plan(self))
            self.bytes = lane_bytes(shape)
            dev.free -= self.bytes
            lanes.append(self)

        def release(self):
            self.released = True
            dev.free += self.bytes

    def run(plan, n, pa, pb, on_host, pu, pv, pval, pout, outputs_on_host, stream):
        a, u, v = buffers[pa], buffers[pu], buffers[pv]
        for k in range(n):  # a request's "field" is its frame's constant value
            u[k] = a[k].mean()
            v[k] = -a[k].mean()
        st = dev.streams[stream]
        st.end = max(dev.tick, st.end) + dev.latency
        runs.append((plan.lane.shape, n))
        return 0

    fake_lib = types.SimpleNamespace(lib=lambda: types.SimpleNamespace(piv_plan_run=run),
                                     check=lambda rc: rc, PIXEL={"u8": 0})
    monkeypatch.setattr(serving, "_torch", lambda: _fake_torch(dev))
    monkeypatch.setattr(serving, "_lib", fake_lib)
    monkeypatch.setattr(serving, "_Lane", Lane)
    return runs, lanes


def _pair(shape, value):
    f = np.full(shape, value, np.uint8)
    return f, f


def test_batches_overlap_and_results_reach_their_requests(monkeypatch):
    dev = _Device(free=1 << 40)
    runs, lanes = _install(monkeypatch, dev, lane_bytes=lambda shape: 1 << 20)
    server = serving.PIVServer({"min_search_size": 16}, max_batch=3, slots_per_shape=2, hbm_reserve=0)
    reqs = [server.submit(*_pair((32, 48), 10 + k)) for k in range(7)]
    reqs += [server.submit(*_pair((40, 40), 100 + k)) for k in range(2)]
    done = server.drain()
    assert len(done) == 9 and all(r.u is not None for r in reqs)
    for r, value in zip(reqs, itertools.chain(range(10, 17), range(100, 102))):
        assert np.all(r.u == value) and np.all(r.v == -value)
        assert r.frame_a is None and r.t_done >= r.t_dispatch >= r.t_arrival
    assert all(n <= 3 for _, n in runs)
    assert sum(n for shape, n in runs if shape == (32, 48)) == 7
    assert [n for shape, n in runs if shape == (32, 48)][:2] == [3, 3]  # both slots took full batches
    assert server.max_in_flight >= 2 and server.overlapping_batches() >= 1
    assert len(lanes) == 2 and server.latency_stats()["count"] == 9
    server.close()
    assert all(l.released for l in lanes) and not server.lanes


def test_admission_waits_for_memory_and_evicts_idle_lanes_oldest_first(monkeypatch):
    est = _lane_estimate
    # Room for the first two lanes plus a spare that holds no third lane.
    dev = _Device(free=1000 + est((32, 32)) + est((32, 33)) + 6000)
    runs, lanes = _install(monkeypatch, dev)
    server = serving.PIVServer({"min_search_size": 16}, max_batch=2, slots_per_shape=1, hbm_reserve=1000)
    assert all(server._estimate(sh) == est(sh) for sh in ((32, 32), (32, 33), (33, 32), (34, 34)))

    a = server.submit(*_pair((32, 32), 1))
    server.step()
    c = server.submit(*_pair((32, 33), 3))
    server.step()
    assert set(server.lanes) == {(32, 32), (32, 33)}
    server.drain()
    assert np.all(a.u == 1) and np.all(c.u == 3)

    # A third size: no room; both lanes are idle, the older one goes.
    d = server.submit(*_pair((33, 32), 4))
    server.step()
    assert lanes[0].released and not lanes[1].released
    assert set(server.lanes) == {(32, 33), (33, 32)}
    server.drain()
    assert np.all(d.u == 4)

    # A fourth size while both lanes are busy: held, nothing is evicted.
    e = server.submit(*_pair((32, 33), 5))
    f = server.submit(*_pair((33, 32), 6))
    server.step()
    g = server.submit(*_pair((34, 34), 7))
    server.step()
    assert server.held_for_memory >= 1 and (34, 34) not in server.lanes and g.u is None
    assert not lanes[1].released and not lanes[2].released
    # Once they finish and go idle, the held request evicts one (the spare
    # and one lane hold it) and runs.
    done = server.drain()
    assert np.all(g.u == 7) and {e, f, g} <= set(done)
    assert (34, 34) in server.lanes and sum(l.released for l in lanes) == 2 and len(server.lanes) == 2


@pytest.mark.parametrize("intervals,expected", [
    ([((1, 1), 0.0, 2.0), ((1, 1), 1.0, 3.0), ((1, 1), 2.5, 4.0)], 2),
    ([((1, 1), 0.0, 1.0), ((1, 1), 1.0, 2.0)], 0),
    ([((1, 1), 0.0, 10.0), ((1, 1), 1.0, 2.0), ((1, 1), 3.0, 4.0)], 2),
])
def test_overlapping_batches(monkeypatch, intervals, expected):
    dev = _Device(free=1 << 40)
    _install(monkeypatch, dev)
    server = serving.PIVServer({"min_search_size": 16})
    server.intervals = list(intervals)
    assert server.overlapping_batches() == expected
