"""Serving form: a continuous-batching PIV request loop on one GPU.

Frame pairs of different sizes arrive over time. Each frame size has a lane:
a ``PIVGPU`` configuration and up to ``slots_per_shape`` plans, each with its
own CUDA stream and pinned staging buffers, whose device workspaces (frames,
deformed frames, predictor fields, spline coefficients) stay resident. A
request waits in its lane's queue until a slot of the lane is free; the slot
then takes every waiting request of its size up to ``max_batch`` (continuous
batching), uploads them and runs the whole multi-pass pipeline
asynchronously, and the loop goes on admitting and dispatching while it runs,
so that work of several sizes and batches overlaps on the device. A lane is
only created when the free device memory, less ``hbm_reserve``, holds its
plans; otherwise its requests wait, and idle lanes are released oldest first
to make room.

Each request's result equals the result of processing the pair alone
(``tests/test_gpu_serving.py``): a plan run treats the pairs of a batch
independently.
"""

import collections
import time

import numpy as np

from . import _lib
from .gpu_process import PIVGPU, _torch

__all__ = ["PIVServer", "Request"]


class Request:
    """One frame pair: arrival time, and after completion its fields and times."""

    __slots__ = ("rid", "frame_a", "frame_b", "t_arrival", "t_dispatch", "t_done", "u", "v")

    def __init__(self, rid, frame_a, frame_b, t_arrival):
        self.rid = rid
        self.frame_a = frame_a
        self.frame_b = frame_b
        self.t_arrival = t_arrival
        self.t_dispatch = None
        self.t_done = None
        self.u = None
        self.v = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_arrival


class _Slot:
    def __init__(self, lane, index):
        torch = _torch()
        self.lane = lane
        self.index = index
        self.stream = torch.cuda.Stream()
        self.event = torch.cuda.Event()
        self.t_start = None  # timing events of the batch in flight (device interval)
        self.t_end = None
        self.batch = []
        self.inputs = None
        self.outputs = None

    def busy(self):
        return bool(self.batch)


class _Lane:
    def __init__(self, shape, settings, max_batch, slots, dft):
        self.shape = shape
        kw = dict(settings)
        mss = kw.pop("min_search_size")
        self.proc = PIVGPU(shape, mss, dft=dft, **kw)
        self.max_batch = max_batch
        self.slots = [_Slot(self, k) for k in range(slots)]
        self.queue = collections.deque()
        self.last_used = time.perf_counter()
        m, n = self.proc.piv_fields[-1].field_shape
        torch = _torch()
        for s in self.slots:
            s.inputs = tuple(torch.empty((max_batch,) + shape, dtype=torch.uint8, pin_memory=True) for _ in range(2))
            s.outputs = tuple(torch.empty((max_batch, m, n), dtype=dt, pin_memory=True)
                              for dt in (torch.float64, torch.float64, torch.uint8, torch.uint8))
            self.proc._plan(_lib.PIXEL["u8"], max_batch, slot=s.index)

    def release(self):
        lib = _lib.lib()
        for plan, _ in self.proc._plans.values():
            lib.piv_plan_destroy(plan)
        self.proc._plans.clear()


class PIVServer:
    """Continuous-batching request loop.

    ``settings`` are PIVGPU keyword arguments (``min_search_size`` included);
    frames are 2-D uint8 arrays. ``submit`` queues a pair, ``step`` admits,
    dispatches and collects without blocking, ``drain`` runs until every
    submitted request is done.
    """

    def __init__(self, settings, max_batch=8, slots_per_shape=2, hbm_reserve=2 << 30, dft="tensor"):
        self.settings = dict(settings)
        self.max_batch = int(max_batch)
        self.slots_per_shape = int(slots_per_shape)
        self.hbm_reserve = int(hbm_reserve)
        self.dft = dft
        self.lanes = {}
        self.waiting = collections.deque()   # requests whose lane does not exist yet
        self.done = []
        self._next_id = 0
        self._lane_bytes = {}
        # Evidence of continuous batching: the most batches in flight at
        # once, the requests held back for lack of device memory, and each
        # batch's device interval (ms after the server's reference event).
        self.max_in_flight = 0
        self.held_for_memory = 0
        self.intervals = []
        torch = _torch()
        self._t0 = torch.cuda.Event(enable_timing=True)
        self._t0.record()

    # -- requests ----------------------------------------------------------
    def submit(self, frame_a, frame_b, t_arrival=None):
        frame_a = np.asarray(frame_a)
        frame_b = np.asarray(frame_b)
        assert frame_a.shape == frame_b.shape and frame_a.ndim == 2, "a pair of equally sized 2-D frames"
        assert frame_a.dtype == np.uint8 and frame_b.dtype == np.uint8, "8-bit frames"
        req = Request(self._next_id, frame_a, frame_b, time.perf_counter() if t_arrival is None else t_arrival)
        self._next_id += 1
        lane = self.lanes.get(frame_a.shape)
        (lane.queue if lane is not None else self.waiting).append(req)
        return req

    # -- loop --------------------------------------------------------------
    def step(self):
        """One non-blocking pass: collect finished slots, admit waiting
        requests whose lane fits in memory, dispatch to free slots. Returns
        the number of requests that finished."""
        finished = self._collect()
        self._admit()
        self._dispatch()
        return finished

    def busy(self):
        return bool(self.waiting) or any(l.queue or any(s.busy() for s in l.slots) for l in self.lanes.values())

    def drain(self, poll_interval=0.0):
        while self.busy():
            if not self.step():
                if poll_interval:
                    time.sleep(poll_interval)
        return self.done

    def close(self):
        """Finishes every submitted request, then releases every lane's plans
        and device workspaces."""
        self.drain()
        for lane in self.lanes.values():
            lane.release()
        self.lanes.clear()

    # -- internals ---------------------------------------------------------
    def _collect(self):
        count = 0
        for lane in self.lanes.values():
            for s in lane.slots:
                if s.busy() and s.event.query():
                    now = time.perf_counter()
                    self.intervals.append((lane.shape, self._t0.elapsed_time(s.t_start),
                                           self._t0.elapsed_time(s.t_end)))
                    u, v = s.outputs[0], s.outputs[1]
                    for k, req in enumerate(s.batch):
                        req.u = u[k].numpy().copy()
                        req.v = v[k].numpy().copy()
                        req.t_done = now
                        req.frame_a = req.frame_b = None
                        self.done.append(req)
                    count += len(s.batch)
                    s.batch = []
                    lane.last_used = now
        return count

    def _estimate(self, shape):
        if shape not in self._lane_bytes:
            ht, wd = shape
            # 8-bit frames, float32 deformed frames and spline coefficients
            # (two frames each) per pair and slot, with a margin for fields.
            self._lane_bytes[shape] = int(1.25 * self.slots_per_shape * self.max_batch * ht * wd * (2 + 8 + 8))
        return self._lane_bytes[shape]

    def _admit(self):
        if not self.waiting:
            return
        torch = _torch()
        kept = collections.deque()
        while self.waiting:
            req = self.waiting.popleft()
            shape = req.frame_a.shape
            lane = self.lanes.get(shape)
            if lane is None:
                need = self._estimate(shape)
                free, _ = torch.cuda.mem_get_info()
                while free - need < self.hbm_reserve and self._evict_idle(exclude=shape):
                    free, _ = torch.cuda.mem_get_info()
                if free - need < self.hbm_reserve:
                    kept.append(req)
                    self.held_for_memory += 1
                    continue
                lane = _Lane(shape, self.settings, self.max_batch, self.slots_per_shape, self.dft)
                self.lanes[shape] = lane
            lane.queue.append(req)
        self.waiting = kept

    def _evict_idle(self, exclude):
        idle = [l for sh, l in self.lanes.items()
                if sh != exclude and not l.queue and not any(s.busy() for s in l.slots)]
        if not idle:
            return False
        lane = min(idle, key=lambda l: l.last_used)
        lane.release()
        del self.lanes[lane.shape]
        return True

    def _dispatch(self):
        lib = _lib.lib()
        for lane in self.lanes.values():
            for s in lane.slots:
                if not lane.queue:
                    break
                if s.busy():
                    continue
                batch = [lane.queue.popleft() for _ in range(min(self.max_batch, len(lane.queue)))]
                now = time.perf_counter()
                ia, ib = (t.numpy() for t in s.inputs)
                for k, req in enumerate(batch):
                    ia[k] = req.frame_a
                    ib[k] = req.frame_b
                    req.t_dispatch = now
                plan = lane.proc._plan(_lib.PIXEL["u8"], self.max_batch, slot=s.index)
                u, v, val, out = s.outputs
                torch = _torch()
                s.t_start = torch.cuda.Event(enable_timing=True)
                s.t_end = torch.cuda.Event(enable_timing=True)
                s.t_start.record(s.stream)
                _lib.check(lib.piv_plan_run(plan, len(batch), ia.ctypes.data, ib.ctypes.data, 1, u.data_ptr(),
                                            v.data_ptr(), val.data_ptr(), out.data_ptr(), 2, s.stream.cuda_stream))
                s.t_end.record(s.stream)
                s.event.record(s.stream)
                s.batch = batch
                lane.last_used = now
        in_flight = sum(s.busy() for lane in self.lanes.values() for s in lane.slots)
        self.max_in_flight = max(self.max_in_flight, in_flight)

    # -- reporting ---------------------------------------------------------
    def overlapping_batches(self):
        """Pairs of completed batches whose device intervals (first to last
        operation of the run on its slot's stream) overlap in time."""
        iv = sorted(self.intervals, key=lambda t: t[1])
        count = 0
        for i in range(len(iv)):
            for j in range(i + 1, len(iv)):
                if iv[j][1] >= iv[i][2]:
                    break
                count += 1
        return count

    def latency_stats(self):
        lat = np.array([r.latency for r in self.done if r.latency is not None])
        if lat.size == 0:
            return {}
        return {"count": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3)}


def serve_arrivals(server, frames, arrivals, poll_interval=0.0):
    """Feeds ``frames[k]`` (a pair) at wall-clock offset ``arrivals[k]``
    seconds from the call while running the loop; returns (requests, seconds)."""
    t0 = time.perf_counter()
    k = 0
    while k < len(arrivals) or server.busy():
        now = time.perf_counter() - t0
        while k < len(arrivals) and arrivals[k] <= now:
            server.submit(frames[k][0], frames[k][1], t_arrival=t0 + arrivals[k])
            k += 1
        if not server.step() and poll_interval:
            time.sleep(poll_interval)
    return server.done, time.perf_counter() - t0
