"""Batched form: one submission of many pairs of uneven frame sizes.

Pairs are grouped by frame size; the groups run under one ``piv_batch``
(``include/piv_gb300.h``): each group has its own plan and CUDA stream for its
per-field stages (predictor, deformation, validation, replacement,
smoothing), and every pass on a tensor engine runs ONE correlation launch over
the windows of every pair of every size (a segment table of the sizes travels
in the kernel parameters). The submission is captured once as a CUDA graph and
replayed. Results come back per pair, in submission order, and equal the
pair's single-pair result.
"""

import ctypes

import numpy as np

from . import _lib
from .gpu_process import PIVGPU, _torch

__all__ = ["PIVMixedBatch"]


class _Group:
    def __init__(self, shape, indices, settings, dft):
        torch = _torch()
        kw = dict(settings)
        mss = kw.pop("min_search_size")
        self.shape = shape
        self.indices = list(indices)
        self.proc = PIVGPU(shape, mss, dft=dft, **kw)
        B = len(self.indices)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.fa = torch.empty((B,) + shape, dtype=torch.uint8, device=dev)
        self.fb = torch.empty_like(self.fa)
        m, n = self.proc.piv_fields[-1].field_shape
        self.u = torch.empty((B, m, n), dtype=torch.float64, device=dev)
        self.v = torch.empty_like(self.u)
        self.val = torch.empty((B, m, n), dtype=torch.uint8, device=dev)
        self.out = torch.empty_like(self.val)

    def config(self):
        """The group's piv_config (keeps its iteration array alive on self)."""
        cfg, self._keep = self.proc._config(_lib.PIXEL["u8"], len(self.indices))
        return cfg


class PIVMixedBatch:
    """Runs a fixed layout of mixed-size 8-bit pairs as one graph replay.

    ``shapes`` lists the frame size of every pair of a submission (the layout
    is fixed at construction); ``settings`` are PIVGPU keyword arguments
    (``min_search_size`` included). ``load(pairs)`` copies a submission's
    frames to the device, ``run()`` replays the captured graph, ``results()``
    returns [(u, v)] per pair as NumPy arrays in submission order.

    ``schedule``: "joint" (one correlation launch per pass over every size),
    "streams" (each size on its own stream throughout) or "auto" (``capture``
    times both graphs on the loaded frames and keeps the faster one; the
    choice is in ``self.schedule``).
    """

    def __init__(self, shapes, settings, dft="tensor", schedule="auto"):
        if schedule not in ("auto", "joint", "streams"):
            raise ValueError(f"schedule must be 'auto', 'joint' or 'streams', not {schedule!r}")
        self.schedule = schedule
        self.schedule_ms = {}
        torch = _torch()
        self.shapes = [tuple(s) for s in shapes]
        order = {}
        for k, s in enumerate(self.shapes):
            order.setdefault(s, []).append(k)
        self.groups = [_Group(s, idx, settings, dft) for s, idx in order.items()]
        G = len(self.groups)
        cfgs = (_lib.PivConfig * G)(*[g.config() for g in self.groups])
        self.batch = ctypes.c_void_p()
        _lib.check(_lib.lib().piv_batch_create(cfgs, G, ctypes.byref(self.batch)))
        ptrs = lambda name: (ctypes.c_void_p * G)(*[getattr(g, name).data_ptr() for g in self.groups])
        self._args = ((ctypes.c_int * G)(*[len(g.indices) for g in self.groups]), ptrs("fa"), ptrs("fb"),
                      ptrs("u"), ptrs("v"), ptrs("val"), ptrs("out"))
        self.stream = torch.cuda.Stream()
        self.graph = False
        self.kernel_nodes = None

    def __del__(self):
        try:
            _lib.lib().piv_batch_destroy(self.batch)
        except Exception:
            pass

    @property
    def windows(self):
        """Interrogation windows per submission, summed over the passes."""
        return sum(len(g.indices) * sum(f.n_wins for f in g.proc.piv_fields) for g in self.groups)

    def load(self, pairs):
        torch = _torch()
        assert len(pairs) == len(self.shapes)
        with torch.cuda.stream(self.stream):
            for g in self.groups:
                fa = np.stack([pairs[k][0] for k in g.indices])
                fb = np.stack([pairs[k][1] for k in g.indices])
                assert fa.shape[1:] == g.shape and fa.dtype == np.uint8
                g.fa.copy_(torch.from_numpy(fa), non_blocking=False)
                g.fb.copy_(torch.from_numpy(fb), non_blocking=False)
        self.stream.synchronize()

    def _capture(self, joint):
        lib = _lib.lib()
        _lib.check(lib.piv_batch_set_schedule(self.batch, int(joint)))
        _lib.check(lib.piv_batch_run(self.batch, *self._args, self.stream.cuda_stream))
        self.stream.synchronize()
        nk = ctypes.c_int(0)
        _lib.check(lib.piv_batch_graph_capture(self.batch, *self._args, ctypes.byref(nk), self.stream.cuda_stream))
        self.kernel_nodes = nk.value
        self.graph = True

    def _time(self, reps=3):
        torch = _torch()
        self.run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        for _ in range(reps):
            self.run()
        e1.record(self.stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def capture(self):
        """Runs once directly (plans configure their kernels), then captures the
        submission as one CUDA graph (with schedule "auto", both schedules are
        captured and timed and the faster one is kept)."""
        if self.schedule != "auto":
            self._capture(self.schedule == "joint")
            return
        for name in ("streams", "joint"):
            self._capture(name == "joint")
            self.schedule_ms[name] = self._time()
        best = min(self.schedule_ms, key=self.schedule_ms.get)
        if best != "joint":
            self._capture(False)
        self.schedule = best

    def run(self):
        lib = _lib.lib()
        if self.graph:
            _lib.check(lib.piv_batch_graph_launch(self.batch, self.stream.cuda_stream))
        else:
            _lib.check(lib.piv_batch_run(self.batch, *self._args, self.stream.cuda_stream))

    def status(self):
        st = ctypes.c_int(0)
        _lib.check(_lib.lib().piv_batch_status(self.batch, ctypes.byref(st), self.stream.cuda_stream))
        return st.value

    def results(self):
        self.stream.synchronize()
        out = [None] * len(self.shapes)
        for g in self.groups:
            u, v = g.u.cpu().numpy(), g.v.cpu().numpy()
            for j, k in enumerate(g.indices):
                out[k] = (u[j], v[j])
        return out
