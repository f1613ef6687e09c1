"""Batched form: one submission of many pairs of uneven frame sizes.

Pairs are grouped by frame size. Each group runs the whole multi-pass
pipeline for all of its pairs in one plan run (one launch per stage and pass
over every window of the group's pairs), the groups run on their own CUDA
streams so that they overlap on the device, and the submission (fork, the
groups' runs, join) is captured once as a single CUDA graph and replayed.
Results come back per pair, in submission order.
"""

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
        self.plan = self.proc._plan(_lib.PIXEL["u8"], B)
        self.stream = torch.cuda.Stream()
        self.done = torch.cuda.Event()

    def launch(self, stream):
        B = len(self.indices)
        _lib.check(_lib.lib().piv_plan_run(self.plan, B, self.fa.data_ptr(), self.fb.data_ptr(), 0,
                                           self.u.data_ptr(), self.v.data_ptr(), self.val.data_ptr(),
                                           self.out.data_ptr(), 0, stream.cuda_stream))


class PIVMixedBatch:
    """Runs a fixed layout of mixed-size 8-bit pairs as one graph replay.

    ``shapes`` lists the frame size of every pair of a submission (the layout
    is fixed at construction); ``settings`` are PIVGPU keyword arguments
    (``min_search_size`` included). ``load(pairs)`` copies a submission's
    frames to the device, ``run()`` replays the captured graph, ``results()``
    returns [(u, v)] per pair as NumPy arrays in submission order.
    """

    def __init__(self, shapes, settings, dft="tensor"):
        torch = _torch()
        self.shapes = [tuple(s) for s in shapes]
        order = {}
        for k, s in enumerate(self.shapes):
            order.setdefault(s, []).append(k)
        self.groups = [_Group(s, idx, settings, dft) for s, idx in order.items()]
        self.stream = torch.cuda.Stream()
        self.fork = torch.cuda.Event()
        self.graph = None

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

    def _submit(self):
        self.fork.record(self.stream)
        for g in self.groups:
            g.stream.wait_event(self.fork)
            g.launch(g.stream)
            g.done.record(g.stream)
        for g in self.groups:
            self.stream.wait_event(g.done)

    def capture(self):
        """Runs once directly (plans allocate and configure their kernels), then
        captures the submission as one CUDA graph."""
        torch = _torch()
        with torch.cuda.stream(self.stream):
            self._submit()
        self.stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._submit()
        torch.cuda.synchronize()

    def run(self):
        torch = _torch()
        if self.graph is None:
            with torch.cuda.stream(self.stream):
                self._submit()
        else:
            with torch.cuda.stream(self.stream):
                self.graph.replay()

    def results(self):
        self.stream.synchronize()
        out = [None] * len(self.shapes)
        for g in self.groups:
            u, v = g.u.cpu().numpy(), g.v.cpu().numpy()
            for j, k in enumerate(g.indices):
                out[k] = (u[j], v[j])
        return out
