"""Serving form: requests of mixed frame sizes go through the continuous-
batching loop, and every request's result equals the result of processing its
pair alone (bit for bit: a plan run treats the pairs of a batch independently).
The loop is continuous batching, not a queue: several batches are in flight at
once and their device intervals overlap; a request whose frame size has no
room in device memory (less the reserve) is held back until room is made."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dft", ["tensor", "tensor_refined"])
def test_results_same_alone_and_in_the_mix(dft):
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.gpu_process import PIVGPU
    from openpiv_gpu.serving import PIVServer

    _build.build()
    torch.cuda.set_device(0)
    settings = dict(synthetic.CONFIGS[5]["piv"])
    shapes = [(96, 128), (128, 160), (160, 96)]
    pairs = [synthetic.config_case(5, k, shape=shapes[k % 3])[:2] for k in range(11)]
    server = PIVServer(settings, max_batch=3, slots_per_shape=2, hbm_reserve=0, dft=dft)
    reqs = []
    for k, (a, b) in enumerate(pairs):
        reqs.append(server.submit(a, b))
        if k % 4 == 3:
            server.step()  # later requests arrive while earlier ones run
    done = server.drain()
    assert len(done) == len(pairs)
    assert server.max_in_flight >= 2, "never more than one batch in flight"
    assert server.overlapping_batches() >= 1, f"no two batches overlapped on the device: {server.intervals}"
    stats = server.latency_stats()
    assert stats["count"] == len(pairs) and stats["p99_ms"] >= stats["p50_ms"] > 0
    kw = dict(settings)
    mss = kw.pop("min_search_size")
    for req, (a, b) in zip(reqs, pairs):
        alone = PIVGPU(a.shape, mss, dft=dft, **kw)
        u, v = alone.run_batch(a[None], b[None], host_out=True)
        np.testing.assert_array_equal(req.u, u[0])
        np.testing.assert_array_equal(req.v, v[0])
    server.close()
    assert not server.lanes


def test_admission_waits_for_device_memory():
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.serving import PIVServer

    _build.build()
    torch.cuda.set_device(0)
    settings = dict(synthetic.CONFIGS[5]["piv"])
    a, b = synthetic.config_case(5, 0, shape=(96, 128))[:2]
    free, _ = torch.cuda.mem_get_info()
    server = PIVServer(settings, max_batch=2, slots_per_shape=1, hbm_reserve=free + (1 << 30))
    req = server.submit(a, b)
    for _ in range(3):
        server.step()
    assert server.held_for_memory >= 1 and not server.lanes and req.u is None, "admitted without room"
    server.hbm_reserve = 0  # room is made: the held request goes through
    server.drain()
    assert req.u is not None and np.isfinite(req.u).all()
