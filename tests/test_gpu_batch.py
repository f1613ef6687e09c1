"""A batch of pairs in one plan run gives each pair's single-pair result, and
the CUDA-graph replay of a run gives the same fields as the direct run."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_equals_single_pairs():
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    torch.cuda.set_device(0)
    pairs = [synthetic.config_case(2, k, shape=(256, 256))[:2] for k in range(3)]
    kw = dict(synthetic.CONFIGS[2]["piv"])
    mss = kw.pop("min_search_size")
    fa = np.stack([p[0] for p in pairs])
    fb = np.stack([p[1] for p in pairs])
    proc = PIVGPU((256, 256), mss, **kw)
    ub, vb = proc.run_batch(fa, fb)
    for k in range(3):
        single = PIVGPU((256, 256), mss, **kw)
        u, v = single(pairs[k][0], pairs[k][1])
        np.testing.assert_array_equal(ub[k].cpu().numpy(), u.cpu().numpy())
        np.testing.assert_array_equal(vb[k].cpu().numpy(), v.cpu().numpy())


def test_graph_replay_equals_direct_run():
    import torch

    from openpiv_gpu import _build, _lib, synthetic
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    lib = _lib.load()
    pairs = [synthetic.config_case(2, k, shape=(256, 256))[:2] for k in range(2)]
    kw = dict(synthetic.CONFIGS[2]["piv"])
    mss = kw.pop("min_search_size")
    fa = torch.as_tensor(np.stack([p[0] for p in pairs])).cuda()
    fb = torch.as_tensor(np.stack([p[1] for p in pairs])).cuda()
    proc = PIVGPU((256, 256), mss, **kw)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ud, vd = proc.run_batch(fa, fb)
    s.synchronize()
    plan = proc.plan_handle(fa, 2)
    m, n = proc.piv_fields[-1].field_shape
    u = torch.zeros((2, m, n), dtype=torch.float64, device="cuda")
    v = torch.zeros_like(u)
    val = torch.zeros((2, m, n), dtype=torch.uint8, device="cuda")
    out = torch.zeros_like(val)
    nk = ctypes.c_int(0)
    _lib.check(lib.piv_plan_graph_capture(plan, 2, fa.data_ptr(), fb.data_ptr(), u.data_ptr(), v.data_ptr(),
                                          val.data_ptr(), out.data_ptr(), ctypes.byref(nk), s.cuda_stream))
    assert nk.value > 10
    _lib.check(lib.piv_plan_graph_launch(plan, s.cuda_stream))
    s.synchronize()
    np.testing.assert_array_equal(u.cpu().numpy(), ud.cpu().numpy())
    np.testing.assert_array_equal(v.cpu().numpy(), vd.cpu().numpy())


def test_pipelined_batches_equal_single_runs():
    """PIVGPU.run_batches (two plans, two streams, asynchronous host copies)
    returns, batch by batch and in order, the fields of separate run_batch
    calls; the plans' device status stays PIV_OK."""
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    torch.cuda.set_device(0)
    kw = dict(synthetic.CONFIGS[2]["piv"])
    mss = kw.pop("min_search_size")
    batches = []
    for b in range(5):
        pairs = [synthetic.config_case(2, 3 * b + k, shape=(192, 224))[:2] for k in range(2)]
        fa = torch.as_tensor(np.stack([p[0] for p in pairs])).pin_memory().numpy()
        fb = torch.as_tensor(np.stack([p[1] for p in pairs])).pin_memory().numpy()
        batches.append((fa, fb))
    ref = PIVGPU((192, 224), mss, **kw, dft="tensor")
    expect = [tuple(x.copy() for x in ref.run_batch(fa, fb, host_out=True)) for fa, fb in batches]
    proc = PIVGPU((192, 224), mss, **kw, dft="tensor")
    got = [(u.copy(), v.copy()) for u, v in proc.run_batches(iter(batches))]
    assert len(got) == len(expect)
    for (u, v), (ue, ve) in zip(got, expect):
        np.testing.assert_array_equal(u, ue)
        np.testing.assert_array_equal(v, ve)
    assert proc.status() == 0 and ref.status() == 0


MIXED_SHAPES = [(128, 160), (96, 96), (128, 160), (160, 224), (96, 96), (128, 160)]
# Ten sizes: more than the eight segments of one launch, so passes on a tensor
# engine take two joint launches.
MANY_SHAPES = [(96 + 16 * (k % 5), 96 + 32 * (k // 5)) for k in range(10)] + [(96, 96)]


@pytest.mark.parametrize("dft,shapes,schedule", [
    ("tensor", MIXED_SHAPES, "joint"), ("tensor", MIXED_SHAPES, "streams"), ("tensor_split", MIXED_SHAPES, "joint"),
    ("fft", MIXED_SHAPES, "joint"), ("tensor", MANY_SHAPES, "joint"), ("tensor", MIXED_SHAPES, "auto"),
    ("tensor_refined", MIXED_SHAPES, "joint"), ("tensor_refined", MANY_SHAPES, "joint"),
    ("tensor_refined", MIXED_SHAPES, "streams")])
def test_mixed_size_submission_equals_single_runs(dft, shapes, schedule):
    """PIVMixedBatch: pairs of several frame sizes in one submission (one
    correlation launch per pass over every size on the tensor engines),
    captured as one CUDA graph; every pair's result equals processing it
    alone."""
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.batching import PIVMixedBatch
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    torch.cuda.set_device(0)
    pairs = [synthetic.config_case(4, k, shape=sh)[:2] for k, sh in enumerate(shapes)]
    settings = dict(synthetic.CONFIGS[4]["piv"])
    batch = PIVMixedBatch(shapes, settings, dft=dft, schedule=schedule)
    batch.load(pairs)
    batch.capture()
    batch.run()
    got = batch.results()
    assert batch.status() == 0
    kw = dict(settings)
    mss = kw.pop("min_search_size")
    for (a, b), (u, v) in zip(pairs, got):
        ue, ve = PIVGPU(a.shape, mss, dft=dft, **kw).run_batch(a[None], b[None], host_out=True)
        np.testing.assert_array_equal(u, ue[0])
        np.testing.assert_array_equal(v, ve[0])
    print(f"{dft}, {len(set(shapes))} sizes, {batch.schedule} {batch.schedule_ms}: {batch.kernel_nodes} kernel nodes")


def test_batch_rejects_configurations_with_different_passes():
    """piv_batch_create: the size groups must share the passes (search, window
    and transform sizes), dtype and correlation engine."""
    import ctypes as ct

    from openpiv_gpu import _build, _lib, synthetic
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    kw = dict(synthetic.CONFIGS[4]["piv"])
    mss = kw.pop("min_search_size")
    a = PIVGPU((128, 160), mss, **kw, dft="tensor")
    b = PIVGPU((160, 224), 2 * mss, **kw, dft="tensor")  # other search sizes
    c = PIVGPU((96, 96), mss, **kw, dft="fft")         # other engine
    for other in (b, c):
        (ca, ka), (cb, kb) = a._config(_lib.PIXEL["u8"], 2), other._config(_lib.PIXEL["u8"], 2)
        cfgs = (_lib.PivConfig * 2)(ca, cb)
        batch = ct.c_void_p()
        assert _lib.lib().piv_batch_create(cfgs, 2, ct.byref(batch)) == _lib.PIV_E_ARG
        assert "differs" in _lib.last_error()
