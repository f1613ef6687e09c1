"""Generates the golden vectors under tests/golden/ from the reference itself.

Run from the repository root on a machine that has the reference source:

    python tests/golden/make_golden.py /path/to/openpiv-python-gpu [case ...]

(with case names, only those fixtures are written).

The reference package is imported unmodified; ``cupy_shim`` maps CuPy to
NumPy/SciPy and restates its four RawModule kernels. Stage outputs are
captured by wrapping methods of the reference's classes (``CorrelationGPU.
__call__``, ``ValidationGPU.__call__``, ``SmoothnGPU.__call__``); the source is
not edited. Each case stores its inputs (small frames), settings and outputs in
``<case>.npz``. Full-size cases store SHA-256 digests of the frames instead of
the frames: the test regenerates the frames from the seed and skips the case
if the digests differ.
"""

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    """(name, cfg, shape, pair_index, overrides, store_frames)."""
    small = (128, 160)
    return [
        ("cfg1_256", 1, (256, 256), 0, {}, True),
        ("cfg1_512", 1, None, 0, {}, False),
        ("cfg2_256", 2, (256, 256), 0, {"deforming_order": 1}, True),
        ("cfg2_1024", 2, None, 0, {"deforming_order": 1}, False),
        ("multi_iter", 2, (192, 224), 1, {"deforming_order": 1, "search_size_iters": (2, 2),
                                           "num_replacing_iters": 1, "revalidate": False}, True),
        ("parabolic_centroid", 2, (192, 192), 2, {"deforming_order": 1,
                                                  "subpixel_method": ("parabolic", "centroid", "gaussian")}, True),
        ("validation_mix", 2, small, 3, {"deforming_order": 1, "median_tol": 1.0, "mad_tol": 3.0,
                                         "mean_tol": 1.5, "rms_tol": 3.0, "replacing_method": "median",
                                         "num_replacing_iters": 3, "revalidate": False}, True),
        ("mean_replace", 2, small, 4, {"deforming_order": 1, "median_tol": 0.7, "replacing_method": "mean",
                                       "num_replacing_iters": 2, "revalidate": True}, True),
        ("spring_heavy", 2, small, 5, {"deforming_order": 1, "median_tol": 0.3, "num_replacing_iters": 2,
                                       "revalidate": True}, True),
        ("s2n_energy", 1, (160, 192), 6, {"s2n_tol": 2.5, "s2n_method": "peak2energy", "median_tol": None}, True),
        ("s2n_mean", 1, (160, 192), 7, {"s2n_tol": 1.2, "s2n_method": "peak2mean"}, True),
        ("float64", 2, (192, 192), 8, {"deforming_order": 1, "dtype_f": "float64"}, True),
        ("deforming_par_1", 2, (160, 160), 9, {"deforming_order": 1, "deforming_par": 1.0,
                                               "search_size_iters": (1, 1)}, True),
        ("deforming_par_0", 2, (160, 160), 10, {"deforming_order": 1, "deforming_par": 0,
                                                "search_size_iters": (1, 1)}, True),
        ("scaled_fixed_s", 2, (160, 192), 11, {"deforming_order": 1, "dt": 2.0, "scaling_par": 0.5,
                                               "smoothing_par": 0.8}, True),
        ("nfft1_nonorm", 1, (160, 160), 12, {"n_fft": 1, "normalize": False, "min_search_size": 16}, True),
        ("nfft1_norm", 1, (160, 160), 13, {"n_fft": 1, "normalize": True, "min_search_size": 16}, True),
        ("not_centered", 2, (150, 170), 14, {"deforming_order": 1, "center": False}, True),
        ("overlap_075", 3, (160, 160), 15, {"overlap_ratio": 0.75, "search_size_iters": (1, 1)}, True),
        ("window8", 2, (96, 96), 16, {"deforming_order": 1, "min_search_size": 8, "search_size_iters": (1, 1)},
         True),
        ("shrink", 2, (160, 160), 17, {"deforming_order": 1, "shrink_ratio": 0.5, "search_size_iters": (1, 1)},
         True),
        ("masked64", 2, (192, 192), 18, {"deforming_order": 1, "dtype_f": "float64", "mask": "disc"}, True),
        ("blank_region", 1, (128, 128), 19, {"median_tol": 2, "blank": True}, True),
        ("validation5x5", 2, small, 20, {"deforming_order": 1, "validation_size": 2, "median_tol": 1.2,
                                         "replacing_method": "median", "replacing_size": 2,
                                         "num_replacing_iters": 2, "revalidate": True}, True),
        ("overlap_per_pass", 2, (160, 160), 21, {"deforming_order": 1, "search_size_iters": (1, 1),
                                                 "overlap_ratio": (0.5, 0.75)}, True),
        ("nfft_real", 2, (160, 160), 22, {"deforming_order": 1, "search_size_iters": (1, 1),
                                          "n_fft": (1.5, 3)}, True),
        ("uint16", 2, small, 23, {"deforming_order": 1, "u16": True}, True),
    ]


def _disc_mask(shape):
    ht, wd = shape
    y, x = np.mgrid[0:ht, 0:wd]
    return ((x - 0.45 * wd) ** 2 + (y - 0.55 * ht) ** 2) < (0.18 * min(ht, wd)) ** 2


def build_case(syn, cfg, shape, pair_index, overrides):
    a, b, field, piv = syn.config_case(cfg, pair_index, shape=shape)
    piv = dict(piv)
    ov = dict(overrides)
    blank = ov.pop("blank", False)
    if blank:  # a constant region: zero-variance windows exercise the all-equal argmax tie
        a = a.copy()
        b = b.copy()
        a[:48, :64] = 7
        b[:48, :64] = 7
    if ov.pop("u16", False):  # 16-bit frames over the full range (x 257 maps 255 to 65535)
        a = a.astype(np.uint16) * np.uint16(257)
        b = b.astype(np.uint16) * np.uint16(257)
    piv.update(ov)
    if piv.get("mask") == "disc":
        piv["mask"] = _disc_mask(a.shape)
    return a, b, field, piv


def run_reference(ref_root, only=()):
    sys.path.insert(0, HERE)
    import cupy_shim

    cupy_shim.install()
    pkg_dir = os.path.join(ROOT, "openpiv-python-gpu_gb300")
    sys.path.insert(0, pkg_dir)
    from openpiv_gpu import synthetic as syn  # this project's generator

    for mod in [m for m in sys.modules if m == "openpiv_gpu" or m.startswith("openpiv_gpu.")]:
        del sys.modules[mod]
    sys.path.remove(pkg_dir)
    sys.path.insert(0, ref_root)
    import openpiv_gpu.gpu_process as gp
    import openpiv_gpu.gpu_smoothn as gs
    import openpiv_gpu.gpu_validation as gv

    assert os.path.abspath(gp.__file__).startswith(os.path.abspath(ref_root)), gp.__file__

    stages = []

    orig_corr = gp.CorrelationGPU.__call__
    orig_val = gv.ValidationGPU.__call__
    orig_smooth = gs.SmoothnGPU.__call__

    def corr_call(self, *args, **kwargs):
        u, v = orig_corr(self, *args, **kwargs)
        stages.append({"u_corr": np.array(u), "v_corr": np.array(v),
                       "i_peak": np.array(self.i_peak1), "j_peak": np.array(self.j_peak1)})
        return u, v

    def val_call(self, *f, mask=None):
        out = orig_val(self, *f, mask=mask)
        st = stages[-1]
        if "val0" not in st:
            st["val0"] = np.array(out) if out is not None else np.zeros(f[0].shape, bool)
            st["u_sum"], st["v_sum"] = np.array(f[0]), np.array(f[1])
            if self.s2n_ratio is not None:
                st["s2n"] = np.array(self.s2n_ratio)
        return out

    def smooth_call(self, *f):
        st = stages[-1]
        st["u_rep"], st["v_rep"] = np.array(f[0]), np.array(f[1])
        z = orig_smooth(self, *f)
        st["u_smooth"], st["v_smooth"] = np.array(z[0]), np.array(z[1])
        st["smooth_s"] = np.array(float(self.s))
        return z

    gp.CorrelationGPU.__call__ = corr_call
    gv.ValidationGPU.__call__ = val_call
    gs.SmoothnGPU.__call__ = smooth_call
    gp.SmoothnGPU = gs.SmoothnGPU

    for name, cfg, shape, pair_index, overrides, store in cases():
        if only and name not in only:
            continue
        a, b, field, piv = build_case(syn, cfg, shape, pair_index, overrides)
        mss = piv.pop("min_search_size")
        stages.clear()
        proc = gp.piv_gpu(a.shape, mss, **piv)
        u, v = proc(a, b)
        x, y = proc.coords
        out = {
            "u": np.asarray(u), "v": np.asarray(v), "x": np.asarray(x), "y": np.asarray(y),
            "val_locations": np.asarray(proc.val_locations), "outliers": np.asarray(proc.outliers),
            "field_mask": np.asarray(proc.field_mask),
            "sha_a": np.array(_digest(a)), "sha_b": np.array(_digest(b)),
            "n_iters": np.array(len(stages)),
        }
        for k, st in enumerate(stages):
            for key, val in st.items():
                out[f"it{k}_{key}"] = np.asarray(val)
        settings = dict(overrides)
        settings.update({"cfg": cfg, "pair_index": pair_index, "shape": list(a.shape)})
        out["settings"] = np.array(json.dumps(settings))
        if store:
            out["frame_a"], out["frame_b"] = a, b
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: field {u.shape} {u.dtype}, outliers0 {int(np.sum(proc.val_locations))}, "
              f"iters {len(stages)}", flush=True)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the openpiv-python-gpu source tree> [case ...]")
    run_reference(sys.argv[1], tuple(sys.argv[2:]))
