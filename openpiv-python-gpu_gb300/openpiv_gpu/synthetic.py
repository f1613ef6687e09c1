"""Seeded synthetic particle-image pairs for tests and benchmarks.

Particle model (one frame pair):

* ``n = round(density * H * W)`` particles at uniform random positions over the
  frame plus a margin wide enough that particles enter and leave at the edges;
* diameters ``d ~ N(d_mean, d_std)`` clipped to ``>= 0.5`` px, peak intensities
  ``I0 ~ U[150, 255]``, Gaussian profile ``I0 * exp(-8 r^2 / d^2)``;
* frame B holds the same particles moved by the displacement field evaluated
  at their frame-A position;
* additive Gaussian noise ``N(0, noise)``, then rounding and clipping to uint8.

Pixel centres sit on integer coordinates (x = column, y = row), the convention
the reference's frame deformation uses (``openpiv_gpu/gpu_process.py:1153``).
Every generator takes a seed and uses NumPy's PCG64 stream, so a pair is a
pure function of its arguments.
"""

import math

import numpy as np

__all__ = [
    "render_pair",
    "lamb_oseen",
    "sinusoidal_shear",
    "streamfunction_field",
    "uniform_field",
    "config_case",
    "CONFIGS",
]


# ----------------------------------------------------------------------------
# Displacement fields: callables (x, y) -> (u, v) in pixels.
# ----------------------------------------------------------------------------
class _Field:
    def __init__(self, fn, description):
        self._fn = fn
        self.description = description

    def __call__(self, x, y):
        return self._fn(np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64))


def lamb_oseen(center, core_radius, max_speed, uniform=(0.0, 0.0)):
    """Lamb-Oseen vortex: tangential speed A (1 - exp(-r^2/rc^2)) / r, scaled so
    its maximum (at r = 1.1209 rc) equals ``max_speed`` px, plus a uniform shift."""
    xc, yc = center
    rc = float(core_radius)
    peak = (1.0 - math.exp(-1.1209 ** 2)) / 1.1209  # max of (1-exp(-s^2))/s
    amp = max_speed * rc / peak
    u0, v0 = uniform

    def fn(x, y):
        dx, dy = x - xc, y - yc
        r2 = dx * dx + dy * dy
        with np.errstate(invalid="ignore", divide="ignore"):
            ut_over_r = np.where(r2 > 0, amp * (1.0 - np.exp(-r2 / (rc * rc))) / np.maximum(r2, 1e-300), 1.0 * amp / (rc * rc))
        return -ut_over_r * dy + u0, ut_over_r * dx + v0

    return _Field(fn, f"lamb-oseen(center={center}, rc={rc:.3f}, max={max_speed}, uniform={uniform})")


def sinusoidal_shear(u_amp=6.0, u_period=256.0, v_amp=2.0, v_period=512.0):
    """u = u_amp sin(2 pi y / u_period), v = v_amp cos(2 pi x / v_period)."""

    def fn(x, y):
        return u_amp * np.sin(2 * np.pi * y / u_period), v_amp * np.cos(2 * np.pi * x / v_period)

    return _Field(fn, f"shear(u={u_amp}sin(2pi y/{u_period}), v={v_amp}cos(2pi x/{v_period}))")


def uniform_field(u0, v0):
    def fn(x, y):
        return np.full(np.broadcast(x, y).shape, float(u0)), np.full(np.broadcast(x, y).shape, float(v0))

    return _Field(fn, f"uniform({u0}, {v0})")


def streamfunction_field(shape, n_modes, max_speed, seed):
    """Divergence-free field u = d(psi)/dy, v = -d(psi)/dx from a seeded
    streamfunction psi = sum_k a_k sin(kx_k x + ky_k y + phi_k), scaled so the
    largest displacement over the frame equals ``max_speed`` px."""
    ht, wd = shape
    rng = np.random.Generator(np.random.PCG64(seed))
    wavelength = rng.uniform(0.15, 0.6, n_modes) * max(ht, wd)
    angle = rng.uniform(0, 2 * np.pi, n_modes)
    kx = 2 * np.pi / wavelength * np.cos(angle)
    ky = 2 * np.pi / wavelength * np.sin(angle)
    phase = rng.uniform(0, 2 * np.pi, n_modes)
    amp = rng.normal(0, 1, n_modes) * wavelength

    def raw(x, y):
        u = np.zeros(np.broadcast(x, y).shape)
        v = np.zeros_like(u)
        for k in range(n_modes):
            c = amp[k] * np.cos(kx[k] * x + ky[k] * y + phase[k])
            u += c * ky[k]
            v -= c * kx[k]
        return u, v

    gy, gx = np.mgrid[0:ht:8, 0:wd:8].astype(np.float64)
    u, v = raw(gx, gy)
    scale = max_speed / max(np.sqrt(u * u + v * v).max(), 1e-12)

    def fn(x, y):
        u, v = raw(x, y)
        return u * scale, v * scale

    return _Field(fn, f"streamfunction({n_modes} modes, max={max_speed}, seed={seed})")


# ----------------------------------------------------------------------------
# Rendering.
# ----------------------------------------------------------------------------
def _render(shape, px, py, d, i0, chunk=20000):
    ht, wd = shape
    img = np.zeros(ht * wd, dtype=np.float64)
    for s in range(0, px.size, chunk):
        cx, cy, cd, ci = px[s:s + chunk], py[s:s + chunk], d[s:s + chunk], i0[s:s + chunk]
        rad = int(math.ceil(1.3 * cd.max())) + 1
        off = np.arange(-rad, rad + 1)
        bx = np.floor(cx).astype(np.int64)[:, None, None] + off[None, None, :]
        by = np.floor(cy).astype(np.int64)[:, None, None] + off[None, :, None]
        r2 = (bx - cx[:, None, None]) ** 2 + (by - cy[:, None, None]) ** 2
        val = ci[:, None, None] * np.exp(-8.0 * r2 / (cd[:, None, None] ** 2))
        inside = (bx >= 0) & (bx < wd) & (by >= 0) & (by < ht)
        bx, by = np.broadcast_to(bx, val.shape), np.broadcast_to(by, val.shape)
        flat = (by * wd + bx)[inside]
        img += np.bincount(flat, weights=val[inside], minlength=ht * wd)
    return img.reshape(ht, wd)


def render_pair(shape, field, seed, density=0.02, d_mean=2.5, d_std=0.5, noise=2.0, max_disp=None):
    """Renders one seeded uint8 frame pair moved by ``field``.

    Returns ``(frame_a, frame_b)``, both uint8 arrays of ``shape``.
    """
    ht, wd = shape
    rng = np.random.Generator(np.random.PCG64(seed))
    if max_disp is None:
        gy, gx = np.mgrid[0:ht:16, 0:wd:16].astype(np.float64)
        u, v = field(gx, gy)
        max_disp = float(np.sqrt(u * u + v * v).max())
    margin = max_disp + 4.0
    area = (ht + 2 * margin) * (wd + 2 * margin)
    n = int(round(density * area))
    px = rng.uniform(-margin, wd + margin, n)
    py = rng.uniform(-margin, ht + margin, n)
    d = np.maximum(rng.normal(d_mean, d_std, n), 0.5)
    i0 = rng.uniform(150.0, 255.0, n)
    u, v = field(px, py)
    img_a = _render(shape, px, py, d, i0)
    img_b = _render(shape, px + u, py + v, d, i0)
    img_a += rng.normal(0.0, noise, img_a.shape)
    img_b += rng.normal(0.0, noise, img_b.shape)
    frame_a = np.clip(np.rint(img_a), 0, 255).astype(np.uint8)
    frame_b = np.clip(np.rint(img_b), 0, 255).astype(np.uint8)
    return frame_a, frame_b


# ----------------------------------------------------------------------------
# The five benchmark workloads (seed = 1000 * config + pair index).
# ----------------------------------------------------------------------------
_CFG1_PIV = dict(min_search_size=32, search_size_iters=1, overlap_ratio=0.5, n_fft=2, subpixel_method="gaussian",
                 median_tol=2, validation_size=1, num_replacing_iters=1, dtype_f="float32")
_CFG2_PIV = dict(min_search_size=16, search_size_iters=(1, 1, 1), overlap_ratio=0.5, n_fft=2,
                 subpixel_method="gaussian", deforming_order=(1, 3, 3), median_tol=2, validation_size=1,
                 num_replacing_iters=2, revalidate=True, smoothing_par=None, dtype_f="float32")
_CFG3_PIV = dict(min_search_size=16, search_size_iters=(1, 1), overlap_ratio=0.75, n_fft=2,
                 subpixel_method="gaussian", median_tol=2, validation_size=1, num_replacing_iters=2,
                 revalidate=True, dtype_f="float32")
_MULTI_PIV = dict(min_search_size=16, search_size_iters=(1, 1, 1), overlap_ratio=0.5, n_fft=2,
                  subpixel_method="gaussian", median_tol=2, validation_size=1, num_replacing_iters=2,
                  revalidate=True, dtype_f="float32")

CONFIGS = {
    1: dict(name="single-pass 512x512, 32 px windows @50%", piv=_CFG1_PIV),
    2: dict(name="three-pass 1024x1024, 64->32->16 @50%, deformation, smoothn", piv=_CFG2_PIV),
    3: dict(name="two-pass 2048x2048, 32->16 @75%", piv=_CFG3_PIV),
    4: dict(name="mixed-size batch, 64->32->16 @50%", piv=_MULTI_PIV),
    5: dict(name="serving stream, 64->32->16 @50%", piv=_MULTI_PIV),
}

_CFG4_SHAPES = [(512, 512), (800, 1280), (768, 1024), (2048, 2048)]
_CFG5_SHAPES = [(480, 640), (800, 1280), (1080, 1920), (1600, 2560), (2160, 4096)]


def config_case(cfg, pair_index=0, shape=None):
    """Returns ``(frame_a, frame_b, field, piv_kwargs)`` for workload ``cfg``.

    ``shape`` overrides the frame size (used for small parity cases that keep a
    workload's particle model and settings).
    """
    seed = 1000 * cfg + pair_index
    piv = dict(CONFIGS[cfg]["piv"])
    if cfg == 1:
        shape = shape or (512, 512)
        ht, wd = shape
        field = lamb_oseen(((wd - 1) / 2.0, (ht - 1) / 2.0), 0.1 * min(ht, wd), 4.0, uniform=(1.5, -0.7))
        a, b = render_pair(shape, field, seed, density=0.02, d_mean=2.5, d_std=0.5)
    elif cfg == 2:
        shape = shape or (1024, 1024)
        field = sinusoidal_shear()
        a, b = render_pair(shape, field, seed, density=0.03, d_mean=2.5, d_std=0.5)
    elif cfg == 3:
        shape = shape or (2048, 2048)
        field = streamfunction_field(shape, 8, 8.0, seed)
        a, b = render_pair(shape, field, seed, density=0.05, d_mean=3.0, d_std=0.8)
    elif cfg in (4, 5):
        rng = np.random.Generator(np.random.PCG64(seed + 500))
        if shape is None:
            shapes = _CFG4_SHAPES if cfg == 4 else _CFG5_SHAPES
            shape = shapes[pair_index % len(shapes)] if cfg == 4 else shapes[rng.integers(len(shapes))]
        ht, wd = shape
        lo, hi = (2.0, 10.0) if cfg == 4 else (2.0, 12.0)
        vmax = rng.uniform(lo, hi)
        density = rng.uniform(0.01, 0.05) if cfg == 4 else rng.uniform(0.01, 0.04)
        if rng.integers(2) == 0:
            field = lamb_oseen((wd * rng.uniform(0.3, 0.7), ht * rng.uniform(0.3, 0.7)), 0.1 * min(ht, wd), vmax)
        else:
            field = sinusoidal_shear(u_amp=vmax, u_period=ht / 2.0, v_amp=vmax / 3.0, v_period=float(wd))
        a, b = render_pair(shape, field, seed, density=density, d_mean=2.5, d_std=0.5)
    else:
        raise ValueError(f"unknown workload {cfg}")
    return a, b, field, piv
