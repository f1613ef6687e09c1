"""Writes twiddles.h: W_256^k = exp(-2 pi i k / 256) for k in [0, 256), as
float and double tables. Each value is derived from an angle reduced to the
first octant so that the exact points (0, +-1, +-sqrt(1/2)) come out exact."""

import math
import os

import numpy as np


def w256(k):
    k %= 256
    q, r = divmod(k, 32)  # octant
    a = math.pi * (r if q % 2 == 0 else 32 - r) / 128.0
    c, s = math.cos(a), math.sin(a)
    if r == 0 and q % 2 == 0:
        c, s = 1.0, 0.0
    if r == 0 and q % 2 == 1:
        c, s = math.sqrt(0.5), math.sqrt(0.5)
    # Map octant (c, s) = (cos a, sin a), a in [0, pi/4], to angle theta = 2 pi k / 256.
    octant = [(c, s), (s, c), (-s, c), (-c, s), (-c, -s), (-s, -c), (s, -c), (c, -s)]
    cos_t, sin_t = octant[q]
    return cos_t, -sin_t


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    vals = [w256(k) for k in range(256)]
    for k in range(256):
        ref = np.exp(-2j * np.pi * k / 256)
        assert abs(vals[k][0] - ref.real) < 1e-15 and abs(vals[k][1] - ref.imag) < 1e-15, k
    lines = ["// Generated by gen_twiddles.py: W_256^k = exp(-2 pi i k / 256).", "#pragma once", ""]
    lines.append("static __constant__ double2 c_tw256_d[256] = {")
    lines += [f"  {{{c!r}, {s!r}}}," for c, s in vals]
    lines.append("};")
    lines.append("static __constant__ float2 c_tw256_f[256] = {")
    lines += [f"  {{{float(np.float32(c))!r}f, {float(np.float32(s))!r}f}}," for c, s in vals]
    lines.append("};")
    with open(os.path.join(here, "twiddles.h"), "w") as fh:
        fh.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
