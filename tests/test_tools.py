"""Frame readers (openpiv_gpu.tools.imread): TIFF and PNG round trips written
by small encoders here, and the reference's tutorial frames
(`openpiv_gpu/tutorials` of the reference checkout, located by the
OPENPIV_TUTORIALS environment variable; skipped when unset): shape, type,
pixel sum and digest recorded from the readers' first run on them (cv2.imread,
which the tutorials use, is not installed here)."""

import hashlib
import os
import struct
import zlib

import numpy as np
import pytest

from openpiv_gpu.tools import imread


def _write_tiff(path, img, order="<", rows_per_strip=None, packbits=False):
    h, w = img.shape
    bits = img.dtype.itemsize * 8
    body = img.astype(order + ("u1" if bits == 8 else "u2")).tobytes()
    rps = rows_per_strip or h
    strips = [body[r * w * img.dtype.itemsize:(r + rps) * w * img.dtype.itemsize] for r in range(0, h, rps)]
    if packbits:  # literal runs of up to 128 bytes
        enc = []
        for s in strips:
            out = bytearray()
            for i in range(0, len(s), 128):
                chunk = s[i:i + 128]
                out += bytes([len(chunk) - 1]) + chunk
            enc.append(bytes(out))
        strips = enc
    head = (b"II*\x00" if order == "<" else b"MM\x00*")
    data = bytearray(head + b"\x00" * 4)
    offsets = []
    for s in strips:
        offsets.append(len(data))
        data += s
    if len(data) % 2:
        data += b"\x00"
    off_arr = len(data)
    data += struct.pack(order + "I" * len(strips), *offsets)
    cnt_arr = len(data)
    data += struct.pack(order + "I" * len(strips), *[len(s) for s in strips])
    ifd = len(data)

    def entry(tag, typ, n, val):
        if typ == 3 and n == 1:
            v = struct.pack(order + "H", val) + b"\x00\x00"
        else:
            v = struct.pack(order + "I", val)
        return struct.pack(order + "HHI", tag, typ, n) + v

    ents = [entry(256, 4, 1, w), entry(257, 4, 1, h), entry(258, 3, 1, bits),
            entry(259, 3, 1, 32773 if packbits else 1), entry(262, 3, 1, 1),
            entry(273, 4, len(strips), off_arr if len(strips) > 1 else offsets[0]), entry(277, 3, 1, 1),
            entry(278, 4, 1, rps), entry(279, 4, len(strips), cnt_arr if len(strips) > 1 else len(strips[0]))]
    data += struct.pack(order + "H", len(ents)) + b"".join(ents) + b"\x00" * 4
    data[4:8] = struct.pack(order + "I", ifd)
    with open(path, "wb") as fh:
        fh.write(bytes(data))


def _paeth(a, b, c):
    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def _write_png(path, img, ctype=0):
    """Encoder applying filter (row % 5) to row `row` (none, sub, up, average, Paeth)."""
    h, w = img.shape[:2]
    depth = img.dtype.itemsize * 8
    px = img.astype(">u2").view(np.uint8) if depth == 16 else img
    raw = np.ascontiguousarray(px).reshape(h, -1).astype(np.int32)
    ch = {0: 1, 2: 3, 6: 4}[ctype]
    bpp = ch * depth // 8
    out = bytearray()
    prev = np.zeros(raw.shape[1], np.int32)
    for y in range(h):
        f = y % 5
        line = raw[y]
        enc = np.zeros_like(line)
        for x in range(len(line)):
            a = line[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            p = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
            enc[x] = (line[x] - p) & 0xFF
        out += bytes([f]) + enc.astype(np.uint8).tobytes()
        prev = line

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    data += chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(data)


@pytest.mark.parametrize("order", ["<", ">"])
@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("rps,packbits", [(None, False), (7, False), (5, True)])
def test_tiff_round_trip(tmp_path, order, dtype, rps, packbits):
    rng = np.random.default_rng(3)
    img = rng.integers(0, np.iinfo(dtype).max, (23, 37), dtype=np.int64).astype(dtype)
    path = tmp_path / "f.tif"
    _write_tiff(path, img, order, rps, packbits)
    got = imread(path)
    assert got.dtype == dtype and got.shape == img.shape
    np.testing.assert_array_equal(got, img)


@pytest.mark.parametrize("dtype,ctype", [(np.uint8, 0), (np.uint16, 0), (np.uint8, 2), (np.uint8, 6)])
def test_png_round_trip(tmp_path, dtype, ctype):
    rng = np.random.default_rng(4)
    ch = {0: 1, 2: 3, 6: 4}[ctype]
    img = rng.integers(0, np.iinfo(dtype).max, (17, 29, ch), dtype=np.int64).astype(dtype)
    path = tmp_path / "f.png"
    _write_png(path, img[:, :, 0] if ch == 1 else img, ctype)
    got = imread(path)
    np.testing.assert_array_equal(got, img[:, :, 0])


TUTORIAL = os.environ.get("OPENPIV_TUTORIALS", "")
FRAMES = [
    ("test0/jh_0000_a.tiff", (512, 1608), np.uint16, 3596764887, "8e64a55b23338b53"),
    ("test0/jh_0000_b.tiff", (512, 1608), np.uint16, 3591312713, "96409745445087b7"),
    ("test1/B005_1.tif", (512, 512), np.uint8, 1760928, "84954fb7cc6fc684"),
    ("test1/B005_2.tif", (512, 512), np.uint8, 1754776, "6dfdaca47a5dad29"),
    ("test2/airfoil_mask.png", (2052, 4603), np.uint8, 569553975, "4368a11f0c8d46f5"),
]


@pytest.mark.parametrize("name,shape,dtype,total,digest", FRAMES)
def test_reference_tutorial_frames(name, shape, dtype, total, digest):
    path = os.path.join(TUTORIAL, name)
    if not TUTORIAL or not os.path.exists(path):
        pytest.skip("OPENPIV_TUTORIALS does not point at the reference's tutorial frames")
    img = imread(path)
    assert img.shape == shape and img.dtype == dtype
    assert int(img.astype(np.int64).sum()) == total
    assert hashlib.sha256(img.tobytes()).hexdigest()[:16] == digest
