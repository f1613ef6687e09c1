"""Frame readers without OpenCV or Pillow.

The reference's tutorials read their frames with ``cv2.imread(path,
cv2.IMREAD_ANYDEPTH)``: 16-bit TIFFs (``tutorials/test0``), 8-bit TIFFs
(``tutorials/test1``) and an 8-bit PNG mask (``tutorials/test2``). ``imread``
returns the same single-channel arrays (uint8 or uint16, shape (rows,
columns)) for baseline TIFF (uncompressed or PackBits strips, either byte
order, 8/16-bit grayscale) and PNG (8/16-bit grayscale, grey + alpha, RGB,
RGBA or palette, non-interlaced; colour images are reduced to their first
channel like the reference's single-channel use).
"""

import struct
import zlib

import numpy as np

__all__ = ["imread"]


def imread(path):
    """Read a TIFF or PNG frame as a 2-D uint8/uint16 array."""
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        return _read_png(data)
    if data[:4] in (b"II*\x00", b"MM\x00*"):
        return _read_tiff(data)
    raise ValueError(f"{path}: not a TIFF or PNG file")


# ---------------------------------------------------------------------------
# TIFF (baseline, strips).
# ---------------------------------------------------------------------------
_TIFF_TYPES = {1: ("B", 1), 3: ("H", 2), 4: ("I", 4), 16: ("Q", 8)}


def _read_tiff(data):
    bo = "<" if data[:2] == b"II" else ">"
    (ifd,) = struct.unpack(bo + "I", data[4:8])
    (count,) = struct.unpack(bo + "H", data[ifd:ifd + 2])
    tags = {}
    for k in range(count):
        e = ifd + 2 + 12 * k
        tag, typ, n = struct.unpack(bo + "HHI", data[e:e + 8])
        if typ not in _TIFF_TYPES:
            continue
        code, size = _TIFF_TYPES[typ]
        if n * size <= 4:
            raw = data[e + 8:e + 8 + n * size]
        else:
            (off,) = struct.unpack(bo + "I", data[e + 8:e + 12])
            raw = data[off:off + n * size]
        tags[tag] = list(struct.unpack(bo + code * n, raw))
    width, height = tags[256][0], tags[257][0]
    bits = tags.get(258, [1])[0]
    compression = tags.get(259, [1])[0]
    spp = tags.get(277, [1])[0]
    if bits not in (8, 16):
        raise ValueError(f"TIFF with {bits} bits per sample is not supported")
    if compression not in (1, 32773):
        raise ValueError(f"TIFF compression {compression} is not supported (uncompressed and PackBits are)")
    offsets, counts = tags[273], tags[279]
    body = b"".join(_unpackbits(data[o:o + c]) if compression == 32773 else data[o:o + c]
                    for o, c in zip(offsets, counts))
    dt = np.dtype(np.uint8 if bits == 8 else (bo + "u2"))
    img = np.frombuffer(body, dtype=dt, count=width * height * spp).reshape(height, width, spp)[:, :, 0]
    return img.astype(np.uint8 if bits == 8 else np.uint16)


def _unpackbits(src):
    """PackBits run-length decoding (TIFF compression 32773)."""
    out = bytearray()
    i = 0
    while i < len(src):
        n = src[i]
        i += 1
        if n < 128:
            out += src[i:i + n + 1]
            i += n + 1
        elif n > 128:
            out += bytes([src[i]]) * (257 - n)
            i += 1
    return bytes(out)


# ---------------------------------------------------------------------------
# PNG.
# ---------------------------------------------------------------------------
_PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _read_png(data):
    i = 8
    idat = []
    palette = None
    while i < len(data):
        (length,) = struct.unpack(">I", data[i:i + 4])
        kind = data[i + 4:i + 8]
        body = data[i + 8:i + 8 + length]
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        i += 12 + length
    if interlace:
        raise ValueError("interlaced PNG is not supported")
    if depth not in (8, 16):
        raise ValueError(f"PNG with bit depth {depth} is not supported")
    ch = _PNG_CHANNELS[ctype]
    bpp = ch * depth // 8                       # bytes per pixel (filter unit)
    stride = width * bpp
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    rows = _unfilter(raw, height, stride, bpp)
    if depth == 16:
        img = rows.view(">u2").reshape(height, width, ch).astype(np.uint16)
    else:
        img = rows.reshape(height, width, ch)
    img = img[:, :, 0]
    if ctype == 3:
        img = palette[img][:, :, 0]
    return np.ascontiguousarray(img)


def _unfilter(raw, height, stride, bpp):
    """Undo the five PNG row filters (none, sub, up, average, Paeth)."""
    out = np.zeros((height, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    pos = 0
    for y in range(height):
        ftype = raw[pos]
        line = raw[pos + 1:pos + 1 + stride].astype(np.int32)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        elif ftype == 1:
            # Sub: a running sum along each byte lane of the pixel, modulo 256.
            cur = (np.cumsum(line.reshape(-1, bpp), axis=0).reshape(-1)) & 0xFF
        else:
            cur = np.zeros(stride, dtype=np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                if ftype == 1:
                    p = a
                elif ftype == 3:
                    p = (a + b) >> 1
                elif ftype == 4:
                    c = prev[x - bpp] if x >= bpp else 0
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                else:
                    raise ValueError(f"unknown PNG filter {ftype}")
                cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out
