"""Record a band of the reference's golden image as a test fixture.

The reference pins its offline path tracer with ``tests/golden/cornell_box.png``:
``examples/cornell_box.cpp`` rendered at 1920x1080, 16 spp, Sobol sampler,
denoiser off, read back after 19 frames (three frames in flight, so the image
holds samples 0..15), then downscaled to 640x360 with PIL's bilinear filter
(``tests/golden/render_golden.py``). This script decodes that PNG (zlib, no
PIL) and stores output rows 100..139 (RGB, uint8) in
``tests/golden/cornell_example_band.npz`` for ``tests/test_oracle_golden_image.py``.
Run in a container that has the reference checkout:

    python tests/golden/make_golden_image.py
"""
import os
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_PNG = os.path.join(os.environ.get("OHAO_REFERENCE_ROOT", "/root/reference"), "tests/golden/cornell_box.png")
OUT = os.path.join(HERE, "cornell_example_band.npz")
ROWS = (100, 140)


def _paeth(a, b, c):
    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
    return a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)


def read_png(path):
    """8-bit RGB or RGBA PNG -> (h, w, 3) uint8 (the five row filters of the PNG specification)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
    w, h, depth, ctype, _, _, interlace = hdr
    assert depth == 8 and ctype in (2, 6) and interlace == 0, hdr
    bpp = 3 if ctype == 2 else 4
    raw = zlib.decompress(idat)
    stride = w * bpp + 1
    out = np.zeros((h, w * bpp), np.int64)
    prev = np.zeros(w * bpp, np.int64)
    for y in range(h):
        f = raw[y * stride]
        line = np.frombuffer(raw[y * stride + 1:(y + 1) * stride], np.uint8).astype(np.int64)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros_like(line)
            for x in range(w * bpp):
                a = int(cur[x - bpp]) if x >= bpp else 0
                b = int(prev[x])
                c = int(prev[x - bpp]) if x >= bpp else 0
                p = a if f == 1 else ((a + b) >> 1 if f == 3 else _paeth(a, b, c))
                cur[x] = (int(line[x]) + p) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, bpp)[:, :, :3].astype(np.uint8)


def main():
    img = read_png(REF_PNG)
    assert img.shape == (360, 640, 3), img.shape
    np.savez_compressed(OUT, rows=np.array(ROWS, np.int32), band=img[ROWS[0]:ROWS[1]],
                        mean_rgb=img.reshape(-1, 3).mean(axis=0))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
