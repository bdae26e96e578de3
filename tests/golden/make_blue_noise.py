"""Generates tests/golden/blue_noise_asset.npz: the reference's blue-noise
texture (assets/blue_noise.png, 256 x 256 RGBA8, loaded by the reference at
src/gfx/renderer.ixx:101-110) decoded to RGBA8 by this library's PNG decoder
(mrt_png_load_rgba8) and cross-checked against an independent decode with
Python's zlib and the PNG scanline filters.  The reference tree is not
present where the GPU tests and the bench run, so they read the fixture.

    python tests/golden/make_blue_noise.py [/path/to/reference]
"""
import os
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
# where the reference tree lies (read only by this script and the test that
# re-checks the fixture when the tree is present)
REFERENCE = Path(os.environ.get("MRT_REFERENCE", "/root/reference"))
ASSET = REFERENCE / "assets" / "blue_noise.png"


def python_decode(data: bytes) -> np.ndarray:
    """8-bit non-interlaced colour type 6 PNG -> (h, w, 4) uint8, stdlib only."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        typ, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and ctype == 6 and inter == 0
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    out = np.zeros((h, 4 * w), np.int32)
    for y in range(h):
        f, cur = raw[y, 0], raw[y, 1:].astype(np.int32)
        up = out[y - 1] if y else np.zeros(4 * w, np.int32)
        row = np.zeros(4 * w, np.int32)
        for i in range(4 * w):
            a = row[i - 4] if i >= 4 else 0
            b = up[i]
            c = up[i - 4] if (i >= 4 and y) else 0
            if f == 0:
                pr = 0
            elif f == 1:
                pr = a
            elif f == 2:
                pr = b
            elif f == 3:
                pr = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            row[i] = (cur[i] + pr) & 255
        out[y] = row
    return out.astype(np.uint8).reshape(h, w, 4)


def main(ref_root=None):
    from minotert_gb300 import build
    build.build()
    from minotert_gb300.scene import load_png
    path = Path(ref_root) / "assets" / "blue_noise.png" if ref_root else ASSET
    img = load_png(path)
    assert img.shape == (256, 256, 4), img.shape
    assert np.array_equal(img, python_decode(path.read_bytes())), "decoders disagree"
    np.savez_compressed(HERE / "blue_noise_asset.npz", rgba=img)
    print(f"wrote {HERE / 'blue_noise_asset.npz'}: {img.shape}, channel means {img.reshape(-1, 4).mean(0)}")


if __name__ == "__main__":
    main(*sys.argv[1:])
