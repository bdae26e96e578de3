"""The PNG decoder behind the blue-noise asset loader (mrt_png_decode_rgba8,
the role lodepng plays at src/gfx/renderer.ixx:101-110): synthetic PNGs of
every colour type it reads, every scanline filter and every DEFLATE block
type decode to the pixels they were made from; corrupt or unsupported files
are refused; and the committed fixture is the reference's asset decoded."""
import ctypes as C
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from minotert_gb300._lib import MRT_EINVAL, MRT_ERANGE, MrtError, lib, ptr
from minotert_gb300.scene import blue_noise_tile, load_png

GOLDEN = Path(__file__).resolve().parent / "golden"
CHANNELS = {0: 1, 4: 2, 2: 3, 6: 4}


def _chunk(typ: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + typ + body + struct.pack(">I", zlib.crc32(typ + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _encode(img: np.ndarray, ctype: int, filters, compress) -> bytes:
    h, w, ch = img.shape
    rows = img.reshape(h, w * ch).astype(np.int32)
    raw = bytearray()
    for y in range(h):
        f = filters[y % len(filters)]
        cur = rows[y]
        up = rows[y - 1] if y else np.zeros_like(cur)
        a = np.concatenate([np.zeros(ch, np.int32), cur[:-ch]])
        c = np.concatenate([np.zeros(ch, np.int32), up[:-ch]])
        pred = [np.zeros_like(cur), a, up, (a + up) // 2, _paeth(a, up, c)][f]
        raw.append(f)
        raw += ((cur - pred) & 255).astype(np.uint8).tobytes()
    ihdr = struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)
    return b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", compress(bytes(raw))) + _chunk(b"IEND", b"")


def _rgba(img, ctype):
    h, w, ch = img.shape
    out = np.full((h, w, 4), 255, np.uint8)
    if ch <= 2:
        out[..., :3] = img[..., :1]
        if ch == 2:
            out[..., 3] = img[..., 1]
    else:
        out[..., :ch] = img
    return out


def _fixed(data):
    c = zlib.compressobj(6, zlib.DEFLATED, 15, 9, zlib.Z_FIXED)
    return c.compress(data) + c.flush()


COMPRESSORS = {"stored": lambda d: zlib.compress(d, 0), "fixed": _fixed, "dynamic": lambda d: zlib.compress(d, 9)}


@pytest.mark.parametrize("ctype", [0, 4, 2, 6])
@pytest.mark.parametrize("blocks", ["stored", "fixed", "dynamic"])
def test_png_decode_round_trip(built_lib, ctype, blocks):
    rng = np.random.default_rng(ctype * 7 + len(blocks))
    h, w = 37, 53
    # smooth gradients plus noise, so every filter sees real predictions
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.stack([(xx * 3 + yy * 5 + k * 40) % 256 for k in range(CHANNELS[ctype])], -1)
    img = (img + rng.integers(0, 4, img.shape)) % 256
    img = img.astype(np.uint8)
    png = _encode(img, ctype, filters=[0, 1, 2, 3, 4], compress=COMPRESSORS[blocks])
    assert np.array_equal(load_png(png), _rgba(img, ctype))


def test_png_decode_refuses_corrupt_and_unsupported_files(built_lib):
    img = np.arange(8 * 8 * 4, dtype=np.uint8).reshape(8, 8, 4)
    good = _encode(img, 6, [4], COMPRESSORS["dynamic"])
    assert np.array_equal(load_png(good), img)
    w, h = C.c_uint32(0), C.c_uint32(0)

    def rc_of(data: bytes, out_bytes=None):
        buf = np.zeros(max(out_bytes if out_bytes is not None else 8 * 8 * 4, 1), np.uint8)
        d = np.frombuffer(data, np.uint8)
        return lib().mrt_png_decode_rgba8(ptr(d), d.nbytes, ptr(buf), out_bytes if out_bytes is not None else buf.nbytes,
                                          C.byref(w), C.byref(h))

    bad = bytearray(good)
    bad[60] ^= 0x01  # inside IDAT: the chunk CRC no longer matches
    assert rc_of(bytes(bad)) == MRT_EINVAL
    assert rc_of(good[:40]) == MRT_EINVAL  # truncated
    assert rc_of(b"not a png at all, not a png at all, not a png") == MRT_EINVAL
    # a deflate stream whose Adler-32 does not match, with valid chunk CRCs
    raw = zlib.decompress(good[good.index(b"IDAT") + 4:good.index(b"IEND") - 8])
    z = bytearray(zlib.compress(raw, 9))
    z[-1] ^= 0xFF
    ihdr = struct.pack(">IIBBBBB", 8, 8, 8, 6, 0, 0, 0)
    forged = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", bytes(z)) + _chunk(b"IEND", b"")
    assert rc_of(forged) == MRT_EINVAL
    # 16-bit samples and interlacing are not read
    for depth, inter in ((16, 0), (8, 1)):
        ihdr = struct.pack(">IIBBBBB", 8, 8, depth, 6, 0, 0, inter)
        assert rc_of(b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", ihdr) + _chunk(b"IDAT", zlib.compress(raw))
                     + _chunk(b"IEND", b"")) == MRT_EINVAL
    assert rc_of(good, out_bytes=8 * 8 * 4 - 1) == MRT_ERANGE
    with pytest.raises(MrtError):
        load_png(GOLDEN / "does_not_exist.png")


def test_blue_noise_fixture_is_the_reference_asset(built_lib):
    fx = np.load(GOLDEN / "blue_noise_asset.npz")["rgba"]
    assert fx.shape == (256, 256, 4) and fx.dtype == np.uint8
    # every channel holds each of the 256 levels equally often (a rank map)
    for ch in range(4):
        assert np.array_equal(np.bincount(fx[..., ch].ravel(), minlength=256), np.full(256, 256))
    assert np.array_equal(blue_noise_tile(fx, 64), fx[:64, :64])
    from golden.make_blue_noise import ASSET as asset
    if not asset.exists():
        pytest.skip("reference tree not present")
    assert np.array_equal(load_png(asset), fx)
