"""The image writers of the C ABI (omv_save_image, host code, no GPU):
decoded pixels against the oracle's 8-bit conversion of the same image,
written the way saveImage does with flipVerticallyOnWrite(true)."""
import ctypes as C
import struct
import zlib

import numpy as np
import pytest
from conftest import golden


def _save(omv, path, img):
    a = np.ascontiguousarray(img, dtype=np.float32)
    return omv.lib().omv_save_image(str(path).encode(), a.ctypes.data_as(C.POINTER(C.c_float)), a.shape[1],
                                    a.shape[0])


def _read_png(path):
    b = open(path, "rb").read()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(b):
        n, t = struct.unpack(">I4s", b[pos:pos + 8])
        data = b[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", b[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(t + data) & 0xFFFFFFFF, t
        if t == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", data)
        elif t == b"IDAT":
            idat += data
        pos += 12 + n
    w, h, depth, ctype = hdr[:4]
    assert (depth, ctype) == (8, 6)
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 4)


def _read_bmp(path):
    b = open(path, "rb").read()
    off, = struct.unpack("<I", b[10:14])
    w, h, planes, bpp = struct.unpack("<iiHH", b[18:30])
    assert bpp == 32
    px = np.frombuffer(b[off:off + 4 * w * h], dtype=np.uint8).reshape(h, w, 4)[::-1]
    return px[..., [2, 1, 0, 3]]


def _read_tga(path):
    b = open(path, "rb").read()
    w, h = struct.unpack("<HH", b[12:16])
    assert b[2] == 2 and b[16] == 32 and b[17] & 0x20
    px = np.frombuffer(b[18:18 + 4 * w * h], dtype=np.uint8).reshape(h, w, 4)
    return px[..., [2, 1, 0, 3]]


@pytest.mark.parametrize("ext,reader", [("png", _read_png), ("bmp", _read_bmp), ("tga", _read_tga)])
def test_8bit_writers_hold_the_reference_pixels(omv, oracle, tmp_path, ext, reader):
    g = golden("post")
    img = g["tonemap_0.5"]
    path = tmp_path / f"out.{ext}"
    assert _save(omv, path, img) == 0
    # flipVerticallyOnWrite(true): the buffer's last row is the picture's top row
    assert np.array_equal(reader(path), g["rgba8"][::-1])


def test_pfm_writer_matches_savepfm(omv, tmp_path):
    img = golden("post")["image"]
    path = tmp_path / "out.pfm"
    assert _save(omv, path, img) == 0
    b = open(path, "rb").read()
    head = b"PF\n23 37\n-1.000000\n"
    assert b[:len(head)] == head
    rgb = np.frombuffer(b[len(head):], dtype="<f4").reshape(37, 23, 3)
    assert np.array_equal(rgb.view(np.uint32), img[..., :3].view(np.uint32))


def test_large_png_spans_several_deflate_blocks(omv, tmp_path):
    rng = np.random.default_rng(3)
    img = rng.uniform(0, 1, (130, 200, 4)).astype(np.float32)
    path = tmp_path / "big.png"
    assert _save(omv, path, img) == 0
    want = np.clip(255.0 * img, 0, 255).astype(np.uint8)[::-1]
    assert np.array_equal(_read_png(path), want)


def test_writer_argument_errors(omv, tmp_path):
    img = np.zeros((2, 2, 4), dtype=np.float32)
    assert _save(omv, tmp_path / "x.jpg", img) == 1
    assert b"extension" in omv.lib().omv_last_error()
    assert omv.lib().omv_save_image(b"x.png", None, 2, 2) == 1
    assert _save(omv, tmp_path / "no_such_dir" / "x.png", img) == 1
