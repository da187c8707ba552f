"""Radiance .hdr decoding (scenes.decode_hdr) against the reference's own
loader: stb_image's stbi_loadf as HDRBackground calls it (HdrBackground.cpp:42),
run on flat and run-length files, both signatures, extra header lines, the
widths at the run-length limits, the fallback to flat pixels after a scanline
without the run-length marker, and zero exponents (tests/golden/hdr.npz, made
by tests/golden/make_golden.py through oracle/golden_harness.cpp)."""
import importlib
import os

import numpy as np
import pytest
from conftest import golden


@pytest.fixture(scope="module")
def gl():
    return importlib.import_module("openmaterial-validation_gb300.gltf")


def test_decode_matches_stb(scenes):
    g = golden("hdr")
    for i in range(int(g["count"])):
        got = scenes.decode_hdr(g[f"file{i}"].tobytes())
        want = g[f"rgb{i}"]
        assert got.shape == want.shape, i
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), i


def test_writer_round_trip_flat_and_run_length(scenes, tmp_path):
    rng = np.random.default_rng(4)
    img = scenes.rgbe_quantize(np.exp(rng.normal(size=(6, 200, 3))).astype(np.float32))
    img[:, 20:180] = img[:, 20:21]
    img[0, 0] = (2.0, 1.0, 0.5)
    for rle in (False, True):
        p = str(tmp_path / f"x{int(rle)}.hdr")
        scenes.write_hdr(p, img, rle=rle)
        assert np.array_equal(scenes.read_hdr(p), img)
    assert os.path.getsize(str(tmp_path / "x1.hdr")) < os.path.getsize(str(tmp_path / "x0.hdr"))


def test_malformed_files_raise(scenes):
    g = golden("hdr")
    raw = g["file1"].tobytes()
    with pytest.raises(ValueError):
        scenes.decode_hdr(raw[:-7])  # ends inside the pixel data
    with pytest.raises(ValueError):
        scenes.decode_hdr(b"#?RADIANCE\nFORMAT=32-bit_rgbe\n\n-Y 1 +X 1\n\x80\x80\x80\x80")
    with pytest.raises(ValueError):
        scenes.decode_hdr(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n+X 1 -Y 1\n\x80\x80\x80\x80")
    with pytest.raises(ValueError):
        scenes.decode_hdr(b"P6\n1 1\n255\n\x00\x00\x00")


def test_load_hdri_sets_the_reference_background(gl, scenes, tmp_path):
    g = golden("hdr")
    p = str(tmp_path / "sky.hdr")
    with open(p, "wb") as fh:
        fh.write(g["file3"].tobytes())
    h = gl.load_hdri(p)
    assert np.array_equal(h.rgb, g["rgb3"])
    assert np.array_equal(h.rotation, np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], np.float32))
    assert h.scale == float(np.float32(np.pi))
