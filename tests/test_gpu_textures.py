"""Textured PBR materials on the GPU (base colour with texture transform and
wrapping, packed metallic-roughness-occlusion, normal maps, separate occlusion,
emission, texture-alpha masking and blending, a second coordinate set) against
the oracle, which reproduces the reference's film of the same scene bit for bit
(tests/test_oracle.py).  The bitmap lookup and everything decided by it before
any random draw (masked hits, the validation subjects) are bit-exact; images are
statistical like every other render."""
import os

import numpy as np
import pytest
from conftest import golden

from test_gpu_render import _params, _render, _zstats

pytestmark = pytest.mark.gpu


def test_device_texture_lookup_matches_reference(gpu):
    g = golden("texture")
    for k in range(3):
        y = gpu.texture_sample(g[f"img{k}"], g[f"uv{k}"])
        assert np.array_equal(y.view(np.uint32), g[f"y{k}"].view(np.uint32)), k


@pytest.fixture(scope="module")
def textured(gpu, oracle, scenes):
    sc = scenes.scene_textured(48, 48, 1)
    return sc, gpu.RenderScene(sc), oracle.OracleScene(sc)


def test_texture_masked_hits_match_oracle(gpu, oracle, textured):
    """Primary hits skip texels of the MASK material below the cutoff exactly
    where the reference does."""
    sc, rs, osc = textured
    seed = 77
    rays, o_hits = osc.render_ids(seed=seed)
    jitter = oracle.mt_uniforms(seed, 2 * sc.camera.width * sc.camera.height)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    hits, _ = r.render_ids(gpu.PinholeCamera.from_spec(sc.camera), jitter=jitter)
    assert np.array_equal(hits["inst"], o_hits["inst"]) and np.array_equal(hits["prim"], o_hits["prim"])
    masked_mesh = 2  # ball2 carries the MASK material
    seen = hits["geom"] == masked_mesh
    assert 0 < seen.mean() < 0.2


@pytest.mark.parametrize("name", ["rmp", "mmp", "in"])
def test_textured_validation_subjects_match_oracle(gpu, textured, name):
    sc, rs, osc = textured
    code = gpu.fc_subject(name)
    o_rgba, o_args, uni, _ = osc.render_fc(code)
    rgba, args, _ = gpu.render_fc(rs, gpu.PinholeCamera.from_spec(sc.camera), code, uniforms=uni)
    assert np.array_equal(args, o_args)
    assert np.array_equal(rgba.view(np.uint32), o_rgba.view(np.uint32))
    if name != "in":
        assert len(np.unique(o_args)) > 20  # texture-modulated factors


def test_textured_scene_statistically_matches_oracle(gpu, oracle, textured):
    sc, rs, osc = textured
    n_cpu = 4096
    film, sumsq, _ = osc.render(params=_params(oracle, sc, n_cpu), mode=1, threads=os.cpu_count() or 8, seed=5,
                                variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n = 8192
    _, s, q, cnt, st = _render(gpu, sc, n, seed=2)
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


def test_emission_adds_radiance(gpu, scenes):
    import dataclasses

    sc = scenes.scene_textured(32, 32, 1)
    dark = dataclasses.replace(sc, materials=[dataclasses.replace(m, emissive_factor=(0.0, 0.0, 0.0))
                                              for m in sc.materials])
    a = _render(gpu, sc, 256, seed=3)[1].mean()
    b = _render(gpu, dark, 256, seed=3)[1].mean()
    assert a > b


def test_adjoint_rejects_textured_materials(gpu, textured):
    import ctypes as C

    torch = pytest.importorskip("torch")
    sc, rs, _ = textured
    cam = gpu.PinholeCamera.from_spec(sc.camera).to_c()
    p = gpu.RendererParameters.for_scene(sc, samplesPerPixel=1).to_c()
    a = torch.zeros((sc.camera.height, sc.camera.width, 3), dtype=torch.float32, device="cuda")
    g = torch.zeros((len(sc.materials), 11), dtype=torch.float32, device="cuda")
    st = gpu.lib().omv_adjoint(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(a.data_ptr()),
                               C.c_void_p(g.data_ptr()), None)
    assert st == 1 and b"untextured" in gpu.lib().omv_last_error()


def test_textured_scene_deep_paths_statistically_match_oracle(gpu, oracle, scenes):
    """Seven camera bounces on the alpha-masked textured scene under a sky (no
    point light), rendered in calls of 2^18 paths: from bounce 3 on the tail
    kernel takes over (one thread per path to its end, masked hits retried)
    and the image still matches the oracle's."""
    import dataclasses
    import math

    sc = scenes.scene_textured(32, 32, 1)
    R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], dtype=np.float32)
    sky = scenes.make_sky(256, 128, np.random.default_rng(4), suns=False)
    sc = dataclasses.replace(sc, lights=[], hdri=scenes.Hdri(sky, R, float(np.float32(math.pi))),
                             render=dataclasses.replace(sc.render, camera_bounces=7, max_path_length=9))
    osc = oracle.OracleScene(sc)
    n_cpu = 4096
    film, sumsq, _ = osc.render(params=_params(oracle, sc, n_cpu), mode=1, threads=os.cpu_count() or 8, seed=6,
                                variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n, chunk = 8192, 256
    s = q = 0.0
    for off in range(0, n, chunk):
        _, s1, q1, _, st = _render(gpu, sc, chunk, seed=3, sample_offset=off)
        assert st["tail_bounce"] == 3 and st["tail_nodes_visited"] > 0
        s, q = s + s1, q + q1
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
