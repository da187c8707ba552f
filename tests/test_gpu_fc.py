"""The device false-colour pass (k_fc through omv_render_fc) and the light-box
views against the oracle, which reproduces the reference's -F and -V output
bit for bit (tests/test_fc.py).  The device is given the oracle's uniforms, so
hits, ids, names, flags, clamped material factors and their colours are
bit-exact; the density and gradient subjects go through device logf / powf and
agree to 1e-5.  The light box: bounds and cameras bit-exact, the 8 views as one
batch equal to 8 separate renders, and view 0 statistically equal to the
oracle."""
import os

import numpy as np
import pytest

from test_fc import SUBJECTS, _palette_from_film, _world_bounds
from test_gpu_render import _zstats

pytestmark = pytest.mark.gpu

FLOAT_ATOL = 1e-5


@pytest.fixture(scope="module")
def fc(gpu, oracle, scenes):
    sc = scenes.scene_validation(64, 48)
    return sc, gpu.RenderScene(sc), oracle.OracleScene(sc)


def _palette(n, seed=3):
    rng = np.random.default_rng(seed)
    return rng.integers(1, 0xFFFFFF, size=n, dtype=np.uint32)


@pytest.mark.parametrize("name", list(SUBJECTS))
def test_fc_pass_matches_oracle(gpu, fc, name):
    sc, rs, osc = fc
    code = SUBJECTS[name]
    pal = _palette(4000)
    o_rgba, o_args, uni, o_hits = osc.render_fc(code, palette=pal)
    rgba, args, hits = gpu.render_fc(rs, gpu.PinholeCamera.from_spec(sc.camera), code, palette=pal, uniforms=uni)
    assert np.array_equal(hits["inst"], o_hits["inst"]) and np.array_equal(hits["prim"], o_hits["prim"])
    hit = (hits["inst"] != 0xFFFFFFFF).reshape(args.shape)
    assert hit.mean() > 0.3
    assert np.all(args[~hit] == 0) and np.all(rgba[~hit][:, :3] == 0) and np.all(rgba[..., 3] == 1)
    if name in ("md", "sg"):
        f, of = args.view(np.float32), o_args.view(np.float32)
        assert np.all(np.abs(f - of) <= FLOAT_ATOL), np.abs(f - of).max()
        assert np.all(np.abs(rgba - o_rgba) <= FLOAT_ATOL)
        assert len(np.unique(of[hit])) > 10
    elif name == "in":
        # the missing material's flag depends on a hemisphere direction built
        # with device sincosf: a direction within rounding of the face plane
        # may flip; the other materials use the camera ray and are exact
        missing = (hits["material"] == len(sc.materials)).reshape(args.shape)
        assert np.array_equal(args[~missing], o_args[~missing])
        assert np.mean(args[missing] == o_args[missing]) >= 0.99
        assert args[hit & ~missing].any()  # the inside-out ball
    else:
        assert np.array_equal(args, o_args)
        assert np.array_equal(rgba.view(np.uint32), o_rgba.view(np.uint32))


def test_fc_pass_reproduces_reference_film(gpu, fc):
    """Device colours on the reference's own uniforms and recovered palettes
    equal the reference's -F films (the md/sg subjects to 1e-5)."""
    from conftest import golden

    sc, rs, osc = fc
    g = golden("fc")
    for name, code in SUBJECTS.items():
        _, o_args, uni, o_hits = osc.render_fc(code)
        hit = (o_hits["inst"] != 0xFFFFFFFF).reshape(o_args.shape)
        pal = None
        if name in ("pid", "gid", "mid"):
            pal = _palette_from_film(g[name][hit], o_args[hit], missing_pink=name == "mid")
        rgba, _, _ = gpu.render_fc(rs, gpu.PinholeCamera.from_spec(sc.camera), code, palette=pal, uniforms=uni)
        tol = FLOAT_ATOL if name in ("md", "sg") else 0.0
        if name == "in":
            missing = o_hits["material"].reshape(o_args.shape) == len(sc.materials)
            assert np.mean(np.all(rgba == g[name], axis=-1)[missing]) >= 0.99
            assert np.array_equal(rgba[~missing], g[name][~missing])
        else:
            assert np.all(np.abs(rgba - g[name]) <= tol), name


def test_fc_philox_pass_and_density_extremes(gpu, fc):
    sc, rs, osc = fc
    cam = gpu.PinholeCamera.from_spec(sc.camera)
    a1 = gpu.render_fc(rs, cam, "gid", seed=5)[1]
    a2 = gpu.render_fc(rs, cam, "gid", seed=5)[1]
    assert np.array_equal(a1, a2)
    _, args, hits = gpu.render_fc(rs, cam, "md", seed=5)
    hit = (hits["inst"] != 0xFFFFFFFF).reshape(args.shape)
    f = args.view(np.float32)[hit]
    assert np.all((f >= 0) & (f <= 1)) and f.max() > 0.9 and f.min() < 0.1
    assert gpu.fc_subject("nosuch") == 0


def test_fc_argument_errors(gpu, fc):
    sc, rs, _ = fc
    cam = gpu.PinholeCamera.from_spec(sc.camera)
    with pytest.raises(gpu.OmvError, match="subject"):
        gpu.render_fc(rs, cam, 42)
    with pytest.raises(ValueError):
        gpu.render_fc(rs, cam, "pid", uniforms=np.zeros(5, np.float32))


def test_scene_bounds_match_reference_arithmetic(gpu, scenes):
    for sc in (scenes.scene_mixed(32, 32, 1), scenes.scene_validation(16, 16),
               scenes.scene_c2(32, 32, 1, tri_scale=0.01, suns=False, sky_size=(64, 32))):
        lo, hi = gpu.RenderScene(sc).bounds()
        rlo, rhi = _world_bounds(sc)
        assert np.array_equal(lo, rlo) and np.array_equal(hi, rhi), (lo, rlo, hi, rhi)


@pytest.fixture(scope="module")
def lightbox(gpu, scenes):
    import torch

    from conftest import golden

    g = golden("lightbox")
    sc = scenes.scene_mixed(32, 32, int(g["spp"]))
    rs = gpu.RenderScene(sc)
    lo, hi = rs.bounds()
    return torch, g, sc, rs, gpu.lightbox_cameras(lo, hi, 32, 32)


def test_lightbox_cameras_from_device_bounds_match_reference(lightbox):
    torch, g, sc, rs, cams = lightbox
    pos = np.array([c.position[:] for c in cams], dtype=np.float32)
    rot = np.array([[c.rotation[r][:] for r in range(3)] for c in cams], dtype=np.float32)
    assert np.array_equal(pos, g["position"]) and np.array_equal(rot, g["rotation"])
    assert [np.float32(c.focus) for c in cams] == list(g["focus"])


def test_lightbox_batch_equals_separate_renders(gpu, lightbox):
    torch, g, sc, rs, cams = lightbox
    spp = 64
    br = gpu.BatchRenderer(rs, gpu.RendererParameters.for_scene(sc))

    def films():
        return [(torch.zeros((32, 32, 3), dtype=torch.float64, device="cuda"), None,
                 torch.zeros((32, 32), dtype=torch.int32, device="cuda")) for _ in cams]

    batch = films()
    br.render([br.job(c, spp, f, seed=11) for c, f in zip(cams, batch)])
    single = films()
    for c, f in zip(cams, single):
        br.render([br.job(c, spp, f, seed=11)])
    torch.cuda.synchronize()
    for a, b in zip(batch, single):
        assert torch.equal(a[2], b[2]) and bool((a[2] == spp).all())
        # shadow contributions are FP32 atomics: equal up to their rounding
        assert float((a[0] - b[0]).abs().max()) <= 1e-6 * max(1e-30, float(b[0].abs().max()))


def test_lightbox_view0_statistically_matches_oracle(gpu, oracle, lightbox):
    torch, g, sc, rs, cams = lightbox
    cam = cams[0]
    n_cpu = 4096
    p = oracle.capi.params_for(sc, spp=n_cpu)
    film, sumsq, _ = oracle.OracleScene(sc).render(camera=cam, params=p, mode=1, threads=os.cpu_count() or 8,
                                                   seed=5, variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n = 8192
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=n, seed=2, accumulate_variance=True))
    _, s, q, cnt = r.render(_Cam(cam), sums=True)
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


class _Cam:
    """A C camera where the renderer expects a PinholeCamera."""

    def __init__(self, c):
        self.c = c

    def to_c(self):
        return self.c
