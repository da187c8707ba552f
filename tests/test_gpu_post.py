"""Device image development (post.cu through the C ABI) against the
reference's outputs (tests/golden/post.npz) and the oracle's restatement:
the median and the 8-bit conversion are bit-exact; gamma correction agrees to
2e-6 relative, the error bound of the device powf against the host's."""
import importlib

import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu

TONEMAP_RTOL = 2e-6


@pytest.fixture(scope="module")
def post(gpu):
    torch = pytest.importorskip("torch")
    return torch, importlib.import_module("openmaterial-validation_gb300.post")


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(torch, t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


@pytest.mark.parametrize("name,gamma", [("tonemap_0.5", 0.5), ("tonemap_0.4545", 0.4545)])
def test_gamma_correction_matches_reference(post, name, gamma):
    torch, P = post
    g = golden("post")
    y = _host(torch, P.gammaCorrection(_dev(torch, g["image"]), 1.0, gamma))
    ref = g[name]
    assert np.all(y[..., 3] == 1.0)
    assert np.all(np.abs(y - ref) <= TONEMAP_RTOL * np.abs(ref)), np.max(np.abs(y - ref) / np.maximum(ref, 1e-30))
    # clamped and black pixels are exact
    sat = (ref == 1.0) | (ref == 0.0)
    assert np.array_equal(y[sat], ref[sat])


def test_median_matches_reference(post):
    torch, P = post
    g = golden("post")
    y = _host(torch, P.SimpleDenoiserMedian(_dev(torch, g["tonemap_0.5"]), 1))
    assert np.array_equal(y, g["median"])


@pytest.mark.parametrize("half", [1, 2, 3])
@pytest.mark.parametrize("shape", [(7, 5), (67, 45), (300, 171)])
def test_median_matches_oracle_on_ragged_sizes(post, oracle, half, shape):
    torch, P = post
    rng = np.random.default_rng(half * 1000 + shape[0])
    img = rng.uniform(0, 1, shape + (4,)).astype(np.float32)
    img[..., :3] = np.round(img[..., :3] * 16) / 16  # many ties
    y = _host(torch, P.SimpleDenoiserMedian(_dev(torch, img), half))
    assert np.array_equal(y, oracle.median(img, half))


def test_rgba8_matches_reference(post):
    torch, P = post
    g = golden("post")
    x = _dev(torch, g["tonemap_0.5"])
    assert np.array_equal(_host(torch, P.rgba8(x)), g["rgba8"])
    assert np.array_equal(_host(torch, P.rgba8(x, flip=True)), g["rgba8"][::-1])


def test_develop_matches_resolve_tonemap_and_conversion(post, oracle):
    torch, P = post
    rng = np.random.default_rng(5)
    H, W = 131, 77
    count = rng.integers(0, 40, (H, W)).astype(np.int32)
    s = (rng.lognormal(-1.0, 1.5, (H, W, 3)) * count[..., None]).astype(np.float64)
    out = P.develop(_dev(torch, s), _dev(torch, count), gamma=0.5)
    lin = _host(torch, out["linear"])
    c = count.astype(np.float64)[..., None]
    want = np.concatenate([(s * np.where(c < 0.5, 1.0, 1.0 / np.maximum(c, 1))).astype(np.float32),
                           np.ones((H, W, 1), np.float32)], axis=-1)
    assert np.array_equal(lin, want)
    ref = oracle.tonemap(lin, 0.5)
    tm = _host(torch, out["tonemapped"])
    assert np.all(np.abs(tm - ref) <= TONEMAP_RTOL * np.abs(ref))
    assert np.array_equal(_host(torch, out["rgba8"]), _host(torch, P.rgba8(out["tonemapped"], flip=True)))


def test_develop_of_a_render_equals_the_render_image(post, gpu, scenes):
    """omv_develop's linear image of a device film is omv_render's image."""
    torch, P = post
    sc = scenes.scene_c1(64, 48, 4)
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_parameters(gpu.RendererParameters.for_scene(sc, seed=3))
    r.set_scene(rs)
    img, s, _, cnt = r.render(gpu.PinholeCamera.from_spec(sc.camera), sums=True)
    out = P.develop(_dev(torch, s), _dev(torch, cnt.astype(np.int32)), linear=True, tonemapped=False, rgba8=False)
    assert np.array_equal(_host(torch, out["linear"]), img)


def test_full_hd_properties(post, oracle):
    """1920x1080: gamma 1 is the clamp alone, and the median equals the oracle's."""
    torch, P = post
    rng = np.random.default_rng(8)
    img = rng.lognormal(-1.0, 1.0, (1080, 1920, 4)).astype(np.float32)
    x = _dev(torch, img)
    y = _host(torch, P.gammaCorrection(x.clone(), 1.0, 1.0))
    want = np.clip(img, 0, 1)
    want[..., 3] = 1.0
    assert np.array_equal(y, want)
    t = oracle.tonemap(img, 0.5)
    m = _host(torch, P.SimpleDenoiserMedian(_dev(torch, t), 1))
    assert np.array_equal(m, oracle.median(t, 1))


def test_argument_errors(post, gpu):
    torch, P = post
    L = gpu.lib()
    x = torch.zeros((4, 4, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(gpu.OmvError, match="half"):
        P.SimpleDenoiserMedian(x, 4)
    assert L.omv_denoise_median(x.data_ptr(), x.data_ptr(), 4, 4, 1, None) == 1
    assert L.omv_develop(None, None, 4, 4, 1.0, 0.5, None, None, None, 0, None) == 1
    assert L.omv_rgba8(x.data_ptr(), None, 4, 4, 0, None) == 1
    assert L.omv_tonemap(x.data_ptr(), 0, 1.0, 0.5, None) == 0
