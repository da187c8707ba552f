"""The GPU wavefront BDPT against the reference estimator.

Random streams differ (counter-based Philox on the GPU, one std::mt19937 in the
reference), so image parity is statistical: per pixel and channel
z = (gpu - ref) / sqrt(se_gpu^2 + se_ref^2).  This estimator is heavy-tailed
(rare light-vertex connections, the missing material's albedo 1000), so a
per-pixel sample variance taken from a few hundred samples underestimates the
spread: two CPU runs of the identical algorithm at 256 and 4096 spp put 3.7% of
the pixel-channels of the mixed scene beyond 3 sigma.  Bars therefore:
  * both sides >= 4096 spp, each with its own sample variance: at most 1% of
    pixel-channels beyond 3 sigma, image mean within 4 combined standard errors (false-alarm rate 6e-5);
  * against the reference's own film (mean only, 1024 spp; the GPU variance
    stands in for both sides): at most 2% beyond 3 sigma (the CPU-vs-CPU spread
    of the same estimator) and the image mean within 4 standard errors;
  * pixels a side never saw a non-zero sample in count as outliers when the
    other side's mean differs (rare events)."""
import os

import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu


def _render(gpu, sc, spp, seed=1, variance=True, **kw):
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=seed,
                                                      accumulate_variance=variance, **kw))
    img, s, q, cnt = r.render(gpu.PinholeCamera.from_spec(sc.camera), sums=True)
    return img, s, q, cnt, r.last_stats


def _zstats(mean_a, n_a, var_a, mean_b, n_b, var_b):
    """Returns (fraction of pixel-channels beyond 3 sigma, global z)."""
    # non-finite means come from infinite samples (the reference's film has one:
    # a single infinite contribution overflowed its FP32 sum); they are excluded
    # and must stay rare
    fin = np.isfinite(mean_a) & np.isfinite(mean_b) & np.isfinite(var_a) & np.isfinite(var_b)
    assert np.count_nonzero(~fin) <= 1e-4 * mean_a.size + 3, np.count_nonzero(~fin)
    mean_a, mean_b = np.where(fin, mean_a, 0.0), np.where(fin, mean_b, 0.0)
    var_a, var_b = np.where(fin, var_a, 0.0), np.where(fin, var_b, 0.0)
    se2 = var_a / n_a + var_b / n_b
    live = se2 > 0
    z = np.zeros_like(mean_a)
    z[live] = (mean_a[live] - mean_b[live]) / np.sqrt(se2[live])
    dead_out = (~live) & (np.abs(mean_a - mean_b) > 1e-6 * max(1.0, float(np.abs(mean_b).max())))
    frac3 = (np.count_nonzero(np.abs(z[live]) > 3) + np.count_nonzero(dead_out)) / mean_a.size
    tot_se = np.sqrt(se2.sum())
    glob = (mean_a.sum() - mean_b.sum()) / tot_se if tot_se > 0 else 0.0
    return frac3, glob


def test_c1_statistically_matches_reference(gpu, scenes):
    g = golden("film_c1_64x1024")
    n_ref = int(g["spp"])
    sc = scenes.scene_c1(64, 64, 1)
    n = 16384
    img, s, q, cnt, st = _render(gpu, sc, n)
    assert (cnt == n).all()
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    ref = g["film"][..., :3].astype(np.float64)
    frac3, glob = _zstats(mean, n, var, ref, n_ref, var)
    assert frac3 < 0.02, frac3
    assert abs(glob) < 4, glob
    assert np.allclose(img[..., :3], mean, rtol=1e-6, atol=1e-6)
    assert st["shadow_rays"] > 0 and st["light_rays"] > 0


def test_mixed_materials_statistically_match_oracle(gpu, oracle, scenes):
    sc = scenes.scene_mixed(48, 48, 1)
    n_cpu = 4096
    film, sumsq, _ = oracle.OracleScene(sc).render(params=_params(oracle, sc, n_cpu), mode=1,
                                                   threads=os.cpu_count() or 8, seed=5, variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n = 8192
    _, s, q, cnt, _ = _render(gpu, sc, n, seed=2)
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


def _params(oracle, sc, spp):
    p = oracle.capi.params_for(sc, spp=spp)
    return p


def test_environment_scene_statistically_matches_oracle(gpu, oracle, scenes):
    """Instanced PBR scene lit by an HDRI (escape term, GGX/diffuse branches,
    rotated and scaled instances), GPU vs oracle."""
    sc = scenes.scene_c2(40, 24, 1, tri_scale=0.02, suns=False, sky_size=(256, 128))
    n_cpu = 8192
    film, sumsq, _ = oracle.OracleScene(sc).render(params=_params(oracle, sc, n_cpu), mode=1,
                                                   threads=os.cpu_count() or 8, seed=3, variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n_cpu - ref ** 2, 0.0)
    n = 32768
    _, s, q, cnt, st = _render(gpu, sc, n, seed=4)
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n_cpu, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
    assert st["shadow_rays"] == 0 and st["light_rays"] == 0


def test_benchmark_scene_with_sun_lobes_statistically_matches_oracle(gpu, oracle, scenes):
    """The benchmark frame's own scene: all 1,048,576 triangles in 64 instances
    and the 2048x1024 sky with its three 1e4 sun lobes, at 96x54 (the camera
    and everything else as in the 1920x1080 frame).  Equal sample counts on
    both sides: with the sun lobes the per-pixel sample variance of the side
    with fewer samples underestimates its spread (two CPU runs of 8192 and
    32768 spp put 1.07% of pixel-channels beyond 3 sigma; 8192 vs 8192,
    three seed pairs: 0.35-0.50%, global z within 2.3)."""
    sc = scenes.scene_c2(96, 54, 1)
    assert sc.num_triangles == 1_048_576 and sc.hdri.rgb.shape[:2] == (1024, 2048)
    n = 8192
    film, sumsq, _ = oracle.OracleScene(sc).render(params=_params(oracle, sc, n), mode=1,
                                                   threads=os.cpu_count() or 8, seed=13, variance=True)
    ref = film[..., :3].astype(np.float64)
    var_ref = np.maximum(sumsq / n - ref ** 2, 0.0)
    _, s, q, cnt, st = _render(gpu, sc, n, seed=14)
    assert (cnt == n).all()
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    frac3, glob = _zstats(mean, n, var, ref, n, var_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


def test_same_seed_same_image_and_partition_invariance(gpu, scenes):
    sc = scenes.scene_c1(64, 64, 1)
    _, a, _, _, _ = _render(gpu, sc, 64, seed=9, variance=False)
    _, b, _, _, _ = _render(gpu, sc, 64, seed=9, variance=False)
    _, c, _, _, _ = _render(gpu, sc, 64, seed=9, variance=False, wave_paths=10007)
    _, d, _, _, _ = _render(gpu, sc, 64, seed=10, variance=False)
    scale = np.abs(a).max()
    assert np.abs(a - b).max() <= 1e-6 * scale
    assert np.abs(a - c).max() <= 1e-6 * scale
    assert np.abs(a - d).max() > 1e-3 * scale


def test_sample_offset_continues_the_sequence(gpu, scenes):
    """Rendering spp in two calls (sample_offset) equals one call."""
    sc = scenes.scene_c1(32, 32, 1)
    _, a, _, _, _ = _render(gpu, sc, 32, seed=3, variance=False)
    _, b1, _, _, _ = _render(gpu, sc, 16, seed=3, variance=False)
    _, b2, _, _, _ = _render(gpu, sc, 16, seed=3, variance=False, sample_offset=16)
    assert np.abs(a - (b1 + b2)).max() <= 1e-6 * np.abs(a).max()


def test_large_scene_frame_properties(gpu, scenes):
    sc = scenes.scene_c2(192, 108, 1)
    img, s, q, cnt, st = _render(gpu, sc, 8, variance=False)
    assert (cnt == 8).all()
    assert np.isfinite(img).all() and (img[..., :3] >= 0).all()
    assert (img[..., 3] == 1).all()
    assert st["paths"] == 192 * 108 * 8
    assert st["extension_rays"] >= st["paths"]
    assert st["stack_overflows"] == 0
    assert img[..., :3].mean() > 0


def test_benchmark_frame_partition_invariance(gpu, scenes):
    """The benchmark frame at full size (1920x1080, 64 spp, 1,048,576 triangles
    in 64 instances, 132.7M paths): one wave, waves of 30,000,001 paths (wave
    boundaries inside pixels) and two calls of 32 samples (sample_offset) give
    the same film up to FP64 summation order, every pixel with 64 samples."""
    sc = scenes.scene_c2(1920, 1080, 64)
    _, a, _, ca, st = _render(gpu, sc, 64, seed=5, variance=False)
    _, b, _, cb, _ = _render(gpu, sc, 64, seed=5, variance=False, wave_paths=30_000_001)
    _, c1, _, cc1, _ = _render(gpu, sc, 32, seed=5, variance=False)
    _, c2, _, cc2, _ = _render(gpu, sc, 32, seed=5, variance=False, sample_offset=32)
    assert st["paths"] == 1920 * 1080 * 64
    assert (ca == 64).all() and (cb == 64).all() and ((cc1 + cc2) == 64).all()
    assert np.isfinite(a).all() and (a >= 0).all()
    scale = np.abs(a).max()
    assert np.abs(a - b).max() <= 1e-9 * scale
    assert np.abs(a - (c1 + c2)).max() <= 1e-9 * scale


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "golden", "film_c1_256x4096.npz")),
                    reason="4096-spp reference film not generated")
def test_c1_full_resolution_4096spp_rel_rmse(gpu, scenes):
    """C1 at 256x256 and 4096 spp on both sides: every pixel within the
    combined Monte Carlo error (3 sigma, at most 1% outliers) and relative RMSE
    of the GPU image against the reference image under 1%."""
    g = golden("film_c1_256x4096")
    sc = scenes.scene_c1(256, 256, 1)
    n = 4096
    _, s, q, cnt, _ = _render(gpu, sc, n, seed=21)
    mean = s / n
    var = np.maximum(q / n - mean ** 2, 0.0)
    ref = g["film"][..., :3].astype(np.float64)
    frac3, glob = _zstats(mean, n, var, ref, int(g["spp"]), var)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
    fin = np.isfinite(ref)
    rel_rmse = np.sqrt(np.mean((mean - ref)[fin] ** 2)) / ref[fin].mean()
    assert rel_rmse < 0.01, rel_rmse


def test_wave_that_does_not_fit_is_out_of_memory_and_the_handle_recovers(gpu, scenes):
    """A requested wave whose path state exceeds the device memory (2e9 paths,
    hundreds of GB) fails with OMV_ERR_OUT_OF_MEMORY before any launch; the
    same renderer then renders normally, identical to a fresh one."""
    sc = scenes.scene_c1(32, 32, 1)
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    huge = scenes.camera_default(1920, 1080)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=1024, wave_paths=2_000_000_000))
    with pytest.raises(gpu.OmvError) as e:
        r.render(gpu.PinholeCamera.from_spec(huge))
    assert "status 3" in str(e.value)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=16, seed=4))
    a = r.render(gpu.PinholeCamera.from_spec(sc.camera))
    b = _render(gpu, sc, 16, seed=4, variance=False)[0]
    assert np.isfinite(a).all()
    assert np.abs(a - b).max() <= 1e-6 * np.abs(b).max()
