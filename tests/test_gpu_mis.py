"""The MIS estimator (OMV_ESTIMATOR_MIS): HDRI alias-table connections at PBR
camera vertices weighted against the reference sampler by the power
heuristic.  Both strategies estimate the reference sampler's own integrand and
the connection ray is traced as a sampled ray in that direction would be, so
the image must converge to the reference estimator's (statistical checks on
the same scene at high sample counts) while its variance falls where the
environment has small bright features.

Statistics: per pixel and channel z = (mis - ref) / sqrt(se_mis^2 + se_ref^2)
(tests/test_gpu_render.py) on scenes the reference estimator samples well;
under the sun lobes (a pixel sees a 1e4 lobe through a few samples in 32768)
only the image mean and the variance are compared."""
import dataclasses

import numpy as np
import pytest

from test_gpu_render import _zstats

pytestmark = pytest.mark.gpu


def _render(gpu, sc, spp, seed, estimator):
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=seed, accumulate_variance=True,
                                                      estimator=estimator))
    _, s, q, _ = r.render(gpu.PinholeCamera.from_spec(sc.camera), sums=True)
    mean = s / spp
    return mean, np.maximum(q / spp - mean ** 2, 0.0)


def _plane(scenes, rough, metal):
    """A 100 x 100 plane under the sky, seen by a camera whose forward vector
    is not unit length (so camera rays are not unit length either)."""
    F32 = np.float32
    base = scenes.scene_c2(40, 24, 1, tri_scale=0.02, suns=False, sky_size=(256, 128))
    qv = np.array([[-50, -2, -50], [50, -2, -50], [50, -2, 50], [-50, -2, 50]], F32)
    qf = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)
    cam = dataclasses.replace(scenes.camera_default(40, 24, 60.0),
                              rotation=scenes.default_view((0, 0, 0), (0, -0.6, -1), (0, 1, 0)))
    mat = scenes.Material(type=0, base_color=(0.8, 0.6, 0.4, 1.0), metallic=metal, roughness=rough)
    mesh = scenes.Mesh(positions=qv, faces=qf, normals=np.tile(np.array([0, 1, 0], F32), (4, 1)), material=0)
    return dataclasses.replace(base, meshes=[mesh], instances=[scenes.Instance(np.eye(4, dtype=F32), 0)],
                               materials=[mat], lights=[], camera=cam, render=scenes.RenderSpec(1, 2, 2, 3))


@pytest.mark.parametrize("rough,metal", [(1.0, 0.0), (0.35, 1.0), (0.6, 0.3)])
def test_mis_plane_matches_the_reference_estimator(gpu, scenes, rough, metal):
    """Diffuse, glossy metal and mixed: the glossy lobe's density needs the
    unit incoming direction, and grazing sampled rays re-hit the plane from
    the reference's shifted origin, which the connections must reproduce."""
    sc = _plane(scenes, rough, metal)
    n = 16384
    m_mis, v_mis = _render(gpu, sc, n, 3, gpu.ESTIMATOR_MIS)
    m_ref, v_ref = _render(gpu, sc, n, 4, gpu.ESTIMATOR_REFERENCE)
    frac3, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
    assert v_mis.mean() < v_ref.mean(), (v_mis.mean(), v_ref.mean())


def test_mis_converges_to_the_reference_estimator(gpu, scenes):
    sc = scenes.scene_c2(40, 24, 1, tri_scale=0.02, suns=False, sky_size=(256, 128))
    n = 32768
    m_mis, v_mis = _render(gpu, sc, n, 7, gpu.ESTIMATOR_MIS)
    m_ref, v_ref = _render(gpu, sc, n, 8, gpu.ESTIMATOR_REFERENCE)
    frac3, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
    assert v_mis.mean() < v_ref.mean(), (v_mis.mean(), v_ref.mean())


def test_mis_under_suns_matches_and_cuts_variance(gpu, scenes):
    """Three 1e4 sun lobes: connections find them, sampled escapes rarely do.
    Per pixel the reference is too heavy-tailed at this sample count for a z
    test (a pixel whose samples missed the lobes understates both its mean and
    its variance, and one that hit them gets a variance that hides any
    difference), so the bars are the image mean (31M samples a side) and the
    variance, which must fall at least 10x."""
    sc = scenes.scene_c2(40, 24, 1, tri_scale=0.02, suns=True, sky_size=(256, 128))
    n = 32768
    m_mis, v_mis = _render(gpu, sc, n, 7, gpu.ESTIMATOR_MIS)
    m_ref, v_ref = _render(gpu, sc, n, 8, gpu.ESTIMATOR_REFERENCE)
    _, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert abs(glob) < 4, glob
    assert v_mis.mean() < 0.1 * v_ref.mean(), (v_mis.mean(), v_ref.mean())


def test_mis_with_point_light_matches_the_reference_estimator(gpu, scenes):
    """Sky and a point light: light-vertex connections and environment rays
    share the shadow queue."""
    sc = scenes.scene_materials(32, 32, 1, tris=20_000, bounces=4, sky=True)
    n = 8192
    m_mis, v_mis = _render(gpu, sc, n, 5, gpu.ESTIMATOR_MIS)
    m_ref, v_ref = _render(gpu, sc, n, 6, gpu.ESTIMATOR_REFERENCE)
    frac3, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


def test_mis_with_alpha_masked_textures_matches_the_reference_estimator(gpu, scenes):
    """Texture-masked and alpha-masked materials under a sky: environment rays
    then take sceneIntersect's closest hit with masked-material retries, as
    the sampled rays do; textured PBR vertices connect with their texel values."""
    import math

    sc = scenes.scene_textured(32, 32, 1)
    R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], dtype=np.float32)
    sky = scenes.make_sky(256, 128, np.random.default_rng(3), suns=False)
    sc = dataclasses.replace(sc, hdri=scenes.Hdri(sky, R, float(np.float32(math.pi))))
    n = 8192
    m_mis, v_mis = _render(gpu, sc, n, 5, gpu.ESTIMATOR_MIS)
    m_ref, v_ref = _render(gpu, sc, n, 6, gpu.ESTIMATOR_REFERENCE)
    frac3, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob


def test_mis_batch_matches_separate_renders(gpu, scenes):
    """A batch under the MIS estimator, captured as a graph on its first call
    (the environment table is built before the capture), gives each job the
    film of a separate MIS render: counts exactly, sums to FP32 rounding of the
    shadow contributions' atomic order."""
    import ctypes as C

    torch = pytest.importorskip("torch")
    sc = scenes.scene_materials(32, 32, 1, tris=20_000, bounces=4, sky=True)
    sets = scenes.material_variants(sc, 2, seed=5)
    rs = gpu.RenderScene(sc)
    br = gpu.BatchRenderer(rs, gpu.RendererParameters.for_scene(sc, estimator=gpu.ESTIMATOR_MIS))
    br.set_material_sets(sets)
    specs = [(32, 24, 4, 11, -1), (16, 16, 9, 12, 0), (24, 40, 5, 13, 1)]
    films, jobs = [], []
    for w, h, spp, seed, ms in specs:
        f = (torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"), None,
             torch.zeros((h, w), dtype=torch.int32, device="cuda"))
        cam = gpu.PinholeCamera.from_spec(sc.camera)
        cam.width, cam.height = w, h
        cam.adjust_to_resolution()
        films.append((f, cam))
        jobs.append(br.job(cam, spp, f, seed=seed, material_set=ms))
    br.render(jobs, graph=True)
    torch.cuda.synchronize()
    for (w, h, spp, seed, ms), (f, cam) in zip(specs, films):
        mats = sc.materials if ms < 0 else sets[ms]
        rs2 = gpu.RenderScene(dataclasses.replace(sc, materials=mats))
        s = torch.zeros((h, w, 3), dtype=torch.float64, device="cuda")
        c = torch.zeros((h, w), dtype=torch.int32, device="cuda")
        p = gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=seed, estimator=gpu.ESTIMATOR_MIS).to_c()
        cc = cam.to_c()
        gpu.check(gpu.lib().omv_render_device(rs2.handle, C.byref(cc), C.byref(p), C.c_void_p(s.data_ptr()), None,
                                              C.c_void_p(c.data_ptr()), None, None))
        torch.cuda.synchronize()
        assert bool((f[2] == c).all())
        assert float((f[0] - s).abs().max()) <= 1e-5 * float(s.abs().max())


def test_mis_scene_without_environment_is_the_reference(gpu, scenes):
    sc = scenes.scene_c1(16, 16, 1)
    a, _ = _render(gpu, sc, 64, 3, gpu.ESTIMATOR_MIS)
    b, _ = _render(gpu, sc, 64, 3, gpu.ESTIMATOR_REFERENCE)
    assert np.array_equal(a, b)


def test_mis_rejected_where_unsupported(gpu, scenes):
    import ctypes as C

    torch = pytest.importorskip("torch")
    sc = scenes.scene_c2(8, 8, 1, tri_scale=0.01, suns=False, sky_size=(64, 32))
    rs = gpu.RenderScene(sc)
    cam = gpu.PinholeCamera.from_spec(sc.camera).to_c()
    p = gpu.RendererParameters.for_scene(sc, samplesPerPixel=1, estimator=gpu.ESTIMATOR_MIS).to_c()
    s = torch.zeros((8, 8, 3), dtype=torch.float64, device="cuda")
    n = torch.zeros((8, 8), dtype=torch.int32, device="cuda")
    L = gpu.lib()
    assert L.omv_render_device_static(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(s.data_ptr()), None,
                                      C.c_void_p(n.data_ptr()), None) == 1
    assert b"MIS" in L.omv_last_error()
    # the adjoint replays the reference estimator only (8 materials: within its limits)
    sm = scenes.scene_materials(8, 8, 1, tris=20_000, bounces=4, sky=True)
    rm = gpu.RenderScene(sm)
    cm = gpu.PinholeCamera.from_spec(sm.camera).to_c()
    pm = gpu.RendererParameters.for_scene(sm, samplesPerPixel=1, estimator=gpu.ESTIMATOR_MIS).to_c()
    adj = torch.zeros((cm.height, cm.width, 3), dtype=torch.float32, device="cuda")
    grad = torch.zeros((len(sm.materials), 11), dtype=torch.float32, device="cuda")
    assert L.omv_adjoint(rm.handle, C.byref(cm), C.byref(pm), C.c_void_p(adj.data_ptr()),
                         C.c_void_p(grad.data_ptr()), None) == 1
    assert b"reference estimator" in L.omv_last_error()
    p.estimator = 7
    assert L.omv_render(rs.handle, C.byref(cam), C.byref(p), None, None, None, None, None) == 1


def test_mis_in_the_tail_kernel_matches_the_reference_estimator(gpu, scenes):
    """Frames of at most 2^18 paths: from bounce 3 on the tail kernel runs
    the MIS estimator's vertices and environment rays (one thread per path),
    and the image still converges to the reference estimator's."""
    sc = scenes.scene_c2(40, 24, 1, tri_scale=0.02, suns=False, sky_size=(256, 128))
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    cam = gpu.PinholeCamera.from_spec(sc.camera)
    n, chunk = 8192, 256
    s = q = 0.0
    for off in range(0, n, chunk):
        r.set_parameters(gpu.RendererParameters.for_scene(sc, samplesPerPixel=chunk, seed=11, sample_offset=off,
                                                          accumulate_variance=True, estimator=gpu.ESTIMATOR_MIS))
        _, s1, q1, _ = r.render(cam, sums=True)
        assert r.last_stats["tail_bounce"] == 3
        s, q = s + s1, q + q1
    m_mis = s / n
    v_mis = np.maximum(q / n - m_mis ** 2, 0.0)
    m_ref, v_ref = _render(gpu, sc, n, 12, gpu.ESTIMATOR_REFERENCE)
    frac3, glob = _zstats(m_mis, n, v_mis, m_ref, n, v_ref)
    assert frac3 < 0.01, frac3
    assert abs(glob) < 4, glob
