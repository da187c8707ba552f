"""Groups of scenes in one handle (omv_scene_create_group): batch jobs and
adjoint jobs that pick their scene.  A job's film (and a replayed gradient)
depends only on its scene, camera, materials, samples and seed, so every job
of a group batch must reproduce the film of its scene rendered alone through
omv_render_device, and every adjoint job the gradient of omv_adjoint on that
scene alone.  Shadow contributions reach a path's radiance through FP32
atomics, so films agree to FP32 summation order (1e-5 of the film's largest
value) and counts exactly; gradients are reduced with atomics too (1e-4)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes(scenes):
    # three different scenes: other geometry seeds, sizes and materials
    return [scenes.scene_materials(40, 32, 1, tris=12_000, bounces=4, n_materials=4, seed=s) for s in (1, 2, 3)]


def _alone(gpu, torch, sc, spp, seed):
    rs = gpu.RenderScene(sc)
    cam = gpu.PinholeCamera.from_spec(sc.camera).to_c()
    p = gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=seed).to_c()
    H, W = cam.height, cam.width
    s = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
    c = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    gpu.check(gpu.lib().omv_render_device(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(s.data_ptr()), None,
                                          C.c_void_p(c.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                          None))
    torch.cuda.synchronize()
    return rs, cam, p, s, c


def test_group_batch_renders_every_scene_as_alone(gpu, scenes):
    torch = pytest.importorskip("torch")
    parts = _scenes(scenes)
    group = gpu.RenderScene.group(parts)
    assert group.material_offsets == [0, 4, 8]
    br = gpu.BatchRenderer(group, gpu.RendererParameters.for_scene(parts[0]))
    jobs, films, want = [], [], []
    for p, sc in enumerate(parts):
        spp, seed = 8 + 4 * p, 40 + p
        _, cam, _, s, c = _alone(gpu, torch, sc, spp, seed)
        want.append((s, c))
        f = (torch.zeros_like(s), None, torch.zeros_like(c))
        films.append(f)
        jobs.append(br.job(cam, spp, f, seed=seed, part=p))
    # the same scene twice in one batch, in reversed order, plus the graph path
    for graph in (False, True):
        for f in films:
            f[0].zero_()
            f[2].zero_()
        br.render(jobs[::-1], graph=graph)
        torch.cuda.synchronize()
        for (s, c), f in zip(want, films):
            assert torch.equal(c, f[2])
            assert float((s - f[0]).abs().max()) <= 1e-5 * float(s.abs().max())


def test_group_scene_zero_answers_the_single_frame_calls(gpu, oracle, scenes):
    """omv_trace_rays on a group traces scene 0: bit-exact hits against the
    oracle on scene 0 alone."""
    parts = _scenes(scenes)
    group = gpu.RenderScene.group(parts)
    rng = np.random.default_rng(3)
    n = 20_000
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3] = rng.uniform([-4, -1, -9], [4, 2, 0], (n, 3))
    d = rng.normal(size=(n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 7] = np.float32(3.402823466e38)
    a, b = group.trace(r), oracle.OracleScene(parts[0]).trace(r)
    for k in ("inst", "prim", "material"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))


def test_group_adjoint_jobs_match_each_scene_alone(gpu, scenes):
    torch = pytest.importorskip("torch")
    parts = _scenes(scenes)
    group = gpu.RenderScene.group(parts)
    br = gpu.BatchRenderer(group, gpu.RendererParameters.for_scene(parts[0]))
    rng = np.random.default_rng(7)
    jobs, adjs, grads, want = [], [], [], []
    for p, sc in enumerate(parts):
        spp, seed = 16, 70 + p
        rs, cam, prm, _, _ = _alone(gpu, torch, sc, spp, seed)
        a = torch.tensor(rng.uniform(-1, 1, (cam.height, cam.width, 3)), dtype=torch.float32, device="cuda")
        g = torch.zeros((len(sc.materials), 11), dtype=torch.float32, device="cuda")
        gpu.check(gpu.lib().omv_adjoint(rs.handle, C.byref(cam), C.byref(prm), C.c_void_p(a.data_ptr()),
                                        C.c_void_p(g.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        want.append(g)
        jobs.append(br.job(cam, spp, (torch.zeros(1, device="cuda"), None, torch.zeros(1, device="cuda")),
                           seed=seed, part=p))
        adjs.append(a)
        grads.append(torch.zeros_like(g))
    br.adjoint(jobs, adjs, grads)
    torch.cuda.synchronize()
    for g, w in zip(grads, want):
        scale = float(w.abs().max())
        assert scale > 0
        assert float((g - w).abs().max()) <= 1e-4 * scale


def test_group_rejects_mixed_lighting_and_bad_parts(gpu, scenes):
    parts = _scenes(scenes)
    dark = scenes.scene_materials(16, 16, 1, tris=2_000, bounces=2, n_materials=2, seed=9)
    dark.lights = []
    with pytest.raises(gpu.OmvError, match="point lights"):
        gpu.RenderScene.group([parts[0], dark])
    torch = pytest.importorskip("torch")
    group = gpu.RenderScene.group(parts[:2])
    br = gpu.BatchRenderer(group, gpu.RendererParameters.for_scene(parts[0]))
    cam = gpu.PinholeCamera.from_spec(parts[0].camera)
    f = (torch.zeros((cam.height, cam.width, 3), dtype=torch.float64, device="cuda"), None,
         torch.zeros((cam.height, cam.width), dtype=torch.int32, device="cuda"))
    with pytest.raises(gpu.OmvError, match="part"):
        br.render([br.job(cam, 4, f, part=2)])


def test_unlit_group_batch_in_the_tail_kernel_matches_each_scene_alone(gpu, scenes):
    """Two scenes under one sky (no point light) as a group batch small enough
    (at most 2^18 paths) that from bounce 3 on the tail kernel runs each path
    to its end with its job's scene, camera and materials: every job still
    reproduces its scene rendered alone (to FP32 summation order)."""
    import dataclasses

    torch = pytest.importorskip("torch")
    a = scenes.scene_c2(24, 16, 1, seed=1, tri_scale=0.01, suns=False, sky_size=(128, 64))
    b = dataclasses.replace(scenes.scene_c2(24, 16, 1, seed=2, tri_scale=0.01, suns=False, sky_size=(128, 64)),
                            hdri=a.hdri)
    parts = [a, b]
    group = gpu.RenderScene.group(parts)
    br = gpu.BatchRenderer(group, gpu.RendererParameters.for_scene(a))
    jobs, films, want = [], [], []
    for p, sc in enumerate(parts):
        spp, seed = 64, 90 + p
        _, cam, _, s, c = _alone(gpu, torch, sc, spp, seed)
        want.append((s, c))
        f = (torch.zeros_like(s), None, torch.zeros_like(c))
        films.append(f)
        jobs.append(br.job(cam, spp, f, seed=seed, part=p))
    st = br.render(jobs, stats=True)
    torch.cuda.synchronize()
    assert st.tail_bounce == 3 and st.tail_nodes_visited > 0
    for (s, c), f in zip(want, films):
        assert torch.equal(c, f[2])
        assert float((s - f[0]).abs().max()) <= 1e-5 * float(s.abs().max())
