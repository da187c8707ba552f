"""Batched rendering (omv_render_batch) against rendering each job on its own.

A batch concatenates the jobs' paths into shared waves; every path keeps the
random numbers of its (job seed, pixel, sample), its job's camera and material
set, and lands in its job's film.  So each job's film must equal a separate
omv_render_device of that job on a scene built with the job's materials: sample
counts exactly, sums up to the order of the FP64 film additions."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _film(torch, w, h):
    return (torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w, 3), dtype=torch.float64, device="cuda"),
            torch.zeros((h, w), dtype=torch.int32, device="cuda"))


def _camera(gpu, sc, w, h):
    cam = gpu.PinholeCamera.from_spec(sc.camera)
    cam.width, cam.height = w, h
    cam.adjust_to_resolution()
    cam.set_y_fov(45.0)
    return cam


def _single(gpu, torch, sc, materials, cam, spp, seed, offset, variance=True):
    """One job on its own scene (built with the job's materials)."""
    import dataclasses
    sc2 = dataclasses.replace(sc, materials=materials)
    rs = gpu.RenderScene(sc2)
    film = _film(torch, cam.width, cam.height)
    p = gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=seed, sample_offset=offset,
                                         accumulate_variance=variance).to_c()
    c = cam.to_c()
    gpu.check(gpu.lib().omv_render_device(rs.handle, C.byref(c), C.byref(p), C.c_void_p(film[0].data_ptr()),
                                          C.c_void_p(film[1].data_ptr()), C.c_void_p(film[2].data_ptr()), None,
                                          None))
    torch.cuda.synchronize()
    return film


def _same(a, b):
    assert bool((a[2] == b[2]).all())
    for k in (0, 1):
        scale = float(a[k].abs().max())
        assert scale > 0
        assert float((a[k] - b[k]).abs().max()) <= 1e-9 * scale


@pytest.fixture(scope="module")
def setup(gpu, scenes):
    torch = pytest.importorskip("torch")
    sc = scenes.scene_materials(32, 32, 4, tris=20_000, bounces=4)
    sets = scenes.material_variants(sc, 3, seed=5)
    rs = gpu.RenderScene(sc)
    br = gpu.BatchRenderer(rs, gpu.RendererParameters.for_scene(sc, accumulate_variance=True))
    br.set_material_sets(sets)
    specs = [(32, 24, 4, 11, -1, 0), (48, 40, 7, 12, 0, 0), (16, 16, 16, 13, 1, 3), (40, 30, 33, 14, 2, 0),
             (24, 24, 9, 15, 0, 5)]
    return torch, sc, sets, rs, br, specs


def test_batch_jobs_match_separate_renders(gpu, setup):
    torch, sc, sets, rs, br, specs = setup
    films, jobs = [], []
    for w, h, spp, seed, ms, off in specs:
        f = _film(torch, w, h)
        films.append(f)
        jobs.append(br.job(_camera(gpu, sc, w, h), spp, f, seed=seed, material_set=ms, sample_offset=off))
    st = br.render(jobs, stats=True)
    torch.cuda.synchronize()
    assert st.paths == sum(w * h * spp for w, h, spp, *_ in specs)
    for (w, h, spp, seed, ms, off), f in zip(specs, films):
        mats = sc.materials if ms < 0 else sets[ms]
        ref = _single(gpu, torch, sc, mats, _camera(gpu, sc, w, h), spp, seed, off)
        assert int(f[2].min()) == spp and int(f[2].max()) == spp
        _same(f, ref)


def test_batch_graph_replay_accumulates_identically(gpu, setup):
    torch, sc, sets, rs, br, specs = setup
    once, twice, jobs1, jobs2 = [], [], [], []
    for w, h, spp, seed, ms, off in specs[:3]:
        a, b = _film(torch, w, h), _film(torch, w, h)
        once.append(a)
        twice.append(b)
        cam = _camera(gpu, sc, w, h)
        jobs1.append(br.job(cam, spp, a, seed=seed, material_set=ms, sample_offset=off))
        jobs2.append(br.job(cam, spp, b, seed=seed, material_set=ms, sample_offset=off))
    br.render(jobs1)
    br.render(jobs2, graph=True)  # capture
    br.render(jobs2, graph=True)  # replay
    torch.cuda.synchronize()
    for a, b in zip(once, twice):
        assert bool((b[2] == 2 * a[2]).all())
        assert float((b[0] - 2 * a[0]).abs().max()) <= 1e-12 * float(a[0].abs().max())


def test_batch_wave_split_and_autotune(gpu, setup):
    """Jobs split across waves (a small wave size) give the same films."""
    torch, sc, sets, rs, br, specs = setup
    fa, fb, ja, jb = [], [], [], []
    for w, h, spp, seed, ms, off in specs:
        a, b = _film(torch, w, h), _film(torch, w, h)
        fa.append(a)
        fb.append(b)
        cam = _camera(gpu, sc, w, h)
        ja.append(br.job(cam, spp, a, seed=seed, material_set=ms, sample_offset=off))
        jb.append(br.job(cam, spp, b, seed=seed, material_set=ms, sample_offset=off))
    br.render(ja)
    chosen = br.autotune(jb)  # renders jb several times
    assert chosen > 0
    for b in fb:
        for t in b:
            t.zero_()
    br.render(jb)
    torch.cuda.synchronize()
    for a, b in zip(fa, fb):
        _same(a, b)


def test_batch_rejects_bad_jobs(gpu, setup):
    torch, sc, sets, rs, br, specs = setup
    f = _film(torch, 8, 8)
    bad = br.job(_camera(gpu, sc, 8, 8), 4, f, material_set=7)
    with pytest.raises(gpu.OmvError, match="material set"):
        br.render([bad])
    bad = br.job(_camera(gpu, sc, 8, 8), 0, f)
    with pytest.raises(gpu.OmvError, match="no samples"):
        br.render([bad])
