"""Checkpoint / resume of a progressive render (ProgressiveFilm): the saved
state (FP64 sums, counts, next sample index) reloads exactly; on the GPU,
16 samples, a save and reload, then 16 more give the 32-sample film."""
import numpy as np
import pytest


def test_save_and_load_round_trip(omv, tmp_path):
    f = omv.ProgressiveFilm(7, 5, variance=True, next_sample=48)
    rng = np.random.default_rng(1)
    f.sum[...] = rng.random(f.sum.shape)
    f.sumsq[...] = rng.random(f.sumsq.shape)
    f.count[...] = 48
    p = str(tmp_path / "film.npz")
    f.save(p)
    g = omv.ProgressiveFilm.load(p)
    assert g.next_sample == 48
    assert np.array_equal(g.sum, f.sum) and np.array_equal(g.sumsq, f.sumsq) and np.array_equal(g.count, f.count)
    assert np.allclose(g.image()[..., :3], f.sum / 48)


def test_checkpoint_keeps_the_image_parameters_and_refuses_others(omv, tmp_path):
    """The parameters that define the image (seed, bounces, estimator, light
    model, cut-off) are saved with the film; resuming with different ones
    raises before anything is rendered."""
    f = omv.ProgressiveFilm(4, 3)
    p0 = omv.RendererParameters(seed=3, estimator=0)
    f.params = omv.ProgressiveFilm._image_params(p0)
    path = str(tmp_path / "film.npz")
    f.save(path)
    g = omv.ProgressiveFilm.load(path)
    assert g.params == f.params

    class Stub:  # only the parameters are read before a mismatch raises
        def __init__(self, params):
            self.params = params

    cam = omv.PinholeCamera(4, 3)
    for change in ({"seed": 4}, {"estimator": 1}, {"cameraBouncesN": 3}, {"lightDistanceAttenuation": 2},
                   {"rayCutPixValue": 0.0}):
        bad = omv.RendererParameters(seed=3, estimator=0)
        for k, v in change.items():
            setattr(bad, k, v)
        with pytest.raises(ValueError, match=next(iter(change))):
            g.add(Stub(bad), cam, 4)


@pytest.mark.gpu
def test_resumed_render_equals_one_render(gpu, scenes, tmp_path):
    sc = scenes.scene_c1(24, 24, 1)
    rs = gpu.RenderScene(sc)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    r.set_parameters(gpu.RendererParameters.for_scene(sc, seed=6))
    cam = gpu.PinholeCamera.from_spec(sc.camera)
    f = gpu.ProgressiveFilm(24, 24)
    f.add(r, cam, 16)
    p = str(tmp_path / "ckpt.npz")
    f.save(p)
    g = gpu.ProgressiveFilm.load(p)
    g.add(r, cam, 16)
    one = gpu.ProgressiveFilm(24, 24)
    one.add(r, cam, 32)
    assert g.next_sample == 32 and (g.count == 32).all()
    assert np.abs(g.sum - one.sum).max() <= 1e-6 * np.abs(one.sum).max()
