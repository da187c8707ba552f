"""omv_render_device_static (the render without device allocation) through the
C ABI, against omv_render_device on the same scene, camera and parameters.

The file sorts last so that, in a full run, these calls also come after every
other GPU test in the same process; each test builds its own scene, so the file
passes alone as well.  Films differ between the two entry points only in the
order of the FP64 atomic additions (the static scratch may split the frame into
more waves), so sums agree to 1e-9 of the film's largest value and sample counts
exactly."""
import ctypes as C
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

OMV_ERR_INVALID_ARGUMENT = 1


def _setup(gpu, scenes, spp=16, **kw):
    torch = pytest.importorskip("torch")
    sc = scenes.scene_c1(64, 64, 1)
    scene = gpu.RenderScene(sc)
    cam = gpu.PinholeCamera.from_spec(sc.camera).to_c()
    params = gpu.RendererParameters.for_scene(sc, samplesPerPixel=spp, seed=5, accumulate_variance=True, **kw).to_c()
    return torch, sc, scene, cam, params


def _film(torch, npix):
    return (torch.zeros(3 * npix, dtype=torch.float64, device="cuda"),
            torch.zeros(3 * npix, dtype=torch.float64, device="cuda"),
            torch.zeros(npix, dtype=torch.int32, device="cuda"))


def _render(gpu, torch, entry, scene, cam, params, film):
    L = gpu.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptrs = [C.c_void_p(t.data_ptr()) for t in film]
    if entry == "static":
        st = L.omv_render_device_static(scene.handle, C.byref(cam), C.byref(params), *ptrs, stream)
    else:
        st = L.omv_render_device(scene.handle, C.byref(cam), C.byref(params), *ptrs, stream, None)
    torch.cuda.synchronize()
    return st


def _assert_same_film(a, b, spp):
    scale = float(a[0].abs().max())
    assert scale > 0
    assert float((a[0] - b[0]).abs().max()) <= 1e-9 * scale
    assert float((a[1] - b[1]).abs().max()) <= 1e-9 * float(a[1].abs().max())
    assert bool((a[2] == b[2]).all()) and int(a[2].min()) == spp


def test_static_render_matches_device_render_on_two_calls_in_a_row(gpu, scenes):
    torch, sc, scene, cam, params = _setup(gpu, scenes)
    npix = cam.width * cam.height
    ref = _film(torch, npix)
    gpu.check(_render(gpu, torch, "device", scene, cam, params, ref))
    for _ in range(2):
        out = _film(torch, npix)
        gpu.check(_render(gpu, torch, "static", scene, cam, params, out))
        _assert_same_film(ref, out, params.samples_per_pixel)


def test_static_render_with_explicit_wave_matches(gpu, scenes):
    torch, sc, scene, cam, params = _setup(gpu, scenes, wave_paths=3001)
    npix = cam.width * cam.height
    ref = _film(torch, npix)
    gpu.check(_render(gpu, torch, "device", scene, cam, params, ref))
    out = _film(torch, npix)
    gpu.check(_render(gpu, torch, "static", scene, cam, params, out))
    _assert_same_film(ref, out, params.samples_per_pixel)


def test_static_render_leaves_free_device_memory_unchanged(gpu, scenes):
    torch, sc, scene, cam, params = _setup(gpu, scenes)
    npix = cam.width * cam.height
    films = [_film(torch, npix) for _ in range(3)]
    gpu.check(_render(gpu, torch, "static", scene, cam, params, films[0]))  # first call per device: setup
    free0 = torch.cuda.mem_get_info()[0]
    for f in films[1:]:
        gpu.check(_render(gpu, torch, "static", scene, cam, params, f))
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_render_rejects_a_wave_beyond_the_scratch(gpu, scenes):
    torch, sc, scene, cam, params = _setup(gpu, scenes, spp=1024, wave_paths=1 << 22)
    film = _film(torch, cam.width * cam.height)
    st = _render(gpu, torch, "static", scene, cam, params, film)
    assert st == OMV_ERR_INVALID_ARGUMENT
    assert b"static scratch holds" in gpu.lib().omv_last_error()
    assert int(film[2].sum()) == 0  # nothing was launched
    params.wave_paths = 0
    params.time_kernels = 1
    assert _render(gpu, torch, "static", scene, cam, params, film) == OMV_ERR_INVALID_ARGUMENT


_FRESH = r"""
import ctypes as C, importlib, sys
import torch
sys.path.insert(0, sys.argv[1])
omv = importlib.import_module("openmaterial-validation_gb300")
S = omv.scenes
L = omv.lib()

def setup(sc):
    scene = omv.RenderScene(sc)
    cam = omv.PinholeCamera.from_spec(sc.camera).to_c()
    params = omv.RendererParameters.for_scene(sc, samplesPerPixel=8, seed=2).to_c()
    n = cam.width * cam.height
    film = [torch.zeros(3 * n, dtype=torch.float64, device="cuda"), None,
            torch.zeros(n, dtype=torch.int32, device="cuda")]
    return scene, cam, params, film

def static(scene, cam, params, film):
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    omv.check(L.omv_render_device_static(scene.handle, C.byref(cam), C.byref(params),
                                         C.c_void_p(film[0].data_ptr()), None, C.c_void_p(film[2].data_ptr()),
                                         stream))
    torch.cuda.synchronize()

lit = setup(S.scene_c1(32, 32, 1))       # point light, opaque materials
masked = setup(S.scene_mixed(32, 32, 1))  # point light, an alpha-blended material
assert any(m.alpha_mode != 0 for m in masked[0].spec.materials)
torch.cuda.synchronize()
static(*lit)  # the first call in this process: loads the module and the wave kernels
free0 = torch.cuda.mem_get_info()[0]
static(*masked)  # masked shadow rays: a kernel the first frame did not launch
static(*lit)
free1 = torch.cuda.mem_get_info()[0]
assert int(lit[3][2].min()) == 16 and int(masked[3][2].min()) == 8, "film counts"
print("FREE", free0, free1)
"""


def test_static_render_first_in_a_fresh_process_allocates_nothing_later(gpu, scenes):
    """In a process whose first render is the static one (lazy module loading
    has loaded nothing yet), a later frame on a scene with alpha-masked
    materials, which launches kernels the first frame did not, still leaves
    free device memory unchanged."""
    pytest.importorskip("torch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("FREE")][-1].split()
    assert int(line[1]) == int(line[2]), line
