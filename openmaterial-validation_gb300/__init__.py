"""GB300-native render path of the OpenMATERIAL validation pathtracer.

Host-side mirror of the reference's renderer facade over the C ABI in
include/omv.h (libomv.so, hand-written CUDA for sm_103a):

  RenderScene      RenderScene::allocate / set* / commitScene   (RenderScene.h:109-204)
  PinholeCamera    PinholeCamera + ViewPoint                   (PinholeCamera.h, RenderSensor.h)
  RendererParameters                                            (RendererParameters.h:20-96)
  BDPTRenderer     setParameters / setScene / render            (BDPTRenderer.h:147-155)

There is no CPU fallback: every call goes through libomv.so and raises
OmvError when the library is missing or a call fails.
"""
from __future__ import annotations

import concurrent.futures
import ctypes as C
import dataclasses
import json
import math
import os
import subprocess
from typing import Optional

import numpy as np

from . import capi, scenes

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libomv.so")
SOURCES = ["bvh_build.cu", "scene.cu", "render.cu", "adjoint.cu", "fc.cu", "post.cu", "capi.cu"]
HEADERS = ["bvh_build.h", "omv_device.cuh", "omv_types.h", "scene.h", "trace.cuh", "shade.cuh", "dual.cuh", "crmath.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
# translation units whose device float math must round like the reference
# (no implicit FMA contraction; explicit fmaf() calls in the traversal stay fused)
NO_CONTRACT = {"render.cu", "scene.cu", "adjoint.cu", "fc.cu", "post.cu"}


class OmvError(RuntimeError):
    pass


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(REPO_DIR, "include", "omv.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles libomv.so for sm_103a in-tree (one object per translation unit,
    compiled in parallel, then linked).  Returns the library path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        extra = ["--fmad=false"] if src in NO_CONTRACT else []
        cmd = [nvcc, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise OmvError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    r = subprocess.run([nvcc, ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise OmvError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    """The loaded libomv.so (raises OmvError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = os.environ.get("OMV_LIBRARY", LIB_PATH)  # a separately built libomv.so
    if not os.path.exists(path):
        raise OmvError(f"{path} is missing: run build() first (no CPU fallback exists)")
    L = C.CDLL(path)
    vp = C.c_void_p
    st = C.c_int32
    L.omv_scene_create.argtypes = [C.POINTER(capi.SceneDesc), C.c_int32, C.POINTER(vp)]
    L.omv_scene_destroy.argtypes = [vp]
    L.omv_scene_get_info.argtypes = [vp, C.POINTER(capi.SceneInfo)]
    L.omv_render.argtypes = [vp, C.POINTER(capi.Camera), C.POINTER(capi.Params), capi.f32p, C.POINTER(C.c_double),
                             C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(capi.Stats)]
    L.omv_render_device.argtypes = [vp, C.POINTER(capi.Camera), C.POINTER(capi.Params), vp, vp, vp, vp,
                                    C.POINTER(capi.Stats)]
    L.omv_render_device_static.argtypes = [vp, C.POINTER(capi.Camera), C.POINTER(capi.Params), vp, vp, vp, vp]
    L.omv_batch_set_materials.argtypes = [vp, C.c_int32, C.POINTER(capi.MaterialDesc)]
    L.omv_render_batch.argtypes = [vp, C.c_int32, C.POINTER(capi.Job), C.POINTER(capi.Params), vp, C.c_int32,
                                   C.POINTER(capi.Stats)]
    L.omv_batch_autotune.argtypes = [vp, C.c_int32, C.POINTER(capi.Job), C.POINTER(capi.Params), vp,
                                     C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    L.omv_scene_set_materials.argtypes = [vp, C.c_int32, C.POINTER(capi.MaterialDesc)]
    L.omv_adjoint.argtypes = [vp, C.POINTER(capi.Camera), C.POINTER(capi.Params), vp, vp, vp]
    L.omv_scene_create_group.argtypes = [C.c_int32, C.POINTER(capi.SceneDesc), C.c_int32, C.POINTER(vp)]
    L.omv_adjoint_batch.argtypes = [vp, C.c_int32, C.POINTER(capi.AdjointJob), C.POINTER(capi.Params), vp]
    L.omv_trace_rays.argtypes = [vp, C.c_int64, capi.f32p, C.POINTER(capi.Hit)]
    L.omv_render_ids.argtypes = [vp, C.POINTER(capi.Camera), capi.f32p, C.c_uint64, C.POINTER(capi.Hit),
                                 C.POINTER(C.c_uint32)]
    for n in ("omv_brdf_eval_direct", "omv_brdf_sample_indirect", "omv_om_fresnel"):
        getattr(L, n).argtypes = [C.c_int64, capi.f32p, capi.f32p]
    L.omv_library_function.argtypes = [C.c_int32, C.c_int64, capi.f32p, capi.f32p]
    L.omv_camera_rays.argtypes = [C.POINTER(capi.Camera), capi.f32p, capi.f32p]
    L.omv_env_radiance.argtypes = [vp, C.c_int64, capi.f32p, capi.f32p]
    L.omv_fc_subject_from_name.argtypes = [C.c_char_p]
    L.omv_fc_subject_from_name.restype = C.c_int32
    L.omv_render_fc.argtypes = [vp, C.POINTER(capi.Camera), C.c_int32, capi.f32p, C.c_uint64,
                                C.POINTER(C.c_uint32), C.c_int32, capi.f32p, C.POINTER(C.c_uint32),
                                C.POINTER(capi.Hit)]
    L.omv_scene_bounds.argtypes = [vp, capi.f32p, capi.f32p]
    L.omv_texture_sample.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int64, capi.f32p, capi.f32p]
    L.omv_lightbox_cameras.argtypes = [capi.f32p, capi.f32p, C.c_int32, C.c_int32, C.POINTER(capi.Camera)]
    L.omv_develop.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_float, C.c_float, vp, vp, vp, C.c_int32, vp]
    L.omv_tonemap.argtypes = [vp, C.c_int64, C.c_float, C.c_float, vp]
    L.omv_denoise_median.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32, vp]
    L.omv_rgba8.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32, vp]
    L.omv_save_image.argtypes = [C.c_char_p, capi.f32p, C.c_int32, C.c_int32]
    L.omv_last_error.restype = C.c_char_p
    L.omv_version.restype = C.c_char_p
    L.omv_params_default.argtypes = [C.POINTER(capi.Params)]
    L.omv_params_default.restype = None
    L.omv_struct_sizes.argtypes = [C.POINTER(C.c_int64), C.c_int32]
    for n in ("omv_scene_create", "omv_scene_destroy", "omv_scene_get_info", "omv_render", "omv_render_device",
              "omv_render_device_static", "omv_batch_set_materials", "omv_render_batch", "omv_batch_autotune",
              "omv_scene_set_materials", "omv_adjoint",
              "omv_trace_rays", "omv_render_ids", "omv_brdf_eval_direct",
              "omv_brdf_sample_indirect", "omv_om_fresnel", "omv_library_function", "omv_camera_rays", "omv_env_radiance", "omv_struct_sizes",
              "omv_develop", "omv_tonemap", "omv_denoise_median", "omv_rgba8", "omv_save_image",
              "omv_render_fc", "omv_scene_bounds", "omv_lightbox_cameras", "omv_texture_sample"):
        getattr(L, n).restype = st
    L.omv_set_log_callback.argtypes = [LogCallback, C.c_void_p]
    L.omv_set_log_callback.restype = st
    _lib = L
    return L


# omv_log_fn: (user, status, message)
LogCallback = C.CFUNCTYPE(None, C.c_void_p, C.c_int32, C.c_char_p)
_log_keep = None


def set_log_callback(fn) -> None:
    """fn(status, message) is called for every failing library call (None
    removes it): omv_set_log_callback."""
    global _log_keep
    cb = LogCallback(lambda _user, status, msg: fn(int(status), msg.decode(errors="replace"))) if fn else None
    check(lib().omv_set_log_callback(cb if cb is not None else LogCallback(), None))
    _log_keep = cb


def check(status: int) -> None:
    if status != 0:
        raise OmvError(f"omv status {status}: {lib().omv_last_error().decode(errors='replace')}")


# ------------------------------------------------------------ parameters --

ESTIMATOR_REFERENCE = 0  # BDPTRenderer's estimator
ESTIMATOR_MIS = 1  # plus environment connections weighted by the power heuristic


@dataclasses.dataclass
class RendererParameters:
    """RendererParameters (RendererParameters.h:20-96) plus the build's keys."""
    cameraBouncesN: int = 10
    lightBouncesN: int = 10
    maxPathLength: int = 8
    samplesPerPixel: int = 20
    lightDistanceAttenuation: int = 1
    lightScaleValue: float = 100.0
    lightMinDistance: float = 0.01
    rayCutPixValue: float = 0.002
    seed: int = 0
    sample_offset: int = 0
    accumulate_variance: bool = False
    wave_paths: int = 0
    estimator: int = 0  # OMV_ESTIMATOR_REFERENCE (0) or OMV_ESTIMATOR_MIS (1)

    def to_c(self) -> capi.Params:
        return capi.Params(camera_bounces=self.cameraBouncesN, light_bounces=self.lightBouncesN, time_kernels=0,
                           max_path_length=self.maxPathLength, samples_per_pixel=self.samplesPerPixel,
                           light_distance_attenuation=self.lightDistanceAttenuation,
                           light_scale=self.lightScaleValue, light_min_distance=self.lightMinDistance,
                           ray_cut_value=self.rayCutPixValue, seed=self.seed, estimator=self.estimator,
                           sample_offset=self.sample_offset, accumulate_variance=1 if self.accumulate_variance else 0,
                           wave_paths=self.wave_paths)

    @classmethod
    def for_scene(cls, scene: scenes.Scene, **kw) -> "RendererParameters":
        r = scene.render
        p = cls(cameraBouncesN=r.camera_bounces, lightBouncesN=r.light_bounces, maxPathLength=r.max_path_length,
                samplesPerPixel=r.samples_per_pixel)
        for k, v in kw.items():
            setattr(p, k, v)
        return p


# ---------------------------------------------------------------- camera --

class PinholeCamera:
    """PinholeCamera (PinholeCamera.cpp): resolution, ViewPoint (position +
    rotation with columns left/up/forward), half sizes and focus."""

    def __init__(self, width: int, height: int, position=(0.0, 0.0, 0.0), forward=(0.0, 0.0, -1.0),
                 up=(0.0, 1.0, 0.0)) -> None:
        self.width, self.height = max(1, int(width)), max(1, int(height))
        self.position = tuple(float(x) for x in position)
        self.rotation = scenes.default_view(position, forward, up)
        self.half_width = 0.0
        self.half_height = 0.0
        self.focus = 0.0

    @classmethod
    def from_spec(cls, spec: scenes.CameraSpec) -> "PinholeCamera":
        c = cls(spec.width, spec.height, spec.position)
        c.rotation = np.asarray(spec.rotation, dtype=np.float32)
        c.half_width, c.half_height, c.focus = spec.half_width, spec.half_height, spec.focus
        return c

    def adjust_to_resolution(self) -> None:
        self.half_height = float(np.float32(0.5) * np.float32(self.height))
        self.half_width = float(np.float32(0.5) * np.float32(self.width))

    def set_y_fov(self, yfov: float) -> None:
        """PinholeCamera::setYFoV: focus = half_height / tan(fov/2)."""
        if not (0.0 < yfov < 180.0):
            raise ValueError("Field-of-view should be greater than zero and smaller than the straight angle.")
        arg = np.float32(np.float32(np.float32(0.5) * np.float32(yfov)) * np.float32(math.pi)) / np.float32(180.0)
        self.focus = float(np.float32(self.half_height) / np.float32(scenes.tanf(arg)))

    def load_properties(self, path: str) -> None:
        """PinholeCamera::loadProperties: pinhole.{aspect, focus, y-fov}."""
        with open(path) as fh:
            j = json.load(fh)
        p = j.get("pinhole", {})
        spec = scenes.camera_from_json(self.width, self.height, float(p.get("aspect", 0.0)),
                                       float(p.get("focus", self.focus)), float(p.get("y-fov", 0.0)), self.position)
        self.half_width, self.half_height, self.focus = spec.half_width, spec.half_height, spec.focus

    def to_c(self) -> capi.Camera:
        spec = scenes.CameraSpec(self.width, self.height, self.position, np.asarray(self.rotation), self.half_width,
                                 self.half_height, self.focus)
        return capi.camera_struct(spec)


# ----------------------------------------------------------------- scene --

class RenderScene:
    """Device scene behind omv_scene_create (RenderScene::commitScene plus the
    GPU acceleration build)."""

    def __init__(self, scene: scenes.Scene, device: int = 0, bvh_builder: int = capi.BVH_SAH) -> None:
        """bvh_builder: capi.BVH_SAH (device, default), BVH_PLOC (device),
        BVH_LBVH (device) or BVH_HOST_SAH (host threads); hits do not depend on it."""
        self.spec = scene
        self._holder = capi.DescHolder(scene, bvh_builder)
        h = C.c_void_p()
        check(lib().omv_scene_create(C.byref(self._holder.desc), device, C.byref(h)))
        self.handle = h

    @classmethod
    def group(cls, scenes_: list, device: int = 0, bvh_builder: int = capi.BVH_SAH) -> "RenderScene":
        """Several scenes in one handle (omv_scene_create_group): batch and
        adjoint jobs pick one by `part`; materials are numbered scene after
        scene (material_offsets)."""
        self = cls.__new__(cls)
        self.spec = scenes_[0]
        self.parts = list(scenes_)
        self._holders = [capi.DescHolder(sc, bvh_builder) for sc in scenes_]
        arr = (capi.SceneDesc * len(scenes_))(*[h.desc for h in self._holders])
        self._arr = arr
        h = C.c_void_p()
        check(lib().omv_scene_create_group(len(scenes_), arr, device, C.byref(h)))
        self.handle = h
        return self

    @property
    def material_offsets(self) -> list:
        """First material of each scene in the group's material order."""
        parts = getattr(self, "parts", [self.spec])
        out, k = [], 0
        for sc in parts:
            out.append(k)
            k += len(sc.materials)
        return out

    def info(self) -> dict:
        i = capi.SceneInfo()
        check(lib().omv_scene_get_info(self.handle, C.byref(i)))
        return {"triangles": i.num_triangles, "blas_nodes": i.num_blas_nodes, "device_bytes": i.device_bytes,
                "build_ms": i.build_ms}

    def close(self) -> None:
        if getattr(self, "handle", None) and self.handle.value:
            lib().omv_scene_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    # closest-hit queries (sceneIntersect) for given rays: (n, 8) org,tnear,dir,tfar
    def trace(self, rays8: np.ndarray) -> np.ndarray:
        rays8 = np.ascontiguousarray(rays8, dtype=np.float32)
        hits = np.zeros(len(rays8), dtype=capi.HIT_DTYPE)
        check(lib().omv_trace_rays(self.handle, len(rays8), capi.fptr(rays8),
                                   hits.ctypes.data_as(C.POINTER(capi.Hit))))
        return hits

    def bounds(self):
        """World bounding box of the valid instances (AssetGeometry::getBBox)."""
        lo = np.zeros(3, dtype=np.float32)
        hi = np.zeros(3, dtype=np.float32)
        check(lib().omv_scene_bounds(self.handle, capi.fptr(lo), capi.fptr(hi)))
        return lo, hi

    def env_radiance(self, dirs: np.ndarray) -> np.ndarray:
        dirs = np.ascontiguousarray(dirs, dtype=np.float32)
        out = np.zeros((len(dirs), 3), dtype=np.float32)
        check(lib().omv_env_radiance(self.handle, len(dirs), capi.fptr(dirs), capi.fptr(out)))
        return out


class BatchRenderer:
    """Many render jobs of one scene through omv_render_batch: each job has its
    own camera, samples per pixel, seed and material set and a device film
    (torch tensors on the scene's GPU: sums (H, W, 3) float64, counts (H, W)
    int32)."""

    def __init__(self, scene: RenderScene, params: RendererParameters) -> None:
        self.scene = scene
        self.params = params
        self._keep: list = []

    def set_material_sets(self, sets) -> None:
        keep: list = []
        descs = capi.material_set_descs(sets, keep)
        check(lib().omv_batch_set_materials(self.scene.handle, len(sets), descs))
        self._keep = keep

    @staticmethod
    def job(camera: "PinholeCamera", spp: int, film, seed: int = 0, material_set: int = -1,
            sample_offset: int = 0, part: int = 0) -> "capi.Job":
        j = capi.Job()
        j.camera = camera.to_c() if hasattr(camera, "to_c") else camera
        j.samples_per_pixel, j.sample_offset, j.seed, j.material_set = spp, sample_offset, seed, material_set
        j.part = part
        j.d_sum_rgb = film[0].data_ptr()
        j.d_sumsq_rgb = film[1].data_ptr() if film[1] is not None else None
        j.d_count = film[2].data_ptr()
        return j

    def render(self, jobs, stream=None, graph: bool = False, stats: bool = False):
        arr = (capi.Job * len(jobs))(*jobs)
        p = self.params.to_c()
        st = capi.Stats() if stats else None
        check(lib().omv_render_batch(self.scene.handle, len(jobs), arr, C.byref(p), stream,
                                     capi.OMV_BATCH_GRAPH if graph else 0, C.byref(st) if st else None))
        return st

    def adjoint(self, jobs, adjoints, grads, stream=None) -> None:
        """omv_adjoint_batch: for every job its adjoint image (H, W, 3) float32
        and its gradient buffer (scene materials, 11) float32, device tensors."""
        arr = (capi.AdjointJob * len(jobs))()
        for i, (j, a, g) in enumerate(zip(jobs, adjoints, grads)):
            arr[i].job = j
            arr[i].d_adjoint_rgb = a.data_ptr()
            arr[i].d_grad = g.data_ptr()
        p = self.params.to_c()
        check(lib().omv_adjoint_batch(self.scene.handle, len(jobs), arr, C.byref(p), stream))

    def autotune(self, jobs, stream=None) -> int:
        """Picks the wave size and shading block size for these jobs; returns
        the wave size (the block size is in self.block_threads)."""
        arr = (capi.Job * len(jobs))(*jobs)
        p = self.params.to_c()
        chosen = C.c_int64(0)
        threads = C.c_int32(0)
        check(lib().omv_batch_autotune(self.scene.handle, len(jobs), arr, C.byref(p), stream, C.byref(chosen),
                                       C.byref(threads)))
        self.block_threads = threads.value
        return chosen.value


class BDPTRenderer:
    """BDPTRenderer facade (BDPTRenderer.h:147-155) over omv_render."""

    def __init__(self) -> None:
        self.params: Optional[RendererParameters] = None
        self.scene: Optional[RenderScene] = None
        self.last_stats: Optional[dict] = None

    def set_parameters(self, p: RendererParameters) -> None:
        self.params = p

    def set_scene(self, s: RenderScene) -> None:
        self.scene = s

    def render(self, camera: PinholeCamera, sums: bool = False):
        """Renders one frame; returns the normalised RGBA image (H, W, 4) like
        PinholeCamera::getImpression after stop().  With sums=True returns
        (image, sum_rgb, sumsq_rgb or None, count)."""
        if self.params is None or self.scene is None:
            raise OmvError("set_parameters and set_scene first")
        cam = camera.to_c()
        p = self.params.to_c()
        H, W = cam.height, cam.width
        img = np.zeros((H, W, 4), dtype=np.float32)
        s = np.zeros((H, W, 3), dtype=np.float64) if sums else None
        q = np.zeros((H, W, 3), dtype=np.float64) if (sums and self.params.accumulate_variance) else None
        cnt = np.zeros((H, W), dtype=np.uint32) if sums else None
        st = capi.Stats()
        dp = C.POINTER(C.c_double)
        check(lib().omv_render(self.scene.handle, C.byref(cam), C.byref(p), capi.fptr(img),
                               s.ctypes.data_as(dp) if s is not None else None,
                               q.ctypes.data_as(dp) if q is not None else None,
                               cnt.ctypes.data_as(C.POINTER(C.c_uint32)) if cnt is not None else None, C.byref(st)))
        self.last_stats = {"paths": st.paths, "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
                           "light_rays": st.light_rays, "render_ms": st.render_ms,
                           "kernel_launches": st.kernel_launches, "stack_overflows": st.stack_overflows,
                           "nodes_visited": st.nodes_visited, "triangles_tested": st.triangles_tested,
                           "tail_bounce": st.tail_bounce, "tail_nodes_visited": st.tail_nodes_visited}
        if sums:
            return img, s, q, cnt
        return img

    def render_ids(self, camera: PinholeCamera, jitter: Optional[np.ndarray] = None, seed: int = 0):
        """Primary-hit identification buffers (pid/gid/mid validation modes):
        returns (hits structured array (H*W,), global primitive ids (H*W,))."""
        cam = camera.to_c()
        n = cam.width * cam.height
        hits = np.zeros(n, dtype=capi.HIT_DTYPE)
        gp = np.zeros(n, dtype=np.uint32)
        j = None
        if jitter is not None:
            j = np.ascontiguousarray(jitter, dtype=np.float32).reshape(-1)
            if len(j) != 2 * n:
                raise ValueError("jitter must hold 2 uniforms per pixel")
        check(lib().omv_render_ids(self.scene.handle, C.byref(cam), capi.fptr(j) if j is not None else None, seed,
                                   hits.ctypes.data_as(C.POINTER(capi.Hit)), gp.ctypes.data_as(C.POINTER(C.c_uint32))))
        return hits, gp


class ProgressiveFilm:
    """Checkpoint / resume of a progressive render.  The whole state of a
    render in progress is its FP64 film (sums, optional sums of squares,
    sample counts) and the next sample index: samples are keyed by (pixel,
    sample), so `add` continues the sequence (sample_offset) and the film
    after 16 + 16 samples, saved and reloaded in between, is the 32-sample
    film.  The reference has no counterpart (it renders a fixed spp)."""

    # the renderer parameters that define the image: samples rendered with
    # other values belong to another image (another estimator, seed, bounce
    # limit or light model) and must not be summed into this film
    IMAGE_KEYS = ("cameraBouncesN", "lightBouncesN", "maxPathLength", "lightDistanceAttenuation",
                  "lightScaleValue", "lightMinDistance", "rayCutPixValue", "seed", "estimator")

    def __init__(self, width: int, height: int, variance: bool = False, next_sample: int = 0) -> None:
        self.sum = np.zeros((height, width, 3), dtype=np.float64)
        self.sumsq = np.zeros((height, width, 3), dtype=np.float64) if variance else None
        self.count = np.zeros((height, width), dtype=np.uint32)
        self.next_sample = int(next_sample)
        self.params: Optional[dict] = None  # IMAGE_KEYS of the first add(), then fixed

    @classmethod
    def _image_params(cls, p: "RendererParameters") -> dict:
        return {k: getattr(p, k) for k in cls.IMAGE_KEYS}

    def add(self, renderer: BDPTRenderer, camera: PinholeCamera, spp: int) -> None:
        """Renders `spp` more samples per pixel with `renderer`'s scene and
        parameters, continuing at next_sample, and accumulates them."""
        if (camera.height, camera.width) != self.count.shape:
            raise ValueError("camera resolution differs from the film's")
        keep = renderer.params
        ip = self._image_params(keep)
        if self.params is not None and ip != self.params:
            diff = sorted(k for k in ip if ip[k] != self.params[k])
            raise ValueError(f"renderer parameters differ from the film's ({', '.join(diff)}): "
                             "their samples would estimate another image")
        p = dataclasses.replace(keep, samplesPerPixel=int(spp), sample_offset=self.next_sample,
                                accumulate_variance=self.sumsq is not None)
        renderer.set_parameters(p)
        try:
            _, s, q, cnt = renderer.render(camera, sums=True)
        finally:
            renderer.set_parameters(keep)
        self.sum += s
        if self.sumsq is not None:
            self.sumsq += q
        self.count += cnt
        self.next_sample += int(spp)
        self.params = ip

    def image(self) -> np.ndarray:
        """The normalised RGBA image (PinholeCamera::stop)."""
        img = np.zeros(self.count.shape + (4,), dtype=np.float32)
        n = np.maximum(self.count, 1)[..., None]
        img[..., :3] = np.where(self.count[..., None] >= 1, self.sum / n, 0.0)
        img[..., 3] = 1.0
        return img

    def save(self, path: str) -> None:
        extra = {"sumsq": self.sumsq} if self.sumsq is not None else {}
        if self.params is not None:
            extra["params"] = np.array(json.dumps(self.params))
        np.savez(path, sum=self.sum, count=self.count, next_sample=np.int64(self.next_sample), **extra)

    @classmethod
    def load(cls, path: str) -> "ProgressiveFilm":
        with np.load(path) as z:
            H, W = z["count"].shape
            f = cls(W, H, variance="sumsq" in z.files, next_sample=int(z["next_sample"]))
            f.sum[...] = z["sum"]
            f.count[...] = z["count"]
            if f.sumsq is not None:
                f.sumsq[...] = z["sumsq"]
            if "params" in z.files:
                f.params = json.loads(str(z["params"]))
        return f


# --------------------------------------------------- validation (-F / -V) --

FC_SUBJECTS = ("pid", "gid", "mid", "mmp", "rmp", "md", "sg", "mn", "in")


def fc_subject(name: str) -> int:
    """Subject code of an -F name (0, the empty subject, for unknown names)."""
    return int(lib().omv_fc_subject_from_name(name.encode()))


def render_fc(scene: "RenderScene", camera, subject, palette=None, uniforms=None, seed: int = 0):
    """The false-colour pass (main.cpp:261-270 with -F <subject>): returns
    (rgba (H, W, 4) float32, args (H, W) uint32, hits (H*W,)).  `subject` is a
    name or an OMV_FC_* code; `palette` 0xRRGGBB per id for pid/gid/mid;
    `uniforms` (H, W, 4) replaces the device's Philox draws."""
    code = fc_subject(subject) if isinstance(subject, str) else int(subject)
    cam = camera.to_c() if hasattr(camera, "to_c") else camera
    W, H = cam.width, cam.height
    rgba = np.zeros((H, W, 4), dtype=np.float32)
    args = np.zeros((H, W), dtype=np.uint32)
    hits = np.zeros(W * H, dtype=capi.HIT_DTYPE)
    pal = None if palette is None else np.ascontiguousarray(palette, dtype=np.uint32)
    uni = None
    if uniforms is not None:
        uni = np.ascontiguousarray(uniforms, dtype=np.float32).reshape(-1)
        if len(uni) != 4 * W * H:
            raise ValueError("uniforms must hold 4 floats per pixel")
    check(lib().omv_render_fc(scene.handle, C.byref(cam), code, capi.fptr(uni) if uni is not None else None, seed,
                              pal.ctypes.data_as(C.POINTER(C.c_uint32)) if pal is not None else None,
                              0 if pal is None else len(pal), capi.fptr(rgba),
                              args.ctypes.data_as(C.POINTER(C.c_uint32)), hits.ctypes.data_as(C.POINTER(capi.Hit))))
    return rgba, args, hits


def lightbox_cameras(lo, hi, width: int, height: int):
    """The 8 light-box views (-V, main.cpp:434-458) of the box [lo, hi] as C
    cameras, in BoundingBox::getCorners order."""
    cams = (capi.Camera * 8)()
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    check(lib().omv_lightbox_cameras(capi.fptr(lo), capi.fptr(hi), width, height, cams))
    return list(cams)


# ------------------------------------------------------ kernel test hooks --

def _hook(name: str, win: int, wout: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, win)
    out = np.zeros((len(x), wout), dtype=np.float32)
    check(getattr(lib(), name)(len(x), capi.fptr(x), capi.fptr(out)))
    return out


def brdf_eval_direct(x: np.ndarray) -> np.ndarray:
    return _hook("omv_brdf_eval_direct", 17, 3, x)


def brdf_sample_indirect(x: np.ndarray) -> np.ndarray:
    return _hook("omv_brdf_sample_indirect", 24, 6, x)


def om_fresnel(x: np.ndarray) -> np.ndarray:
    return _hook("omv_om_fresnel", 7, 3, x)


# omv_library_function's OMV_FN_* (include/omv.h)
FN_SIN, FN_COS, FN_ASIN, FN_ACOS, FN_POW5, FN_POW_M2 = range(6)


def library_function(fn: int, x: np.ndarray) -> np.ndarray:
    """The device's correctly rounded std::sin / cos / asin / acos /
    pow(x, 5) / pow(x, -2) of float inputs (FN_* selects)."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    out = np.zeros_like(x)
    check(lib().omv_library_function(fn, len(x), capi.fptr(x), capi.fptr(out)))
    return out


def texture_sample(img: np.ndarray, uv: np.ndarray) -> np.ndarray:
    """BitmapTexture::texture on the device: (H, W, 4) uint8 image, (n, 2) coordinates."""
    a = np.ascontiguousarray(img, dtype=np.uint8)
    x = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
    out = np.zeros((len(x), 4), dtype=np.float32)
    check(lib().omv_texture_sample(a.shape[1], a.shape[0], a.ctypes.data_as(C.POINTER(C.c_uint8)), len(x),
                                   capi.fptr(x), capi.fptr(out)))
    return out


def camera_rays(camera: PinholeCamera, jitter: np.ndarray) -> np.ndarray:
    cam = camera.to_c()
    j = np.ascontiguousarray(jitter, dtype=np.float32)
    out = np.zeros((cam.width * cam.height, 6), dtype=np.float32)
    check(lib().omv_camera_rays(C.byref(cam), capi.fptr(j), capi.fptr(out)))
    return out


__all__ = ["build", "lib", "OmvError", "RendererParameters", "PinholeCamera", "RenderScene", "BDPTRenderer",
           "BatchRenderer", "render_fc", "fc_subject", "lightbox_cameras", "FC_SUBJECTS",
           "brdf_eval_direct", "brdf_sample_indirect", "om_fresnel", "camera_rays", "scenes", "capi"]
