"""ORACLE -- test infrastructure only.

ctypes wrapper of liboracle.so, the C restatement of the reference renderer's
hot path (oc_render.c / oc_bvh.c) and of its image post-processing (oc_post.c).  Used by the tests as the checker, by
__graft_entry__.smoke() as the checker and by bench.py as the timed CPU
reference; never by the product path.
"""
from __future__ import annotations

import ctypes as C
import importlib
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
capi = importlib.import_module("openmaterial-validation_gb300.capi")

LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BUILD = os.path.join(HERE, "_ref")
REFERENCE_SEED = 3254638  # RenderScene.cpp:20


def reference_tree():
    """The reference source tree: $OMV_REFERENCE, else the tree `make ref`
    last built from (recorded in _ref/REFERENCE_TREE); None when neither
    exists (then the tests that read the reference's own files skip)."""
    cands = [os.environ.get("OMV_REFERENCE")]
    marker = os.path.join(REF_BUILD, "REFERENCE_TREE")
    if os.path.exists(marker):
        with open(marker) as f:
            cands.append(f.read().strip())
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "pathtracer", "src")):
            return c
    return None

_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    for f in ("oc_render.c", "oc_bvh.c", "oc_post.c", "oc_core.h", "oc_bvh.h", "oc_render.h"):
        if os.path.getmtime(os.path.join(HERE, f)) > t:
            return True
    return os.path.getmtime(os.path.join(ROOT, "include", "omv.h")) > t


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.oc_scene_create.restype = vp
        L.oc_scene_create.argtypes = [C.POINTER(capi.SceneDesc)]
        L.oc_scene_destroy.argtypes = [vp]
        L.oc_render.argtypes = [vp, C.POINTER(capi.Camera), C.POINTER(capi.Params), C.c_int32, C.c_uint32,
                                C.c_int32, C.c_int32, C.c_int32, capi.f32p, C.POINTER(C.c_double),
                                C.POINTER(C.c_uint64)]
        L.oc_film_stop.argtypes = [capi.f32p, C.c_int64]
        L.oc_render_ids.argtypes = [vp, C.POINTER(capi.Camera), C.c_uint32, capi.f32p, C.POINTER(capi.Hit)]
        L.oc_trace_rays.argtypes = [vp, C.c_int64, capi.f32p, C.POINTER(capi.Hit)]
        for n in ("oc_brdf_eval_direct", "oc_brdf_sample_indirect", "oc_om_fresnel"):
            getattr(L, n).argtypes = [C.c_int64, capi.f32p, capi.f32p]
        L.oc_camera_rays.argtypes = [C.POINTER(capi.Camera), capi.f32p, capi.f32p]
        L.oc_env_radiance.argtypes = [vp, C.c_int64, capi.f32p, capi.f32p]
        L.oc_mt_uniforms.argtypes = [C.c_uint32, C.c_int64, capi.f32p]
        L.oc_ior_lookup.restype = C.c_float
        L.oc_ior_lookup.argtypes = [capi.f32p, C.c_int32, C.c_float]
        L.oc_scene_mesh_info.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32)]
        L.oc_scene_mesh_vertices.argtypes = [vp, C.c_int32, capi.f32p]
        L.oc_scene_normal_matrix.argtypes = [vp, C.c_int32, capi.f32p]
        L.oc_render_fc.argtypes = [vp, C.POINTER(capi.Camera), C.c_uint32, C.c_int32, C.POINTER(C.c_uint32),
                                   C.c_int32, capi.f32p, C.POINTER(C.c_uint32), capi.f32p, C.POINTER(capi.Hit)]
        L.oc_density_range.argtypes = [vp, capi.f32p]
        L.oc_texture_sample.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_uint8), C.c_int64, capi.f32p, capi.f32p]
        L.oc_render_views.argtypes = [vp, C.c_int32, C.POINTER(capi.Camera), C.POINTER(capi.Params), C.c_uint32,
                                      capi.f32p]
        L.oc_tonemap.argtypes = [capi.f32p, C.c_int64, C.c_float, C.c_float]
        L.oc_median.argtypes = [capi.f32p, C.c_int, C.c_int, C.c_int]
        L.oc_rgba8.argtypes = [capi.f32p, C.c_int64, C.POINTER(C.c_uint8)]
        _lib = L
    return _lib


class OracleScene:
    def __init__(self, scene) -> None:
        self.scene = scene
        self._holder = capi.DescHolder(scene)
        self.h = lib().oc_scene_create(C.byref(self._holder.desc))
        if not self.h:
            raise RuntimeError("oracle: scene has no valid instance")

    def close(self) -> None:
        if self.h:
            lib().oc_scene_destroy(self.h)
            self.h = None

    def __del__(self) -> None:
        try:
            self.close()
        except Exception:
            pass

    def render(self, camera=None, params=None, mode: int = 0, seed: int = REFERENCE_SEED, threads: int = 1,
               rows=None, variance: bool = False, normalize: bool = True):
        """Returns (film W*H*4 float32 [normalised like PinholeCamera::stop when
        normalize], sumsq or None, ray count)."""
        cam = capi.camera_struct(camera or self.scene.camera)
        p = params or capi.params_for(self.scene)
        W, H = cam.width, cam.height
        r0, r1 = rows if rows is not None else (0, H)
        film = np.zeros((H, W, 4), dtype=np.float32)
        sumsq = np.zeros((H, W, 3), dtype=np.float64) if variance else None
        rays = C.c_uint64(0)
        rc = lib().oc_render(self.h, C.byref(cam), C.byref(p), mode, seed, threads, r0, r1, capi.fptr(film),
                             sumsq.ctypes.data_as(C.POINTER(C.c_double)) if variance else None, C.byref(rays))
        if rc != 0:
            raise RuntimeError("oracle render failed")
        if normalize:
            lib().oc_film_stop(capi.fptr(film), W * H)
        return film, sumsq, int(rays.value)

    def render_ids(self, camera=None, seed: int = REFERENCE_SEED):
        cam = capi.camera_struct(camera or self.scene.camera)
        n = cam.width * cam.height
        rays = np.zeros((n, 6), dtype=np.float32)
        hits = np.zeros(n, dtype=capi.HIT_DTYPE)
        lib().oc_render_ids(self.h, C.byref(cam), seed, capi.fptr(rays), hits.ctypes.data_as(C.POINTER(capi.Hit)))
        return rays, hits

    def render_fc(self, subject: int, palette=None, camera=None, seed: int = REFERENCE_SEED):
        """The false-colour pass: (rgba (H, W, 4), args uint32 (H, W), uniforms
        (H, W, 4), hits (H*W,))."""
        cam = capi.camera_struct(camera or self.scene.camera)
        W, H = cam.width, cam.height
        rgba = np.zeros((H, W, 4), dtype=np.float32)
        args = np.zeros((H, W), dtype=np.uint32)
        uni = np.zeros((H, W, 4), dtype=np.float32)
        hits = np.zeros(W * H, dtype=capi.HIT_DTYPE)
        pal = None if palette is None else np.ascontiguousarray(palette, dtype=np.uint32)
        lib().oc_render_fc(self.h, C.byref(cam), seed, subject,
                           pal.ctypes.data_as(C.POINTER(C.c_uint32)) if pal is not None else None,
                           0 if pal is None else len(pal), capi.fptr(rgba), args.ctypes.data_as(C.POINTER(C.c_uint32)),
                           capi.fptr(uni), hits.ctypes.data_as(C.POINTER(capi.Hit)))
        return rgba, args, uni, hits

    def density_range(self):
        out = np.zeros(2, dtype=np.float32)
        lib().oc_density_range(self.h, capi.fptr(out))
        return out

    def render_views(self, cams, params=None, seed: int = REFERENCE_SEED):
        """Light-box loop: normalised films (n, H, W, 4) of the cameras rendered
        in turn from one generator."""
        arr = (capi.Camera * len(cams))(*cams)
        p = params or capi.params_for(self.scene)
        W, H = cams[0].width, cams[0].height
        films = np.zeros((len(cams), H, W, 4), dtype=np.float32)
        if lib().oc_render_views(self.h, len(cams), arr, C.byref(p), seed, capi.fptr(films)) != 0:
            raise RuntimeError("oracle render_views failed")
        return films

    def trace(self, rays8: np.ndarray):
        rays8 = np.ascontiguousarray(rays8, dtype=np.float32)
        hits = np.zeros(len(rays8), dtype=capi.HIT_DTYPE)
        lib().oc_trace_rays(self.h, len(rays8), capi.fptr(rays8), hits.ctypes.data_as(C.POINTER(capi.Hit)))
        return hits

    def env_radiance(self, dirs: np.ndarray) -> np.ndarray:
        dirs = np.ascontiguousarray(dirs, dtype=np.float32)
        out = np.zeros((len(dirs), 3), dtype=np.float32)
        lib().oc_env_radiance(self.h, len(dirs), capi.fptr(dirs), capi.fptr(out))
        return out

    def mesh_vertices(self, mesh: int) -> np.ndarray:
        vn, fn, mat = C.c_int32(), C.c_int32(), C.c_int32()
        lib().oc_scene_mesh_info(self.h, mesh, C.byref(vn), C.byref(fn), C.byref(mat))
        out = np.zeros((vn.value, 10), dtype=np.float32)
        lib().oc_scene_mesh_vertices(self.h, mesh, capi.fptr(out))
        return out

    def mesh_material(self, mesh: int) -> int:
        vn, fn, mat = C.c_int32(), C.c_int32(), C.c_int32()
        lib().oc_scene_mesh_info(self.h, mesh, C.byref(vn), C.byref(fn), C.byref(mat))
        return mat.value

    def normal_matrix(self, inst: int) -> np.ndarray:
        out = np.zeros(9, dtype=np.float32)
        lib().oc_scene_normal_matrix(self.h, inst, capi.fptr(out))
        return out.reshape(3, 3)


def _batch(fn, width_in: int, width_out: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, width_in)
    out = np.zeros((len(x), width_out), dtype=np.float32)
    fn(len(x), capi.fptr(x), capi.fptr(out))
    return out


def brdf_eval_direct(x: np.ndarray) -> np.ndarray:
    return _batch(lib().oc_brdf_eval_direct, 17, 3, x)


def brdf_sample_indirect(x: np.ndarray) -> np.ndarray:
    return _batch(lib().oc_brdf_sample_indirect, 24, 6, x)


def om_fresnel(x: np.ndarray) -> np.ndarray:
    return _batch(lib().oc_om_fresnel, 7, 3, x)


def camera_rays(camera, jitter: np.ndarray) -> np.ndarray:
    cam = capi.camera_struct(camera)
    jitter = np.ascontiguousarray(jitter, dtype=np.float32)
    out = np.zeros((cam.width * cam.height, 6), dtype=np.float32)
    lib().oc_camera_rays(C.byref(cam), capi.fptr(jitter), capi.fptr(out))
    return out


def mt_uniforms(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    lib().oc_mt_uniforms(seed, n, capi.fptr(out))
    return out


def ior_lookup(table: np.ndarray, wl: float) -> float:
    t = np.ascontiguousarray(table, dtype=np.float32)
    return float(lib().oc_ior_lookup(capi.fptr(t), len(t), wl))


def tonemap(img: np.ndarray, gamma: float, A: float = 1.0) -> np.ndarray:
    """gammaCorrection (ToneMapping.cpp:24) of an (H, W, 4) float image, returned as a copy."""
    out = np.array(img, dtype=np.float32, order="C", copy=True)
    lib().oc_tonemap(capi.fptr(out), out.size // 4, A, gamma)
    return out


def median(img: np.ndarray, half: int = 1) -> np.ndarray:
    """SimpleDenoiserMedian<half> (Denoiser.h:24) of an (H, W, 4) float image, as a copy."""
    out = np.array(img, dtype=np.float32, order="C", copy=True)
    lib().oc_median(capi.fptr(out), out.shape[1], out.shape[0], half)
    return out


def rgba8(img: np.ndarray) -> np.ndarray:
    """saveImage's conversion (main.cpp:92): unsigned char(255 f) per channel."""
    x = np.ascontiguousarray(img, dtype=np.float32)
    out = np.zeros(x.shape, dtype=np.uint8)
    lib().oc_rgba8(capi.fptr(x), x.size, out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out


def texture_sample(img: np.ndarray, uv: np.ndarray) -> np.ndarray:
    """BitmapTexture::texture of an (H, W, 4) uint8 image at n (u, v) pairs."""
    a = np.ascontiguousarray(img, dtype=np.uint8)
    x = np.ascontiguousarray(uv, dtype=np.float32).reshape(-1, 2)
    out = np.zeros((len(x), 4), dtype=np.float32)
    lib().oc_texture_sample(a.shape[1], a.shape[0], a.ctypes.data_as(C.POINTER(C.c_uint8)), len(x), capi.fptr(x),
                            capi.fptr(out))
    return out
