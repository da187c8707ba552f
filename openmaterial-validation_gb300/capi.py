"""ctypes mirror of include/omv.h (the C ABI of the render path) and helpers
that turn a :class:`scenes.Scene` into an ``omv_scene_desc``.

Struct layouts must match omv.h field for field; tests/test_capi.py checks the
sizes against the library's own ``sizeof`` reports.
"""
from __future__ import annotations

import ctypes as C
from typing import Any, List

import numpy as np

f32p = C.POINTER(C.c_float)
u32p = C.POINTER(C.c_uint32)

OMV_OK = 0
OMV_MATERIAL_PBR = 0
OMV_MATERIAL_OPENMATERIAL = 1


class MeshDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_int32), ("num_faces", C.c_int32), ("faces", u32p),
                ("positions", f32p), ("position_stride", C.c_int32),
                ("normals", f32p), ("normal_stride", C.c_int32),
                ("tangents", f32p), ("tangent_stride", C.c_int32),
                ("texcoord0", f32p), ("texcoord_stride", C.c_int32),
                ("material", C.c_int32), ("texcoord1", f32p)]


class InstanceDesc(C.Structure):
    _fields_ = [("transform", (C.c_float * 4) * 4), ("mesh", C.c_int32)]


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgba", C.POINTER(C.c_uint8))]


class TextureRef(C.Structure):
    _fields_ = [("texture", C.c_int32), ("texcoord", C.c_int32), ("has_transform", C.c_int32),
                ("transform", (C.c_float * 3) * 2)]


TEXTURE_SLOTS = ("base_color_texture", "metallic_roughness_texture", "normal_texture", "occlusion_texture",
                 "emissive_texture")


class MaterialDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("base_color", C.c_float * 4), ("metallic", C.c_float),
                ("roughness", C.c_float), ("ior", C.c_float), ("alpha_mode", C.c_int32),
                ("alpha_cutoff", C.c_float), ("double_sided", C.c_int32), ("temperature", C.c_float),
                ("ior_n_count", C.c_int32), ("ior_n", f32p), ("ior_k_count", C.c_int32), ("ior_k", f32p)] + \
        [(n, TextureRef) for n in TEXTURE_SLOTS] + \
        [("normal_scale", C.c_float), ("occlusion_strength", C.c_float), ("emissive_factor", C.c_float * 3)]


class LightDesc(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("intensity", C.c_float * 3), ("range", C.c_float)]


class HdriDesc(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", f32p),
                ("rotation", (C.c_float * 3) * 3), ("scale", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("num_meshes", C.c_int32), ("meshes", C.POINTER(MeshDesc)),
                ("num_instances", C.c_int32), ("instances", C.POINTER(InstanceDesc)),
                ("num_materials", C.c_int32), ("materials", C.POINTER(MaterialDesc)),
                ("num_lights", C.c_int32), ("lights", C.POINTER(LightDesc)),
                ("hdri", C.POINTER(HdriDesc)), ("num_textures", C.c_int32),
                ("textures", C.POINTER(TextureDesc)), ("bvh_builder", C.c_int32)]


BVH_SAH, BVH_PLOC, BVH_LBVH, BVH_HOST_SAH = 0, 1, 2, 3


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_int64), ("num_blas_nodes", C.c_int64), ("num_tlas_nodes", C.c_int64),
                ("device_bytes", C.c_int64), ("build_ms", C.c_double)]


class Camera(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("position", C.c_float * 3),
                ("rotation", (C.c_float * 3) * 3), ("half_width", C.c_float), ("half_height", C.c_float),
                ("focus", C.c_float)]


class Params(C.Structure):
    _fields_ = [("camera_bounces", C.c_int32), ("light_bounces", C.c_int32), ("max_path_length", C.c_int32),
                ("samples_per_pixel", C.c_int32), ("light_distance_attenuation", C.c_int32),
                ("light_scale", C.c_float), ("light_min_distance", C.c_float), ("ray_cut_value", C.c_float),
                ("seed", C.c_uint64), ("estimator", C.c_int32), ("sample_offset", C.c_int32),
                ("accumulate_variance", C.c_int32), ("wave_paths", C.c_int32), ("time_kernels", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("extension_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("light_rays", C.c_int64), ("render_ms", C.c_double), ("kernel_launches", C.c_int64),
                ("nodes_visited", C.c_int64), ("triangles_tested", C.c_int64), ("extend_ms", C.c_double),
                ("extend_launches", C.c_int64), ("shadow_ms", C.c_double), ("shadow_launches", C.c_int64),
                ("stack_overflows", C.c_int64), ("shadow_nodes_visited", C.c_int64),
                ("shadow_triangles_tested", C.c_int64), ("tail_bounce", C.c_int64),
                ("tail_nodes_visited", C.c_int64), ("tail_triangles_tested", C.c_int64), ("tail_ms", C.c_double)]


class Hit(C.Structure):
    _fields_ = [("inst", C.c_uint32), ("geom", C.c_uint32), ("prim", C.c_uint32), ("material", C.c_uint32),
                ("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("pad", C.c_uint32)]


HIT_DTYPE = np.dtype([("inst", "<u4"), ("geom", "<u4"), ("prim", "<u4"), ("material", "<u4"),
                      ("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("pad", "<u4")])


class Job(C.Structure):
    _fields_ = [("camera", Camera), ("samples_per_pixel", C.c_int32), ("sample_offset", C.c_int32),
                ("seed", C.c_uint64), ("material_set", C.c_int32), ("part", C.c_int32),
                ("d_sum_rgb", C.c_void_p), ("d_sumsq_rgb", C.c_void_p), ("d_count", C.c_void_p)]


class AdjointJob(C.Structure):
    _fields_ = [("job", Job), ("d_adjoint_rgb", C.c_void_p), ("d_grad", C.c_void_p)]


OMV_BATCH_GRAPH = 1


def fptr(a: np.ndarray):
    return a.ctypes.data_as(f32p)


def default_params() -> Params:
    """RendererParameters defaults (RendererParameters.h:56-89)."""
    return Params(camera_bounces=10, light_bounces=10, max_path_length=8, samples_per_pixel=20,
                  light_distance_attenuation=1, light_scale=100.0, light_min_distance=0.01,
                  ray_cut_value=0.002, seed=0, estimator=0, sample_offset=0, accumulate_variance=0,
                  wave_paths=0, time_kernels=0)


def params_for(scene, spp: int = None, seed: int = 0, variance: bool = False) -> Params:
    p = default_params()
    r = scene.render
    p.camera_bounces = r.camera_bounces
    p.light_bounces = r.light_bounces
    p.max_path_length = r.max_path_length
    p.samples_per_pixel = r.samples_per_pixel if spp is None else spp
    p.seed = seed
    p.accumulate_variance = 1 if variance else 0
    return p


def camera_struct(cam) -> Camera:
    if isinstance(cam, Camera):
        return cam
    c = Camera()
    c.width, c.height = cam.width, cam.height
    for i in range(3):
        c.position[i] = cam.position[i]
        for j in range(3):
            c.rotation[i][j] = float(cam.rotation[i, j])
    c.half_width, c.half_height, c.focus = cam.half_width, cam.half_height, cam.focus
    return c


def material_descs(materials, keep: List[Any]):
    """omv_material_desc array for a list of scenes.Material; the IOR tables
    are appended to `keep`."""
    mats = (MaterialDesc * max(1, len(materials)))()
    for i, mat in enumerate(materials):
        md = mats[i]
        md.type = mat.type
        for c in range(4):
            md.base_color[c] = mat.base_color[c]
        md.metallic, md.roughness, md.ior = mat.metallic, mat.roughness, mat.ior
        md.alpha_mode, md.alpha_cutoff = mat.alpha_mode, mat.alpha_cutoff
        md.double_sided = 1 if mat.double_sided else 0
        md.temperature = mat.temperature
        md.normal_scale = getattr(mat, "normal_scale", 1.0)
        md.occlusion_strength = getattr(mat, "occlusion_strength", 1.0)
        for c in range(3):
            md.emissive_factor[c] = getattr(mat, "emissive_factor", (0.0, 0.0, 0.0))[c]
        for slot in TEXTURE_SLOTS:
            ref = getattr(mat, slot, None)
            if ref is None:
                continue
            tr = getattr(md, slot)
            tr.texture = int(ref.texture) + 1
            tr.texcoord = int(ref.texcoord)
            if ref.transform is not None:
                tr.has_transform = 1
                T = np.asarray(ref.transform, dtype=np.float32)
                for r in range(2):
                    for c in range(3):
                        tr.transform[r][c] = float(T[r, c])
        if mat.ior_n is not None:
            tn = np.ascontiguousarray(np.asarray(mat.ior_n, dtype=np.float64).astype(np.float32))
            tk = np.ascontiguousarray(np.asarray(mat.ior_k, dtype=np.float64).astype(np.float32))
            keep += [tn, tk]
            md.ior_n_count, md.ior_n = len(tn), fptr(tn)
            md.ior_k_count, md.ior_k = len(tk), fptr(tk)
    return mats


def material_set_descs(sets, keep: List[Any]):
    """Flat omv_material_desc array of several material sets (set after set)."""
    flat = [m for row in sets for m in row]
    return material_descs(flat, keep)


class DescHolder:
    """Keeps every numpy buffer referenced by an omv_scene_desc alive."""

    def __init__(self, scene, bvh_builder: int = BVH_SAH) -> None:
        self.keep: List[Any] = []
        meshes = (MeshDesc * max(1, len(scene.meshes)))()
        for i, m in enumerate(scene.meshes):
            md = meshes[i]
            pos = np.ascontiguousarray(m.positions, dtype=np.float32)
            fac = np.ascontiguousarray(m.faces, dtype=np.uint32)
            self.keep += [pos, fac]
            md.num_vertices, md.num_faces = len(pos), len(fac)
            md.faces = fac.ctypes.data_as(u32p)
            md.positions, md.position_stride = fptr(pos), 3
            if m.normals is not None:
                n = np.ascontiguousarray(m.normals, dtype=np.float32)
                self.keep.append(n)
                md.normals, md.normal_stride = fptr(n), 3
            if m.tangents is not None:
                t = np.ascontiguousarray(m.tangents, dtype=np.float32)
                self.keep.append(t)
                md.tangents, md.tangent_stride = fptr(t), 4
            if m.texcoord0 is not None:
                uv = np.ascontiguousarray(m.texcoord0, dtype=np.float32)
                self.keep.append(uv)
                md.texcoord0, md.texcoord_stride = fptr(uv), 2
            if getattr(m, "texcoord1", None) is not None:
                if m.texcoord0 is None:
                    raise ValueError("texcoord1 needs texcoord0")
                uv1 = np.ascontiguousarray(m.texcoord1, dtype=np.float32)
                self.keep.append(uv1)
                md.texcoord1 = fptr(uv1)
            md.material = m.material
        insts = (InstanceDesc * max(1, len(scene.instances)))()
        for i, inst in enumerate(scene.instances):
            M = np.asarray(inst.transform, dtype=np.float32)
            for r in range(4):
                for c in range(4):
                    insts[i].transform[r][c] = float(M[r, c])
            insts[i].mesh = inst.mesh
        mats = material_descs(scene.materials, self.keep)
        lights = (LightDesc * max(1, len(scene.lights)))()
        for i, l in enumerate(scene.lights):
            for c in range(3):
                lights[i].position[c] = l.position[c]
                lights[i].intensity[c] = l.intensity[c]
            lights[i].range = l.range
        self.hdri = None
        if scene.hdri is not None:
            h = HdriDesc()
            rgb = np.ascontiguousarray(scene.hdri.rgb, dtype=np.float32)
            self.keep.append(rgb)
            h.height, h.width = rgb.shape[0], rgb.shape[1]
            h.rgb = fptr(rgb)
            for r in range(3):
                for c in range(3):
                    h.rotation[r][c] = float(scene.hdri.rotation[r, c])
            h.scale = scene.hdri.scale
            self.hdri = h
        self.keep += [meshes, insts, mats, lights]
        d = SceneDesc()
        d.num_meshes, d.meshes = len(scene.meshes), meshes
        d.num_instances, d.instances = len(scene.instances), insts
        d.num_materials, d.materials = len(scene.materials), mats
        d.num_lights, d.lights = len(scene.lights), lights
        d.hdri = C.pointer(self.hdri) if self.hdri is not None else None
        texs = getattr(scene, "textures", None) or []
        if texs:
            tds = (TextureDesc * len(texs))()
            for i, t in enumerate(texs):
                a = np.ascontiguousarray(t, dtype=np.uint8)
                if a.ndim != 3 or a.shape[2] != 4:
                    raise ValueError("textures are (H, W, 4) uint8 RGBA")
                self.keep.append(a)
                tds[i].height, tds[i].width = a.shape[0], a.shape[1]
                tds[i].rgba = a.ctypes.data_as(C.POINTER(C.c_uint8))
            self.keep.append(tds)
            d.num_textures, d.textures = len(texs), tds
        d.bvh_builder = int(bvh_builder)
        self.desc = d
