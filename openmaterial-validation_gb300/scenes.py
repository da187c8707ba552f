"""Seeded synthetic scenes of the benchmark shapes, in two forms:

* flattened arrays, exactly as the reference's RenderScene holds them after
  main.cpp has flattened the glTF asset (main.cpp:285-416) -- what the C ABI
  (omv_scene_create) takes;
* glTF 2.0 + OpenMATERIAL files (geometry .gltf/.bin, OpenMATERIAL material and
  IOR tables, KHR_lights_punctual point lights, a pinhole camera JSON and a
  Radiance RGBE .hdr environment) that the reference renderer loads itself, so
  both renderers consume identical inputs.

Scenes (sizes from the benchmark definitions):

* ``c1``: icosphere (4 midpoint subdivisions, 5,120 triangles, radius 1) with an
  OpenMATERIAL conductor whose IOR table gives n=(0.18,0.42,1.37),
  k=(3.42,2.35,1.77) at the RGB wavelengths 650/510/440 nm, on a 10x10 diffuse
  ground quad (PBR, base colour 0.5, metallic 0, roughness 1) at y=-1; one point
  light at (2,4,2), white, intensity 50; pinhole camera, y-fov 45 deg, 256x256,
  16 spp, camera/light bounces 6, max path length 6.  The whole asset sits under
  a root node translated by (0,0,-5) so that the reference's fixed camera (origin,
  looking down -z, main.cpp:459-476) sees it.  The conductor's GGX roughness 0.3
  has no counterpart in the reference's OpenMATERIAL model (a perfect mirror,
  OpenMaterial.cpp:72-93) and is therefore not represented.
* ``c2``: 64 meshes (32 tori of 12,288 triangles, 32 noise-displaced icospheres
  of 20,480 triangles: 1,048,576 triangles) under uniform random rotations,
  scale U[0.5,2] and positions U[-20,20]^3 m around the camera (at least 8 m
  from it, so the camera is outside every object); PBR
  materials baseColor U[0,1]^3, roughness U[0.05,1], metallic Bernoulli(0.5);
  a 2048x1024 equirectangular HDRI (log-normal sky, mu=0 sigma=1, plus three
  Gaussian sun lobes of peak 1e4) stored as RGBE; 1920x1080, 64 spp, max path
  length 10, camera bounces 10, no point lights.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import dataclasses
import functools
import json
import math
import os
import re
import struct
from typing import List, Optional

import numpy as np

F32 = np.float32

# Constants.h:53 -- wavelengths of the three base channels [m]
RGB_WAVELENGTHS = (6.50000004e-07, 5.10000007e-07, 4.40000008e-07)


_LIBM_F = {}


def _libm_f(name: str):
    """A float function of the C library (tanf, cosf, sinf)."""
    f = _LIBM_F.get(name)
    if f is None:
        lib = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        f = getattr(lib, name)
        f.restype = ctypes.c_float
        f.argtypes = [ctypes.c_float]
        _LIBM_F[name] = f
    return f


def tanf(x: float) -> float:
    """float tangent through the C library, as std::tan(float) evaluates it."""
    return float(_libm_f("tanf")(float(F32(x))))


def cosf(x: float) -> float:
    return float(_libm_f("cosf")(float(F32(x))))


def sinf(x: float) -> float:
    return float(_libm_f("sinf")(float(F32(x))))


# ----------------------------------------------------------------- geometry --

@functools.lru_cache(maxsize=8)
def _icosphere_cached(subdivisions: int):
    v, f = _icosphere(subdivisions)
    v.setflags(write=False)
    f.setflags(write=False)
    return v, f


def icosphere(subdivisions: int):
    v, f = _icosphere_cached(subdivisions)
    return v.copy(), f.copy()


def _icosphere(subdivisions: int):
    """Unit icosphere by repeated midpoint subdivision of an icosahedron, all
    vertices projected onto the unit sphere (computed in float64, stored f32)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
             (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
             (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
             (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
             (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}
        new_faces = []

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = new_faces
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.uint32)


def torus(R: float, r: float, nu: int, nv: int):
    u = np.arange(nu) * (2 * np.pi / nu)
    v = np.arange(nv) * (2 * np.pi / nv)
    uu, vv = np.meshgrid(u, v, indexing="ij")
    cx, cz = np.cos(uu), np.sin(uu)
    pos = np.stack([(R + r * np.cos(vv)) * cx, r * np.sin(vv), (R + r * np.cos(vv)) * cz], -1).reshape(-1, 3)
    nrm = np.stack([np.cos(vv) * cx, np.sin(vv), np.cos(vv) * cz], -1).reshape(-1, 3)
    idx = np.arange(nu * nv).reshape(nu, nv)
    i0 = idx
    i1 = np.roll(idx, -1, axis=0)
    i2 = np.roll(idx, -1, axis=1)
    i3 = np.roll(np.roll(idx, -1, axis=0), -1, axis=1)
    f = np.concatenate([np.stack([i0, i2, i1], -1).reshape(-1, 3), np.stack([i1, i2, i3], -1).reshape(-1, 3)])
    return pos, nrm, f.astype(np.uint32)


def displaced_icosphere(subdivisions: int, rng: np.random.Generator, amplitude: float = 0.18, modes: int = 6):
    v, f = icosphere(subdivisions)
    disp = np.zeros(len(v))
    for _ in range(modes):
        k = rng.normal(size=3)
        k *= rng.uniform(1.5, 5.0) / np.linalg.norm(k)
        disp += np.sin(v @ k + rng.uniform(0, 2 * np.pi)) / modes ** 0.5
    return v * (1.0 + amplitude * disp)[:, None], f


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


# -------------------------------------------------------------- data model --

@dataclasses.dataclass
class Mesh:
    positions: np.ndarray                 # (V,3) f32
    faces: np.ndarray                     # (F,3) u32
    normals: Optional[np.ndarray] = None  # (V,3) f32 or None (derived at commit)
    tangents: Optional[np.ndarray] = None  # (V,4) f32 or None (derived at commit)
    texcoord0: Optional[np.ndarray] = None
    material: int = -1
    name: str = "mesh"
    texcoord1: Optional[np.ndarray] = None


@dataclasses.dataclass
class Instance:
    transform: np.ndarray  # (4,4) f32 object-to-world
    mesh: int


@dataclasses.dataclass
class Material:
    type: int                      # 0 PBR, 1 OpenMATERIAL
    base_color: tuple = (1.0, 1.0, 1.0, 1.0)
    metallic: float = 1.0
    roughness: float = 1.0
    ior: float = 1.5
    alpha_mode: int = 0
    alpha_cutoff: float = 0.5
    double_sided: bool = False
    temperature: float = 300.0
    ior_n: Optional[np.ndarray] = None  # (K,2) wavelength[m], n
    ior_k: Optional[np.ndarray] = None
    name: str = "material"
    # PBR texture slots (TextureRef or None) and their factors
    base_color_texture: Optional["TextureRef"] = None
    metallic_roughness_texture: Optional["TextureRef"] = None
    normal_texture: Optional["TextureRef"] = None
    occlusion_texture: Optional["TextureRef"] = None
    emissive_texture: Optional["TextureRef"] = None
    normal_scale: float = 1.0
    occlusion_strength: float = 1.0
    emissive_factor: tuple = (0.0, 0.0, 0.0)


@dataclasses.dataclass
class TextureRef:
    """A material's use of scene texture `texture` through TEXCOORD_`texcoord`,
    with KHR_texture_transform (offset, rotation, scale) when given."""
    texture: int
    texcoord: int = 0
    offset: Optional[tuple] = None
    rotation: Optional[float] = None
    scale: Optional[tuple] = None

    @property
    def transform(self) -> Optional[np.ndarray]:
        """Rows 0-1 of getTextureTransform's matrix (PbrMaterial.cpp:25-57), float32."""
        if self.offset is None and self.rotation is None and self.scale is None:
            return None
        off = [F32(x) for x in (self.offset or (0.0, 0.0))]
        sc = [F32(x) for x in (self.scale or (1.0, 1.0))]
        rot = F32(self.rotation or 0.0)
        c, s = F32(cosf(rot)), F32(sinf(rot))
        return np.array([[sc[0] * c, sc[0] * s, off[0]], [-(sc[1] * s), sc[1] * c, off[1]]], dtype=F32)


@dataclasses.dataclass
class Light:
    position: tuple
    intensity: tuple
    range: float = 0.0  # <= 0: unlimited


@dataclasses.dataclass
class Hdri:
    rgb: np.ndarray          # (H,W,3) f32, already RGBE-quantised
    rotation: np.ndarray     # (3,3)
    scale: float


@dataclasses.dataclass
class CameraSpec:
    width: int
    height: int
    position: tuple
    rotation: np.ndarray     # (3,3): columns left, up, forward (ViewPoint)
    half_width: float
    half_height: float
    focus: float
    json_props: Optional[dict] = None


@dataclasses.dataclass
class RenderSpec:
    samples_per_pixel: int
    camera_bounces: int
    light_bounces: int
    max_path_length: int


@dataclasses.dataclass
class Scene:
    name: str
    meshes: List[Mesh]
    instances: List[Instance]
    materials: List[Material]
    lights: List[Light]
    hdri: Optional[Hdri]
    camera: CameraSpec
    render: RenderSpec
    gltf_nodes: list = dataclasses.field(default_factory=list)  # for the writer
    textures: list = dataclasses.field(default_factory=list)    # (H, W, 4) uint8 RGBA images

    @property
    def num_triangles(self) -> int:
        return int(sum(len(self.meshes[i.mesh].faces) for i in self.instances))


# ----------------------------------------------------------------- cameras --

def default_view(position=(0.0, 0.0, 0.0), forward=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """ViewPoint as main.cpp:459-476 builds it: left = forward x up,
    up' = left x forward; rotation columns (left, up', forward)."""
    f = np.array(forward, dtype=F32)
    u = np.array(up, dtype=F32)

    def cross(a, b):
        return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], dtype=F32)

    left = cross(f, u)
    up2 = cross(left, f)
    return np.stack([left, up2, f], axis=1).astype(F32)


def camera_from_json(width, height, aspect, focus, yfov, position=(0.0, 0.0, 0.0)) -> CameraSpec:
    """PinholeCamera::loadProperties (PinholeCamera.cpp:115-148)."""
    focus32 = F32(focus)
    half_h = F32(focus32 * F32(tanf(F32(F32(F32(0.5) * F32(yfov)) * F32(math.pi)) / F32(180.0))))
    half_w = F32(F32(aspect) * half_h)
    return CameraSpec(width, height, tuple(position), default_view(position), float(half_w), float(half_h),
                      float(focus32), json_props={"pinhole": {"aspect": aspect, "focus": focus, "y-fov": yfov}})


def camera_default(width, height, yfov=60.0, position=(0.0, 0.0, 0.0)) -> CameraSpec:
    """PinholeCamera::adjustToResolution + setYFoV(60) (main.cpp:485-486,
    PinholeCamera.cpp:156-174)."""
    half_h = F32(F32(0.5) * F32(height))
    half_w = F32(F32(0.5) * F32(width))
    arg = F32(F32(F32(0.5) * F32(yfov)) * F32(math.pi)) / F32(180.0)
    focus = F32(half_h / F32(tanf(arg)))
    return CameraSpec(width, height, tuple(position), default_view(position), float(half_w), float(half_h),
                      float(focus))


# ---------------------------------------------------------------- builders --

def _om_conductor(n_rgb, k_rgb, name="om_conductor") -> Material:
    """IOR tables with points exactly at the three RGB wavelengths (so
    AssetMaterialIor::getIor returns the given n,k), bracketed by 380 nm and
    780 nm points so the range check passes (AssetMaterialIor.cpp:140)."""
    wl = [3.8e-07, RGB_WAVELENGTHS[2], RGB_WAVELENGTHS[1], RGB_WAVELENGTHS[0], 7.8e-07]
    nv = [n_rgb[2], n_rgb[2], n_rgb[1], n_rgb[0], n_rgb[0]]
    kv = [k_rgb[2], k_rgb[2], k_rgb[1], k_rgb[0], k_rgb[0]]
    return Material(type=1, ior_n=np.array(list(zip(wl, nv)), dtype=np.float64),
                    ior_k=np.array(list(zip(wl, kv)), dtype=np.float64), name=name)


def scene_c1(width: int = 256, height: int = 256, spp: int = 16) -> Scene:
    v, f = icosphere(4)
    sphere = Mesh(positions=v.astype(F32), normals=(v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F32),
                  faces=f, material=0, name="icosphere")
    qv = np.array([[-5, -1, -5], [5, -1, -5], [5, -1, 5], [-5, -1, 5]], dtype=F32)
    qf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32)
    ground = Mesh(positions=qv, normals=np.tile(np.array([0, 1, 0], dtype=F32), (4, 1)), faces=qf, material=1,
                  name="ground")
    conductor = _om_conductor((0.18, 0.42, 1.37), (3.42, 2.35, 1.77))
    diffuse = Material(type=0, base_color=(0.5, 0.5, 0.5, 1.0), metallic=0.0, roughness=1.0, name="ground_diffuse")
    root_t = np.eye(4, dtype=F32)
    root_t[2, 3] = -5.0
    inst = [Instance(root_t.copy(), 0), Instance(root_t.copy(), 1)]
    light = Light(position=(2.0, 4.0, -3.0), intensity=(50.0, 50.0, 50.0))
    focus = (height / 2.0) / math.tan(math.radians(22.5))
    cam = camera_from_json(width, height, width / height, focus, 45.0)
    nodes = {"root_translation": (0.0, 0.0, -5.0), "light_translation": (2.0, 4.0, 2.0),
             "light_color": (1.0, 1.0, 1.0), "light_intensity": 50.0}
    return Scene("c1", [sphere, ground], inst, [conductor, diffuse], [light], None, cam,
                 RenderSpec(spp, 6, 6, 6), gltf_nodes=[nodes])


def gltf_light_intensity(color, intensity) -> tuple:
    """The RGB intensity the reference gives a KHR_lights_punctual point light:
    colour x intensity with the green and blue entries exchanged (main.cpp:360-362
    reads getLightGreen / getLightBlue, which return m_color[2] / m_color[1],
    PointLight.h:52-56), in float32."""
    c = np.asarray(color, dtype=F32)
    i = F32(intensity)
    return (float(c[0] * i), float(c[2] * i), float(c[1] * i))


def scene_lights(width: int = 48, height: int = 48, spp: int = 16) -> Scene:
    """C1's geometry and materials under three coloured point lights of
    different power, one with a glTF range: the light pick by the luminance
    CDF of their power (RenderScene.cpp:274-279, DistanceRandom.h:98-115), the
    green/blue order of coloured lights and the ranged attenuation branches
    (BDPTRenderer.cpp:104-126, RenderLightPoint.cpp:20-26)."""
    base = scene_c1(width, height, spp)
    root = (0.0, 0.0, -5.0)
    spec = [{"translation": (2.0, 4.0, 2.0), "color": (1.0, 0.8, 0.55), "intensity": 60.0},
            {"translation": (-3.0, 2.5, 1.0), "color": (0.2, 0.45, 1.0), "intensity": 25.0, "range": 7.5},
            {"translation": (0.5, 6.0, -2.0), "color": (0.9, 0.15, 0.35), "intensity": 90.0}]
    lights = []
    for lt in spec:
        pos = tuple(float(F32(F32(root[k]) + F32(lt["translation"][k]))) for k in range(3))
        lights.append(Light(position=pos, intensity=gltf_light_intensity(lt["color"], lt["intensity"]),
                            range=float(lt.get("range", 0.0))))
    nodes = {"root_translation": root, "lights": spec}
    return Scene("lights", base.meshes, base.instances, base.materials, lights, None, base.camera,
                 RenderSpec(spp, 6, 6, 6), gltf_nodes=[nodes])


def make_sky(width: int, height: int, rng: np.random.Generator, suns: bool = True) -> np.ndarray:
    """Log-normal sky (mu=0, sigma=1 of the log) from a smooth Gaussian field on
    the sphere, plus three Gaussian sun lobes of peak 1e4, in the equirect
    parametrisation HDRBackground::getRadiance reads (row 0 = zenith)."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    elev = (0.5 - v) * np.pi
    phi = u * 2 * np.pi
    ee, pp = np.meshgrid(elev, phi, indexing="ij")
    d = np.stack([np.cos(ee) * np.cos(pp), np.cos(ee) * np.sin(pp), np.sin(ee)], -1)
    g = np.zeros((height, width))
    modes = 24
    for _ in range(modes):
        k = rng.normal(size=3)
        k *= rng.uniform(0.5, 6.0) / np.linalg.norm(k)
        g += np.cos(d @ k + rng.uniform(0, 2 * np.pi))
    g *= (2.0 / modes) ** 0.5  # unit variance
    sky = np.exp(g)[..., None] * np.array([0.55, 0.7, 1.0])
    for _ in range(3 if suns else 0):
        e = rng.uniform(0.15, 1.2)
        a = rng.uniform(0, 2 * np.pi)
        s = np.array([np.cos(e) * np.cos(a), np.cos(e) * np.sin(a), np.sin(e)])
        w = math.radians(rng.uniform(1.0, 3.0))
        ang = np.arccos(np.clip(d @ s, -1, 1))
        sky += (1e4 * np.exp(-0.5 * (ang / w) ** 2))[..., None] * np.array([1.0, 0.95, 0.85])
    return rgbe_quantize(sky.astype(F32))


def scene_c2(width: int = 1920, height: int = 1080, spp: int = 64, seed: int = 0,
             tri_scale: float = 1.0, suns: bool = True, sky_size=(2048, 1024)) -> Scene:
    """tri_scale < 1 shrinks the tessellation and suns=False drops the three
    1e4 sun lobes (low-variance variants for parity tests)."""
    rng = np.random.default_rng(seed)
    meshes, insts, mats = [], [], []
    sub = 5 if tri_scale >= 1.0 else max(1, int(round(5 + math.log(tri_scale, 4))))
    nu, nv = max(8, int(round(128 * tri_scale ** 0.5))), max(6, int(round(48 * tri_scale ** 0.5)))
    for i in range(64):
        if i % 2 == 0:
            R = rng.uniform(1.0, 3.0)
            r = rng.uniform(0.2, 0.8)
            p, n, f = torus(R, r, nu, nv)
            m = Mesh(positions=p.astype(F32), normals=n.astype(F32), faces=f, material=i, name=f"torus{i}")
        else:
            p, f = displaced_icosphere(sub, rng)
            m = Mesh(positions=p.astype(F32), normals=None, faces=f, material=i, name=f"blob{i}")
        meshes.append(m)
        rot = random_rotation(rng)
        s = rng.uniform(0.5, 2.0)
        while True:  # U[-20,20]^3 around the camera, keeping the camera outside every object
            t = rng.uniform(-20.0, 20.0, 3)
            if np.linalg.norm(t) > 8.0:
                break
        M = np.eye(4)
        M[:3, :3] = rot * s
        M[:3, 3] = t
        insts.append(Instance(M.astype(F32), i))
        mats.append(Material(type=0, base_color=(float(rng.uniform()), float(rng.uniform()), float(rng.uniform()), 1.0),
                             roughness=float(rng.uniform(0.05, 1.0)), metallic=float(rng.integers(0, 2)),
                             name=f"pbr{i}"))
    sky = make_sky(sky_size[0], sky_size[1], rng, suns)
    R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], dtype=F32)  # main.cpp:401-405 (y-up)
    hdri = Hdri(sky, R, float(F32(math.pi)))
    cam = camera_default(width, height)
    return Scene("c2", meshes, insts, mats, [], hdri, cam, RenderSpec(spp, 10, 10, 10))


def _tessellation_for(tris: int):
    """(icosphere subdivision, torus nu, nv) for 4 icospheres and 4 tori of
    about `tris` triangles in total: the icospheres take the largest power-of-4
    size within half the budget, the tori the rest."""
    sub = 1
    while sub < 7 and 4 * 20 * 4 ** (sub + 1) <= tris // 2:
        sub += 1
    per_torus = max(96, (tris - 4 * 20 * 4 ** sub) // 4)
    nv = max(6, int(round((per_torus / 2 / 2.67) ** 0.5)))
    nu = max(8, int(round(per_torus / 2 / nv)))
    return sub, nu, nv


def scene_materials(width: int = 512, height: int = 512, spp: int = 32, tris: int = 100_000,
                    n_materials: int = 8, seed: int = 0, bounces: int = 6, sky: bool = False) -> Scene:
    """Material-study scene (batched sweeps, adjoint, inverse fits): 8 objects
    (tori and displaced icospheres, about `tris` triangles in total) on a
    10x10 ground quad under one point light, seen by a 45-degree pinhole camera.
    Materials alternate glTF PBR (base colour, roughness, metallic) and
    OpenMATERIAL conductors (complex IOR at the RGB wavelengths); the ground
    uses material 0.  With `sky`, a 512x256 log-normal sky (no sun lobes) lights
    the scene as well, so the mirror-like conductors show something to fit."""
    rng = np.random.default_rng(seed)
    sub, nu, nv = _tessellation_for(tris)
    meshes, insts = [], []
    for i in range(8):
        if i % 2 == 0:
            R = rng.uniform(0.5, 0.8)
            p, n, f = torus(R, rng.uniform(0.15, 0.3), nu, nv)
            m = Mesh(positions=p.astype(F32), normals=n.astype(F32), faces=f, material=i % n_materials,
                     name=f"torus{i}")
        else:
            p, f = displaced_icosphere(sub, rng, amplitude=0.12)
            p = (p * 0.7).astype(F32)
            m = Mesh(positions=p, normals=None, faces=f, material=i % n_materials, name=f"blob{i}")
        meshes.append(m)
        M = np.eye(4)
        M[:3, :3] = random_rotation(rng)
        M[:3, 3] = (-3.0 + 2.0 * (i % 4), -0.2 + 0.3 * rng.uniform(), -4.0 - 2.2 * (i // 4))
        insts.append(Instance(M.astype(F32), i))
    qv = np.array([[-6, -1, 1], [6, -1, 1], [6, -1, -11], [-6, -1, -11]], dtype=F32)
    qf = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)
    meshes.append(Mesh(positions=qv, normals=np.tile(np.array([0, 1, 0], dtype=F32), (4, 1)), faces=qf,
                       material=0, name="ground"))
    insts.append(Instance(np.eye(4, dtype=F32), 8))
    mats = []
    for i in range(n_materials):
        if i % 2 == 0:
            mats.append(Material(type=0, base_color=(float(rng.uniform(0.2, 0.9)), float(rng.uniform(0.2, 0.9)),
                                                     float(rng.uniform(0.2, 0.9)), 1.0),
                                 roughness=float(rng.uniform(0.2, 0.9)), metallic=float(rng.uniform(0.0, 1.0)),
                                 name=f"pbr{i}"))
        else:
            mats.append(_om_conductor(tuple(rng.uniform(0.1, 4.0, 3)), tuple(rng.uniform(0.1, 4.0, 3)),
                                      name=f"om{i}"))
    light = Light(position=(2.0, 4.0, 0.0), intensity=(50.0, 50.0, 50.0))
    focus = (height / 2.0) / math.tan(math.radians(22.5))
    cam = camera_from_json(width, height, width / height, focus, 45.0, position=(0.0, 1.5, 4.0))
    hdri = None
    if sky:
        R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], dtype=F32)  # main.cpp:401-405 (y-up)
        hdri = Hdri(make_sky(512, 256, np.random.default_rng(seed + 7), suns=False), R, float(F32(math.pi)))
    return Scene("materials", meshes, insts, mats, [light], hdri, cam, RenderSpec(spp, bounces, bounces, bounces))


def material_variants(scene: Scene, n_sets: int, seed: int = 1) -> List[List[Material]]:
    """Per-job material sets for a batched sweep: conductors get n, k in
    U[0.1, 4] per RGB channel, PBR materials a roughness in U[0.02, 1] (other
    fields as in the scene)."""
    rng = np.random.default_rng(seed)
    sets = []
    for _ in range(n_sets):
        row = []
        for m in scene.materials:
            if m.type == 1:
                row.append(_om_conductor(tuple(rng.uniform(0.1, 4.0, 3)), tuple(rng.uniform(0.1, 4.0, 3)), m.name))
            else:
                row.append(dataclasses.replace(m, roughness=float(rng.uniform(0.02, 1.0))))
        sets.append(row)
    return sets


def scene_mixed(width: int = 32, height: int = 32, spp: int = 8) -> Scene:
    """Parity scene covering every material branch of the reference: the
    OpenMATERIAL conductor, a rough PBR metal (specular GGX branch), a
    double-sided PBR dielectric (transmission branch, BRDFModel.h:291-310), a
    BLEND PBR with alpha 0.5, a mesh without material (the missing-material
    diffuse, DiffuseColorMaterial.cpp) and the diffuse ground; C1's light and
    camera model, bounces 4, max path length 5."""
    v, f = icosphere(2)
    v32 = v.astype(F32)
    n32 = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F32)
    meshes = []
    centers = [(-1.6, -0.3, 0.0), (0.0, -0.3, -0.8), (1.6, -0.3, 0.0), (-0.8, 0.9, -1.2), (0.9, 0.9, -1.5)]
    scale = F32(0.7)
    for i, c in enumerate(centers):
        p = (v32 * scale + np.array(c, dtype=F32)).astype(F32)
        meshes.append(Mesh(positions=p, normals=n32.copy(), faces=f, material=[0, 1, 2, 3, -1][i], name=f"ball{i}"))
    qv = np.array([[-5, -1, -5], [5, -1, -5], [5, -1, 5], [-5, -1, 5]], dtype=F32)
    qf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32)
    meshes.append(Mesh(positions=qv, normals=None, faces=qf, material=4, name="ground"))
    mats = [_om_conductor((0.18, 0.42, 1.37), (3.42, 2.35, 1.77)),
            Material(type=0, base_color=(0.9, 0.6, 0.3, 1.0), metallic=1.0, roughness=0.3, name="rough_metal"),
            Material(type=0, base_color=(0.8, 0.9, 1.0, 1.0), metallic=0.0, roughness=0.15, double_sided=True,
                     name="dielectric"),
            Material(type=0, base_color=(0.2, 0.8, 0.3, 0.5), metallic=0.2, roughness=0.5, alpha_mode=2,
                     name="blend"),
            Material(type=0, base_color=(0.5, 0.5, 0.5, 1.0), metallic=0.0, roughness=1.0, name="ground_diffuse")]
    root_t = np.eye(4, dtype=F32)
    root_t[2, 3] = -5.0
    inst = [Instance(root_t.copy(), i) for i in range(len(meshes))]
    light = Light(position=(2.0, 4.0, -3.0), intensity=(50.0, 50.0, 50.0))
    focus = (height / 2.0) / math.tan(math.radians(22.5))
    cam = camera_from_json(width, height, width / height, focus, 45.0)
    nodes = {"root_translation": (0.0, 0.0, -5.0), "light_translation": (2.0, 4.0, 2.0),
             "light_color": (1.0, 1.0, 1.0), "light_intensity": 50.0}
    return Scene("mixed", meshes, inst, mats, [light], None, cam, RenderSpec(spp, 4, 4, 5), gltf_nodes=[nodes])


def scene_validation(width: int = 64, height: int = 48) -> Scene:
    """Scene for the false-colour subjects: triangle densities over three
    orders of magnitude (icospheres of 80, 320 and 1280 faces, a 2-face
    ground), one ball wound inside out with outward vertex normals (inverted
    normals, surface gradient 1), an OpenMATERIAL conductor, PBR materials with
    distinct metallic / roughness factors (one roughness above 1, clamped by the
    subject) and a mesh without material.  C1's light and camera model."""
    meshes = []
    specs = [(2, (-1.6, -0.3, 0.0), 0, False), (1, (0.0, -0.3, -0.8), 1, False), (3, (1.6, -0.3, 0.0), 2, False),
             (1, (-0.8, 0.9, -1.2), 3, True), (2, (0.9, 0.9, -1.5), -1, False)]
    scale = F32(0.7)
    for i, (sub, c, mat, flip) in enumerate(specs):
        v, f = icosphere(sub)
        n = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F32)
        p = (v.astype(F32) * scale + np.array(c, dtype=F32)).astype(F32)
        faces = f[:, [0, 2, 1]].copy() if flip else f
        meshes.append(Mesh(positions=p, normals=n, faces=np.ascontiguousarray(faces), material=mat, name=f"ball{i}"))
    qv = np.array([[-5, -1, -5], [5, -1, -5], [5, -1, 5], [-5, -1, 5]], dtype=F32)
    qf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32)
    meshes.append(Mesh(positions=qv, normals=None, faces=qf, material=4, name="ground"))
    mats = [_om_conductor((0.18, 0.42, 1.37), (3.42, 2.35, 1.77)),
            Material(type=0, base_color=(0.9, 0.6, 0.3, 1.0), metallic=1.0, roughness=0.3, name="rough_metal"),
            Material(type=0, base_color=(0.8, 0.9, 1.0, 1.0), metallic=0.25, roughness=1.3, double_sided=True,
                     name="over_rough"),
            Material(type=0, base_color=(0.2, 0.8, 0.3, 1.0), metallic=0.6, roughness=0.8, name="inside_out"),
            Material(type=0, base_color=(0.5, 0.5, 0.5, 1.0), metallic=0.0, roughness=1.0, name="ground_diffuse")]
    root_t = np.eye(4, dtype=F32)
    root_t[2, 3] = -5.0
    inst = [Instance(root_t.copy(), i) for i in range(len(meshes))]
    light = Light(position=(2.0, 4.0, -3.0), intensity=(50.0, 50.0, 50.0))
    focus = (height / 2.0) / math.tan(math.radians(22.5))
    cam = camera_from_json(width, height, width / height, focus, 45.0)
    nodes = {"root_translation": (0.0, 0.0, -5.0), "light_translation": (2.0, 4.0, 2.0),
             "light_color": (1.0, 1.0, 1.0), "light_intensity": 50.0}
    return Scene("validation", meshes, inst, mats, [light], None, cam, RenderSpec(1, 1, 1, 8), gltf_nodes=[nodes])


def _texture_images(seed: int = 7) -> List[np.ndarray]:
    """Seeded RGBA8 images: base colour with a varying alpha (64x32), packed
    occlusion/roughness/metallic (32x32), a tangent-space normal map including
    texels with z <= 0.5 (32x32), a separate occlusion map (16x16) and an
    emission map (16x16)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:32, 0:64]
    base = np.zeros((32, 64, 4), np.uint8)
    chk = ((x // 8 + y // 8) % 2).astype(np.float64)
    base[..., 0] = np.clip(60 + 160 * chk + rng.integers(0, 30, chk.shape), 0, 255)
    base[..., 1] = np.clip(200 - 120 * chk + rng.integers(0, 30, chk.shape), 0, 255)
    base[..., 2] = rng.integers(20, 200, chk.shape)
    base[..., 3] = np.clip(255 * (0.5 + 0.5 * np.sin(x / 5.0) * np.cos(y / 3.0)), 0, 255)
    y2, x2 = np.mgrid[0:32, 0:32]
    mr = np.zeros((32, 32, 4), np.uint8)
    mr[..., 0] = 128 + (127 * np.cos(x2 / 4.0)).astype(np.int64)
    mr[..., 1] = np.clip(40 + 7 * x2, 0, 255)
    mr[..., 2] = np.clip(255 - 8 * y2, 0, 255)
    mr[..., 3] = 255
    nrm = np.zeros((32, 32, 4), np.uint8)
    nx = 0.6 * np.sin(x2 / 3.0)
    ny = 0.6 * np.cos(y2 / 2.0)
    nz = np.sqrt(np.clip(1.0 - nx ** 2 - ny ** 2, 0.0, 1.0))
    nz[:4, :4] = -0.2  # stored z below 0.5: clamped to 0.5 + FLT_EPSILON
    nrm[..., 0] = np.clip(np.rint(127.5 * (nx + 1.0)), 0, 255)
    nrm[..., 1] = np.clip(np.rint(127.5 * (ny + 1.0)), 0, 255)
    nrm[..., 2] = np.clip(np.rint(127.5 * (nz + 1.0)), 0, 255)
    nrm[..., 3] = 255
    occ = np.full((16, 16, 4), 255, np.uint8)
    occ[..., 0] = rng.integers(60, 256, (16, 16))
    em = np.zeros((16, 16, 4), np.uint8)
    em[..., :3] = rng.integers(0, 256, (16, 16, 3)) * (rng.random((16, 16, 1)) < 0.3)
    em[..., 3] = 255
    return [base, mr, nrm, occ, em]


def _sphere_uv(v: np.ndarray) -> np.ndarray:
    d = v / np.linalg.norm(v, axis=1, keepdims=True)
    u = 0.5 + np.arctan2(d[:, 2], d[:, 0]) / (2 * math.pi)
    w = 0.5 - np.arcsin(np.clip(d[:, 1], -1, 1)) / math.pi
    return np.stack([u, w], 1).astype(F32)


def scene_textured(width: int = 32, height: int = 32, spp: int = 8) -> Scene:
    """Parity scene for the PBR texture paths: base colour (with KHR texture
    transform and wrapping coordinates), packed metallic-roughness-occlusion,
    a normal map, a separate occlusion map, an emissive ball, an alpha-masked
    and an alpha-blended textured material, a second coordinate set, and the
    OpenMATERIAL conductor; C1's light and camera model, bounces 4."""
    v, f = icosphere(2)
    n = (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F32)
    uv = _sphere_uv(v)
    uv1 = (uv * F32(2.0) + F32(0.25)).astype(F32)
    meshes = []
    centers = [(-1.6, -0.3, 0.0), (0.0, -0.3, -0.8), (1.6, -0.3, 0.0), (-0.8, 0.9, -1.2), (0.9, 0.9, -1.5)]
    mats_of = [1, 2, 3, 4, 5]
    scale = F32(0.7)
    for i, c in enumerate(centers):
        p = (v.astype(F32) * scale + np.array(c, dtype=F32)).astype(F32)
        meshes.append(Mesh(positions=p, normals=n.copy(), faces=f, material=mats_of[i], name=f"ball{i}",
                           texcoord0=uv.copy(), texcoord1=uv1.copy() if i == 3 else None))
    qv = np.array([[-5, -1, -5], [5, -1, -5], [5, -1, 5], [-5, -1, 5]], dtype=F32)
    qf = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32)
    quv = np.array([[-1.5, -1.5], [2.5, -1.5], [2.5, 2.5], [-1.5, 2.5]], dtype=F32)
    meshes.append(Mesh(positions=qv, normals=None, faces=qf, material=0, name="ground", texcoord0=quv))
    T = TextureRef
    mats = [
        Material(type=0, base_color=(0.9, 0.9, 0.9, 1.0), metallic=0.8, roughness=0.9, name="ground_textured",
                 base_color_texture=T(0, 0, offset=(0.1, 0.2), rotation=0.3, scale=(2.0, 1.5)),
                 metallic_roughness_texture=T(1), normal_texture=T(2), normal_scale=0.8,
                 occlusion_texture=T(3, scale=(3.0, 3.0)), occlusion_strength=0.7),
        _om_conductor((0.18, 0.42, 1.37), (3.42, 2.35, 1.77)),
        Material(type=0, base_color=(1.0, 0.8, 0.6, 1.0), metallic=1.0, roughness=1.0, name="emissive_ball",
                 base_color_texture=T(0), metallic_roughness_texture=T(1), occlusion_texture=T(1),
                 occlusion_strength=0.5, emissive_texture=T(4, rotation=1.0), emissive_factor=(1.0, 0.5, 0.2)),
        Material(type=0, base_color=(0.8, 0.9, 1.0, 0.9), metallic=0.1, roughness=0.4, alpha_mode=1,
                 alpha_cutoff=0.5, double_sided=True, name="masked", base_color_texture=T(0, 0, scale=(3.0, 2.0))),
        Material(type=0, base_color=(0.9, 0.9, 0.9, 0.8), metallic=0.3, roughness=0.6, alpha_mode=2, name="blend",
                 base_color_texture=T(0, 1), normal_texture=T(2, 1), normal_scale=1.2),
        Material(type=0, base_color=(0.5, 0.7, 0.9, 1.0), metallic=0.0, roughness=0.5, name="second_set",
                 metallic_roughness_texture=T(1, offset=(0.5, 0.5))),
    ]
    root_t = np.eye(4, dtype=F32)
    root_t[2, 3] = -5.0
    inst = [Instance(root_t.copy(), i) for i in range(len(meshes))]
    light = Light(position=(2.0, 4.0, -3.0), intensity=(50.0, 50.0, 50.0))
    focus = (height / 2.0) / math.tan(math.radians(22.5))
    cam = camera_from_json(width, height, width / height, focus, 45.0)
    nodes = {"root_translation": (0.0, 0.0, -5.0), "light_translation": (2.0, 4.0, 2.0),
             "light_color": (1.0, 1.0, 1.0), "light_intensity": 50.0}
    return Scene("textured", meshes, inst, mats, [light], None, cam, RenderSpec(spp, 4, 4, 5), gltf_nodes=[nodes],
                 textures=_texture_images())


SCENES = {"c1": scene_c1, "c2": scene_c2, "mixed": scene_mixed, "validation": scene_validation,
          "textured": scene_textured}


# -------------------------------------------------------------------- RGBE --

def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    rgb = np.asarray(rgb, dtype=np.float64)
    v = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), dtype=np.uint8)
    ok = v > 1e-32
    m, e = np.frexp(v[ok])
    scale = m * 256.0 / v[ok]
    out[ok, :3] = np.clip(np.floor(rgb[ok] * scale[:, None]), 0, 255).astype(np.uint8)
    out[ok, 3] = (e + 128).astype(np.uint8)
    return out


def rgbe_decode(rgbe: np.ndarray) -> np.ndarray:
    """Radiance RGBE to float, as stb_image's HDR loader converts it:
    value = byte * 2^(e - 136), zero when e == 0."""
    e = rgbe[..., 3].astype(np.int32)
    f = np.ldexp(np.float32(1.0), e - 136).astype(F32)
    out = rgbe[..., :3].astype(F32) * f[..., None]
    out[e == 0] = 0.0
    return out.astype(F32)


def rgbe_quantize(rgb: np.ndarray) -> np.ndarray:
    return rgbe_decode(rgbe_encode(rgb))


def _rle_channel(vals: np.ndarray) -> bytes:
    """One channel of a new-style RLE scanline: runs of 3..127 equal bytes as
    (128 + n, value), everything else as literal dumps of at most 128 bytes."""
    out = bytearray()
    n, i = len(vals), 0
    lit = []
    while i < n:
        r = 1
        while i + r < n and r < 127 and vals[i + r] == vals[i]:
            r += 1
        if r >= 3:
            while lit:
                out.append(min(len(lit), 128))
                out.extend(lit[:128])
                lit = lit[128:]
            out += bytes((128 + r, int(vals[i])))
            i += r
        else:
            lit.append(int(vals[i]))
            i += 1
    while lit:
        out.append(min(len(lit), 128))
        out.extend(lit[:128])
        lit = lit[128:]
    return bytes(out)


def write_hdr(path: str, rgb: np.ndarray, rle: bool = False) -> None:
    """Radiance .hdr: flat RGBE scanlines, or (rle, widths 8..32767) new-style
    run-length scanlines as Radiance writes them.  A flat file's first pixel
    must not start with the RLE marker bytes 2, 2."""
    h, w, _ = rgb.shape
    data = rgbe_encode(rgb)
    with open(path, "wb") as fh:
        fh.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        fh.write(f"-Y {h} +X {w}\n".encode())
        if rle:
            if not 8 <= w < 32768:
                raise ValueError("run-length scanlines need 8 <= width < 32768")
            for j in range(h):
                fh.write(bytes((2, 2, w >> 8, w & 255)))
                for k in range(4):
                    fh.write(_rle_channel(data[j, :, k]))
        else:
            if data[0, 0, 0] == 2 and data[0, 0, 1] == 2:
                raise ValueError("first pixel would read as an RLE marker")
            fh.write(data.tobytes())


def decode_hdr(raw: bytes) -> np.ndarray:
    """A Radiance .hdr file as the reference loads it (stbi_loadf with 0
    requested channels, HdrBackground.cpp:42, through stb_image's HDR loader):
    signature #?RADIANCE or #?RGBE, header lines up to an empty one (one must
    be FORMAT=32-bit_rle_rgbe), then "-Y H +X W".  Widths 8..32767 read
    new-style run-length scanlines; a scanline that does not start with
    (2, 2, length < 32768) makes stb decode the whole image again as flat
    pixels from there (that scanline's 4 bytes become pixel 0).  Other widths
    are flat.  A file that ends inside the pixel data raises ValueError (stb
    then repeats whatever its 4-byte read buffer last held).
    Returns (H, W, 3) float32: byte * 2^(e - 136), zero when e == 0."""
    n = len(raw)
    pos = 0

    def get8():
        nonlocal pos
        if pos >= n:
            raise ValueError("truncated HDR pixel data")
        pos += 1
        return raw[pos - 1]

    def token():
        nonlocal pos
        end = raw.find(b"\n", pos)
        end = n if end < 0 else end
        t = raw[pos:end][:1023]
        pos = min(end + 1, n)
        return t.decode("latin-1")

    if token() not in ("#?RADIANCE", "#?RGBE"):
        raise ValueError("not a Radiance HDR file")
    valid = False
    while True:
        t = token()
        if not t:
            break
        valid = valid or t == "FORMAT=32-bit_rle_rgbe"
    if not valid:
        raise ValueError("unsupported HDR format")
    def strtol(x):  # C strtol: leading white space, sign, digits; (0, x) when none
        m = re.match(r"[ \t\n\v\f\r]*([+-]?[0-9]+)", x)
        return (int(m.group(1)), x[m.end():]) if m else (0, x)

    t = token()
    if not t.startswith("-Y "):
        raise ValueError("unsupported HDR data layout")
    height, rest = strtol(t[3:])
    rest = rest.lstrip(" ")
    if not rest.startswith("+X "):
        raise ValueError("unsupported HDR data layout")
    width, _ = strtol(rest[3:])
    if width <= 0 or height <= 0:
        raise ValueError("bad HDR size")
    total = width * height
    px = np.zeros((total, 4), dtype=np.uint8)

    def flat(first: int) -> None:
        nonlocal pos
        need = 4 * (total - first)
        if pos + need > n:
            raise ValueError("truncated HDR pixel data")
        px[first:] = np.frombuffer(raw[pos:pos + need], dtype=np.uint8).reshape(-1, 4)
        pos += need

    if width < 8 or width >= 32768:
        flat(0)
    else:
        line = np.zeros((width, 4), dtype=np.uint8)
        for j in range(height):
            c1, c2, ln = get8(), get8(), get8()
            if c1 != 2 or c2 != 2 or (ln & 0x80):
                px[0] = (c1, c2, ln, get8())
                flat(1)
                break
            ln = (ln << 8) | get8()
            if ln != width:
                raise ValueError("invalid decoded scanline length")
            for k in range(4):
                i = 0
                while i < width:
                    count = get8()
                    if count > 128:
                        count -= 128
                        if count > width - i:
                            raise ValueError("bad RLE data in HDR")
                        line[i:i + count, k] = get8()
                    else:
                        if count > width - i:
                            raise ValueError("bad RLE data in HDR")
                        if pos + count > n:
                            raise ValueError("truncated HDR pixel data")
                        line[i:i + count, k] = np.frombuffer(raw[pos:pos + count], dtype=np.uint8)
                        pos += count
                    i += count
            px[j * width:(j + 1) * width] = line
    return rgbe_decode(px.reshape(height, width, 4))


def read_hdr(path: str) -> np.ndarray:
    with open(path, "rb") as fh:
        return decode_hdr(fh.read())


# -------------------------------------------------------------- glTF writer --

def _hexid(tag: str) -> str:
    h = 0xcbf29ce484222325
    for ch in tag.encode():
        h = ((h ^ ch) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return f"{h:016x}{(h * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF:016x}"


def _asset_info(asset_type: str, title: str) -> dict:
    return {"version": "2.0", "generator": "omv synthetic scene generator",
            "extensions": {"OpenMaterial_asset_info": {
                "asset_type": asset_type, "id": _hexid(title), "title": title, "asset_version": "1",
                "asset_variation": "1", "creator": "omv", "description": title}}}


def _write_om_material(dirname: str, mat: Material) -> str:
    ior_file = f"{mat.name}_ior.gltf"

    def table(a):
        return [[float(w), float(x)] for w, x in a]

    with open(os.path.join(dirname, ior_file), "w") as fh:
        json.dump({"asset": _asset_info("material_ior", f"IOR {mat.name}"),
                   "extensions": {"OpenMaterial_ior_data": {"data": [
                       {"temperature": float(mat.temperature), "n": table(mat.ior_n), "k": table(mat.ior_k)}]}}},
                  fh, indent=1)
    mat_file = f"{mat.name}.gltf"
    params = {
        "user_preferences": {
            "geometrical_optics": True, "include_diffraction": False, "include_numerical_simulation": False,
            "material_scheme": "surface", "material_classification": "solid-metal",
            "material_type": {"isotropic": True, "homogeneous": True, "magnetic": False},
            "temperature": float(mat.temperature), "surface_displacement_uri": "",
            "surface_roughness": {"surface_height_rms": 0.0, "surface_correlation_length": 0.0},
            "lambert_emission": 0.0, "subsurface": {"subsurface": False, "subsurface_thickness": 0.0},
            "ingredients": [{"material_ref": "", "order": ""}],
            "coating_materials": [{"layer_thickness": 0.0, "material_ref": ""}]},
        "physical_properties": {
            "refractive_index_uri": ior_file, "mean_free_path": 1e-6, "particle_density": 1.0,
            "particle_cross_section": 1.0, "emissive_coefficient_uri": "",
            "detection_wavelength_ranges": [{"min": 3e-07, "max": 8e-07, "typical_sensor": "camera"}],
            "applicable_sensors": ["camera"], "effective_particle_area": 1.0, "relative_permittivity_uri": "",
            "relative_permeability_uri": "", "conductivity_uri": "", "acoustic_impedance": 1.0,
            "shear_velocity": 1.0}}
    with open(os.path.join(dirname, mat_file), "w") as fh:
        json.dump({"asset": _asset_info("material", mat.name),
                   "materials": [{"name": mat.name, "extensions": {"OpenMaterial_material_parameters": params}}],
                   "extensionsUsed": ["OpenMaterial_asset_info", "OpenMaterial_material_parameters"]}, fh, indent=1)
    return mat_file


def write_png(path: str, rgba: np.ndarray) -> None:
    """8-bit RGBA PNG (filter 0 on every row, zlib-compressed)."""
    import struct
    import zlib

    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = a.shape[:2]
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(t: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)

    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
                 chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def _gltf_texture_info(ref: "TextureRef", extra: dict = None) -> dict:
    info = {"index": int(ref.texture), "texCoord": int(ref.texcoord)}
    if extra:
        info.update(extra)
    if ref.offset is not None or ref.rotation is not None or ref.scale is not None:
        t = {}
        if ref.offset is not None:
            t["offset"] = [float(x) for x in ref.offset]
        if ref.rotation is not None:
            t["rotation"] = float(ref.rotation)
        if ref.scale is not None:
            t["scale"] = [float(x) for x in ref.scale]
        info["extensions"] = {"KHR_texture_transform": t}
    return info


def write_gltf(scene: Scene, dirname: str) -> dict:
    """Writes <name>.gltf/.bin (+ material, IOR, camera and HDR files) and returns
    the reference command-line flags (main.cpp:161-193) that render it."""
    os.makedirs(dirname, exist_ok=True)
    blob = bytearray()
    accessors, views = [], []

    def add(arr: np.ndarray, comp: int, typ: str, minmax: bool = False) -> int:
        while len(blob) % 4:
            blob.append(0)
        off = len(blob)
        blob.extend(arr.tobytes())
        views.append({"buffer": 0, "byteOffset": off, "byteLength": arr.nbytes})
        acc = {"bufferView": len(views) - 1, "componentType": comp, "count": int(arr.shape[0]), "type": typ}
        if minmax:
            acc["min"] = [float(x) for x in arr.min(axis=0)]
            acc["max"] = [float(x) for x in arr.max(axis=0)]
        accessors.append(acc)
        return len(accessors) - 1

    gl_meshes, gl_mats = [], []
    mat_index = {}
    for mi, mat in enumerate(scene.materials):
        if mat.type == 1:
            uri = _write_om_material(dirname, mat)
            gl_mats.append({"name": mat.name, "extensions": {"OpenMaterial_reference_link": {
                "id": _hexid(mat.name), "title": mat.name, "uri": uri}}})
        else:
            gm = {"name": mat.name, "pbrMetallicRoughness": {
                "baseColorFactor": [float(c) for c in mat.base_color], "metallicFactor": float(mat.metallic),
                "roughnessFactor": float(mat.roughness)}}
            if mat.double_sided:
                gm["doubleSided"] = True
            if mat.alpha_mode:
                gm["alphaMode"] = ["OPAQUE", "MASK", "BLEND"][mat.alpha_mode]
                gm["alphaCutoff"] = float(mat.alpha_cutoff)
            pmr = gm["pbrMetallicRoughness"]
            if mat.base_color_texture is not None:
                pmr["baseColorTexture"] = _gltf_texture_info(mat.base_color_texture)
            if mat.metallic_roughness_texture is not None:
                pmr["metallicRoughnessTexture"] = _gltf_texture_info(mat.metallic_roughness_texture)
            if mat.normal_texture is not None:
                gm["normalTexture"] = _gltf_texture_info(mat.normal_texture, {"scale": float(mat.normal_scale)})
            if mat.occlusion_texture is not None:
                gm["occlusionTexture"] = _gltf_texture_info(mat.occlusion_texture,
                                                            {"strength": float(mat.occlusion_strength)})
            if mat.emissive_texture is not None:
                gm["emissiveTexture"] = _gltf_texture_info(mat.emissive_texture)
            if any(float(x) != 0.0 for x in mat.emissive_factor):
                gm["emissiveFactor"] = [float(x) for x in mat.emissive_factor]
            gl_mats.append(gm)
        mat_index[mi] = mi
    for m in scene.meshes:
        attrs = {"POSITION": add(np.ascontiguousarray(m.positions, dtype=F32), 5126, "VEC3", True)}
        if m.normals is not None:
            attrs["NORMAL"] = add(np.ascontiguousarray(m.normals, dtype=F32), 5126, "VEC3")
        if m.tangents is not None:
            attrs["TANGENT"] = add(np.ascontiguousarray(m.tangents, dtype=F32), 5126, "VEC4")
        if m.texcoord0 is not None:
            attrs["TEXCOORD_0"] = add(np.ascontiguousarray(m.texcoord0, dtype=F32), 5126, "VEC2")
            if m.texcoord1 is not None:
                attrs["TEXCOORD_1"] = add(np.ascontiguousarray(m.texcoord1, dtype=F32), 5126, "VEC2")
        ind = add(np.ascontiguousarray(m.faces, dtype=np.uint32).reshape(-1), 5125, "SCALAR")
        prim = {"attributes": attrs, "indices": ind}
        if 0 <= m.material < len(scene.materials):
            prim["material"] = mat_index[m.material]
        gl_meshes.append({"name": m.name, "primitives": [prim]})

    extensions, nodes, scene_nodes = {}, [], []
    used = ["OpenMaterial_reference_link"] if any(x.type == 1 for x in scene.materials) else []
    if scene.gltf_nodes:
        # one root node (translated) holding a node per mesh and the light node
        cfg = scene.gltf_nodes[0]
        nm = len(scene.meshes)
        lights = cfg.get("lights") or [{"translation": cfg["light_translation"], "color": cfg["light_color"],
                                        "intensity": cfg["light_intensity"]}]
        nodes.append({"name": "root", "translation": list(cfg["root_translation"]),
                      "children": list(range(1, nm + 1 + len(lights)))})
        for i, m in enumerate(scene.meshes):
            nodes.append({"name": m.name, "mesh": i})
        gl_lights = []
        for i, lt in enumerate(lights):
            nodes.append({"name": f"light{i}" if i else "light", "translation": list(lt["translation"]),
                          "extensions": {"KHR_lights_punctual": {"light": i}}})
            rec = {"type": "point", "color": list(lt["color"]), "intensity": lt["intensity"]}
            if lt.get("range"):
                rec["range"] = lt["range"]
            gl_lights.append(rec)
        extensions["KHR_lights_punctual"] = {"lights": gl_lights}
        used.append("KHR_lights_punctual")
        scene_nodes = [0]
    else:
        for i, inst in enumerate(scene.instances):
            M = np.asarray(inst.transform, dtype=F32)
            nodes.append({"name": f"n{i}", "mesh": inst.mesh,
                          "matrix": [float(M[r, c]) for c in range(4) for r in range(4)]})
            scene_nodes.append(i)
    bin_name = f"{scene.name}.bin"
    doc = {"asset": {"version": "2.0", "generator": "omv synthetic scene generator"},
           "scene": 0, "scenes": [{"nodes": scene_nodes}], "nodes": nodes, "meshes": gl_meshes,
           "materials": gl_mats, "accessors": accessors, "bufferViews": views,
           "buffers": [{"uri": bin_name, "byteLength": len(blob)}]}
    if scene.textures:
        images = []
        for i, img in enumerate(scene.textures):
            name = f"{scene.name}_tex{i}.png"
            write_png(os.path.join(dirname, name), img)
            images.append({"uri": name})
        doc["images"] = images
        doc["samplers"] = [{}]
        doc["textures"] = [{"source": i, "sampler": 0} for i in range(len(images))]
        refs = [getattr(m, slot) for m in scene.materials for slot in
                ("base_color_texture", "metallic_roughness_texture", "normal_texture", "occlusion_texture",
                 "emissive_texture")]
        if any(r is not None and (r.offset is not None or r.rotation is not None or r.scale is not None)
               for r in refs):
            used.append("KHR_texture_transform")
    if extensions:
        doc["extensions"] = extensions
    if used:
        doc["extensionsUsed"] = used
    with open(os.path.join(dirname, bin_name), "wb") as fh:
        fh.write(bytes(blob))
    gltf = os.path.join(dirname, f"{scene.name}.gltf")
    with open(gltf, "w") as fh:
        json.dump(doc, fh)
    r = scene.render
    aspect = scene.camera.width / scene.camera.height
    flags = ["-i", gltf, "-r", str(scene.camera.width), "-a", repr(F32(aspect).item()),
             "-S", str(r.samples_per_pixel), "-q", str(r.max_path_length), "-B", str(r.camera_bounces),
             "-b", str(r.light_bounces)]
    if scene.lights:
        flags.append("-L")
    if scene.camera.json_props is not None:
        cam_path = os.path.join(dirname, f"{scene.name}_camera.json")
        with open(cam_path, "w") as fh:
            json.dump(scene.camera.json_props, fh)
        flags += ["-l", cam_path]
    if scene.hdri is not None:
        hdr_path = os.path.join(dirname, f"{scene.name}_sky.hdr")
        write_hdr(hdr_path, scene.hdri.rgb)
        flags += ["-H", hdr_path]
    return {"gltf": gltf, "flags": flags}
