"""Generates the golden fixtures in this directory by running the reference
renderer's own code (built from its unmodified sources by oracle/Makefile
`make ref` against the Embree-API shim).  Needs the reference tree where
the oracle recipe finds it (its REF, or OMV_REFERENCE) and runs on the
development host only; the
fixtures it writes are committed and are all the tests need elsewhere.

    python tests/golden/make_golden.py [--only name,...] [--big]

Fixtures (numpy .npz):
  mt.npz            RandomSampler draws (std::mt19937 + uniform_real_distribution<float>)
  brdf_eval.npz     BSDFModel<GGX>::evaluateDirect on seeded inputs
  brdf_sample.npz   BSDFModel<GGX>::sampleIndirect with RandomSampler(seed) per case
  om.npz            OpenMaterial::getBrdf (Fresnel of a complex IOR) for the C1 conductor
  ior.npz           AssetMaterialIor::getIor on a synthetic IOR table
  env.npz           HDRBackground::getRadiance on a synthetic RGBE image
  camera.npz        PinholeCamera::loadProperties + getRay (one RandomSampler)
  scene_<s>.npz     the committed RenderScene of scene <s> (vertex block, normal
                    matrices, material ids, lights) dumped after commitScene
  film_<s>.npz      linear film (PinholeCamera after stop) of a -C 1 render + ray count
  ids_c1_64.npz     primary rays and hits of the false-colour (-F mid) pass
  post.npz          gammaCorrection (two gammas), SimpleDenoiserMedian<1> and
                    saveImage's 8-bit conversion on a seeded 23x37 HDR image
  texture.npz       BitmapTexture::texture on seeded images and coordinates
                    (wrapping, negative, texel-centre and edge cases)
  film_textured_32x8.npz / scene_textured.npz
                    -C 1 film and committed scene of the textured PBR scene
  film_lights_32x4_A<a>.npz / scene_lights.npz
                    -C 1 films at -A 0, 1, 2 and the committed scene of three
                    coloured point lights (one with a glTF range)
  png.npz           stb_image's RGBA decode (as tinygltf loads images) of seeded PNG
                    files of every colour type, depth and row filter
  assets.npz        digests of the reference's committed scene for each of its own
                    objects/ and scenes/ assets (pathtracer -L, the OMV_REF_SCENE dump)
  fc.npz            false-colour films (-F pid gid mid mmp rmp md sg mn in, and an
                    unknown name) of the validation scene, before tone mapping
  lightbox.npz      the 8 light-box views (-V) of the mixed scene: cameras
                    (ViewPoint, half sizes, focus) and linear films
"""
from __future__ import annotations

import argparse
import importlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
S = importlib.import_module("openmaterial-validation_gb300.scenes")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF = None  # the reference tree, set by main() after the recipe has built it
BIN = os.path.join(ROOT, "oracle", "_ref")


def run(cmd, env=None):
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed ({r.returncode}):\n{r.stdout[-3000:]}\n{r.stderr[-3000:]}")
    return r


def harness(*args):
    return run([os.path.join(BIN, "golden_harness"), *map(str, args)])


def f32file(d, name, arr):
    p = os.path.join(d, name)
    np.ascontiguousarray(arr, dtype=np.float32).tofile(p)
    return p


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def gen_mt(tmp):
    out = os.path.join(tmp, "mt.bin")
    harness("mt", 3254638, 20000, out)
    np.savez_compressed(os.path.join(HERE, "mt.npz"), seed=3254638, u=np.fromfile(out, dtype=np.float32))


def gen_brdf(tmp):
    rng = np.random.default_rng(1)
    n = 4000
    N = unit(rng, n)
    V = unit(rng, n)
    V[: n * 3 // 4] = np.where((np.sum(V * N, 1) < 0)[:, None], -V, V)[: n * 3 // 4]
    L = unit(rng, n)
    L[: n * 3 // 4] = np.where((np.sum(L * N, 1) < 0)[:, None], -L, L)[: n * 3 // 4]
    I = -V
    color = np.concatenate([rng.uniform(0, 1, (n, 3)), np.ones((n, 1))], 1)
    metal = rng.uniform(0, 1, n)
    metal[::5] = 0.0
    metal[1::5] = 1.0
    rough = rng.uniform(0.02, 1.0, n)
    alpha = rough ** 2
    x = np.zeros((n, 17), dtype=np.float32)
    x[:, 0:3], x[:, 3:6], x[:, 6:9], x[:, 9:13], x[:, 13], x[:, 14] = I, L, N, color, metal, alpha
    out = os.path.join(tmp, "eval.out")
    harness("eval", f32file(tmp, "eval.in", x), out)
    np.savez_compressed(os.path.join(HERE, "brdf_eval.npz"), x=x, y=np.fromfile(out, dtype=np.float32).reshape(n, 3))
    # sampleIndirect: random frames, both facing sides, transmissive cases
    N = unit(rng, n)
    T = unit(rng, n)
    T = T - N * np.sum(T * N, 1, keepdims=True)
    T /= np.linalg.norm(T, axis=1, keepdims=True)
    V = unit(rng, n)
    I = -V
    color = np.concatenate([rng.uniform(0, 1, (n, 3)), np.where(rng.uniform(0, 1, (n, 1)) < 0.3,
                                                                 rng.uniform(0.1, 1, (n, 1)), 1.0)], 1)
    x = np.zeros((n, 24), dtype=np.float32)
    x[:, 0:3], x[:, 3:6], x[:, 6:9], x[:, 9:13] = I, N, T, color
    x[:, 13] = rng.uniform(0, 1, n)
    x[:, 14] = rng.uniform(0.02, 1.0, n) ** 2
    x[:, 15] = np.where(rng.uniform(0, 1, n) < 0.5, 1.0 / 1.5, 1.0)
    x[:, 16] = (rng.uniform(0, 1, n) < 0.4).astype(np.float32)
    seeds = np.arange(1000, 1000 + n, dtype=np.uint32)
    x[:, 17] = seeds.view(np.float32)
    out = os.path.join(tmp, "sample.out")
    harness("sample", f32file(tmp, "sample.in", x), out)
    np.savez_compressed(os.path.join(HERE, "brdf_sample.npz"), x=x, seeds=seeds,
                        y=np.fromfile(out, dtype=np.float32).reshape(n, 6))


def gen_om(tmp):
    sc = S.scene_c1(8, 8, 1)
    d = os.path.join(tmp, "om")
    S.write_gltf(sc, d)
    mat = sc.materials[0]
    c = np.concatenate([np.linspace(1e-3, 1.0, 400), np.random.default_rng(2).uniform(0, 1, 600)]).astype(np.float32)
    out = os.path.join(tmp, "om.out")
    harness("om", os.path.join(d, f"{mat.name}.gltf"), f32file(tmp, "om.in", c), out)
    np.savez_compressed(os.path.join(HERE, "om.npz"), cos=c, y=np.fromfile(out, dtype=np.float32).reshape(-1, 3),
                        n=np.array([0.18, 0.42, 1.37], dtype=np.float32),
                        k=np.array([3.42, 2.35, 1.77], dtype=np.float32))


def gen_ior(tmp):
    rng = np.random.default_rng(3)
    wl = np.sort(rng.uniform(2.0e-7, 1.2e-6, 60))
    nv = 1.0 + np.cumsum(rng.uniform(-0.05, 0.08, 60)).clip(-0.5, 3)
    kv = np.abs(2.0 + np.cumsum(rng.uniform(-0.1, 0.1, 60)))
    mat = S.Material(type=1, ior_n=np.stack([wl, nv], 1), ior_k=np.stack([wl, kv], 1), name="synthetic")
    d = os.path.join(tmp, "ior")
    os.makedirs(d, exist_ok=True)
    S._write_om_material(d, mat)
    q = np.stack([np.full(500, 300.0), np.concatenate([rng.uniform(wl[0], wl[-1], 496),
                                                       np.float32(wl[[0, 5, 30, -1]])])], 1).astype(np.float32)
    out = os.path.join(tmp, "ior.out")
    harness("ior", os.path.join(d, "synthetic_ior.gltf"), f32file(tmp, "ior.in", q), out)
    tab_n = np.stack([wl, nv], 1).astype(np.float32)
    tab_k = np.stack([wl, kv], 1).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "ior.npz"), q=q, y=np.fromfile(out, dtype=np.float32).reshape(-1, 2),
                        table_n=tab_n, table_k=tab_k)


def gen_env(tmp):
    rng = np.random.default_rng(4)
    img = S.make_sky(64, 32, rng) * np.float32(0.001)
    img = S.rgbe_quantize(img)
    hdr = os.path.join(tmp, "env.hdr")
    S.write_hdr(hdr, img)
    dirs = np.concatenate([unit(rng, 3000), np.eye(3), -np.eye(3),
                           [[0.0, 1.0, 1e-7], [1e-7, 1.0, 0.0], [0.0, -1.0, 0.0]]]).astype(np.float32)
    R = np.array([[1, 0, 0], [0, 0, 1], [0, -1, 0]], dtype=np.float32)
    scale = np.float32(np.pi)
    inp = np.concatenate([R.reshape(-1), [scale], dirs.reshape(-1)]).astype(np.float32)
    out = os.path.join(tmp, "env.out")
    harness("env", hdr, f32file(tmp, "env.in", inp), out)
    np.savez_compressed(os.path.join(HERE, "env.npz"), image=S.read_hdr(hdr), rotation=R, scale=scale, dirs=dirs,
                        y=np.fromfile(out, dtype=np.float32).reshape(-1, 3))


def gen_camera(tmp):
    sc = S.scene_c1(48, 40, 1)
    d = os.path.join(tmp, "cam")
    S.write_gltf(sc, d)
    out = os.path.join(tmp, "cam.out")
    harness("camera", os.path.join(d, "c1_camera.json"), 48, 40, 777, out)
    y = np.fromfile(out, dtype=np.float32)
    np.savez_compressed(os.path.join(HERE, "camera.npz"), width=48, height=40, seed=777, sizes=y[:3],
                        rays=y[3:].reshape(-1, 6), json=str(sc.camera.json_props))


def read_scene_dump(path):
    raw = open(path, "rb").read()
    off = 0

    def i32():
        nonlocal off
        v = int(np.frombuffer(raw, np.int32, 1, off)[0])
        off += 4
        return v

    def f32(n):
        nonlocal off
        v = np.frombuffer(raw, np.float32, n, off).copy()
        off += 4 * n
        return v

    assert i32() == 0x4F4D5631
    ok = i32()
    out = {"ok": ok}
    nm = i32()
    verts, faces, mesh_mat = [], [], []
    for _ in range(nm):
        mid, vn, fn, mat, stride = i32(), i32(), i32(), i32(), i32()
        mesh_mat.append(mat)
        if vn > 0 and fn > 0:
            faces.append(np.frombuffer(raw, np.uint32, 3 * fn, off).reshape(fn, 3).copy())
            off += 12 * fn
            verts.append(f32(10 * vn).reshape(vn, 10))
        else:
            faces.append(np.zeros((0, 3), np.uint32))
            verts.append(np.zeros((0, 10), np.float32))
    ni = i32()
    xf, nmx, imesh = [], [], []
    for _ in range(ni):
        i32()
        imesh.append(i32())
        xf.append(f32(16).reshape(4, 4))
        nmx.append(f32(9).reshape(3, 3))
    nmat = i32()
    mtype, mrec = [], []
    for _ in range(nmat):
        mtype.append(i32())
        mrec.append(f32(16))
    nl = i32()
    lights = [f32(8) for _ in range(nl)]
    out["has_background"] = i32()
    out.update(mesh_material=np.array(mesh_mat, np.int32), inst_mesh=np.array(imesh, np.int32),
               inst_xf=np.array(xf, np.float32).reshape(-1, 4, 4), inst_nrm=np.array(nmx, np.float32).reshape(-1, 3, 3),
               mat_type=np.array(mtype, np.int32), mat_rec=np.array(mrec, np.float32).reshape(-1, 16),
               lights=np.array(lights, np.float32).reshape(-1, 8))
    for i, (v, f) in enumerate(zip(verts, faces)):
        out[f"verts{i}"] = v
        out[f"faces{i}"] = f
    return out


def render_reference(sc, tmp, exe="pathtracer", extra=(), log=None):
    d = os.path.join(tmp, f"{sc.name}_{sc.camera.width}_{sc.render.samples_per_pixel}_{exe}")
    out = S.write_gltf(sc, d)
    env = dict(os.environ, OMV_REF_FILM=os.path.join(d, "film.bin"), OMV_REF_SCENE=os.path.join(d, "scene.bin"))
    if log:
        env["OMV_SHIM_LOG"] = log
    r = run([os.path.join(BIN, exe), *out["flags"], "-C", "1", "-o", os.path.join(d, "out.png"), *extra], env=env)
    line = [l for l in r.stderr.splitlines() if l.startswith("OMV_REF_RENDER")][0].split()
    hdr = np.fromfile(os.path.join(d, "film.bin"), dtype=np.int32, count=2)
    film = np.fromfile(os.path.join(d, "film.bin"), dtype=np.float32)[2:].reshape(hdr[1], hdr[0], 4)
    return film, float(line[1]), int(line[2]), read_scene_dump(os.path.join(d, "scene.bin"))


def gen_lights(tmp):
    """Three coloured point lights, one ranged, at attenuation modes 0, 1, 2
    (-A): films and the committed scene (light positions, G/B-ordered
    intensities, ranges, powers)."""
    sc = S.scene_lights(32, 32, 4)
    for A in (0, 1, 2):
        film, secs, rays, dump = render_reference(sc, tmp, extra=["-A", str(A)])
        np.savez_compressed(os.path.join(HERE, f"film_lights_32x4_A{A}.npz"), film=film, seconds=secs, rays=rays,
                            width=32, height=32, spp=4, attenuation=A)
    np.savez_compressed(os.path.join(HERE, "scene_lights.npz"), **dump)


def gen_films(tmp, big=False):
    jobs = [("film_c1_32x4", S.scene_c1(32, 32, 4)), ("film_mixed_32x8", S.scene_mixed(32, 32, 8)),
            ("film_c1_64x1024", S.scene_c1(64, 64, 1024))]
    if big:
        jobs.append(("film_c1_256x4096", S.scene_c1(256, 256, 4096)))
    for name, sc in jobs:
        film, secs, rays, dump = render_reference(sc, tmp)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), film=film, seconds=secs, rays=rays,
                            width=sc.camera.width, height=sc.camera.height, spp=sc.render.samples_per_pixel)
        if name in ("film_c1_32x4", "film_mixed_32x8"):
            np.savez_compressed(os.path.join(HERE, f"scene_{sc.name}.npz"), **dump)
        print(name, film.shape, secs, rays)


def gen_ids(tmp):
    sc = S.scene_c1(64, 64, 1)
    log = os.path.join(tmp, "shim.log")
    if os.path.exists(log):
        os.remove(log)
    render_reference(sc, tmp, exe="pathtracer_fc", extra=["-F", "mid"], log=log)
    rec = np.fromfile(log, dtype=np.uint8).reshape(-1, 64)
    f = rec[:, :32].copy().view(np.float32).reshape(-1, 8)
    u = rec[:, 32:48].copy().view(np.uint32).reshape(-1, 4)
    g = rec[:, 48:60].copy().view(np.float32).reshape(-1, 3)
    assert len(rec) == 64 * 64, len(rec)
    np.savez_compressed(os.path.join(HERE, "ids_c1_64.npz"), rays=f, hit=u[:, 0], geom=u[:, 1], inst=u[:, 2],
                        prim=u[:, 3], u=g[:, 0], v=g[:, 1], t=g[:, 2])


def gen_post(tmp):
    rng = np.random.default_rng(9)
    W, H = 23, 37
    img = rng.lognormal(-1.5, 1.5, size=(H, W, 4)).astype(np.float32)
    img[rng.random((H, W)) < 0.08] = 0.0                       # black pixels: l = 0
    img[rng.random((H, W)) < 0.04, :3] = np.float32(1e-8)       # below FLT_EPSILON
    img[rng.random((H, W)) < 0.05] *= np.float32(40.0)          # fireflies, clamped
    img[:4, :4, :3] = np.floor(img[:4, :4, :3] * 4) / 4         # ties in the median windows
    src = f32file(tmp, "post.in", img)
    out = {"image": img}
    for name, g in (("tonemap_0.5", 0.5), ("tonemap_0.4545", 0.4545)):
        o = os.path.join(tmp, name)
        harness("tonemap", W, H, g, src, o)
        out[name] = np.fromfile(o, dtype=np.float32).reshape(H, W, 4)
    tm = f32file(tmp, "post.tm", out["tonemap_0.5"])
    o = os.path.join(tmp, "post.med")
    harness("median", W, H, tm, o)
    out["median"] = np.fromfile(o, dtype=np.float32).reshape(H, W, 4)
    o = os.path.join(tmp, "post.u8")
    harness("rgba8", W, H, tm, o)
    out["rgba8"] = np.fromfile(o, dtype=np.uint8).reshape(H, W, 4)
    np.savez_compressed(os.path.join(HERE, "post.npz"), **out)


def gen_texture(tmp):
    rng = np.random.default_rng(12)
    out = {}
    for k, (W, H) in enumerate(((7, 5), (64, 32), (1, 1))):
        img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
        uv = np.concatenate([rng.uniform(-3.0, 3.0, (3000, 2)),
                             (np.stack(np.meshgrid(np.arange(W + 1), np.arange(H + 1)), -1).reshape(-1, 2) + 0.5)
                             / np.array([W, H]),
                             [[0.0, 0.0], [1.0, 1.0], [-1e-7, 1e-7], [0.5 / W, 0.5 / H], [1.0 - 1e-7, 0.9999999]]]
                            ).astype(np.float32)
        pi = os.path.join(tmp, f"tex{k}.bin")
        img.tofile(pi)
        o = os.path.join(tmp, f"tex{k}.out")
        harness("texture", W, H, pi, f32file(tmp, f"uv{k}.bin", uv), o)
        out[f"img{k}"], out[f"uv{k}"] = img, uv
        out[f"y{k}"] = np.fromfile(o, dtype=np.float32).reshape(-1, 4)
    np.savez_compressed(os.path.join(HERE, "texture.npz"), **out)


def gen_textured(tmp):
    sc = S.scene_textured(32, 32, 8)
    film, secs, rays, dump = render_reference(sc, tmp)
    np.savez_compressed(os.path.join(HERE, "film_textured_32x8.npz"), film=film, seconds=secs, rays=rays,
                        width=32, height=32, spp=8)
    np.savez_compressed(os.path.join(HERE, "scene_textured.npz"), **dump)


def write_png_variant(path, samples, ctype, depth, filters, palette=None, trns=None):
    """A PNG file with the given samples (H, W, C), colour type, bit depth and
    per-row filter types (0-4), for decoder checks."""
    import struct
    import zlib

    h, w = samples.shape[:2]
    if depth == 16:
        rows = [samples[y].astype(">u2").tobytes() for y in range(h)]
    elif depth == 8:
        rows = [samples[y].astype(np.uint8).tobytes() for y in range(h)]
    else:
        rows = []
        per = 8 // depth
        for y in range(h):
            b = bytearray((w * depth + 7) // 8)
            for x in range(w):
                b[x // per] |= int(samples[y, x, 0]) << (8 - depth * (x % per + 1))
            rows.append(bytes(b))
    bpp = max(1, (depth * samples.shape[2]) // 8)
    raw = bytearray()
    prev = bytes(len(rows[0]))
    for y, row in enumerate(rows):
        f = filters[y % len(filters)]
        out = bytearray(len(row))
        for x in range(len(row)):
            a = row[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) >> 1
            else:
                q = a + b - c
                pa, pb, pc = abs(q - a), abs(q - b), abs(q - c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            out[x] = (row[x] - p) & 0xFF
        raw.append(f)
        raw += out
        prev = row

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)

    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        data += chunk(b"tRNS", trns)
    data += chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(data)


def gen_png(tmp):
    import struct

    rng = np.random.default_rng(21)
    cases = []
    for ctype, chans in ((0, 1), (2, 3), (4, 2), (6, 4)):
        for depth in (8, 16):
            top = 255 if depth == 8 else 65535
            cases.append((ctype, depth, rng.integers(0, top + 1, (9, 13, chans)), None, None))
    for depth in (1, 2, 4, 8):
        pal = rng.integers(0, 256, (1 << depth, 3))
        trns = bytes(rng.integers(0, 256, max(1, (1 << depth) // 2)).astype(np.uint8))
        cases.append((3, depth, rng.integers(0, 1 << depth, (7, 11, 1)), pal, trns))
    for depth in (1, 2, 4):
        cases.append((0, depth, rng.integers(0, 1 << depth, (6, 10, 1)), None, None))
    key = struct.pack(">HHH", 10, 20, 30)
    s = rng.integers(0, 40, (8, 8, 3))
    s[2, 3] = (10, 20, 30)
    cases.append((2, 8, s, None, key))
    out = {}
    for i, (ct, d, smp, pal, tr) in enumerate(cases):
        p = os.path.join(tmp, f"v{i}.png")
        write_png_variant(p, smp, ct, d, [0, 1, 2, 3, 4], pal, tr)
        o = os.path.join(tmp, f"v{i}.out")
        harness("png", p, o)
        wh = np.fromfile(o, dtype=np.int32, count=2)
        px = np.fromfile(o, dtype=np.uint16, offset=8).reshape(wh[1], wh[0], 4)
        out[f"file{i}"] = np.frombuffer(open(p, "rb").read(), dtype=np.uint8)
        out[f"rgba{i}"] = px
        out[f"bits{i}"] = d
    out["count"] = len(cases)
    np.savez_compressed(os.path.join(HERE, "png.npz"), **out)


def gen_hdr(tmp):
    """Radiance files in every form stb_image's HDR loader takes (flat and
    run-length scanlines, both signatures, extra header lines, widths at the
    RLE limits, the mid-file fallback to flat pixels, zero exponents)."""
    rng = np.random.default_rng(23)

    def sky(h, w):
        img = np.exp(rng.normal(size=(h, w, 3))).astype(np.float32)
        img[:, w // 4:w // 2] = img[:, w // 4:w // 4 + 1]  # runs
        img[0, 0] = (2.0, 1.0, 0.5)                          # not an RLE marker as a flat first pixel
        return img

    def hdr_bytes(img, rle, head=b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n"):
        p = os.path.join(tmp, "w.hdr")
        S.write_hdr(p, img, rle=rle)
        raw = open(p, "rb").read()
        return head + raw[raw.index(b"\n\n") + 2:]

    files = [hdr_bytes(sky(3, 5), False), hdr_bytes(sky(7, 40), True), hdr_bytes(sky(2, 8), True),
             hdr_bytes(sky(3, 300), True,
                       b"#?RGBE\n# written by a test\nEXPOSURE=1.0\nFORMAT=32-bit_rle_rgbe\nGAMMA=1\n\n"),
             hdr_bytes(sky(4, 16), False)]
    a = hdr_bytes(sky(5, 12), True)
    z = S.rgbe_encode(sky(5, 12)).tobytes()
    files.append(a[:a.index(b"\x02\x02\x00\x0c", a.index(b"\x02\x02\x00\x0c") + 1)] + z[:4 * 60])
    dark = sky(2, 9)
    dark[1, 3] = 0.0
    files.append(hdr_bytes(dark, True))
    out = {}
    for i, raw in enumerate(files):
        p = os.path.join(tmp, f"h{i}.hdr")
        open(p, "wb").write(raw)
        o = os.path.join(tmp, f"h{i}.out")
        harness("hdr", p, o)
        whc = np.fromfile(o, dtype=np.int32, count=3)
        out[f"file{i}"] = np.frombuffer(raw, dtype=np.uint8)
        out[f"rgb{i}"] = np.fromfile(o, dtype=np.float32, offset=12).reshape(whc[1], whc[0], 3)
    out["count"] = len(files)
    np.savez_compressed(os.path.join(HERE, "hdr.npz"), **out)


ASSETS = ["objects/" + n for n in (
    "cone_gold", "cube_aluminium", "cube_gold", "cube_pbr_gold", "cubes_pbr", "icospheres_gold_iron_aluminium",
    "icospheres_gold_iron_missing", "monkey_gold", "plane_pointlight", "sphere_aluminium", "sphere_gold",
    "teapot_aluminium", "teapot_gold", "teapot_iron", "torus_aluminium", "torus_gold", "torus_pbr",
    "truck_example", "vehicle_example")] + ["scenes/multiple_instances"]


def scene_digest(meshes_v, meshes_f, mesh_rec, inst_mesh, inst_xf, inst_nrm, lights):
    """What the asset checks compare: per mesh a hash of its committed vertex
    block and faces and the record of its material; instances; lights."""
    import hashlib

    def canon(v):  # one NaN pattern: the payload of a NaN is not part of the contract
        v = np.array(v, np.float32)
        v[np.isnan(v)] = np.float32("nan")
        return v

    mh = np.array([int(hashlib.sha1(canon(v).tobytes() +
                                    np.ascontiguousarray(f, np.uint32).tobytes()).hexdigest()[:15], 16)
                   for v, f in zip(meshes_v, meshes_f)], dtype=np.int64)
    return {"mesh_hash": mh, "mesh_rec": np.asarray(mesh_rec, np.float32).reshape(len(mh), -1),
            "inst_mesh": np.asarray(inst_mesh, np.int32), "inst_xf": np.asarray(inst_xf, np.float32),
            "inst_nrm": np.asarray(inst_nrm, np.float32), "lights": np.asarray(lights, np.float32).reshape(-1, 8)}


def gen_assets(tmp):
    out = {}
    for a in ASSETS:
        path = os.path.join(REF, a + ".gltf")
        dump = os.path.join(tmp, "asset.bin")
        env = dict(os.environ, OMV_REF_SCENE=dump)
        run([os.path.join(BIN, "pathtracer"), "-i", path, "-r", "4", "-a", "1", "-S", "1", "-B", "1", "-b", "1",
             "-L", "-C", "1", "-o", os.path.join(tmp, "asset.png")], env=env)
        d = read_scene_dump(dump)
        nm = len(d["mesh_material"])
        recs = []
        for i in range(nm):
            mi = int(d["mesh_material"][i])
            if 0 <= mi < len(d["mat_type"]) and d["mat_type"][mi] != 2:
                recs.append(np.concatenate([[d["mat_type"][mi]], d["mat_rec"][mi]]).astype(np.float32))
            else:
                recs.append(np.concatenate([[2], np.zeros(16)]).astype(np.float32))
        dg = scene_digest([d[f"verts{i}"] for i in range(nm)], [d[f"faces{i}"] for i in range(nm)], recs,
                          d["inst_mesh"], d["inst_xf"], d["inst_nrm"], d["lights"])
        key = a.replace("/", "__")
        for k, v in dg.items():
            out[f"{key}.{k}"] = v
        print(a, nm, len(d["inst_mesh"]), len(d["lights"]))
    np.savez_compressed(os.path.join(HERE, "assets.npz"), **out)


FC_SUBJECTS = ["pid", "gid", "mid", "mmp", "rmp", "md", "sg", "mn", "in", "nosuch"]


def gen_fc(tmp):
    sc = S.scene_validation(64, 48)
    out = {}
    for name in FC_SUBJECTS:
        film, _, _, dump = render_reference(sc, tmp, exe="pathtracer_fc", extra=["-F", name])
        out[name] = film
    out["width"], out["height"] = sc.camera.width, sc.camera.height
    np.savez_compressed(os.path.join(HERE, "fc.npz"), **out)
    np.savez_compressed(os.path.join(HERE, "scene_validation.npz"), **dump)


def gen_lightbox(tmp):
    sc = S.scene_mixed(32, 32, 32)
    d = os.path.join(tmp, "lightbox")
    o = S.write_gltf(sc, d)
    cams = os.path.join(d, "cameras.bin")
    if os.path.exists(cams):
        os.remove(cams)
    env = dict(os.environ, OMV_REF_FILM=os.path.join(d, "film_%d.bin"), OMV_REF_CAMERAS=cams)
    run([os.path.join(BIN, "pathtracer"), *o["flags"], "-C", "1", "-V", "-o", os.path.join(d, "out.png")], env=env)
    films = []
    for k in range(8):
        p = os.path.join(d, f"film_{k}.bin")
        hdr = np.fromfile(p, dtype=np.int32, count=2)
        films.append(np.fromfile(p, dtype=np.float32)[2:].reshape(hdr[1], hdr[0], 4))
    c = np.fromfile(cams, dtype=np.float32).reshape(-1, 15)
    assert len(c) == 8, c.shape
    np.savez_compressed(os.path.join(HERE, "lightbox.npz"), films=np.stack(films), position=c[:, 0:3],
                        rotation=c[:, 3:12].reshape(8, 3, 3), half_width=c[:, 12], half_height=c[:, 13],
                        focus=c[:, 14], spp=sc.render.samples_per_pixel)


GENS = {"mt": gen_mt, "brdf": gen_brdf, "om": gen_om, "ior": gen_ior, "env": gen_env, "camera": gen_camera,
        "films": gen_films, "ids": gen_ids, "post": gen_post, "fc": gen_fc, "lightbox": gen_lightbox,
        "textured": gen_textured, "texture": gen_texture, "png": gen_png, "hdr": gen_hdr, "assets": gen_assets,
        "lights": gen_lights}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="")
    ap.add_argument("--big", action="store_true", help="also the 256x256 4096-spp C1 reference film")
    a = ap.parse_args()
    global REF
    run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"])
    REF = O.reference_tree()
    if REF is None:
        sys.exit("reference tree not found: set OMV_REFERENCE")
    names = [n for n in a.only.split(",") if n] or list(GENS)
    with tempfile.TemporaryDirectory() as tmp:
        for n in names:
            if n == "films":
                gen_films(tmp, a.big)
            else:
                GENS[n](tmp)
            print("wrote", n)


if __name__ == "__main__":
    main()
