"""glTF / OpenMATERIAL asset loading into the render path's scene description.

Host-side restatement of the reference's asset pipeline, from the file on disk
to the flattened scene main.cpp hands to RenderScene:

  AssetGeometry::loadGltf / loadData / loadNodes / loadMesh / loadMaterial
      (pathtracer/src/assets/AssetGeometry.cpp:303-772): nodes, meshes as
      primitive lists, OpenMATERIAL reference links on nodes (a referenced file
      is loaded once; later references copy its root nodes), materials by
      priority (checkMaterialType, :263-288), KHR_lights_punctual lights, images
  PbrMaterial (PbrMaterial.cpp:25-204): factors, texture slots, KHR_texture_transform
  AssetMaterial / AssetMaterialIor (AssetMaterial.cpp:300-309,
      AssetMaterialIor.cpp:47-98, 104-121): the OpenMATERIAL file, its IOR file
      and the tables of the temperature closest to the material's
  ImageData::load (ImageData.cpp:33-100) after tinygltf/stb: images as RGBA8
  main.cpp:280-395: the scene transformation (setUpTransformation, :47-80),
      material numbering, lights (with their green/blue order, :355-368),
      meshes (:370-389) and instances (iterateAssetGeometryNodes,
      AssetGeometry.h:180-200) in the reference's order.

Transforms are evaluated in float32 in the reference's operation order, so the
flattened instances equal the reference's bit for bit.  Images: PNG (8 and 16
bit, every colour type, non-interlaced); other formats raise ValueError.
"""
from __future__ import annotations

import base64
import dataclasses
import json
import math
import os
import struct
import zlib
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import scenes

F32 = np.float32
FLT_MAX = float(np.finfo(np.float32).max)


# --------------------------------------------------------------- float32 ---

def _mat_mul4(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """multSquareMatrix (UtilityFunctions.h:271-281): C[i][j] = 0 + sum_k A[i][k] B[k][j], in order."""
    C = np.zeros((4, 4), dtype=F32)
    for i in range(4):
        for j in range(4):
            acc = F32(0.0)
            for k in range(4):
                acc = F32(acc + F32(A[i, k] * B[k, j]))
            C[i, j] = acc
    return C


def _matrix_from_quaternion(q) -> np.ndarray:
    """matrixFromQuaternion (UtilityFunctions.h:363-377)."""
    one, two = F32(1.0), F32(2.0)
    q0, q1, q2, q3 = (F32(x) for x in q)
    M = np.zeros((3, 3), dtype=F32)
    M[0, 0] = one - two * F32(F32(q1 * q1) + F32(q2 * q2))
    M[0, 1] = two * F32(F32(q0 * q1) - F32(q2 * q3))
    M[0, 2] = two * F32(F32(q0 * q2) + F32(q1 * q3))
    M[1, 0] = two * F32(F32(q0 * q1) + F32(q2 * q3))
    M[1, 1] = one - two * F32(F32(q0 * q0) + F32(q2 * q2))
    M[1, 2] = two * F32(F32(q1 * q2) - F32(q0 * q3))
    M[2, 0] = two * F32(F32(q0 * q2) - F32(q1 * q3))
    M[2, 1] = two * F32(F32(q1 * q2) + F32(q0 * q3))
    M[2, 2] = one - two * F32(F32(q0 * q0) + F32(q1 * q1))
    return M


def _transformation_from_qts(q, t, s) -> np.ndarray:
    """transformationFromQTS (UtilityFunctions.h:500-516)."""
    R = _matrix_from_quaternion(q)
    M = np.zeros((4, 4), dtype=F32)
    for r in range(3):
        for c in range(3):
            M[r, c] = F32(R[r, c] * F32(s[c]))
        M[r, 3] = F32(t[r])
    M[3, 3] = F32(1.0)
    return M


def _node_matrix(node: dict) -> np.ndarray:
    """AssetGeometry::loadNodes (:549-563): column-major matrix, or T R S."""
    if node.get("matrix"):
        gm = node["matrix"]
        M = np.zeros((4, 4), dtype=F32)
        for i in range(16):
            M[i % 4, i // 4] = F32(gm[i])
        return M
    t = [F32(x) for x in node.get("translation", (0.0, 0.0, 0.0))]
    s = [F32(x) for x in node.get("scale", (1.0, 1.0, 1.0))]
    q = [F32(x) for x in node.get("rotation", (0.0, 0.0, 0.0, 1.0))]
    return _transformation_from_qts(q, t, s)


def _xform_point(M: np.ndarray, v) -> np.ndarray:
    """multVector3(fmat4, v): M[i][0] v0 + M[i][1] v1 + M[i][2] v2 + M[i][3]."""
    out = np.zeros(3, dtype=F32)
    for i in range(3):
        out[i] = F32(F32(F32(F32(M[i, 0] * F32(v[0])) + F32(M[i, 1] * F32(v[1]))) + F32(M[i, 2] * F32(v[2])))
                     + M[i, 3])
    return out


# ------------------------------------------------------------------- PNG ---

def decode_png(data: bytes) -> np.ndarray:
    """A PNG image as stb_image loads it with 4 requested channels, then
    ImageData::load's 8-bit conversion (16-bit samples / 256): (H, W, 4) uint8."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG image (only PNG textures are supported)")
    pos, idat = 8, bytearray()
    hdr = palette = trns = None
    while pos + 8 <= len(data):
        n, t = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if t == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif t == b"PLTE":
            palette = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif t == b"tRNS":
            trns = body
        elif t == b"IDAT":
            idat += body
        elif t == b"IEND":
            break
        pos += 12 + n
    if hdr is None:
        raise ValueError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    if interlace:
        raise ValueError("interlaced PNG images are not supported")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = depth * chans
    stride = (w * bits + 7) // 8
    bpp = max(1, bits // 8)
    raw = zlib.decompress(bytes(idat))
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 0xFF
        elif f == 1 and stride % bpp == 0:  # Sub: a running sum per byte lane
            cur = np.cumsum(line.reshape(-1, bpp), axis=0).reshape(-1) & 0xFF
        else:
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                b = prev[x]
                c = prev[x - bpp] if x >= bpp else 0
                if f == 1:
                    v = a
                elif f == 3:
                    v = (a + b) >> 1
                else:  # Paeth
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    v = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + v) & 0xFF
        out[y] = cur
        prev = cur
    if depth == 16:
        samples = out.view(">u2").reshape(h, w, chans).astype(np.uint32)
        top = 65535
    elif depth == 8:
        samples = out[:, :w * chans].reshape(h, w, chans).astype(np.uint32)
        top = 255
    else:  # 1, 2, 4 bit grey or palette
        per = 8 // depth
        idx = np.unpackbits(out, axis=1) if depth == 1 else None
        vals = np.zeros((h, w), dtype=np.uint32)
        for x in range(w):
            byte = out[:, (x * depth) // 8].astype(np.uint32)
            shift = 8 - depth * (x % per + 1)
            vals[:, x] = (byte >> shift) & ((1 << depth) - 1)
        del idx
        if ctype == 0:  # stb scales low-depth grey to 8 bits
            vals = vals * (255 // ((1 << depth) - 1))
        samples = vals[..., None]
        top = 255
    if ctype == 3:
        if palette is None:
            raise ValueError("palette PNG without PLTE")
        rgb = palette[samples[..., 0]].astype(np.uint32)
        alpha = np.full((h, w), 255, np.uint32)
        if trns is not None:
            ta = np.frombuffer(trns, dtype=np.uint8)
            sel = samples[..., 0] < len(ta)
            alpha[sel] = ta[samples[..., 0][sel]]
        rgba = np.concatenate([rgb, alpha[..., None]], axis=-1)
    else:
        if chans in (1, 2):
            g = samples[..., 0]
            a = samples[..., 1] if chans == 2 else np.full((h, w), top, np.uint32)
            rgba = np.stack([g, g, g, a], axis=-1)
        elif chans == 3:
            rgba = np.concatenate([samples, np.full((h, w, 1), top, np.uint32)], axis=-1)
        else:
            rgba = samples
        if trns is not None and chans in (1, 3):  # colour-key transparency
            key = np.array(struct.unpack(">" + "H" * (len(trns) // 2), trns), dtype=np.uint32)
            if depth < 8 and ctype == 0:
                key = key * (255 // ((1 << depth) - 1))
            hit = np.all(samples[..., :chans] == key[:chans], axis=-1)
            rgba = rgba.copy()
            rgba[..., 3] = np.where(hit, 0, rgba[..., 3])
    if depth == 16:
        rgba = rgba // 256
    return rgba.astype(np.uint8)


# ------------------------------------------------------------- documents ---

class _Doc:
    """One glTF document with its buffers (tinygltf's Model)."""

    def __init__(self, path: str):
        self.path = path
        self.dir = os.path.dirname(path)
        ext = os.path.splitext(path)[1].lower()
        with open(path, "rb") as fh:
            blob = fh.read()
        bin_chunk = None
        if ext == ".glb":
            magic, version, length = struct.unpack("<4sII", blob[:12])
            if magic != b"glTF":
                raise ValueError(f"{path}: not a binary glTF")
            pos, js = 12, None
            while pos < length:
                clen, ctype = struct.unpack("<I4s", blob[pos:pos + 8])
                chunk = blob[pos + 8:pos + 8 + clen]
                if ctype == b"JSON":
                    js = json.loads(chunk.decode("utf-8"))
                elif ctype == b"BIN\x00":
                    bin_chunk = chunk
                pos += 8 + clen
            self.j = js
        elif ext == ".gltf":
            self.j = json.loads(blob.decode("utf-8"))
        else:
            raise ValueError(f"Wrong file extension in file: {path}")
        self.buffers = []
        for b in self.j.get("buffers", []):
            uri = b.get("uri")
            if uri is None:
                self.buffers.append(bin_chunk or b"")
            elif uri.startswith("data:"):
                self.buffers.append(base64.b64decode(uri.split(",", 1)[1]))
            else:
                with open(os.path.join(self.dir, uri), "rb") as fh:
                    self.buffers.append(fh.read())

    def accessor(self, idx: int, dtype, ncomp: int) -> np.ndarray:
        a = self.j["accessors"][idx]
        v = self.j["bufferViews"][a["bufferView"]]
        buf = self.buffers[v["buffer"]]
        off = v.get("byteOffset", 0) + a.get("byteOffset", 0)
        n = a["count"] * ncomp
        return np.frombuffer(buf, dtype=dtype, count=n, offset=off)

    def indices(self, idx: int) -> np.ndarray:
        """copyIndicesFromArray (AssetGeometry.cpp:152-190)."""
        a = self.j["accessors"][idx]
        ct = a["componentType"]
        dt = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5124: np.int32}[ct]
        x = self.accessor(idx, dt, 1)
        if ct == 5120:
            return x.view(np.uint8).astype(np.uint32)
        return x.astype(np.int64).astype(np.uint32)

    def image(self, img: dict) -> Optional[np.ndarray]:
        if "uri" in img:
            uri = img["uri"]
            if uri.startswith("data:"):
                data = base64.b64decode(uri.split(",", 1)[1])
            else:
                with open(os.path.join(self.dir, uri), "rb") as fh:
                    data = fh.read()
        elif "bufferView" in img:
            v = self.j["bufferViews"][img["bufferView"]]
            buf = self.buffers[v["buffer"]]
            data = buf[v.get("byteOffset", 0):v.get("byteOffset", 0) + v["byteLength"]]
        else:
            return None
        return decode_png(data)


@dataclasses.dataclass
class _Node:
    name: str
    uri: str
    M: np.ndarray
    prims: List[int]
    children: List["_Node"] = dataclasses.field(default_factory=list)
    parent: Optional["_Node"] = None

    def copy(self) -> "_Node":
        """Node's copy constructor (Node.h:169-196): children copied deeply."""
        c = _Node(self.name, self.uri, self.M.copy(), list(self.prims))
        for ch in self.children:
            cc = ch.copy()
            cc.parent = c
            c.children.append(cc)
        return c

    def descendants(self) -> List["_Node"]:
        out = list(self.children)
        for ch in self.children:
            if ch.children:
                out += ch.descendants()
        return out

    def global_matrix(self) -> np.ndarray:
        """Node::getGlobalTransformation (Node.h:148-153)."""
        P = self.parent.global_matrix() if self.parent else np.eye(4, dtype=F32)
        return _mat_mul4(P, self.M)


@dataclasses.dataclass
class LoadedAsset:
    """The reference's AssetGeometry after loading, flattened like main.cpp."""
    scene: scenes.Scene
    bbox: Tuple[np.ndarray, np.ndarray]
    transformation: np.ndarray
    material_names: List[str]


class _Loader:
    def __init__(self, priority: str, use_lights: bool):
        if priority not in ("om", "pbr"):
            raise ValueError("Material loading priority has to be 'om' or 'pbr'")
        self.priority = priority
        self.use_lights = use_lights
        self.nodes: List[_Node] = []          # AssetGeometry::m_vpNodes
        self.prims: List[dict] = []           # m_vpPrimitives
        self.materials: List[dict] = []       # m_vpMaterials (OpenMATERIAL dedup by file name)
        self.missing = {"kind": "missing"}
        self.lights: List[Tuple[dict, _Node]] = []
        self.images: Dict[int, np.ndarray] = {}
        self.loaded_files: Dict[str, List[_Node]] = {}

    # AssetGeometry::checkMaterialType (:263-288)
    def _material_type(self, jm: dict) -> str:
        has_om = "OpenMaterial_reference_link" in jm.get("extensions", {})
        has_pbr = "pbrMetallicRoughness" in jm
        if self.priority == "om":
            if has_om:
                return "openMaterial"
            if has_pbr:
                return "pbr"
        else:
            if has_pbr:
                return "pbr"
            if has_om:
                return "openMaterial"
        return "unknown"

    def _load_material(self, doc: _Doc, idx: int) -> dict:
        mats = doc.j.get("materials", [])
        jm = mats[idx] if idx < len(mats) else {}  # a dangling index: the missing material
        kind = self._material_type(jm)
        if kind == "openMaterial":
            fname = doc.dir + os.sep + jm["extensions"]["OpenMaterial_reference_link"]["uri"]
            for m in self.materials:
                if m.get("file") == fname:
                    return m
            m = _load_open_material(fname)
            self.materials.append(m)
            return m
        if kind == "pbr":
            m = _load_pbr(doc, idx)
            self.materials.append(m)
            return m
        return self.missing

    def _load_mesh(self, doc: _Doc, mi: int, loaded_mats: Dict[int, dict]) -> List[int]:
        """AssetGeometry::loadMesh (:611-730)."""
        out = []
        gm = doc.j["meshes"][mi]
        for prim in gm["primitives"]:
            if prim.get("mode", 4) != 4:
                raise ValueError("primitives other than triangles not supported")
            mat = None
            midx = prim.get("material", -1)
            if midx >= 0:
                if midx not in loaded_mats:
                    loaded_mats[midx] = self._load_material(doc, midx)
                mat = loaded_mats[midx]
            p = {"name": gm.get("name", ""), "material": mat, "faces": doc.indices(prim["indices"]).reshape(-1, 3)}
            for attr, acc in prim["attributes"].items():
                a = doc.j["accessors"][acc]
                if attr == "POSITION":
                    p["positions"] = doc.accessor(acc, np.float32, 3).reshape(-1, 3)
                elif attr == "NORMAL":
                    p["normals"] = doc.accessor(acc, np.float32, 3).reshape(-1, 3)
                elif attr == "TANGENT":
                    p["tangents"] = doc.accessor(acc, np.float32, 4)
                elif attr.startswith("TEXCOORD_"):
                    ch = int(attr[9:])
                    if ch < 8:
                        p[f"uv{ch}"] = doc.accessor(acc, np.float32, 2).reshape(-1, 2)
                del a
            out.append(len(self.prims))
            self.prims.append(p)
        return out

    def _load_nodes(self, doc: _Doc) -> List[_Node]:
        """AssetGeometry::loadNodes (:470-609): the file's nodes go to the front."""
        jn = doc.j.get("nodes", [])
        fresh = [_Node(n.get("name", ""), "", np.eye(4, dtype=F32), []) for n in jn]
        self.nodes[0:0] = fresh
        loaded_meshes: Dict[int, List[int]] = {}
        loaded_mats: Dict[int, dict] = {}
        for k, n in enumerate(jn):
            node = fresh[k]
            link = n.get("extensions", {}).get("OpenMaterial_reference_link")
            if isinstance(link, dict) and "uri" in link:
                node.uri = link["uri"]
            mi = n.get("mesh", -1)
            if mi >= 0:
                if mi not in loaded_meshes:
                    loaded_meshes[mi] = self._load_mesh(doc, mi, loaded_mats)
                node.prims += loaded_meshes[mi]
            lp = n.get("extensions", {}).get("KHR_lights_punctual")
            if isinstance(lp, dict) and self.use_lights:
                li = lp["light"]
                self.lights.append((doc.j["extensions"]["KHR_lights_punctual"]["lights"][li], node))
            node.M = _node_matrix(n)
            for c in n.get("children", []):
                if c >= len(fresh):
                    raise ValueError(f"unresolved reference to node {c}")
                fresh[c].parent = node
                node.children.append(fresh[c])
        return fresh

    def load(self, path: str, parent: Optional[_Node] = None) -> None:
        """AssetGeometry::loadGltf (:303-391) with loadData (:433-468)."""
        doc = _Doc(path)
        for i, img in enumerate(doc.j.get("images", [])):  # ids restart per file (:774-782)
            data = doc.image(img)
            if data is not None:
                self.images[i] = data
        new_nodes = self._load_nodes(doc)
        for node in new_nodes:
            ref = node.uri
            if ref in self.loaded_files and ref:
                for child in self.loaded_files[ref]:
                    cp = child.copy()
                    self.nodes.append(cp)
                    self.nodes += cp.descendants()
                    cp.parent = node
                    node.children.append(cp)
                continue
            is_root = node.parent is None
            if parent is not None and is_root:
                node.parent = parent
                parent.children.append(node)
            if is_root and parent is not None and parent.uri:
                self.loaded_files.setdefault(parent.uri, []).append(node)
            if ref:
                self.load(doc.dir + os.sep + ref, node)


def _load_pbr(doc: _Doc, idx: int) -> dict:
    """PbrMaterial::loadPropertiesFromJson (PbrMaterial.cpp:122-204)."""
    jm = doc.j["materials"][idx]
    pmr = jm.get("pbrMetallicRoughness", {})
    mode = jm.get("alphaMode", "OPAQUE")
    if mode not in ("BLEND", "MASK", "OPAQUE"):
        raise ValueError("Invalid alpha-blending mode")

    def clamp01(x):
        x = F32(x)
        m = x if x < F32(1.0) else F32(1.0)
        return float(F32(0.0) if F32(0.0) > m else m)

    def slot(info):
        if not info or info.get("index", -1) < 0:
            return None
        tex = doc.j["textures"][info["index"]]
        t = info.get("extensions", {}).get("KHR_texture_transform")
        ref = scenes.TextureRef(texture=int(tex.get("source", -1)), texcoord=int(info.get("texCoord", 0)))
        if isinstance(t, dict):
            ref.offset = tuple(t["offset"]) if "offset" in t else (0.0, 0.0)
            ref.scale = tuple(t["scale"]) if "scale" in t else (1.0, 1.0)
            ref.rotation = float(t.get("rotation", 0.0))
        return ref

    nt = jm.get("normalTexture", {})
    ot = jm.get("occlusionTexture", {})
    return {
        "kind": "pbr",
        "material": scenes.Material(
            type=0, name=jm.get("name", ""),
            base_color=tuple(float(F32(x)) for x in pmr.get("baseColorFactor", (1.0, 1.0, 1.0, 1.0))),
            metallic=clamp01(pmr.get("metallicFactor", 1.0)), roughness=clamp01(pmr.get("roughnessFactor", 1.0)),
            alpha_mode={"OPAQUE": 0, "MASK": 1, "BLEND": 2}[mode], alpha_cutoff=clamp01(jm.get("alphaCutoff", 0.5)),
            double_sided=bool(jm.get("doubleSided", False)),
            base_color_texture=slot(pmr.get("baseColorTexture")),
            metallic_roughness_texture=slot(pmr.get("metallicRoughnessTexture")),
            normal_texture=slot(nt), occlusion_texture=slot(ot), emissive_texture=slot(jm.get("emissiveTexture")),
            normal_scale=float(F32(nt.get("scale", 1.0))), occlusion_strength=float(F32(ot.get("strength", 1.0))),
            emissive_factor=tuple(float(F32(x)) for x in jm.get("emissiveFactor", (0.0, 0.0, 0.0))))}


def _load_open_material(fname: str) -> dict:
    """AssetMaterial + AssetMaterialIor (AssetMaterial.cpp:248-309,
    AssetMaterialIor.cpp:47-121): the IOR tables of the temperature closest to
    the material's, sorted by wavelength."""
    with open(fname) as fh:
        j = json.load(fh)
    jm = j["materials"][0]
    params = jm["extensions"]["OpenMaterial_material_parameters"]
    temp = float(F32(params["user_preferences"]["temperature"]))
    if temp < 0:
        raise ValueError(f"{fname}: temperature must be non-negative")
    uri = params["physical_properties"]["refractive_index_uri"]
    n_tab = k_tab = None
    if uri:
        with open(os.path.join(os.path.dirname(fname), uri)) as fh:
            ji = json.load(fh)
        data = []
        for it in ji["extensions"]["OpenMaterial_ior_data"]["data"]:
            t = float(F32(it["temperature"]))
            if t < 0:
                raise ValueError("temperature must be non-negative")
            if "n" in it and "k" in it:
                n = np.array([[F32(w), F32(x)] for w, x in it["n"]], dtype=F32)
                k = np.array([[F32(w), F32(x)] for w, x in it["k"]], dtype=F32)
                n = n[np.argsort(n[:, 0], kind="stable")]
                k = k[np.argsort(k[:, 0], kind="stable")]
                data.append((t, n, k))
        data.sort(key=lambda d: d[0])
        if data:
            best, delta = 0, abs(F32(data[0][0] - temp))
            for i in range(1, len(data)):
                d = abs(F32(data[i][0] - temp))
                if d < delta:
                    best, delta = i, d
            _, n_tab, k_tab = data[best]
    mat = scenes.Material(type=1, name=jm.get("name", os.path.basename(fname)), temperature=temp,
                          ior_n=n_tab, ior_k=k_tab)
    return {"kind": "om", "file": fname, "material": mat}


def _bbox(loader: _Loader) -> Tuple[np.ndarray, np.ndarray]:
    """AssetGeometry::getBBox (:230-237, Node.h:132-166, Mesh.cpp:56-65)."""
    lo = np.full(3, np.inf, dtype=F32)
    hi = np.full(3, -np.inf, dtype=F32)

    def rec(node: _Node, ext: np.ndarray):
        M = _mat_mul4(ext, node.M)
        for pi in node.prims:
            for v in loader.prims[pi]["positions"]:
                p = _xform_point(M, v)
                np.minimum(lo, p, out=lo)
                np.maximum(hi, p, out=hi)
        for c in node.children:
            rec(c, M)

    for node in loader.nodes:
        if node.parent is None:
            rec(node, np.eye(4, dtype=F32))
    return lo, hi


def scene_transformation(bbc, rotation_zyx_deg=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0)) -> np.ndarray:
    """setUpTransformation (main.cpp:47-80): rotation about the bounding-box
    centre, then the translation (given as the -T option's values)."""
    deg = F32(F32(3.14159265358979323846) / F32(180.0))
    rot = [F32(x) for x in rotation_zyx_deg]
    a = [F32(rot[2] * deg), F32(rot[1] * deg), F32(rot[0] * deg)]  # reversed order
    s = [F32(scenes.sinf(x)) for x in a]
    c = [F32(scenes.cosf(x)) for x in a]
    one, zer = F32(1.0), F32(0.0)
    Rx = np.array([[one, zer, zer], [zer, c[0], s[0]], [zer, -s[0], c[0]]], dtype=F32)
    Ry = np.array([[c[1], zer, -s[1]], [zer, one, zer], [s[1], zer, c[1]]], dtype=F32)
    Rz = np.array([[c[2], s[2], zer], [-s[2], c[2], zer], [zer, zer, one]], dtype=F32)

    def mul3(A, B):
        C = np.zeros((3, 3), dtype=F32)
        for i in range(3):
            for j in range(3):
                acc = F32(0.0)
                for k in range(3):
                    acc = F32(acc + F32(A[i, k] * B[k, j]))
                C[i, j] = acc
        return C

    R = mul3(mul3(Rz, Ry), Rx)
    t = np.eye(4, dtype=F32)
    t[:3, :3] = R
    bbc = [F32(x) for x in bbc]
    t[0, 3], t[1, 3], t[2, 3] = bbc
    TM = _transformation_inverse(t)
    shift = [F32(-F32(x)) for x in translation]  # the -T values are negated (main.cpp:251)
    for i in range(3):
        TM[i, 3] = F32(TM[i, 3] - F32(shift[i] - bbc[i]))
    return TM


def _inverse3(M: np.ndarray) -> np.ndarray:
    """inverseMatrix3 / detMatrix3 (UtilityFunctions.h:334-349): k = 1.0 / det
    in double (a double literal), then the adjugate terms in float32."""
    m = M.astype(F32)

    def p3(a, b, c):
        return F32(F32(a * b) * c)

    det = F32(F32(F32(F32(F32(p3(m[0, 0], m[1, 1], m[2, 2]) + p3(m[0, 1], m[1, 2], m[2, 0]))
                          + p3(m[0, 2], m[1, 0], m[2, 1])) - p3(m[0, 2], m[1, 1], m[2, 0]))
                  - p3(m[0, 1], m[1, 0], m[2, 2])) - p3(m[0, 0], m[1, 2], m[2, 1]))
    k = F32(1.0 / float(det))

    def d(a, b, c, e):  # a*b - c*e
        return F32(F32(a * b) - F32(c * e))

    def n(a, b, c, e):  # -a*b + c*e
        return F32(F32(F32(-a) * b) + F32(c * e))

    R = np.zeros((3, 3), dtype=F32)
    R[0, 0] = F32(k * d(m[1, 1], m[2, 2], m[1, 2], m[2, 1]))
    R[0, 1] = F32(k * n(m[0, 1], m[2, 2], m[0, 2], m[2, 1]))
    R[0, 2] = F32(k * d(m[0, 1], m[1, 2], m[0, 2], m[1, 1]))
    R[1, 0] = F32(k * n(m[1, 0], m[2, 2], m[1, 2], m[2, 0]))
    R[1, 1] = F32(k * d(m[0, 0], m[2, 2], m[0, 2], m[2, 0]))
    R[1, 2] = F32(k * n(m[0, 0], m[1, 2], m[0, 2], m[1, 0]))
    R[2, 0] = F32(k * d(m[1, 0], m[2, 1], m[1, 1], m[2, 0]))
    R[2, 1] = F32(k * n(m[0, 0], m[2, 1], m[0, 1], m[2, 0]))
    R[2, 2] = F32(k * d(m[0, 0], m[1, 1], m[0, 1], m[1, 0]))
    return R


def _transformation_inverse(M: np.ndarray) -> np.ndarray:
    """transformationInverse (UtilityFunctions.h:519-540)."""
    RSi = _inverse3(M[:3, :3])
    T = M[:3, 3]
    out = np.zeros((4, 4), dtype=F32)
    out[:3, :3] = RSi
    for i in range(3):
        acc = F32(F32(F32(RSi[i, 0] * T[0]) + F32(RSi[i, 1] * T[1])) + F32(RSi[i, 2] * T[2]))
        out[i, 3] = F32(-acc)
    out[3, 3] = F32(1.0)
    return out


# backgrounds are z-up and glTF scenes y-up: the rotation main.cpp:400-404 gives
# every HDR background (applied as dir * R, HdrBackground.cpp:58)
HDRI_Y_UP = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, -1.0, 0.0]], dtype=F32)


def load_hdri(path: str, scale: float = float(F32(math.pi))) -> scenes.Hdri:
    """The -H background as main.cpp:397-406 sets it up: the Radiance file
    decoded as stb_image decodes it (scenes.decode_hdr), the y-up rotation and
    the radiance scale (RendererParameters::hdrScaleValue, pi)."""
    return scenes.Hdri(scenes.read_hdr(path), HDRI_Y_UP.copy(), float(F32(scale)))


def load_gltf(path: str, use_lights: bool = False, priority: str = "om",
              rotation_zyx_deg=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0), lightbox: bool = False,
              camera: Optional[scenes.CameraSpec] = None, render: Optional[scenes.RenderSpec] = None,
              hdri: Optional[scenes.Hdri] = None) -> LoadedAsset:
    """Loads a .gltf / .glb asset (with its OpenMATERIAL references) and
    flattens it like main.cpp:280-395.  `use_lights` is the -L option (lights
    from KHR_lights_punctual; the reference then ignores an HDR background),
    `priority` the -P option, `rotation_zyx_deg` / `translation` the -e / -T
    options (ignored in light-box mode, -V, which uses the identity)."""
    L = _Loader(priority, use_lights)
    L.load(os.path.abspath(path) if os.path.isabs(path) else path)
    lo, hi = _bbox(L)
    bbc = [F32(F32(F32(hi[k] - lo[k]) * F32(0.5)) + lo[k]) for k in range(3)]
    if lightbox:
        TM = np.eye(4, dtype=F32)
    else:
        TM = scene_transformation(bbc, rotation_zyx_deg, translation)
    # material numbering: first use over the primitives (the reference uses
    # the pointer order of a std::map, main.cpp:305-312)
    mat_ids: Dict[int, int] = {}
    materials: List[scenes.Material] = []
    names: List[str] = []
    for p in L.prims:
        m = p["material"]
        if m is None or m is L.missing:
            continue
        if id(m) not in mat_ids:
            mat_ids[id(m)] = len(materials)
            materials.append(m["material"])
            names.append(m["material"].name)
    meshes: List[scenes.Mesh] = []
    for p in L.prims:
        m = p["material"]
        tang = None
        if "tangents" in p:  # main.cpp:384 passes the 4-wide tangents with stride 3
            t = p["tangents"]
            nv = len(p["positions"])
            idx = (np.arange(nv)[:, None] * 3 + np.arange(4)[None, :])
            tang = np.asarray(t, dtype=F32)[np.minimum(idx, len(t) - 1)]
        uv0 = p.get("uv0")
        uv1 = p.get("uv1") if uv0 is not None else None
        meshes.append(scenes.Mesh(positions=np.asarray(p["positions"], dtype=F32),
                                  normals=np.asarray(p["normals"], dtype=F32) if "normals" in p else None,
                                  tangents=tang, texcoord0=uv0, texcoord1=uv1,
                                  faces=np.ascontiguousarray(p["faces"], dtype=np.uint32),
                                  material=mat_ids[id(m)] if (m is not None and m is not L.missing) else -1,
                                  name=p["name"]))
    instances: List[scenes.Instance] = []

    def walk(node: _Node, T: np.ndarray):
        nT = _mat_mul4(T, node.M)
        for pi in node.prims:
            instances.append(scenes.Instance(nT.copy(), pi))
        for c in node.children:
            walk(c, nT)

    for node in L.nodes:  # addSceneNodes (:791-801): every root, in node order
        if node.parent is None:
            walk(node, TM)
    lights: List[scenes.Light] = []
    for jl, node in L.lights:  # main.cpp:355-368, PointLight.h:52-56
        tM = _mat_mul4(TM, node.global_matrix())
        col = [F32(x) for x in jl.get("color", (1.0, 1.0, 1.0))]
        inten = F32(jl.get("intensity", 1.0))
        rgb = (F32(col[0] * inten), F32(col[2] * inten), F32(col[1] * inten))
        rng = float(F32(jl["range"])) if "range" in jl else FLT_MAX
        lights.append(scenes.Light(position=(float(tM[0, 3]), float(tM[1, 3]), float(tM[2, 3])),
                                   intensity=tuple(float(x) for x in rgb), range=rng))
    textures: List[np.ndarray] = []
    if L.images:
        for i in range(max(L.images) + 1):
            textures.append(L.images.get(i, np.zeros((0, 0, 4), np.uint8)))
    cam = camera or scenes.camera_default(800, 600)
    sc = scenes.Scene(os.path.splitext(os.path.basename(path))[0], meshes, instances, materials, lights,
                      None if use_lights else hdri, cam, render or scenes.RenderSpec(20, 10, 10, 8),
                      textures=textures)
    return LoadedAsset(scene=sc, bbox=(lo, hi), transformation=TM, material_names=names)
