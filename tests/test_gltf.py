"""The glTF / OpenMATERIAL loader (openmaterial-validation_gb300/gltf.py)
against the reference's own loading: its stb PNG decode (tests/golden/png.npz),
the committed scenes of files this repository writes (the scene_*.npz dumps),
and - where the reference tree is present - the committed scene of every asset
the reference ships (tests/golden/assets.npz, made by tests/golden/make_golden.py
from its pathtracer run on each file)."""
import importlib
import os
import sys

import numpy as np
import pytest
from conftest import ROOT, golden

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as _oracle  # noqa: E402

REF_TREE = _oracle.reference_tree()


@pytest.fixture(scope="module")
def gl():
    return importlib.import_module("openmaterial-validation_gb300.gltf")


def test_png_decode_matches_stb(gl):
    g = golden("png")
    for i in range(int(g["count"])):
        got = gl.decode_png(g[f"file{i}"].tobytes())
        want = g[f"rgba{i}"]
        if int(g[f"bits{i}"]) == 16:
            want = want // 256  # ImageData::load's 16-bit conversion
        assert np.array_equal(got, want.astype(np.uint8)), i


def _ref_alpha_mode(m):
    return {0: 2, 1: 1, 2: 0}[m.alpha_mode]  # PbrMaterial::AlphaMode: Blend 0, Mask 1, Opaque 2


def _material_record(oracle, scenes, m):
    """The record ref_hooks dumps for a committed material: type, then
    PBR (base colour, metallic, roughness, ior, alpha mode, cutoff, double
    sided) or OpenMATERIAL (n, k at the RGB wavelengths, temperature)."""
    rec = np.zeros(17, np.float32)
    if m is None:
        rec[0] = 2
        return rec
    if m.type == 0:
        rec[0] = 0
        rec[1:5] = m.base_color
        rec[5], rec[6], rec[7] = m.metallic, m.roughness, m.ior
        rec[8], rec[9], rec[10] = _ref_alpha_mode(m), m.alpha_cutoff, 1.0 if m.double_sided else 0.0
    else:
        rec[0] = 1
        for c, w in enumerate(scenes.RGB_WAVELENGTHS):
            rec[1 + c] = oracle.ior_lookup(np.asarray(m.ior_n, np.float32), w)
            rec[4 + c] = oracle.ior_lookup(np.asarray(m.ior_k, np.float32), w)
        rec[7] = m.temperature
    return rec


def _digest(oracle, scenes, sc):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as M

    osc = oracle.OracleScene(sc)
    verts = [osc.mesh_vertices(i) for i in range(len(sc.meshes))]
    faces = [m.faces for m in sc.meshes]
    recs = [_material_record(oracle, scenes, sc.materials[m.material] if 0 <= m.material < len(sc.materials)
                             else None) for m in sc.meshes]
    lights = [[*l.position, *l.intensity] for l in sc.lights]
    return M.scene_digest(verts, faces, recs, [i.mesh for i in sc.instances],
                          [np.asarray(i.transform, np.float32) for i in sc.instances],
                          [osc.normal_matrix(k) for k in range(len(sc.instances))],
                          np.array([l + [0, 0] for l in lights], np.float32))


@pytest.mark.parametrize("name", ["c1", "mixed", "textured"])
def test_loader_reproduces_the_reference_commit_of_written_files(gl, oracle, scenes, tmp_path, name):
    """write_gltf -> load_gltf -> commit equals what the reference committed
    from the same files (vertex blocks, instances, normal matrices, lights)."""
    sc = getattr(scenes, f"scene_{name}")(8, 8, 1)
    out = scenes.write_gltf(sc, str(tmp_path))
    asset = gl.load_gltf(out["gltf"], use_lights=True)
    ls = asset.scene
    g = golden(f"scene_{name}")
    osc = oracle.OracleScene(ls)
    for i in range(len(ls.meshes)):
        assert np.array_equal(osc.mesh_vertices(i).view(np.uint32), g[f"verts{i}"].view(np.uint32)), i
        assert np.array_equal(ls.meshes[i].faces, g[f"faces{i}"])
    for i, inst in enumerate(ls.instances):
        assert np.array_equal(np.asarray(inst.transform, np.float32).view(np.uint32), g["inst_xf"][i].view(np.uint32))
        assert np.array_equal(osc.normal_matrix(i).view(np.uint32), g["inst_nrm"][i].view(np.uint32))
        assert inst.mesh == g["inst_mesh"][i]
    L = g["lights"]
    for i, l in enumerate(ls.lights):
        assert np.array_equal(np.array(l.position, np.float32), L[i, 0:3])
        assert np.array_equal(np.array(l.intensity, np.float32), L[i, 3:6])
    assert len(ls.textures) == len(sc.textures)
    for a, b in zip(ls.textures, sc.textures):
        assert np.array_equal(a, b)
    for me0, me1 in zip(sc.meshes, ls.meshes):  # materials are numbered in first-use order
        m0, m1 = sc.materials[me0.material], ls.materials[me1.material]
        assert m0.type == m1.type
        if m0.type == 0:
            for slot in ("base_color_texture", "metallic_roughness_texture", "normal_texture", "occlusion_texture",
                         "emissive_texture"):
                r0, r1 = getattr(m0, slot), getattr(m1, slot)
                assert (r0 is None) == (r1 is None), slot
                if r0 is not None:
                    assert (r0.texture, r0.texcoord) == (r1.texture, r1.texcoord)
                    t0, t1 = r0.transform, r1.transform
                    assert (t0 is None) == (t1 is None) and (t0 is None or np.array_equal(t0, t1))


def test_loader_renders_like_the_written_scene(gl, oracle, scenes, tmp_path):
    """The loaded textured scene renders the reference's -C 1 film bit for bit."""
    g = golden("film_textured_32x8")
    sc = scenes.scene_textured(32, 32, 8)
    out = scenes.write_gltf(sc, str(tmp_path))
    asset = gl.load_gltf(out["gltf"], use_lights=True, camera=sc.camera, render=sc.render)
    film, _, rays = oracle.OracleScene(asset.scene).render(mode=0)
    assert rays == int(g["rays"])
    assert np.array_equal(film.view(np.uint32), g["film"].view(np.uint32))


def test_scene_transformation_is_identity_without_options(gl):
    T = gl.scene_transformation([1.25, -3.5, 7.0])
    assert np.array_equal(T, np.eye(4, dtype=np.float32))
    R = gl.scene_transformation([0.5, 0.25, -1.0], (30.0, 45.0, 60.0), (1.0, 2.0, 3.0))
    assert np.allclose(R[:3, :3] @ R[:3, :3].T, np.eye(3), atol=1e-6)


def _assets():
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden as M

    return M.ASSETS


@pytest.mark.skipif(REF_TREE is None or not os.path.isdir(os.path.join(REF_TREE, "objects")),
                    reason="reference assets not present")
@pytest.mark.parametrize("asset", _assets())
def test_loader_matches_reference_on_its_assets(gl, oracle, scenes, asset):
    g = golden("assets")
    key = asset.replace("/", "__")
    sc = gl.load_gltf(os.path.join(REF_TREE, asset + ".gltf"), use_lights=True).scene
    d = _digest(oracle, scenes, sc)
    assert np.array_equal(d["mesh_hash"], g[f"{key}.mesh_hash"])
    assert np.array_equal(d["inst_mesh"], g[f"{key}.inst_mesh"])
    assert np.array_equal(d["inst_xf"].view(np.uint32), g[f"{key}.inst_xf"].view(np.uint32))
    assert np.array_equal(d["inst_nrm"].view(np.uint32), g[f"{key}.inst_nrm"].view(np.uint32))
    want = g[f"{key}.mesh_rec"]
    got = d["mesh_rec"]
    assert got.shape == want.shape
    for i in range(len(got)):
        n = 11 if got[i, 0] == 0 else 8
        assert np.array_equal(got[i, :n], want[i, :n]), (i, got[i, :n], want[i, :n])
    gl_ = g[f"{key}.lights"]
    assert len(d["lights"]) == len(gl_)
    for a, b in zip(d["lights"], gl_):
        assert np.array_equal(a[:3], b[:3]) and np.array_equal(a[3:6], b[3:6])
