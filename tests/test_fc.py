"""False-colour validation and the light box on the CPU: the oracle's
restatement of the -F pass and of the -V view loop against the reference's own
films (tests/golden/fc.npz, lightbox.npz), and the C ABI's light-box cameras
against the reference's ViewPoints, all bit for bit."""
import ctypes as C

import numpy as np
import pytest
from conftest import golden

SUBJECTS = {"pid": 1, "gid": 2, "mid": 3, "mmp": 4, "rmp": 5, "md": 6, "sg": 7, "mn": 8, "in": 9, "nosuch": 0}


def _palette_from_film(film, args, missing_pink=False):
    """The reference draws pid/gid/mid colours from an entropy-seeded
    generator; recover its table from its film (every id must map to one
    colour) so that the rest of the pass can be compared exactly."""
    pal = {}
    ids = args.reshape(-1)
    rgb = np.rint(film[..., :3].reshape(-1, 3).astype(np.float64) * 255.0).astype(np.int64)
    for i, c in zip(ids, rgb):
        if missing_pink and i == 0xFFFFFFFF:
            continue
        v = int((c[0] << 16) | (c[1] << 8) | c[2])
        assert pal.setdefault(int(i), v) == v, "one id painted in two colours"
    n = max(pal) + 1 if pal else 0
    table = np.zeros(n, dtype=np.uint32)
    for i, v in pal.items():
        table[i] = v
    return table


@pytest.fixture(scope="module")
def fc_case(oracle, scenes):
    sc = scenes.scene_validation(64, 48)
    return oracle.OracleScene(sc), golden("fc")


@pytest.mark.parametrize("name", ["mmp", "rmp", "md", "sg", "mn", "in", "nosuch"])
def test_oracle_fc_subject_matches_reference(fc_case, name):
    osc, g = fc_case
    rgba, args, _, hits = osc.render_fc(SUBJECTS[name])
    ref = g[name]
    assert np.array_equal(rgba.view(np.uint32), ref.view(np.uint32)), np.argwhere(rgba != ref)[:5]
    if name in ("in", "md", "sg"):  # the subject must actually vary over this scene
        assert len(np.unique(args[hits["inst"].reshape(args.shape) != 0xFFFFFFFF])) > 1


@pytest.mark.parametrize("name", ["pid", "gid", "mid"])
def test_oracle_fc_ids_match_reference(fc_case, name):
    osc, g = fc_case
    _, args, _, hits = osc.render_fc(SUBJECTS[name])
    hit = (hits["inst"] != 0xFFFFFFFF).reshape(args.shape)
    ref = g[name]
    pal = _palette_from_film(ref[hit], args[hit], missing_pink=name == "mid")
    if name == "mid":
        assert np.all(pal >> 16 == 0)  # red channel is zero for material ids
    rgba, _, _, _ = osc.render_fc(SUBJECTS[name], palette=pal)
    assert np.array_equal(rgba.view(np.uint32), ref.view(np.uint32))
    assert len(np.unique(args[hit])) > 3


def test_oracle_fc_density_extremes(fc_case):
    osc, _ = fc_case
    lo, hi = osc.density_range()
    assert 0 < lo < hi


def test_fc_subject_names(omv):
    L = omv.lib()
    for name, code in SUBJECTS.items():
        assert L.omv_fc_subject_from_name(name.encode()) == code
    assert L.omv_fc_subject_from_name(None) == 0


def _world_bounds(sc):
    """AssetGeometry::getBBox of the flattened scene, float32 in the
    reference's operation order (m0 x + m1 y + m2 z + m3)."""
    lo = np.full(3, np.inf, dtype=np.float32)
    hi = np.full(3, -np.inf, dtype=np.float32)
    for inst in sc.instances:
        M = np.asarray(inst.transform, dtype=np.float32)
        v = np.asarray(sc.meshes[inst.mesh].positions, dtype=np.float32)
        p = np.stack([((M[r, 0] * v[:, 0] + M[r, 1] * v[:, 1]) + M[r, 2] * v[:, 2]) + M[r, 3] for r in range(3)], 1)
        lo = np.minimum(lo, p.min(0))
        hi = np.maximum(hi, p.max(0))
    return lo, hi


def _lightbox(omv, lo, hi, w, h):
    cams = (omv.capi.Camera * 8)()
    lo = np.ascontiguousarray(lo, dtype=np.float32)
    hi = np.ascontiguousarray(hi, dtype=np.float32)
    omv.check(omv.lib().omv_lightbox_cameras(omv.capi.fptr(lo), omv.capi.fptr(hi), w, h, cams))
    return list(cams)


def test_lightbox_cameras_match_reference(omv, scenes):
    g = golden("lightbox")
    sc = scenes.scene_mixed(32, 32, 32)
    lo, hi = _world_bounds(sc)
    cams = _lightbox(omv, lo, hi, 32, 32)
    pos = np.array([c.position[:] for c in cams], dtype=np.float32)
    rot = np.array([[c.rotation[r][:] for r in range(3)] for c in cams], dtype=np.float32)
    assert np.array_equal(pos.view(np.uint32), g["position"].view(np.uint32))
    assert np.array_equal(rot.view(np.uint32), g["rotation"].view(np.uint32))
    for c, hw, hh, f in zip(cams, g["half_width"], g["half_height"], g["focus"]):
        assert (np.float32(c.half_width), np.float32(c.half_height), np.float32(c.focus)) == (hw, hh, f)


def test_lightbox_argument_errors(omv):
    cams = (omv.capi.Camera * 8)()
    lo = np.zeros(3, np.float32)
    hi = -np.ones(3, np.float32)
    L = omv.lib()
    assert L.omv_lightbox_cameras(omv.capi.fptr(lo), omv.capi.fptr(hi), 8, 8, cams) == 1
    assert L.omv_lightbox_cameras(omv.capi.fptr(lo), omv.capi.fptr(lo), 0, 8, cams) == 1
    assert L.omv_lightbox_cameras(None, None, 8, 8, cams) == 1


def test_oracle_lightbox_views_match_reference(omv, oracle, scenes):
    """The light-box loop of the oracle (one generator across the 8 views)
    reproduces the reference's 8 films bit for bit."""
    g = golden("lightbox")
    sc = scenes.scene_mixed(32, 32, int(g["spp"]))
    lo, hi = _world_bounds(sc)
    films = oracle.OracleScene(sc).render_views(_lightbox(omv, lo, hi, 32, 32))
    ref = g["films"]
    fin = np.isfinite(ref)
    assert np.array_equal(films[fin].view(np.uint32), ref[fin].view(np.uint32))
    assert np.array_equal(np.isfinite(films), fin)
