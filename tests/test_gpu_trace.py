"""GPU BVH build + traversal: identification (primary-hit) buffers bit-exact
against the reference's false-colour pass and against the oracle's closest-hit
query on the same rays."""
import numpy as np
import pytest
from conftest import golden

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.402823466e38)

# every acceleration-structure builder must give the same hits: the box tests
# are conservative and the hit contract (closest t, then lowest instance and
# primitive) does not depend on the tree
BUILDERS = pytest.mark.parametrize("builder", [0, 1, 2, 3], ids=["sah", "ploc", "lbvh", "host_sah"])


def _hits_equal(a, b):
    for k in ("inst", "geom", "prim", "material"):
        if not np.array_equal(a[k], b[k]):
            bad = np.nonzero(a[k] != b[k])[0]
            return False, f"{k} differs at {bad[:8]} ({len(bad)} rays)"
    for k in ("t", "u", "v"):
        if not np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)):
            bad = np.nonzero(a[k].view(np.uint32) != b[k].view(np.uint32))[0]
            return False, f"{k} differs at {bad[:8]} ({len(bad)} rays)"
    return True, ""


def test_reference_rays_give_reference_ids(gpu, scenes):
    """The exact rays the reference traced in its -F mid pass (logged at the
    Embree boundary) give the same instance/geometry/primitive ids and t,u,v."""
    g = golden("ids_c1_64")
    rs = gpu.RenderScene(scenes.scene_c1(64, 64, 1))
    hits = rs.trace(g["rays"])
    hit = g["hit"].astype(bool)
    assert np.array_equal(hits["inst"] != 0xFFFFFFFF, hit)
    for k in ("geom", "inst", "prim"):
        assert np.array_equal(hits[k][hit], g[k][hit]), k
    for k in ("u", "v", "t"):
        assert np.array_equal(hits[k][hit].view(np.uint32), g[k][hit].view(np.uint32)), k


@BUILDERS
def test_id_pass_with_reference_jitter_full_c1(gpu, oracle, scenes, builder):
    """C1 material-ID pass at 256x256: GPU raygen + trace with the reference's
    jitter stream equals the oracle replay (itself pinned bit-exact to the
    reference binary) for every pixel."""
    sc = scenes.scene_c1(256, 256, 1)
    _, ref = oracle.OracleScene(sc).render_ids()
    jitter = oracle.mt_uniforms(oracle.REFERENCE_SEED, 2 * 256 * 256)
    rs = gpu.RenderScene(sc, bvh_builder=builder)
    r = gpu.BDPTRenderer()
    r.set_scene(rs)
    hits, gprim = r.render_ids(gpu.PinholeCamera.from_spec(sc.camera), jitter=jitter)
    ok, msg = _hits_equal(hits, ref)
    assert ok, msg
    faces = [len(m.faces) for m in sc.meshes]
    pre = np.concatenate([[0], np.cumsum(faces)])
    hit = hits["inst"] != 0xFFFFFFFF
    assert np.array_equal(gprim[hit], pre[hits["geom"][hit]] + hits["prim"][hit])
    assert set(np.unique(hits["material"][hit])) <= {0, 1}


def _random_rays(rng, n, lo, hi, spread=1.0):
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 4:7] = o, d * spread
    r[:, 3] = 0.0
    r[:, 7] = FLT_MAX
    return r


@BUILDERS
def test_large_instanced_scene_matches_oracle(gpu, oracle, scenes, builder):
    """1M-triangle scene, 64 rotated/scaled instances: GPU hits equal the
    oracle's on camera rays and on random rays (bit-exact)."""
    sc = scenes.scene_c2(160, 90, 1)
    rs = gpu.RenderScene(sc, bvh_builder=builder)
    os_ = oracle.OracleScene(sc)
    rng = np.random.default_rng(5)
    cam = rays_from_camera(oracle, sc)
    rnd = _random_rays(rng, 20000, [-25, -25, -65], [25, 25, -15])
    axis = _random_rays(rng, 3000, [-25, -25, -65], [25, 25, -15])
    axis[:, 4:7] = np.eye(3, dtype=np.float32)[rng.integers(0, 3, 3000)] * np.where(
        rng.uniform(size=(3000, 1)) < 0.5, -1, 1)
    # nearly axis-parallel: the other two components tiny (reciprocals up to
    # the box test's 1e20 clamp), where the slab distances are largest
    tilt = axis.copy()
    tiny = rng.choice(np.array([1e-30, 1e-21, 1e-12, 1e-6, 1e-3], np.float32), (3000, 3))
    tilt[:, 4:7] += tiny * np.where(rng.uniform(size=(3000, 3)) < 0.5, -1, 1) * (tilt[:, 4:7] == 0)
    rays = np.concatenate([cam, rnd, axis, tilt])
    ok, msg = _hits_equal(rs.trace(rays), os_.trace(rays))
    assert ok, msg


def rays_from_camera(oracle, sc):
    W, H = sc.camera.width, sc.camera.height
    jr = oracle.camera_rays(sc.camera, np.full(2 * W * H, 0.5, np.float32))
    r = np.zeros((W * H, 8), np.float32)
    r[:, 0:3], r[:, 4:7] = jr[:, 0:3], jr[:, 3:6]
    r[:, 7] = FLT_MAX
    return r


@BUILDERS
def test_edge_cases_match_oracle(gpu, oracle, scenes, builder):
    """Shared edges (ties between the two ground triangles), vertices, grazing
    rays, zero/NaN directions, empty intervals, origins on surfaces."""
    sc = scenes.scene_mixed(8, 8, 1)
    rs = gpu.RenderScene(sc, bvh_builder=builder)
    os_ = oracle.OracleScene(sc)
    rows = []
    # rays through the ground quad's diagonal (shared edge) and its corners
    for t in np.linspace(0.0, 1.0, 41):
        p = np.array([-5 + 10 * t, -1.0, -5 + 10 * t - 5.0], np.float32)
        rows.append([0, 3, -5, 0, *(p - np.array([0, 3, -5], np.float32)), FLT_MAX])
    for c in ([-5, -1, -10], [5, -1, -10], [5, -1, 0], [-5, -1, 0]):
        rows.append([0, 3, -5, 0, c[0], c[1] - 3, c[2] + 5, FLT_MAX])
    # grazing along the ground plane, exactly in and slightly above it
    for dy in (0.0, 1e-7, -1e-7):
        rows.append([-6, -1 + dy, -5, 0, 1, 0, 0, FLT_MAX])
    rows += [[0, 0, 0, 0, 0, 0, 0, FLT_MAX], [0, 0, 0, 0, np.nan, 0, -1, FLT_MAX],
             [0, 0, 0, 5, 0, 0, -1, 1], [0, 0, 0, 0, 0, 0, -1, 0], [0, 0, 0, 0, 0, 0, -1, 4.3]]
    rays = np.array(rows, np.float32)
    rng = np.random.default_rng(9)
    # origins on the spheres, shooting outwards and inwards
    m = sc.meshes[1]
    pts = m.positions[rng.integers(0, len(m.positions), 500)] + np.array([0, 0, -5], np.float32)
    d = rng.normal(size=(500, 3)).astype(np.float32)
    extra = np.zeros((500, 8), np.float32)
    extra[:, 0:3], extra[:, 4:7], extra[:, 7] = pts, d, FLT_MAX
    rays = np.concatenate([rays, extra])
    ok, msg = _hits_equal(rs.trace(rays), os_.trace(rays))
    assert ok, msg


@BUILDERS
def test_alpha_masked_material_is_skipped_like_reference(gpu, oracle, scenes, builder):
    sc = scenes.scene_mixed(8, 8, 1)
    sc.materials[3].alpha_mode = 1  # MASK with base alpha 0.5 < cutoff 0.75
    sc.materials[3].alpha_cutoff = 0.75
    rs = gpu.RenderScene(sc, bvh_builder=builder)
    os_ = oracle.OracleScene(sc)
    rays = rays_from_camera(oracle, scenes.scene_mixed(96, 96, 1))
    a, b = rs.trace(rays), os_.trace(rays)
    ok, msg = _hits_equal(a, b)
    assert ok, msg
    assert not np.any(a["material"] == 3)


@BUILDERS
def test_non_finite_triangles_change_no_hit(gpu, scenes, builder):
    """Triangles with NaN or infinite vertices (appended to a mesh, so every
    valid triangle keeps its id) are never hit and change no other hit, as an
    Embree robust build ignores invalid primitives: the closest-hit query on
    random rays and the camera ID pass are bit-identical with and without them,
    and the frame renders finite."""
    import dataclasses

    sc = scenes.scene_c1(64, 64, 1)
    m = sc.meshes[0]
    rng = np.random.default_rng(12)
    bad_v, bad_f = [], []
    nv = len(m.positions)
    for k, val in enumerate((np.nan, np.inf, -np.inf, np.nan, np.inf)):
        tri = m.positions[m.faces[rng.integers(len(m.faces))]].astype(np.float32).copy()
        if k == 3:
            tri[:, :] = np.nan                           # all three vertices
        else:
            tri[k % 3, k % 3] = val                      # one coordinate
        bad_v.append(tri)
        bad_f.append(nv + 3 * k + np.arange(3))
    pos = np.concatenate([m.positions.astype(np.float32)] + bad_v)
    faces = np.concatenate([m.faces.astype(np.uint32), np.array(bad_f, np.uint32)])
    normals = None if m.normals is None else np.concatenate([m.normals, np.tile(m.normals[:1], (len(bad_v) * 3, 1))])
    sc_bad = dataclasses.replace(sc, meshes=[dataclasses.replace(m, positions=pos, faces=faces, normals=normals)]
                                 + list(sc.meshes[1:]))
    a, b = gpu.RenderScene(sc, bvh_builder=builder), gpu.RenderScene(sc_bad, bvh_builder=builder)
    rays = _random_rays(rng, 200_000, -3.0, 3.0)
    ok, msg = _hits_equal(a.trace(rays), b.trace(rays))
    assert ok, msg
    ids = []
    for rs in (a, b):
        r = gpu.BDPTRenderer()
        r.set_scene(rs)
        ids.append(r.render_ids(gpu.PinholeCamera.from_spec(sc.camera), jitter=np.full(2 * 64 * 64, 0.5, np.float32))[0])
    ok, msg = _hits_equal(ids[0], ids[1])
    assert ok, msg
    r = gpu.BDPTRenderer()
    r.set_scene(b)
    r.set_parameters(gpu.RendererParameters.for_scene(sc_bad, samplesPerPixel=16))
    img = r.render(gpu.PinholeCamera.from_spec(sc.camera))
    assert np.isfinite(img).all()


@BUILDERS
def test_many_meshes_of_every_size_match_oracle(gpu, oracle, scenes, builder):
    """Meshes of 1, 2, 3, 5 ... triangles beside large ones, coincident
    triangles (equal boxes: every clustering distance ties) and meshes shared
    by several instances: one device forest over all meshes, hits bit-exact
    against the oracle."""
    import dataclasses

    rng = np.random.default_rng(21)
    base = scenes.scene_mixed(8, 8, 1)
    meshes, insts = [], []
    for k, nt in enumerate([1, 2, 3, 5, 8, 17, 64, 257, 1000, 4099]):
        c = rng.uniform(-3, 3, 3).astype(np.float32)
        v = (c + rng.normal(size=(3 * nt, 3)) * 0.3).astype(np.float32)
        f = np.arange(3 * nt, dtype=np.uint32).reshape(nt, 3)
        if k == 6:  # 64 copies of one triangle
            v = np.tile(v[:3], (nt, 1))
        meshes.append(scenes.Mesh(positions=v, normals=None, faces=f, material=k % len(base.materials), name=f"m{k}"))
        for r in range(1 + k % 3):
            t = np.eye(4, dtype=np.float32)
            t[:3, 3] = rng.uniform(-2, 2, 3) - np.array([0, 0, 8], np.float32)
            insts.append(scenes.Instance(t, k))
    sc = dataclasses.replace(base, meshes=meshes, instances=insts)
    rs = gpu.RenderScene(sc, bvh_builder=builder)
    os_ = oracle.OracleScene(sc)
    rays = _random_rays(rng, 50_000, [-6, -6, -14], [6, 6, -2])
    ok, msg = _hits_equal(rs.trace(rays), os_.trace(rays))
    assert ok, msg
    assert np.count_nonzero(rs.trace(rays)["inst"] != 0xFFFFFFFF) > 1000
