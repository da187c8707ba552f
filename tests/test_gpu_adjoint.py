"""Path-replay adjoint (omv_adjoint) against central finite differences with
common random numbers (eps 1e-3, the same seed on both sides), through the
torch.autograd.Function of openmaterial-validation_gb300.diff.

With the sampled directions independent of a parameter (base colour,
metallic, conductor n and k) the replayed derivative is the exact derivative
of the same per-sample estimate that the finite difference differentiates,
so the two agree up to the difference quotient's error.  Roughness also
moves the GGX-sampled directions under common random numbers, while the
adjoint keeps them fixed and adds the score of their density: the two agree
in expectation only."""
import dataclasses
import importlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(gpu, scenes):
    torch = pytest.importorskip("torch")
    diff = importlib.import_module("openmaterial-validation_gb300.diff")
    sc = scenes.scene_materials(48, 48, 16, tris=20_000, bounces=4)
    R = diff.MaterialRenderer(sc, spp=64, seed=7)
    P0 = diff.params_from_materials(sc.materials)
    # target: the scene with other parameters, rendered with another seed
    Pt = P0.copy()
    Pt[:, 0:3] = np.clip(Pt[:, 0:3] * 0.7 + 0.1, 0.05, 0.95)
    Pt[:, 4] = 1.0 - Pt[:, 4]
    Pt[:, 5:11] = Pt[:, 5:11] * 0.8
    Rt = diff.MaterialRenderer(sc, spp=256, seed=99)
    Rt.set_params(Pt)
    s, c = Rt.render_sums(torch)
    T = (s / c.unsqueeze(-1)).detach()
    return torch, diff, sc, R, P0, T


def _loss(torch, R, P, T):
    R.set_params(P)
    s, c = R.render_sums(torch)
    I = s / c.unsqueeze(-1)
    return float(((I - T) ** 2).mean())


def test_adjoint_matches_central_differences(case):
    """Every parameter that does not move sampled directions, to 1e-3."""
    torch, diff, sc, R, P0, T = case
    P = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
    I = R.image(P)
    L = ((I - T) ** 2).mean()
    L.backward()
    g_ad = P.grad.detach().cpu().numpy()
    active = diff.active_mask(sc.materials)
    exact = active.copy()
    exact[:, 3] = False  # roughness: expectation check below
    eps = 1e-3
    g_fd = np.zeros_like(g_ad)
    for i, k in zip(*np.nonzero(exact)):
        Pp, Pm = P0.copy(), P0.copy()
        Pp[i, k] += eps
        Pm[i, k] -= eps
        g_fd[i, k] = (_loss(torch, R, Pp, T) - _loss(torch, R, Pm, T)) / (2 * eps)
    R.set_params(P0)
    scale = np.abs(g_fd[exact]).max()
    rel = np.abs(g_ad - g_fd)[exact] / (np.abs(g_fd[exact]) + 1e-3 * scale)
    assert np.all(g_ad[~active] == 0)
    assert float(rel.max()) < 1e-3, (g_ad, g_fd)


def test_adjoint_roughness_in_expectation(case):
    """Roughness under common random numbers moves the GGX-sampled directions,
    so only expectations agree: a linear image loss, many samples and a wider
    difference step."""
    torch, diff, sc, R0, P0, T = case
    R = diff.MaterialRenderer(sc, spp=1024, seed=21)
    rng = np.random.default_rng(4)
    H, W = R.cam.height, R.cam.width
    w = torch.tensor(rng.uniform(0.0, 1.0, (H, W, 3)) / (H * W), dtype=torch.float64, device="cuda")
    P = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
    (R.image(P) * w).sum().backward()
    g_ad = P.grad.detach().cpu().numpy()[:, 3]

    def lin(Px):
        R.set_params(Px)
        s, c = R.render_sums(torch)
        return float(((s / c.unsqueeze(-1)) * w).sum())

    eps = 0.02
    g_fd = np.zeros(len(sc.materials))
    for i in range(len(sc.materials)):
        if sc.materials[i].type != 0:
            continue
        Pp, Pm = P0.copy(), P0.copy()
        Pp[i, 3] += eps
        Pm[i, 3] -= eps
        g_fd[i] = (lin(Pp) - lin(Pm)) / (2 * eps)
    R.set_params(P0)
    out = os.environ.get("OMV_ADJOINT_REPORT")
    if out:
        with open(out, "w") as fh:
            json.dump({"g_ad": g_ad.tolist(), "g_fd": g_fd.tolist()}, fh)
    pbr = np.array([m.type == 0 for m in sc.materials])
    scale = np.abs(g_fd[pbr]).max()
    assert np.all(np.abs(g_ad[pbr] - g_fd[pbr]) <= 0.2 * np.abs(g_fd[pbr]) + 0.05 * scale), (g_ad, g_fd)


def test_adjoint_matches_finite_differences_on_the_reference_renderer(gpu, oracle, scenes):
    """The GPU path-replay gradient of a linear image loss against central
    differences of the same loss on the reference CPU renderer (the oracle,
    which reproduces the reference bit for bit), for every parameter of every
    material: PBR base colour, roughness and metallic, and the OpenMATERIAL
    conductors' n and k at the three RGB wavelengths (changed through the IOR
    tables the reference looks them up in, AssetMaterialIor.cpp:133-178,
    OpenMaterial.cpp:20-38).  Both sides of a difference use common random
    numbers (the oracle's per-row mt19937 streams, same seed); the two
    renderers draw different numbers, so they agree in expectation.  Each side
    is estimated over four independent seeds, its standard error taken from
    their spread, and every component must agree within four combined
    standard errors plus 2% of its value (the O(eps^2) error of the quotient)."""
    torch = pytest.importorskip("torch")
    diff = importlib.import_module("openmaterial-validation_gb300.diff")
    sc = scenes.scene_materials(24, 24, 1, tris=4000, bounces=3, n_materials=4)
    P0 = diff.params_from_materials(sc.materials)
    active = diff.active_mask(sc.materials)
    rng = np.random.default_rng(3)
    H, W = sc.camera.height, sc.camera.width
    w = rng.uniform(0.0, 1.0, (H, W, 3)) / (H * W)
    wt = torch.tensor(w, dtype=torch.float64, device="cuda")
    seeds = 4
    ad = []
    for k in range(seeds):
        R = diff.MaterialRenderer(sc, spp=8192, seed=5 + k)
        P = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
        (R.image(P) * wt).sum().backward()
        ad.append(P.grad.detach().cpu().numpy())
    ad = np.array(ad)

    def loss_cpu(Px, seed):
        s2 = dataclasses.replace(sc, materials=diff.materials_from_params(sc.materials, Px))
        film, _, _ = oracle.OracleScene(s2).render(params=oracle.capi.params_for(s2, spp=1024), mode=1,
                                                   threads=os.cpu_count() or 8, seed=seed)
        return float((film[..., :3].astype(np.float64) * w).sum())

    rows = []
    for i, k in zip(*np.nonzero(active)):
        eps = 0.02 if k == 3 else 0.01
        fd = []
        for sd in range(seeds):
            Pp, Pm = P0.copy(), P0.copy()
            Pp[i, k] += eps
            Pm[i, k] -= eps
            fd.append((loss_cpu(Pp, 100 + sd) - loss_cpu(Pm, 100 + sd)) / (2 * eps))
        fd = np.array(fd)
        a = ad[:, i, k]
        rows.append((int(i), int(k), float(a.mean()), float(a.std(ddof=1) / np.sqrt(seeds)), float(fd.mean()),
                     float(fd.std(ddof=1) / np.sqrt(seeds))))
    out = os.environ.get("OMV_ADJOINT_REPORT")
    if out:
        with open(out, "w") as fh:
            json.dump(rows, fh)
    kinds = {k for _, k, *_ in rows}
    assert kinds == set(range(11)), kinds  # base colour, roughness, metallic, n and k all checked
    bad = [r for r in rows if abs(r[2] - r[4]) > 4.0 * np.hypot(r[3], r[5]) + 0.02 * abs(r[4])]
    assert not bad, bad
