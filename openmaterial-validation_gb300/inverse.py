"""Inverse material fitting by path-replay gradients (config C5): recover the
roughness of the PBR materials and the complex IOR (n, k per RGB channel) of
the OpenMATERIAL conductors of several independent scenes from high-spp
renders made with hidden parameters, with Adam on an L2 image loss.

The scenes are the material-study scenes lit by a point light and one sky
HDRI they share (the conductors are perfect mirrors: under a point light
alone they show little).  Each step renders every scene once (forward) and
replays its paths once (adjoint) with fresh, independent random streams, so
the gradient of the squared error is not biased by the correlation of image
and derivative.

`fit` keeps all scenes in one group (omv_scene_create_group): a step is one
batch render of every scene's job and one batch of adjoint jobs.
`fit_sequential` renders and replays the scenes one after another through
their own handles (the form without a group), for comparison."""
from __future__ import annotations

import importlib
from dataclasses import dataclass
from typing import List

import numpy as np

from . import diff, scenes


@dataclass
class FitResult:
    steps: int
    initial_error: float      # mean absolute parameter error before the fit
    final_error: float        # after it
    per_scene_error: List[float]
    initial_roughness_error: float
    final_roughness_error: float
    initial_ior_error: float  # conductors' n, k
    final_ior_error: float
    initial_loss: float       # mean image loss of the first step
    final_loss: float         # of the last step
    seconds: float


def _free_mask(materials) -> np.ndarray:
    """Slots fitted: roughness of PBR materials, n and k of conductors."""
    m = np.zeros((len(materials), diff.SLOTS), dtype=bool)
    for i, mat in enumerate(materials):
        if mat.type == 0:
            m[i, 3] = True
        else:
            m[i, 5:11] = True
    return m


def make_scenes(n_scenes: int, tris: int, res: int, spp: int, seed: int) -> list:
    """The fit's scenes: independent geometry and materials, one shared sky."""
    out = []
    for j in range(n_scenes):
        sc = scenes.scene_materials(res, res, spp, tris=tris, n_materials=4, seed=seed + 100 + j, bounces=6,
                                    sky=True)
        if out:
            sc.hdri = out[0].hdri
        out.append(sc)
    return out


def fit(n_scenes: int = 32, tris: int = 50_000, res: int = 256, spp: int = 16, target_spp: int = 1024,
        steps: int = 200, lr: float = 1e-2, seed: int = 0) -> FitResult:
    import time

    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    rng = np.random.default_rng(seed)
    scs = make_scenes(n_scenes, tris, res, spp, seed)
    group = omv.RenderScene.group(scs)
    br = omv.BatchRenderer(group, omv.RendererParameters.for_scene(scs[0], samplesPerPixel=spp))
    truths = [diff.params_from_materials(sc.materials) for sc in scs]
    frees = [_free_mask(sc.materials) for sc in scs]
    starts = []
    for t, f in zip(truths, frees):
        x = t.copy()
        x[f] = t[f] * rng.uniform(0.6, 1.4, int(f.sum()))
        starts.append(x)
    keep: list = []

    def set_all(Ps):  # every scene's current parameters, in the group's material order
        mats = []
        for sc, P in zip(scs, Ps):
            mats += diff.materials_from_params(sc.materials, P)
        keep.clear()
        descs = omv.capi.material_descs(mats, keep)
        omv.check(omv.lib().omv_scene_set_materials(group.handle, len(mats), descs))

    films = [(torch.zeros((res, res, 3), dtype=torch.float64, device="cuda"), None,
              torch.zeros((res, res), dtype=torch.int32, device="cuda")) for _ in scs]
    cams = [omv.PinholeCamera.from_spec(sc.camera) for sc in scs]

    def render(n_spp, seeds):
        for f in films:
            f[0].zero_()
            f[2].zero_()
        jobs = [br.job(cams[j], n_spp, films[j], seed=seeds[j], part=j) for j in range(n_scenes)]
        br.render(jobs)
        torch.cuda.synchronize()
        return [f[0] / f[2].clamp(min=1).unsqueeze(-1).to(torch.float64) for f in films]

    set_all(truths)
    T = [x.clone() for x in render(target_spp, [10_000 + j for j in range(n_scenes)])]
    P = [torch.tensor(x, dtype=torch.float64) for x in starts]
    opts = [torch.optim.Adam([p.requires_grad_()], lr=lr) for p in P]
    free_t = [torch.from_numpy(f) for f in frees]
    grads = [torch.zeros((len(sc.materials), diff.SLOTS), dtype=torch.float32, device="cuda") for sc in scs]

    def err(x, truth, free):
        return float(np.mean(np.abs(x[free] - truth[free])))

    def part_err(slots):
        out = []
        for x, t, f in zip(P, truths, frees):
            m = f.copy()
            m[:, [i for i in range(diff.SLOTS) if i not in slots]] = False
            out.append(err(x.detach().numpy(), t, m) if m.any() else 0.0)
        return float(np.mean(out))

    init = [err(x.detach().numpy(), t, f) for x, t, f in zip(P, truths, frees)]
    init_r, init_nk = part_err([3]), part_err(list(range(5, 11)))
    t0 = time.perf_counter()
    first_loss = last_loss = 0.0
    for step in range(steps):
        set_all([p.detach().numpy() for p in P])
        imgs = render(spp, [2 * (step * n_scenes + j) + 1 for j in range(n_scenes)])
        adjs, loss = [], 0.0
        for I, Tj in zip(imgs, T):
            ok = torch.isfinite(Tj) & torch.isfinite(I)
            cnt = max(1, int(ok.sum()))
            d = torch.where(ok, I - torch.where(ok, Tj, torch.zeros_like(Tj)), torch.zeros_like(I))
            loss += float((d ** 2).sum()) / cnt / n_scenes
            adjs.append((2.0 * d / cnt).to(torch.float32).contiguous())
        for g in grads:
            g.zero_()
        jobs = [br.job(cams[j], spp, films[j], seed=2 * (step * n_scenes + j) + 2, part=j) for j in range(n_scenes)]
        br.adjoint(jobs, adjs, grads)
        torch.cuda.synchronize()
        if step == 0:
            first_loss = loss
        last_loss = loss
        for j in range(n_scenes):
            opts[j].zero_grad()
            g = grads[j].detach().to("cpu", torch.float64)
            g[~free_t[j]] = 0.0
            P[j].grad = g
            opts[j].step()
            with torch.no_grad():  # keep the parameters physical
                P[j][:, 3].clamp_(0.02, 1.0)
                P[j][:, 5:11].clamp_(0.05, 8.0)
    secs = time.perf_counter() - t0
    final = [err(x.detach().numpy(), t, f) for x, t, f in zip(P, truths, frees)]
    return FitResult(steps, float(np.mean(init)), float(np.mean(final)), final, init_r, part_err([3]), init_nk,
                     part_err(list(range(5, 11))), first_loss, last_loss, secs)


def fit_sequential(n_scenes: int = 32, tris: int = 50_000, res: int = 256, spp: int = 16,
                   target_spp: int = 1024, steps: int = 200, lr: float = 1e-2, seed: int = 0) -> FitResult:
    import time

    import torch

    rng = np.random.default_rng(seed)
    work = []
    for j, sc in enumerate(make_scenes(n_scenes, tris, res, spp, seed)):
        truth = diff.params_from_materials(sc.materials)
        free = _free_mask(sc.materials)
        tgt = diff.MaterialRenderer(sc, spp=target_spp, seed=10_000 + j)
        tgt.set_params(truth)
        s, c = tgt.render_sums(torch)
        T = (s / c.unsqueeze(-1)).detach()
        del tgt, s, c
        R = diff.MaterialRenderer(sc, spp=spp, seed=0)
        start = truth.copy()
        start[free] = truth[free] * rng.uniform(0.6, 1.4, int(free.sum()))
        work.append((R, T, truth, free, torch.tensor(start, dtype=torch.float64, requires_grad=True)))

    def err(P, truth, free):
        return float(np.mean(np.abs(P[free] - truth[free])))

    def part(slots):
        def f(w):
            m = w[3].copy()
            m[:, [i for i in range(diff.SLOTS) if i not in slots]] = False
            return err(w[4].detach().numpy(), w[2], m) if m.any() else 0.0
        return float(np.mean([f(w) for w in work]))

    init = [err(w[4].detach().numpy(), w[2], w[3]) for w in work]
    init_r, init_nk = part([3]), part(list(range(5, 11)))
    opts = [torch.optim.Adam([w[4]], lr=lr) for w in work]
    t0 = time.perf_counter()
    first_loss, last_loss = 0.0, 0.0
    for step in range(steps):
        for j, (R, T, truth, free, P) in enumerate(work):
            R.set_seeds(2 * (step * n_scenes + j) + 1, 2 * (step * n_scenes + j) + 2)
            opts[j].zero_grad()
            I = R.image(P)
            ok = torch.isfinite(T) & torch.isfinite(I)
            d = torch.where(ok, I - torch.where(ok, T, torch.zeros_like(T)), torch.zeros_like(I))
            L = (d ** 2).sum() / max(1, int(ok.sum()))
            L.backward()
            if step == 0:
                first_loss += float(L.detach()) / n_scenes
            if step == steps - 1:
                last_loss += float(L.detach()) / n_scenes
            with torch.no_grad():
                P.grad[~torch.from_numpy(free)] = 0.0
            opts[j].step()
            with torch.no_grad():  # keep the parameters physical
                P[:, 3].clamp_(0.02, 1.0)
                P[:, 5:11].clamp_(0.05, 8.0)
    secs = time.perf_counter() - t0
    final = [err(w[4].detach().numpy(), w[2], w[3]) for w in work]
    return FitResult(steps, float(np.mean(init)), float(np.mean(final)), final, init_r, part([3]), init_nk,
                     part(list(range(5, 11))), first_loss, last_loss, secs)


def main() -> None:
    import argparse
    import json

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--scenes", type=int, default=32)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--res", type=int, default=256)
    ap.add_argument("--sequential", action="store_true", help="one scene after another instead of one group")
    args = ap.parse_args()
    importlib.import_module("openmaterial-validation_gb300").build()
    f = fit_sequential if args.sequential else fit
    r = f(n_scenes=args.scenes, steps=args.steps, spp=args.spp, res=args.res)
    print(json.dumps(r.__dict__))


if __name__ == "__main__":
    main()
