"""Benchmark of the GB300 BDPT render path on the large plain-BDPT workload.

Workload (one step = one frame): 64 instanced meshes, 1,048,576 triangles,
glTF PBR materials, 2048x1024 RGBE HDRI (log-normal sky + three 1e4 sun lobes),
1920x1080, 64 spp, camera bounces 10, max path length 10, no point lights
(seeded synthetic scene of that shape; see openmaterial-validation_gb300/scenes.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours: K frames on cuda:LOCAL_RANK; value = all ranks' paths / max-over-ranks
device time (CUDA events on the launching stream, L2 flushed between frames,
flush outside the events).  With N > 1 every rank renders its own sample range
of the same frame (replicas, no collective in the timed region).
reference: the CPU reference implementation of the path (the oracle's C port of
the reference renderer, oracle/oc_render.c, all host threads) on bounded row
bands of the same frame; rank 0 only.
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "BDPT Mpaths/s & Mrays/s at equal RMSE; batched/adjoint vs plain on 1 GB300"
WORKLOAD = ("plain BDPT, large scene: 64 instances / 1,048,576 triangles, PBR metallic-roughness, "
            "2048x1024 HDRI, 1920x1080, 64 spp, max path length 10")
HBM_FALLBACK_GBS = 6800.0


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            j = json.load(fh)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def frame_config(scene) -> dict:
    """The workload keys both arms report, identical on both sides (the same
    scene and frame); how each arm runs it is its line's `parallelism`."""
    workload = WORKLOAD if scene.name != "c1" else "plain BDPT, point-light scene (C1 geometry and light)"
    return {"workload": workload, "width": scene.camera.width, "height": scene.camera.height,
            "spp": scene.render.samples_per_pixel, "max_path_length": scene.render.max_path_length,
            "triangles": scene.num_triangles, "instances": len(scene.instances),
            "l2": "flushed by a 256 MiB write between timed frames (GPU arm)", "film": "FP64 sums"}


class Clocks:
    """nvidia-smi sampling during the timed region (50 ms period)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_sample_offset(rank: int, spp: int) -> int:
    """Replicas: rank r renders samples [r spp, (r + 1) spp) of every pixel, so
    the ranks' films are disjoint sample ranges of one image (no collective)."""
    return rank * spp


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's time (the job's time): MAX all-reduce, or x alone."""
    import torch

    if dist is None:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(paths_per_rank: int, ws: int, seconds: float) -> float:
    """Mpaths/s of the whole job: the paths of all ranks over the slowest rank's time."""
    return paths_per_rank * ws / seconds / 1e6


def cpu_reference(oracle, scene, spp: int, target_s: float, seed: int = 7, threads: int = None):
    """Times the oracle port (all host threads) on a centred band of rows sized to
    about target_s seconds.  Returns (Mpaths/s, Mrays/s, cores, rows, seconds)."""
    threads = threads or os.cpu_count() or 1
    os_ = oracle.OracleScene(scene)
    W, H = scene.camera.width, scene.camera.height
    p = oracle.capi.params_for(scene, spp=spp)
    mid = H // 2
    rows = max(1, min(H, threads))
    while True:
        r0 = max(0, mid - rows // 2)
        t0 = time.perf_counter()
        _, _, rays = os_.render(params=p, mode=1, threads=threads, rows=(r0, r0 + rows), seed=seed, normalize=False)
        dt = time.perf_counter() - t0
        if dt >= 0.5 * target_s or rows >= H:
            break
        rows = min(H, max(rows + 1, int(rows * target_s / max(dt, 1e-3))))
    paths = rows * W * spp
    os_.close()
    return paths / dt / 1e6, rays / dt / 1e6, threads, rows, dt


def run_reference(args, scene, rank):
    if rank != 0:
        return
    import oracle

    oracle.build()
    spp = scene.render.samples_per_pixel
    vals, rvals, rows_used, secs = [], [], 0, []
    for i in range(args.warmup + args.steps):
        v, rv, cores, rows, dt = cpu_reference(oracle, scene, spp, target_s=args.ref_step_seconds, seed=100 + i)
        if i >= args.warmup:
            vals.append(v)
            rvals.append(rv)
            secs.append(dt)
            rows_used = rows
    value = statistics.mean(vals)
    sample = f"rows {scene.camera.height // 2 - rows_used // 2}..+{rows_used} of the 1920x1080 frame at {spp} spp"
    line = {"metric": METRIC, "value": round(value, 4), "unit": "Mpaths/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * statistics.mean(secs), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": frame_config(scene), "parallelism": f"{cores} host threads",
            "mrays_per_s": round(statistics.mean(rvals), 4),
            "cpu_baseline": {"value": round(value, 4), "unit": "Mpaths/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batched(args, dev):
    """Batched material sweep: jobs of one 200k-triangle scene (8 materials,
    point light, 6 bounces), square resolution side U{128..1024}, spp U{4..64},
    one material set each, rendered (a) one job per call and (b) as one batch
    (autotuned wave size, captured CUDA graph).  Same estimator, jobs and spp on
    both sides, so the films (and their RMSE) are equal; jobs/s compares them."""
    import numpy as np
    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    S = importlib.import_module("openmaterial-validation_gb300.scenes")
    n = args.batch_jobs
    sc = S.scene_materials(64, 64, 4, tris=200_000, bounces=6)
    rs = omv.RenderScene(sc, dev.index or 0)
    sets = S.material_variants(sc, n, seed=3)
    rng = np.random.default_rng(11)
    sides = rng.integers(128, 1025, size=n)
    spps = rng.integers(4, 65, size=n)
    br = omv.BatchRenderer(rs, omv.RendererParameters.for_scene(sc))
    br.set_material_sets(sets)
    films, jobs = [], []
    for j in range(n):
        w = int(sides[j])
        f = (torch.zeros((w, w, 3), dtype=torch.float64, device=dev), None,
             torch.zeros((w, w), dtype=torch.int32, device=dev))
        cam = omv.PinholeCamera.from_spec(sc.camera)
        cam.width = cam.height = w
        cam.adjust_to_resolution()
        cam.set_y_fov(45.0)
        films.append(f)
        jobs.append(br.job(cam, int(spps[j]), f, seed=j, material_set=j))
    paths = int(sum(int(sides[j]) ** 2 * int(spps[j]) for j in range(n)))

    def zero():
        for f in films:
            f[0].zero_()
            f[2].zero_()

    def timed(fn):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize(dev)
        return time.perf_counter() - t0

    def plain():
        for jb in jobs:
            br.render([jb])

    # one job per call through the single-frame API, as a caller without the
    # batch entry point would do it: the job's materials, then its frame
    L, capi = omv.lib(), omv.capi
    descs = []
    for j in range(n):
        keep: list = []
        descs.append((capi.material_descs(sets[j], keep), len(sets[j]), keep))
    prm = []
    for j in range(n):
        pc = br.params.to_c()
        pc.samples_per_pixel, pc.seed, pc.sample_offset = int(spps[j]), j, 0
        prm.append(pc)
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def per_call():
        for j, jb in enumerate(jobs):
            d, m, _ = descs[j]
            omv.check(L.omv_scene_set_materials(rs.handle, m, d))
            omv.check(L.omv_render_device(rs.handle, C.byref(jb.camera), C.byref(prm[j]), C.c_void_p(jb.d_sum_rgb),
                                          None, C.c_void_p(jb.d_count), stream, None))

    chosen = br.autotune(jobs)
    br.render(jobs, graph=True)  # capture
    zero()
    timed(plain)  # warm-up
    zero()
    t_plain = timed(plain)
    ref_sum = [f[0].clone() for f in films]
    ref_cnt = [f[2].clone() for f in films]
    zero()
    timed(per_call)  # warm-up
    zero()
    t_call = timed(per_call)
    call_sum = [f[0].clone() for f in films]
    call_cnt = [f[2].clone() for f in films]
    keep0: list = []
    omv.check(L.omv_scene_set_materials(rs.handle, len(sc.materials), capi.material_descs(sc.materials, keep0)))
    zero()
    br.render(jobs, graph=True)  # warm-up replay
    zero()
    t_batch = timed(lambda: br.render(jobs, graph=True))
    # shadow-ray contributions reach a path's radiance through FP32 atomics, whose
    # order varies from run to run: a path's radiance is an FP32 sum of up to
    # (light bounces + 1) x camera bounces = 42 terms, each rounding by at most
    # half an ulp of the running sum, on both sides: sums agree to 42 FP32 ulps
    # (5e-6) of the pixel, counts exactly
    counts_match = all(bool((f[2] == c).all()) for f, c in zip(films, ref_cnt))
    rel = max(float((f[0] - r).abs().max()) / max(1e-30, float(r.abs().max())) for f, r in zip(films, ref_sum))
    match = counts_match and rel <= 5e-6
    call_counts = all(bool((f[2] == c).all()) for f, c in zip(films, call_cnt))
    call_rel = max(float((f[0] - r).abs().max()) / max(1e-30, float(r.abs().max())) for f, r in zip(films, call_sum))
    del films, ref_sum, ref_cnt, call_sum, call_cnt
    torch.cuda.empty_cache()
    return {"jobs": n, "paths": paths, "plain_jobs_per_s": round(n / t_plain, 3),
            "batched_jobs_per_s": round(n / t_batch, 3), "speedup": round(t_plain / t_batch, 3),
            "per_call_jobs_per_s": round(n / t_call, 3), "speedup_vs_per_call": round(t_call / t_batch, 3),
            "per_call_films_match": call_counts and call_rel <= 5e-6,
            "plain_mpaths_per_s": round(paths / t_plain / 1e6, 2), "batched_mpaths_per_s": round(paths / t_batch / 1e6, 2),
            "wave_paths": chosen, "shade_block_threads": br.block_threads, "graph": True, "films_match": match,
            "counts_match": counts_match,
            "films_max_rel_diff": rel,
            "timing": "host wall clock with device synchronisation, one pass over all jobs",
            "equal_rmse": "same estimator, jobs and spp: identical films up to summation order",
            "scene": f"{rs.info()['triangles']} triangles, 8 materials (4 PBR, 4 OpenMATERIAL conductors), point light, 6 bounces"}


def run_post(args, dev, film, count, W, H, flush):
    """Image development of the frame just rendered (the reference main's tail,
    main.cpp:505-521): omv_develop (film -> normalised -> gamma 0.5 -> 8-bit,
    flipped) and the 3x3 median, each timed alone with CUDA events on the
    launching stream, L2 flushed before every launch.  Algorithmic bytes per
    pixel: develop 24 + 4 read, 16 + 16 + 4 written; median 16 read, 16 written.
    CPU side: the oracle's gamma correction and median of the same image, one
    thread (the reference runs both single-threaded)."""
    import numpy as np
    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    L = omv.lib()
    npix = W * H
    lin = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    toned = torch.empty_like(lin)
    med = torch.empty_like(lin)
    u8 = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream(dev)
    sp = C.c_void_p(st.cuda_stream)

    def develop():
        omv.check(L.omv_develop(C.c_void_p(film.data_ptr()), C.c_void_p(count.data_ptr()), W, H, 1.0, 0.5,
                                C.c_void_p(lin.data_ptr()), C.c_void_p(toned.data_ptr()), C.c_void_p(u8.data_ptr()),
                                1, sp))

    def median():
        omv.check(L.omv_denoise_median(C.c_void_p(toned.data_ptr()), C.c_void_p(med.data_ptr()), W, H, 1, sp))

    def timed(fn, reps):
        for _ in range(3):
            fn()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            fn()
            e1.record(st)
            torch.cuda.synchronize(dev)
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    hbm, kind = _peaks()
    reps = max(5, args.steps * 4)
    out = {"image": f"{W}x{H}", "l2": "flushed by a 256 MiB write before each launch", "peak_gbs": hbm,
           "peak_source": kind}
    for name, fn, bpp in (("develop", develop, 64), ("median3", median, 32)):
        t = timed(fn, reps)
        gbs = npix * bpp / (t / 1e3) / 1e9
        out[name] = {"ms": round(t, 4), "bytes_per_pixel": bpp, "achieved_gbs": round(gbs, 1),
                     "frac": round(gbs / hbm, 4), "mpix_per_s": round(npix / (t / 1e3) / 1e6, 1)}
    if not args.no_cpu_baseline:
        import oracle

        oracle.build()
        img = lin.cpu().numpy()
        t0 = time.perf_counter()
        tm = oracle.tonemap(img, 0.5)
        t1 = time.perf_counter()
        oracle.median(tm, 1)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "gamma_ms": round((t1 - t0) * 1e3, 2),
                               "median_ms": round((t2 - t1) * 1e3, 2),
                               "sample": f"the whole {W}x{H} image"}
        # parity on the benchmark frame itself
        out["median_matches_oracle"] = bool(np.array_equal(med.cpu().numpy(), oracle.median(toned.cpu().numpy(), 1)))
    return out


def run_adjoint(args, dev):
    """Adjoint: 512x512 L2 loss against a 1024-spp target of a 100k-triangle
    scene with 8 materials (4 PBR: base colour, roughness, metallic; 4
    OpenMATERIAL conductors: n, k per RGB: 44 active parameters of 88 slots),
    32 spp forward.  The path-replay gradient (forward + replay) is timed
    against central differences (eps 1e-3, common random numbers: 2 renders per
    parameter) at the same spp; both are compared with a 512-spp path-replay
    reference gradient, and gradients/s are compared at equal RMSE (time grows
    with the inverse square of the RMSE)."""
    import numpy as np
    import torch

    S = importlib.import_module("openmaterial-validation_gb300.scenes")
    diff = importlib.import_module("openmaterial-validation_gb300.diff")
    spp = args.adjoint_spp
    sc = S.scene_materials(512, 512, spp, tris=100_000, bounces=6)
    P0 = diff.params_from_materials(sc.materials)
    active = diff.active_mask(sc.materials)
    Pt = P0.copy()
    Pt[:, 0:3] = np.clip(Pt[:, 0:3] * 0.7 + 0.1, 0.05, 0.95)
    Pt[:, 3] = np.clip(Pt[:, 3] * 0.8 + 0.1, 0.05, 0.95)
    Pt[:, 4] = 1.0 - Pt[:, 4]
    Pt[:, 5:11] = Pt[:, 5:11] * 0.8
    Rt = diff.MaterialRenderer(sc, spp=1024, seed=99)
    Rt.set_params(Pt)
    s, c = Rt.render_sums(torch)
    T = (s / c.unsqueeze(-1)).detach()
    del Rt, s, c
    R = diff.MaterialRenderer(sc, spp=spp, seed=1)

    # the estimator can produce an infinite sample (so does the reference's):
    # pixels whose target or image is not finite are left out of the loss
    def l2(I):
        ok = torch.isfinite(T) & torch.isfinite(I)
        d = torch.where(ok, I - torch.where(ok, T, torch.zeros_like(T)), torch.zeros_like(I))
        return (d ** 2).sum() / max(1, int(ok.sum()))

    def ad_grad(renderer):
        P = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
        L = l2(renderer.image(P))
        L.backward()
        return P.grad.detach().cpu().numpy()

    def loss(Px):
        R.set_params(Px)
        s_, c_ = R.render_sums(torch)
        return float(l2(s_ / c_.unsqueeze(-1)))

    def fd_grad():
        g = np.zeros_like(P0)
        for i, k in zip(*np.nonzero(active)):
            Pp, Pm = P0.copy(), P0.copy()
            Pp[i, k] += 1e-3
            Pm[i, k] -= 1e-3
            g[i, k] = (loss(Pp) - loss(Pm)) / 2e-3
        return g

    ad_grad(R)  # warm-up
    t0 = time.perf_counter()
    g_ad = ad_grad(R)
    t_ad = time.perf_counter() - t0
    t0 = time.perf_counter()
    g_fd = fd_grad()
    t_fd = time.perf_counter() - t0
    Rref = diff.MaterialRenderer(sc, spp=512, seed=5)
    g_ref = ad_grad(Rref)
    exact = active.copy()
    exact[:, 3] = False

    def rmse(g, m):
        return float(np.sqrt(np.mean((g[m] - g_ref[m]) ** 2)))

    out = {"params": int(active.sum()), "slots": int(active.size), "spp": spp,
           "adjoint_s": round(t_ad, 4), "fd_s": round(t_fd, 4), "fd_renders": int(2 * active.sum())}
    for name, m in (("all", active), ("no_roughness", exact)):
        ra, rf = rmse(g_ad, m), rmse(g_fd, m)
        t_fd_eq = t_fd * max(1.0, (rf / ra) ** 2) if ra > 0 else t_fd
        out[name] = {"rmse_adjoint": ra, "rmse_fd": rf, "adjoint_gradients_per_s": round(1.0 / t_ad, 3),
                     "fd_gradients_per_s_at_equal_rmse": round(1.0 / t_fd_eq, 5),
                     "speedup_at_equal_rmse": round(t_fd_eq / t_ad, 2)}
    out["reference"] = "path-replay gradient at 512 spp, other seed"
    out["timing"] = "host wall clock with device synchronisation"
    return out


def run_mis(args, dev, rs, scene, flush):
    """The MIS estimator (environment connections, power heuristic) against the
    reference estimator on the benchmark frame: device time per frame and the
    per-sample variance of every pixel and channel.  Both estimate the same
    image, so the speed at equal RMSE is (t_ref x var_ref) / (t_mis x var_mis).
    The reference estimator's variance under the sun lobes is heavy-tailed;
    over the 132.7M samples of a frame its mean is still well estimated."""
    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    L, capi = omv.lib(), omv.capi
    W, H = scene.camera.width, scene.camera.height
    spp, npix = scene.render.samples_per_pixel, W * H
    cam = capi.camera_struct(scene.camera)
    s = torch.zeros(3 * npix, dtype=torch.float64, device=dev)
    q = torch.zeros(3 * npix, dtype=torch.float64, device=dev)
    n = torch.zeros(npix, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for name, est in (("reference", omv.ESTIMATOR_REFERENCE), ("mis", omv.ESTIMATOR_MIS)):
        p = capi.params_for(scene, spp=spp, seed=4321)
        p.estimator = est
        p.accumulate_variance = 1

        def once():
            s.zero_()
            q.zero_()
            n.zero_()
            omv.check(L.omv_render_device(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(s.data_ptr()),
                                          C.c_void_p(q.data_ptr()), C.c_void_p(n.data_ptr()),
                                          C.c_void_p(stream.cuda_stream), None))

        once()  # warm-up (the MIS estimator builds its table here)
        times = []
        for _ in range(3):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            once()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1))
        mean = s / spp
        var = torch.clamp(q / spp - mean * mean, min=0.0)
        out[name] = {"ms": round(sorted(times)[1], 3), "var": float(var.mean()), "image_sum": float(mean.sum()),
                     "se": float(torch.sqrt((var / spp).sum()))}
    r, m = out["reference"], out["mis"]
    z = (m["image_sum"] - r["image_sum"]) / max(1e-30, (m["se"] ** 2 + r["se"] ** 2) ** 0.5)
    return {"ms_reference": r["ms"], "ms_mis": m["ms"], "var_reference": r["var"], "var_mis": m["var"],
            "variance_ratio": round(r["var"] / max(m["var"], 1e-30), 2), "image_mean_z": round(z, 2),
            "speedup_at_equal_rmse": round(r["ms"] * r["var"] / max(m["ms"] * m["var"], 1e-30), 2),
            "mis_mpaths_per_s": round(npix * spp / (m["ms"] / 1e3) / 1e6, 1),
            "timing": "CUDA events, median of 3 frames, L2 flushed, per-pixel variance accumulated on both sides"}


def run_lights(args, dev, flush):
    """The point-light path (light subpaths, vertex connections and their
    closest-hit shadow rays, BDPTRenderer.cpp:260-298, 208-235): C1 (256x256,
    16 spp, max path length 6, one point light, 5,122 triangles) and the same
    scene at 1920x1080, 64 spp, which fills the GPU.  Device time per frame
    (CUDA events, median of 3, L2 flushed, per-kernel events on), rays of every
    kind, the shadow kernel's roofline (nodes x 128 B + triangles x 48 B per
    launch over its event time) and the oracle port on the machine's cores beside
    it (C1: the whole frame; full HD: a centred band of rows)."""
    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    S = importlib.import_module("openmaterial-validation_gb300.scenes")
    L, capi = omv.lib(), omv.capi
    hbm, peak_kind = _peaks()
    stream = torch.cuda.current_stream(dev)
    out = {}
    for name, sc in (("c1_256x256x16", S.scene_c1(256, 256, 16)), ("c1_1920x1080x64", S.scene_c1(1920, 1080, 64))):
        rs = omv.RenderScene(sc, dev.index or 0)
        W, H = sc.camera.width, sc.camera.height
        spp, npix = sc.render.samples_per_pixel, W * H
        cam = capi.camera_struct(sc.camera)
        p = capi.params_for(sc, spp=spp, seed=31)
        p.time_kernels = 1
        s = torch.zeros(3 * npix, dtype=torch.float64, device=dev)
        n = torch.zeros(npix, dtype=torch.int32, device=dev)
        runs = []
        for it in range(4):
            s.zero_()
            n.zero_()
            flush.zero_()
            st = capi.Stats()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            omv.check(L.omv_render_device(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(s.data_ptr()), None,
                                          C.c_void_p(n.data_ptr()), C.c_void_p(stream.cuda_stream), C.byref(st)))
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if it:
                runs.append((e0.elapsed_time(e1), st))
        runs.sort(key=lambda r: r[0])
        ms, st = runs[1]
        rays = st.extension_rays + st.shadow_rays + st.light_rays
        sl = max(1, st.shadow_launches)
        sh_bytes = (st.shadow_nodes_visited * 128 + st.shadow_triangles_tested * 48) / sl
        sh_ms = st.shadow_ms / sl
        sh_gbs = sh_bytes / (sh_ms / 1e3) / 1e9 if sh_ms > 0 else 0.0
        rec = {"frame_ms": round(ms, 3), "mpaths_per_s": round(npix * spp / (ms / 1e3) / 1e6, 1),
               "mrays_per_s": round(rays / (ms / 1e3) / 1e6, 1), "extension_rays": st.extension_rays,
               "light_rays": st.light_rays, "shadow_rays": st.shadow_rays, "launches": st.kernel_launches,
               "extend_ms": round(st.extend_ms, 3), "shadow_ms": round(st.shadow_ms, 3),
               "shadow_roofline": {"kernel": "k_shadow (vertex connections)", "bound": "hbm",
                                   "achieved": round(sh_gbs, 1), "peak": hbm, "unit": "GB/s",
                                   "frac": round(sh_gbs / hbm, 4), "peak_source": peak_kind,
                                   "bytes_per_launch": round(sh_bytes), "ms_per_launch": round(sh_ms, 4)}}
        if not args.no_cpu_baseline:
            import oracle

            oracle.build()
            v, rv, cores, rows, dt = cpu_reference(oracle, sc, spp, target_s=min(4.0, args.cpu_seconds))
            rec["cpu_baseline"] = {"value": round(v, 4), "unit": "Mpaths/s", "cores": cores, "kind": "port",
                                   "mrays_per_s": round(rv, 4),
                                   "sample": f"rows {H // 2 - rows // 2}..+{rows} of the {W}x{H} frame at {spp} spp"}
            rec["gpu_over_cpu"] = round(rec["mpaths_per_s"] / max(v, 1e-9), 1)
        out[name] = rec
        rs.close()
        del s, n
    return out


def run_c5(args, dev):
    """Batched inverse material fit (32 scenes x 50k triangles x 4 materials,
    256x256, targets at 1024 spp, 200 Adam steps at lr 1e-2, 16 spp forward
    and adjoint): all scenes in one group, a step being one batch render and
    one batch of adjoint jobs, against the same fit with one scene after
    another through their own handles (timed over its first steps; both
    forms do the same work per step).  Parameter errors against the hidden
    values."""
    inv = importlib.import_module("openmaterial-validation_gb300.inverse")
    g = inv.fit(n_scenes=args.c5_scenes, tris=50_000, res=256, spp=16, target_spp=1024, steps=args.c5_steps,
                lr=1e-2, seed=0)
    seq_steps = max(1, min(10, args.c5_steps))
    q = inv.fit_sequential(n_scenes=args.c5_scenes, tris=50_000, res=256, spp=16, target_spp=1024,
                           steps=seq_steps, lr=1e-2, seed=0)
    per_g, per_q = g.seconds / g.steps, q.seconds / q.steps
    return {"scenes": args.c5_scenes, "steps": g.steps, "group_seconds": round(g.seconds, 2),
            "group_seconds_per_step": round(per_g, 4), "sequential_seconds_per_step": round(per_q, 4),
            "sequential_steps_timed": q.steps, "speedup_per_step": round(per_q / per_g, 2),
            "roughness_error": [round(g.initial_roughness_error, 4), round(g.final_roughness_error, 4)],
            "conductor_nk_error": [round(g.initial_ior_error, 4), round(g.final_ior_error, 4)],
            "parameter_error": [round(g.initial_error, 4), round(g.final_error, 4)],
            "loss": [g.initial_loss, g.final_loss],
            "timing": "host wall clock of the optimisation loop (targets excluded), device synchronised each step"}


def run_builders(args, dev, scene, flush):
    """The four acceleration-structure builders on the benchmark scene: the
    scene creation time (omv_scene_create, which the build dominates) and the
    frame's device time on each tree (CUDA events, median of 3 frames, L2
    flushed), with the nodes each extension ray fetched."""
    import torch

    omv = importlib.import_module("openmaterial-validation_gb300")
    L, capi = omv.lib(), omv.capi
    W, H = scene.camera.width, scene.camera.height
    spp, npix = scene.render.samples_per_pixel, W * H
    cam = capi.camera_struct(scene.camera)
    s = torch.zeros(3 * npix, dtype=torch.float64, device=dev)
    n = torch.zeros(npix, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for name, b in (("sah", capi.BVH_SAH), ("ploc", capi.BVH_PLOC), ("lbvh", capi.BVH_LBVH),
                    ("host_sah", capi.BVH_HOST_SAH)):
        rs = omv.RenderScene(scene, dev.index or 0, bvh_builder=b)
        info = rs.info()
        p = capi.params_for(scene, spp=spp, seed=77)
        times, st = [], capi.Stats()
        for it in range(4):
            s.zero_()
            n.zero_()
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            omv.check(L.omv_render_device(rs.handle, C.byref(cam), C.byref(p), C.c_void_p(s.data_ptr()), None,
                                          C.c_void_p(n.data_ptr()), C.c_void_p(stream.cuda_stream), C.byref(st)))
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if it:
                times.append(e0.elapsed_time(e1))
        ms = sorted(times)[1]
        out[name] = {"build_ms": round(info["build_ms"], 1), "frame_ms": round(ms, 3),
                     "mpaths_per_s": round(npix * spp / (ms / 1e3) / 1e6, 1),
                     "nodes_per_ray": round(st.nodes_visited / max(1, st.extension_rays), 2),
                     "bvh8_nodes": info["blas_nodes"]}
        rs.close()
    out["build_ms_note"] = "omv_scene_create wall time: geometry upload, normals, the BVH build and its validation"
    return out


def run_ours(args, scene, ws, rank, local):
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    omv = importlib.import_module("openmaterial-validation_gb300")
    if rank == 0:
        omv.build()
    if dist:
        dist.barrier()
    L = omv.lib()
    capi = omv.capi
    rs = omv.RenderScene(scene, device=local)
    W, H = scene.camera.width, scene.camera.height
    spp = scene.render.samples_per_pixel
    npix = W * H
    cam = capi.camera_struct(scene.camera)
    params = capi.params_for(scene, spp=spp, seed=1234)
    params.sample_offset = rank_sample_offset(rank, spp)
    params.time_kernels = 1
    dev = torch.device("cuda", local)
    film = torch.zeros(3 * npix, dtype=torch.float64, device=dev)
    count = torch.zeros(npix, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(stats):
        film.zero_()
        count.zero_()
        omv.check(L.omv_render_device(rs.handle, C.byref(cam), C.byref(params), C.c_void_p(film.data_ptr()), None,
                                      C.c_void_p(count.data_ptr()), C.c_void_p(stream.cuda_stream),
                                      C.byref(stats)))

    for _ in range(args.warmup):
        step(capi.Stats())
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    torch.cuda.synchronize(dev)
    evs = []
    agg = {k: 0 for k in ("extension_rays", "shadow_rays", "light_rays", "kernel_launches", "nodes_visited",
                          "triangles_tested", "extend_launches", "stack_overflows", "tail_nodes_visited",
                          "tail_triangles_tested")}
    ext_ms = tail_ms = 0.0
    tail_bounce = 0
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = capi.Stats()
        step(st)
        e1.record(stream)
        evs.append((e0, e1))
        for k in agg:
            agg[k] += getattr(st, k)
        ext_ms += st.extend_ms
        tail_ms += st.tail_ms
        tail_bounce = st.tail_bounce
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    clock = clocks.stop()
    dev_ms = sum(a.elapsed_time(b) for a, b in evs)
    max_ms = max_over_ranks(dev_ms, dist, dev)
    cnt_ok = bool((count == spp).all().item())
    value = whole_job_rate(npix * spp * args.steps, ws, max_ms / 1e3)
    rays = (agg["extension_rays"] + agg["shadow_rays"] + agg["light_rays"]) * ws
    # roofline of the closest-hit kernel: algorithmic bytes = nodes x 128 B + triangles x 48 B
    hbm, peak_kind = _peaks()
    launches = max(1, agg["extend_launches"])
    bytes_per_launch = (agg["nodes_visited"] * 128 + agg["triangles_tested"] * 48) / launches
    ms_per_launch = ext_ms / launches
    achieved = bytes_per_launch / (ms_per_launch / 1e3) / 1e9 if ms_per_launch > 0 else 0.0
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
            "frac": round(achieved / hbm, 4), "traffic": None,
            "traffic_note": "DRAM bytes are not observable inside a timed run; the ncu captures of this kernel "
                            "are summarised under profiles/", "kernel": "k_extend",
            "peak_source": peak_kind, "bytes_per_launch": round(bytes_per_launch), "ms_per_launch": round(ms_per_launch, 4),
            "share_of_step": round(ext_ms / max(dev_ms, 1e-9), 4)}
    # end to end through the public API: host buffers, H2D of the step's inputs, D2H of the image
    e2e = None
    if rank == 0 or ws > 1:
        img = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy()
        p2 = capi.params_for(scene, spp=spp, seed=99)
        p2.sample_offset = rank_sample_offset(rank, spp)
        for _ in range(args.warmup):
            omv.check(L.omv_render(rs.handle, C.byref(cam), C.byref(p2), capi.fptr(img), None, None, None, None))
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            omv.check(L.omv_render(rs.handle, C.byref(cam), C.byref(p2), capi.fptr(img), None, None, None, None))
            times.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(sum(times), dist, dev)
        e2e = {"value": round(whole_job_rate(npix * spp * args.steps, ws, e2e_s), 4), "unit": "Mpaths/s",
               "h2d_bytes_per_step": C.sizeof(capi.Camera) + C.sizeof(capi.Params),
               "d2h_bytes_per_step": int(img.nbytes)}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle

        oracle.build()
        v, rv, cores, rows, dt = cpu_reference(oracle, scene, spp, target_s=args.cpu_seconds)
        cpu = {"value": round(v, 4), "unit": "Mpaths/s", "cores": cores, "kind": "port",
               "sample": f"rows {H // 2 - rows // 2}..+{rows} of the {W}x{H} frame at {spp} spp ({dt:.1f} s)",
               "mrays_per_s": round(rv, 4)}
    if rank == 0:
        info = rs.info()
        line = {"metric": METRIC, "value": round(value, 4), "unit": "Mpaths/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(max_ms / args.steps, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": frame_config(scene), "parallelism": f"replicas x{ws} (disjoint sample ranges)",
                "mrays_per_s": round(rays / (max_ms / 1e3) / 1e6, 4), "film_counts_ok": cnt_ok,
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clock,
                "gpu_launches": agg["kernel_launches"], "scene_build_ms": round(info["build_ms"], 1),
                "stack_overflows": agg["stack_overflows"],
                "tail": {"kernel": "k_camera_tail", "from_bounce": tail_bounce,
                         "ms_per_step": round(tail_ms / args.steps, 4),
                         "share_of_step": round(tail_ms / max(dev_ms, 1e-9), 4),
                         "nodes_per_step": agg["tail_nodes_visited"] // args.steps,
                         "triangles_per_step": agg["tail_triangles_tested"] // args.steps}}
        if ws == 1 and not args.no_lights:
            line["lights"] = run_lights(args, dev, flush)
        if ws == 1 and not args.no_builders:
            line["builders"] = run_builders(args, dev, scene, flush)
        if ws == 1 and not args.no_post:
            line["post"] = run_post(args, dev, film, count, W, H, flush)
        if ws == 1 and not args.no_mis:
            line["mis"] = run_mis(args, dev, rs, scene, flush)
        if ws == 1 and not args.no_batched:
            line["batched"] = run_batched(args, dev)
        if ws == 1 and not args.no_adjoint:
            line["adjoint"] = run_adjoint(args, dev)
        if ws == 1 and not args.no_c5:
            line["c5"] = run_c5(args, dev)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--scene", choices=["c2", "c1"], default="c2",
                    help="c2: the benchmark scene; c1: the point-light scene (for profiling the light path)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched material sweep")
    ap.add_argument("--no-post", action="store_true", help="skip the image development leg")
    ap.add_argument("--no-builders", action="store_true", help="skip the BVH builder comparison leg")
    ap.add_argument("--no-lights", action="store_true", help="skip the point-light leg")
    ap.add_argument("--no-mis", action="store_true", help="skip the MIS-vs-reference estimator leg")
    ap.add_argument("--batch-jobs", type=int, default=256)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-vs-finite-difference leg")
    ap.add_argument("--adjoint-spp", type=int, default=32)
    ap.add_argument("--no-c5", action="store_true", help="skip the batched inverse-fit leg")
    ap.add_argument("--c5-scenes", type=int, default=32)
    ap.add_argument("--c5-steps", type=int, default=200)
    args = ap.parse_args()
    ws, rank, local = _dist()
    if args.impl == "reference" and rank != 0:
        return
    S = importlib.import_module("openmaterial-validation_gb300.scenes")
    if args.scene == "c1":  # the point-light scene (profiling of the light path), not the benchmark frame
        scene = S.scene_c1(args.width, args.height, args.spp)
    else:
        scene = S.scene_c2(args.width, args.height, args.spp)
    if args.impl == "reference":
        run_reference(args, scene, rank)
    else:
        run_ours(args, scene, ws, rank, local)


if __name__ == "__main__":
    main()
