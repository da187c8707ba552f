"""The bench's multi-rank path on CPU (gloo, world size 2): every rank renders
its own sample range of the frame (replicas, no collective inside the timed
region), the job's time is the slowest rank's (MAX all-reduce), the job's rate
counts all ranks' paths, and under the reference arm only rank 0 works."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp
from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local = bench._dist()
    dist.init_process_group("gloo", rank=r, world_size=w)
    slowest = bench.max_over_ranks(10.0 + 5.0 * r, dist, torch.device("cpu"))
    off = bench.rank_sample_offset(r, 64)
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, w, local, slowest, off))


def test_two_ranks_take_disjoint_sample_ranges_and_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [(r, w, l) for r, w, l, _, _ in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(s == 15.0 for *_, s, _ in res)
    offsets = [o for *_, o in res]
    assert offsets == [0, 64]  # [0, 64) and [64, 128): disjoint, together 2 x spp samples


def test_whole_job_rate_counts_every_rank():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.whole_job_rate(1_000_000, 4, 2.0) == pytest.approx(2.0)
    assert bench.max_over_ranks(3.5, None, None) == 3.5


def test_reference_arm_works_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.main() is None
    assert capsys.readouterr().out == ""


def test_both_arms_report_the_same_workload_config():
    """The GPU arm and the reference arm describe their workload with the
    same keys and values (one function builds both); how each runs it is the
    line's separate `parallelism` key."""
    sys.path.insert(0, ROOT)
    import importlib

    import bench

    S = importlib.import_module("openmaterial-validation_gb300.scenes")
    sc = S.scene_c2(48, 27, 4, tri_scale=0.01, suns=False, sky_size=(64, 32))
    a, b = bench.frame_config(sc), bench.frame_config(sc)
    assert a == b
    assert {"workload", "width", "height", "spp", "max_path_length", "triangles", "instances"} <= set(a)
    assert "parallelism" not in a
    assert (a["width"], a["height"], a["spp"]) == (48, 27, 4)
