"""The multi-GPU path of bench.py is replicas only: independent chains, a gloo
group for the barrier and the max over ranks.  Two CPU ranks over gloo check
the reduction, the whole-job rate and that only rank 0 runs the reference arm."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench

    r, w, lr = bench.replica_env()
    dist = bench.replica_group(w)
    ms = 100.0 + 50.0 * r  # this rank's timed region
    ms_max = bench.replica_max(dist, ms)
    rate = bench.whole_job_rate(w, 95 * 10, ms_max)
    dist.barrier()
    # the reference arm: rank 0 alone does work; the others return at once
    class A:
        steps, warmup, gpus = 1, 1, w

    ran = "skipped"
    if r != 0:
        bench.run_reference(A())
        ran = "returned"
    dist.destroy_process_group()
    out.put((r, w, lr, ms_max, rate, ran))


def test_two_gloo_replicas_reduce_to_the_slowest_rank():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, ms_max, rate, ran) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert ms_max == 150.0
        assert abs(rate - 2 * 950 / 0.150) < 1e-9
    assert res[1][5] == "returned"


def test_one_process_needs_no_group():
    import bench

    assert bench.replica_group(1) is None
    assert bench.replica_max(None, 3.5) == 3.5
    assert bench.whole_job_rate(1, 95, 1000.0) == 95.0


def test_hbm_roofline_view(tmp_path):
    import json

    import bench

    peaks = tmp_path / "peaks.json"
    peaks.write_text(json.dumps({"hbm_gbs": 6800.0}))
    r = bench.hbm_roofline(5.0e10, 125.0, str(peaks))  # 50 GB in 125 ms -> 400 GB/s
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["achieved"] - 400.0) < 1e-9 and abs(r["frac"] - 400.0 / 6800.0) < 1e-12
    assert bench.hbm_roofline(None, 125.0, str(peaks)) is None
    assert bench.hbm_roofline(5.0e10, 125.0, str(tmp_path / "missing.json")) is None
