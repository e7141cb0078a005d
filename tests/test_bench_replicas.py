"""Multi-GPU replicas of bench.py on CPU: two gloo ranks check the
max-over-ranks time and the whole-job arithmetic (every rank runs the same
workload on its own GPU; the job's time is the slowest rank's)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist = bench.dist_setup()
    try:
        seconds = [2.0, 3.0][r]             # rank 1 is the slower replica
        out = {
            "world": w, "rank": r, "local": local,
            "max": bench.max_over_ranks(dist, seconds),
            # 4096 trajectories per rank
            "rate": bench.replica_rate(dist, w, 4096.0, seconds),
            # one circuit per step per rank
            "spu": bench.replica_seconds_per_unit(dist, w, 1.0, seconds),
        }
        bench.barrier(dist)
        q.put(out)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_whole_job_arithmetic():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q))
             for r in range(2)]
    for p in procs:
        p.start()
    outs = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["world"] == 2 and o["local"] == o["rank"]
        assert o["max"] == 3.0
        assert o["rate"] == pytest.approx(2 * 4096 / 3.0)
        assert o["spu"] == pytest.approx(3.0 / 2)


def test_gpus_flag_must_match_launcher(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        gpus = 2
    monkeypatch.setenv("WORLD_SIZE", "4")
    with pytest.raises(SystemExit):
        bench.self_launch(A())
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.self_launch(A()) is None
    monkeypatch.delenv("WORLD_SIZE")
    A.gpus = 1
    assert bench.self_launch(A()) is None
