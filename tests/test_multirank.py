"""World-size-2 gloo tests of the bench's multi-rank host logic, and its
side-run commands (CPU only).

Every rank converts its own stream (replicas, weak scaling): no data-path
collective exists; the only cross-rank step is the MAX of the ranks' timed
regions, which these tests exercise over a real gloo process group.
"""
import json
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(times[rank])
    v = bench.job_throughput(1000, 3, world, t)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"r{rank}.json"), "w") as fh:
        json.dump({"t": t, "v": v}, fh)


def test_max_over_ranks_gloo(tmp_path):
    times = [0.25, 0.75]
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, times, str(tmp_path)), nprocs=2,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for r in res:
        assert r["t"] == 0.75                       # every rank sees the slowest rank
        assert r["v"] == pytest.approx(1000 * 3 * 2 / 0.75 / 1e6)


def test_single_process_time_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5) == 1.5
    assert bench.job_throughput(2_000_000, 2, 1, 4.0) == pytest.approx(1.0)


def test_reference_arm_nonzero_rank_is_silent(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1",
                                      "--warmup", "1"])
    bench.run_reference(bench.parse())
    assert capsys.readouterr().out == ""


def test_also_commands():
    """The default run's side workloads: each a subprocess with 3 warm-up and 3
    timed steps; name@f adds the multistream length scale."""
    import bench
    cmd = bench.also_command("samerate128")
    assert cmd[2:] == ["--workload", "samerate128", "--steps", "3", "--warmup", "3"]
    cmd = bench.also_command("multistream64@0.125")
    assert cmd[2:] == ["--workload", "multistream64", "--steps", "3", "--warmup", "3",
                       "--ms-scale", "0.125"]
    for w in bench.ALSO_DEFAULT:
        name = w.partition("@")[0]
        assert name in ("samerate128", "samerate128lp", "dsd256to128", "dsd2pcm128", "precorr128",
                        "dsd512conv6", "diff16", "multistream64")
