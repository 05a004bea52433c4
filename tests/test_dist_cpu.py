"""The multi-rank path of bench.py on CPU: two gloo ranks, each with its own
shard seed; the job's time is the slowest rank's and the whole-job value
counts every rank's columns; the reference arm runs on rank 0 only."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    w, r, loc = bench.dist_setup()
    t = bench.max_over_ranks(1.5 + rank, w, "cpu")          # rank 1 is the slower one
    v = bench.job_value(w, 1000, 10, t)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, loc, bench.rank_seed(2026, r), t, v))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert out[0][3] != out[1][3]                       # own shard per rank
    assert all(o[4] == 2.5 for o in out)                # max over ranks
    assert all(abs(o[5] - 2 * 1000 * 10 / 2.5) < 1e-9 for o in out)


def test_reference_arm_other_ranks_do_nothing(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        ncol, seed, warmup, steps, gpus = 1024, 1, 3, 4, 2
    assert bench.reference_arm(Args(), 2, 1) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_json_line(capsys):
    """Rank 0 of the reference arm times the CPU oracle and prints one JSON
    line with the contract's keys (a small workload: ~10 s of oracle work)."""
    import json
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        ncol, seed, warmup, steps, gpus = 2048, 2026, 1, 16, 1
    bench.reference_arm(Args(), 1, 0)
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    line = json.loads(lines[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
