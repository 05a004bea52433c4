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
    # the same workload config dict as the GPU arm builds from the same inputs
    A, _ = bench.make_inputs(Args.ncol, bench.rank_seed(Args.seed, 0))
    assert line["config"] == json.loads(json.dumps(bench.bench_config(A, Args.ncol)))
    assert "all 2048 columns" in line["cpu_baseline"]["sample"]


def test_soil_gate_passes_on_oracle_states_and_flags_a_planted_error():
    """The bench's correctness gate, fed oracle states in place of the GPU's:
    identical states pass; a planted 1e-7 relative error in one column of the
    one-step state is caught and counted."""
    import copy
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    A, npatch = bench.make_inputs(512, 7)
    o = bench.OracleSoilStepper(A)
    o.step(3)
    G = copy.deepcopy(o.S)
    o.step(1)
    G1 = copy.deepcopy(o.S)
    zero = (np.zeros(512), np.zeros(512))
    gate, rate, _ = bench.soil_gate(A, npatch, G, 3, G1, zero, True, sensitivity_runs=1)
    assert gate["pass"] and rate > 0
    assert gate["trajectory"]["columns_above_tol"] == 0 and gate["one_step_from_evolved_state"]["columns_above_tol"] == 0
    assert all(v == 0.0 for v in gate["trajectory"]["max_rel_err"].values())
    assert gate["balance"]["oracle_errh2o_max_mm"] < 1e-9
    use = gate["one_step_from_evolved_state"]["band_use"]
    assert set(use) == set(bench.GATE_CANCEL) and all(v["columns_above_tol_without_band"] == 0 for v in use.values())
    bad = copy.deepcopy(G1)
    bad["t_soisno"][-1, 100] *= 1.0 + 1e-7
    gate, _, _ = bench.soil_gate(A, npatch, G, 3, bad, zero, True, sensitivity_runs=1)
    assert not gate["pass"] and gate["one_step_from_evolved_state"]["columns_above_tol"] == 1
    assert gate["one_step_from_evolved_state"]["max_rel_err"]["t_soisno"] > 5e-8
    bad = copy.deepcopy(G1)
    bad["xmf"][:] = bad["xmf"] * (1.0 + 1e-6) + 1.0
    gate, _, _ = bench.soil_gate(A, npatch, G, 3, bad, zero, True, sensitivity_runs=1)
    assert not gate["pass"] and gate["one_step_from_evolved_state"]["max_rel_err"]["xmf (conditioned)"] > 1e-9
    assert gate["one_step_from_evolved_state"]["band_use"]["xmf"]["columns_above_tol_without_band"] > 0
    over = (np.full(512, 2e-5), np.zeros(512))
    gate, _, _ = bench.soil_gate(A, npatch, G, 3, G1, over, True, sensitivity_runs=1)
    assert not gate["pass"] and gate["balance"]["columns_above_stop"] == 512
