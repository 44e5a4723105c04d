"""The multi-rank path of bench.py on CPU (gloo, two ranks): every rank
renders its own replica of the workload, the job's time is the slowest
rank's (one all-reduce, no data exchange), and the reference arm runs on
rank 0 alone."""
import argparse
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.dist_setup()
    # rank 1 is the slower replica
    total_ms = bench.max_over_ranks(10.0 + 2.0 * r, w)
    value = bench.job_throughput(w, 2_097_152, 4, total_ms)
    dist.barrier()
    q.put((r, w, local, total_ms, value))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 and o[2] == o[0] for o in out)
    for _, _, _, total_ms, value in out:
        assert total_ms == 12.0
        assert abs(value - 2 * 2_097_152 * 4 / 0.012 / 1e6) < 1e-6


def test_single_rank_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert abs(bench.job_throughput(1, 1000, 10, 5.0) - 2.0) < 1e-12


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(workload="sphere", steps=1, warmup=3)
    assert bench.run_reference(args, 2, 1) == 0
    assert capsys.readouterr().out == ""


def test_reference_arm_line_keeps_the_contract(capsys):
    """The reference arm's one JSON line on rank 0: the metric of the GPU arm,
    the CPU implementation timed (the oracle port here), e2e without copies."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(workload="sphere", steps=2, warmup=3)
    assert bench.run_reference(args, 1, 0) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == "Mtris/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"] == "sphere"
