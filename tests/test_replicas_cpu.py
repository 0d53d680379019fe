"""CPU tests of bench.py's replica path (gloo, world size 2) and of its reference arm.

The column ID does not shard: every rank runs its own matrix or batch, and
the only collective is the max of the ranks' times.  These tests run that
rank logic over gloo on the host: the barrier, the max over ranks, the
whole-job rate, per-rank seeding of the workloads, the reference arm's
rank-0-only rule, and the reference arm's JSON line (one short step).
"""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    ctx = bench.Ctx(None, device_type="cpu")
    ctx.barrier()
    local_ms = 100.0 * (rank + 1)                      # rank 1 is the slow one
    got_max = ctx.max_over_ranks(local_ms)
    value, ms_max = ctx.job_rate(8, local_ms)
    # the batched workload of this rank (small): seeded by the rank
    blocks = W.kernel_blocks_device(4, 16, 48, 0.5, ctx.rank, "cpu")
    shapes = [tuple(A.shape) for A in blocks]
    sums = [float(A.double().sum()) for A in blocks]
    ctx.barrier()
    ctx.close()
    with open(os.path.join(out, f"rank{rank}.json"), "w") as f:
        json.dump(dict(max=got_max, value=value, ms_max=ms_max, shapes=shapes, sums=sums), f)


def test_two_rank_replicas_over_gloo(tmp_path):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["max"] == pytest.approx(200.0)
        assert r["ms_max"] == pytest.approx(200.0)
        # 2 ranks x 8 units over the slowest rank's 0.2 s
        assert r["value"] == pytest.approx(world * 8 / 0.2)
    # independent replicas: each rank's problem set differs from the other's ...
    assert res[0]["shapes"] != res[1]["shapes"] or res[0]["sums"] != res[1]["sums"]
    # ... and equals what the same seed gives in one process
    sys.path.insert(0, ROOT)
    from robust_blockwise_random_pivoting_gb300 import workloads as W
    for rank in range(world):
        shapes = W.kernel_block_shapes(4, 16, 48, rank)
        assert [tuple(s) for s in shapes.tolist()] == [tuple(s) for s in res[rank]["shapes"]]
        ref = [float(W.kernel_block_scaled(int(m), int(n), q, 0.5, rank, np.float32).astype(np.float64).sum())
               for q, (m, n) in enumerate(shapes)]
        np.testing.assert_allclose(res[rank]["sums"], ref, rtol=1e-5)


def _bench(args, rank, world=2):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, env=env,
                          capture_output=True, text=True, timeout=120)


@pytest.mark.parametrize("workload", ["blocks4096", "snn16k"])
def test_reference_arm_runs_on_rank_zero_only(workload):
    """Under torchrun the reference arm's other ranks exit 0 without work or output."""
    p = _bench(["--impl", "reference", "--gpus", "2", "--workload", workload], rank=1)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


@pytest.mark.parametrize("workload", ["adjoint8k", "idcmp16k", "cpqr16k"])
def test_reference_arm_unavailable_lines(workload):
    p = _bench(["--impl", "reference", "--workload", workload], rank=0)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unavailable"]


@pytest.mark.parametrize("workload", ["blocks4096", "gexp1000"])
def test_reference_arm_line_on_cpu(workload):
    """The reference arm (the oracle port on the host cores) prints one complete JSON line."""
    p = _bench(["--impl", "reference", "--workload", workload, "--steps", "1", "--warmup", "0"], rank=0, world=1)
    assert p.returncode == 0, p.stderr
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "matrices/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "matrices/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"].startswith(workload)
