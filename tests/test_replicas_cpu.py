"""The N>1 replica path of bench.py with two gloo ranks on the CPU.

The path does not shard: every rank runs its own replica and the ranks meet
only in barriers and in the max-over-ranks of the timed region.  These tests
run that host logic with world_size 2 (no GPU): the rendezvous on
127.0.0.1, the barrier, the max-reduce, and torchrun launching the reference
arm, where rank 0 alone prints the JSON line.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(10.0 + rank)  # each rank's "elapsed ms"
    d.barrier()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"rank": d.rank, "ws": d.ws, "max": m}, f)
    d.close()


def test_dist_barrier_and_max_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank_main, args=(r, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1]
    assert all(x["ws"] == 2 for x in res)
    # the timed region of the job is the slowest rank's
    assert all(x["max"] == 11.0 for x in res)


def test_torchrun_reference_arm_prints_one_line_from_rank0():
    pytest.importorskip("torch")
    from oracle.build import build_oracle
    build_oracle()
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--workload", "ch2d-128", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["unit"] == "steps/s"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
