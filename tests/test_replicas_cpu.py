"""N > 1 without GPUs: the bench's replica aggregation over a gloo process
group (world size 2), and the reference arm launched under torchrun, where
rank 0 alone measures and prints."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank  # each replica's own timing
    m = bench.reduce_max_ms(ms, dist, "cpu")
    v = bench.aggregate_gst(1_000_000, 4, m, world)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"ms": m, "value": v}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    for r in res:
        assert r["ms"] == 150.0
        # both replicas' points over the slowest replica's time
        assert r["value"] == pytest.approx(2 * 1_000_000 * 4 / 0.150 / 1e9)


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--side", "24", "--iters", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
