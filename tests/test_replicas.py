"""The N>1 path of bench.py on CPU: independent replicas over gloo
(world_size 2).  Ranks exchange only the barrier and the max/sum of their
timings and counts; nothing on the data path."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(world)
    d.barrier()
    res = {"max": d.max(float(rank + 1) * 1.5), "sum": d.sum(float(10 * (rank + 1)))}
    d.barrier()
    d.close()
    (Path(out_dir) / f"rank{rank}.json").write_text(json.dumps(res))


def test_dist_barrier_max_sum_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        res = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert res == {"max": 3.0, "sum": 30.0}


def test_reference_arm_prints_one_line_from_rank0_only(tmp_path):
    lib = ROOT / "trinityrnaseq_gb300" / "lib" / "libtrinkmer_synth.so"
    if not lib.exists():
        pytest.skip("synthetic-input library not built")
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--cpu-pairs", "2000"]
    p = subprocess.run(cmd, cwd=tmp_path, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port" and out["e2e"]["h2d_bytes_per_step"] == 0
