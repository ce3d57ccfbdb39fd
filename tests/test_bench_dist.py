"""bench.py's multi-rank bookkeeping on CPU: two gloo ranks, the timing reduction
is the max over ranks and the update count the sum (weak scaling, independent
domains), and the reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out: str) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist = bench.init_dist(world)
    assert dist.get_backend() == "gloo"
    t = bench.reduce_max(dist, 1.0 + rank)
    s = bench.reduce_sum(dist, 10.0 * (rank + 1))
    bench.barrier(dist)
    Path(out, f"r{rank}").write_text(f"{t} {s}")
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the gloo path is the CPU-only configuration")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in (0, 1):
        t, s = (float(v) for v in (tmp_path / f"r{r}").read_text().split())
        assert t == 2.0 and s == 30.0


def test_reference_arm_prints_on_rank_zero_only(tmp_path):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
