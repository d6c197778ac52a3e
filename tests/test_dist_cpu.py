"""The replica path of bench.py for N > 1 GPUs (one process per GPU, no
collective on the data path): world size 2 over gloo on the CPU. Each rank
pins its own device, the step times are reduced with a max over ranks and
the barrier lines the ranks up, as the benchmark does around its timed
region."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import os, sys
sys.path.insert(0, os.environ["CEOS_ROOT"])
import bench
ws, rank, dist = bench.dist_setup()
assert os.environ["CUDA_VISIBLE_DEVICES"] == os.environ["LOCAL_RANK"]
bench.barrier(dist)
t = bench.max_over_ranks(dist, 1.5 + rank)
print(f"rank {rank} of {ws}: max {t}", flush=True)
assert t == 2.5
dist.destroy_process_group()
'''


def test_replicas_gloo_world_size_2(tmp_path):
    pytest.importorskip("torch")
    script = tmp_path / "replicas.py"
    script.write_text(SCRIPT)
    env = dict(os.environ, CEOS_ROOT=ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=29533", str(script)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=240)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "rank 0 of 2: max 2.5" in r.stdout and "rank 1 of 2: max 2.5" in r.stdout
