"""CPU tests of the benchmark's multi-rank host logic (replicas, one process
per GPU): two gloo ranks on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
import bench
rank, world, local = bench.dist_env()
dist.init_process_group("gloo", rank=rank, world_size=world)
slowest = bench.max_over_ranks(1.5 + rank)      # rank 1 is the slow one
dist.barrier()
dist.destroy_process_group()
print(json.dumps({"rank": rank, "world": world, "local": local, "max": slowest}))
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_with_two_gloo_ranks(tmp_path):
    """Each rank reports its own time; every rank gets the slowest one."""
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    port = str(_free_port())
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port, CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script), ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert all(o["world"] == 2 and o["local"] == o["rank"] for o in outs)
    assert all(o["max"] == 2.5 for o in outs)


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit at once, printing
    nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
