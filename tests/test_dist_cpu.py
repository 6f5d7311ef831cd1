"""The multi-process (replicas) path of bench.py on CPU: world size 2 over
gloo, launched the way torchrun would (RANK / WORLD_SIZE / MASTER_* in the
environment, 127.0.0.1)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
world, rank, local, dist = bench.dist_setup(2, backend="gloo")
bench.barrier(dist, world)
ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, world)     # per-rank timings
bench.barrier(dist, world)
print(json.dumps({{"rank": rank, "world": world, "local": local, "max_ms": ms}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch(code, world, extra_env=None, args=()):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        env.update(extra_env or {})
        cmd = [sys.executable, "-c", code] if code else [sys.executable, *args]
        procs.append(subprocess.Popen(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_replica_timing_is_the_max_over_ranks():
    outs = launch(CHILD.format(root=ROOT), 2)
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o in outs), key=lambda d: d["rank"])
    assert [d["rank"] for d in res] == [0, 1] and all(d["world"] == 2 for d in res)
    assert all(d["max_ms"] == 15.0 for d in res)


def test_reference_arm_runs_on_rank_0_only():
    # rank 1 of a 2-rank reference run exits 0 without output or a process group
    outs = launch(None, 1, extra_env={"WORLD_SIZE": "2", "RANK": "1"},
                  args=("bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"))
    assert outs[0].strip() == ""
