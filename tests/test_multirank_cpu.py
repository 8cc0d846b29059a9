"""The N>1 path of bench.py on CPU: two gloo ranks.  The path tracer shards
as replicas (each rank renders its own frames), so the only cross-rank step
is the final aggregation: the slowest rank's time and the sum of the work.
The reference arm must do nothing on ranks other than 0."""

import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank = int(os.environ["RANK"]); world = int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", rank=rank, world_size=world)
t, p, r = bench.aggregate_ranks(100.0 + 50.0 * rank, 1000 * (rank + 1), 3000 * (rank + 1), world)
print(json.dumps({{"rank": rank, "t": t, "paths": p, "rays": r}}), flush=True)
dist.destroy_process_group()
"""


def _launch(code, world=2, extra_env=None):
    port = _free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_two_rank_aggregation_gloo():
    import json

    outs = _launch(WORKER.format(root=ROOT))
    res = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    for r in res:
        assert r["t"] == 150.0          # slowest rank
        assert r["paths"] == 3000.0     # 1000 + 2000
        assert r["rays"] == 9000.0


def test_reference_arm_other_ranks_exit_without_work():
    code = ("import sys; sys.path.insert(0, %r); sys.argv = ['bench.py', '--impl', 'reference', "
            "'--steps', '1', '--warmup', '0']; import bench; sys.exit(bench.main())" % ROOT)
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_cpu_tile_samples_are_whole_waves_spread_over_the_frame():
    """The CPU legs (cpu_baseline and --impl reference) time the same sample:
    distinct tile ids spread over the whole frame in row-major order, as many
    tiles as the work target asks for, rounded up to whole waves of threads."""
    sys.path.insert(0, ROOT)
    import bench

    total = 30 * 17  # 64x64 tiles of a 1920x1080 frame
    for n in (1, 16, 48, 112, 509, 510, 600):
        ids = bench.spread_tiles(total, n)
        assert len(ids) == min(n, total) == len(set(ids))
        assert ids == sorted(ids) and 0 <= ids[0] and ids[-1] < total
        if len(ids) > 1:
            gaps = [b - a for a, b in zip(ids, ids[1:])]
            assert max(gaps) - min(gaps) <= 1
    for per_tile, target, threads in ((0.7, 12.0, 16), (0.7, 4.0, 16), (0.05, 12.0, 16),
                                      (3.0, 1.0, 8), (1e-9, 12.0, 16)):
        n = bench.cpu_tile_count(per_tile, target, threads, total)
        assert 1 <= n <= total
        assert n == total or n % threads == 0
        assert n == total or n * per_tile / threads >= target * 0.999 or n == threads
