"""The N > 1 host logic of bench.py on the CPU: two ranks over gloo (the GPU
runs use NCCL with the same calls).  The path shards by shot with no data
exchange, so the only collectives are the barrier and the max-over-ranks
timing; each rank runs its own shot(s), and only rank 0 prints."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import __graft_entry__ as ge
    import bench
    ge.package()  # the package under its import name (geometry helpers)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    geom = bench.geometry(64)
    src = bench.shot_source(geom, r)
    shots = bench.batch_shots(4, bench.BATCH_SEED + r)
    ms = bench.max_over_ranks(10.0 + 5.0 * r, dist, "cpu")  # rank 1 is the slowest
    rate = bench.weak_rate(geom.compute_points, 100, w, ms)
    dist.barrier()
    out.put((r, w, local, src, shots[0]["src"], ms, rate))
    dist.destroy_process_group()


def test_two_ranks_shard_by_shot_and_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, src0, bsrc0, ms0, rate0), (r1, w1, l1, src1, bsrc1, ms1, rate1) = got
    assert (r0, r1) == (0, 1) and w0 == w1 == 2 and (l0, l1) == (0, 1)
    assert src0 != src1 and bsrc0 != bsrc1          # independent shots per rank
    assert ms0 == ms1 == 15.0                       # the slowest rank's time
    assert rate0 == rate1
    # weak scaling: the whole job did twice the single-rank work in that time
    # (a 64^3 interior + 48-cell sponge updates 160^3 points per step)
    import bench  # noqa: E402  (the test process has the repo root on sys.path)
    assert rate0 == pytest.approx(2 * bench.weak_rate(160 ** 3, 100, 1,
                                                      15.0))


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0 and p.stdout.strip() == ""
