"""The multi-rank path of bench.py on the CPU: two ranks over gloo (127.0.0.1).
Chains are independent, so ranks share no data: each rank builds its own chain
mix (weak scaling) and the only collectives are the timing barrier, the max of
the per-rank times and the sum of the per-rank work.  The reference arm runs on
rank 0 alone; the other ranks return without work."""
import multiprocessing as mp
import os
import socket
import sys
import types

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    try:
        import bench
        d = bench.Dist(world)
        d.barrier()
        mx = d.max(float(rank + 1))
        sm = d.sum(float(10 * (rank + 1)))
        args = types.SimpleNamespace(workload="batched", chains=8, steps=1, warmup=3, gpus=world)
        specs, _ = bench.build_specs(args, d.rank)
        ref = bench.run_reference(args, d) if rank != 0 else "rank0-skipped"
        q.put((rank, mx, sm, [(s.n, s.chi, round(float(s.p[0]), 12)) for s in specs], ref))
        d.pg.destroy_process_group()
    except Exception as e:  # report to the parent instead of hanging it
        q.put((rank, "error", repr(e), None, None))


def test_two_ranks_share_only_timing_collectives():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        r = q.get(timeout=120)
        out[r[0]] = r
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        assert out[r][1] != "error", out[r][2]
        assert out[r][1] == 2.0  # max over ranks of the per-rank time
        assert out[r][2] == 30.0  # sum over ranks of the per-rank work
    # weak scaling: the same number of chains per rank, different chains
    assert len(out[0][3]) == len(out[1][3]) == 8
    assert out[0][3] != out[1][3]
    # reference arm: rank 1 returns without work
    assert out[1][4] is None
