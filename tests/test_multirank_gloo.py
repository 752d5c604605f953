"""The N > 1 path on CPU: two gloo ranks, as torchrun launches bench.py on two GPUs.

The path shards by storm: ranks are independent replicas with their own storms or
requests, and the only communication is the barrier and the max-over-ranks of the
timed region.  Two processes (spawned) check the rank set-up, the reduction, that the
ranks' batches share no storm, and that the request shards partition the stream.
"""
import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    from his_gb300.serving import shard_requests
    try:
        w, r, _ = bench.dist_init(backend="gloo")
        bench.barrier(w)
        slowest = bench.max_over_ranks(1.5 * (r + 1), w)
        keys = [s.key for s in bench.rank_storms(3, r)]
        shard = shard_requests(list(range(11)), r, w)
        q.put((r, w, slowest, keys, shard))
        bench.barrier(w)
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_two_gloo_ranks_are_independent_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 3.0 for o in out)                       # max over ranks of 1.5, 3.0
    k0, k1 = set(out[0][3]), set(out[1][3])
    assert len(k0) == len(k1) == 3 and not (k0 & k1)            # no storm runs on both ranks
    s0, s1 = out[0][4], out[1][4]
    assert sorted(s0 + s1) == list(range(11)) and not set(s0) & set(s1)
