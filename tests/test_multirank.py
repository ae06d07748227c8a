"""World-size-2 gloo checks of the replicas-only multi-GPU layout (CPU)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from marie_gb300.dist import shard_rhs, max_over_ranks, gather_counts  # noqa: E402


def test_shards_partition():
    for n in (0, 1, 7, 64, 65):
        for w in (1, 2, 3, 8):
            got = []
            for r in range(w):
                a, b = shard_rhs(n, r, w)
                assert 0 <= a <= b <= n
                got.extend(range(a, b))
            assert got == list(range(n))
    with pytest.raises(ValueError):
        shard_rhs(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        a, b = shard_rhs(10, rank, world)
        t = max_over_ranks(1.5 + rank)
        iters = gather_counts([rank * 100 + i for i in range(b - a)])
        q.put((rank, a, b, t, iters))
    finally:
        dist.destroy_process_group()


def test_gloo_world2_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a0, b0, t0, it0), (r1, a1, b1, t1, it1) = res
    assert (a0, b0, a1, b1) == (0, 5, 5, 10)
    assert t0 == t1 == 2.5                           # max over ranks
    assert it0 == it1 == [0, 1, 2, 3, 4, 100, 101, 102, 103, 104]


def _failing_worker(rank, world, port, q):
    """Rank 1 raises before the collective: rank 0's collective must end with
    an error after the process-group timeout, not hang."""
    import datetime
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=5))
    if rank == 1:
        q.put((rank, "raised"))
        q.close()
        q.join_thread()
        os._exit(3)
    try:
        max_over_ranks(1.0)
        q.put((rank, "no error"))
    except Exception as e:  # noqa: BLE001
        q.put((rank, "error: " + type(e).__name__))


def test_gloo_rank_failure_is_detected():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res[1] == "raised"
    assert res[0].startswith("error")
