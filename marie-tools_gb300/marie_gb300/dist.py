"""Multi-GPU layout of the solve: replicas over independent right-hand sides.

The VIE system of one body is solved on one GPU; independent right-hand
sides (coil ports) and independent bodies shard across ranks with no
collective on the data path (ie_solver_vie.m:16-21 solves ports
independently).  Ranks only agree on the shard boundaries and reduce the
timing (max over ranks) and the small per-rhs reports at the end.
"""
from __future__ import annotations


def shard_rhs(n_global: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced [start, stop) of the global right-hand sides owned
    by `rank`; the shards of all ranks partition range(n_global)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("invalid rank/world")
    base, extra = divmod(n_global, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, group=None) -> float:
    """Max of a scalar over ranks (the timing rule of the benchmark)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_counts(local: list[int], group=None) -> list[int]:
    """Concatenate small per-rank integer lists (e.g. iterations per rhs) in
    rank order."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return list(local)
    world = dist.get_world_size(group)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    n = torch.tensor([len(local)], device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(int(s.item()) for s in sizes))
    buf = torch.zeros(mx, dtype=torch.int64, device=dev)
    buf[: len(local)] = torch.tensor(local, dtype=torch.int64)
    outs = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(outs, buf, group=group)
    res = []
    for o, s in zip(outs, sizes):
        res.extend(int(v) for v in o[: int(s.item())].tolist())
    return res
