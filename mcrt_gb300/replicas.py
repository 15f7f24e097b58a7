"""One render replica per GPU (the path does not shard: pixels, samples and views
are independent, so there is no exchange during rendering).

A launcher such as torchrun starts one process per GPU; each renders its own
frames.  The only distributed operations are a barrier around timed regions
and reductions of per-rank figures: the maximum step time and the total
number of samples.  ``split_rows`` divides the rows of one image among ranks
for callers that want one image rendered by several GPUs (each rank renders
its rows, the host concatenates them; no device-to-device traffic).
"""
from __future__ import annotations

import os


def env_ranks():
    """(rank, world_size, local_rank) from the launcher's environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init(backend: str = "nccl", device_index: int | None = None):
    import torch
    import torch.distributed as dist
    rank, world, local = env_ranks()
    if world > 1 and not dist.is_initialized():
        if backend == "nccl":
            torch.cuda.set_device(local if device_index is None else device_index)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
    return rank, world, local


def _tensor(x, device):
    import torch
    return torch.tensor([float(x)], dtype=torch.float64, device=device)


def max_over_ranks(x: float, device="cpu") -> float:
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, device="cpu") -> float:
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = _tensor(x, device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def split_rows(height: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous row range [y0, y1) of `rank`; ranges cover [0, height) exactly once."""
    base, extra = divmod(height, world)
    y0 = rank * base + min(rank, extra)
    return y0, y0 + base + (1 if rank < extra else 0)
