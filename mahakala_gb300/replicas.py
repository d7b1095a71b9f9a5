"""Multi-GPU form: independent replicas.

Rays are independent and the snapshot is read-only, so N GPUs either render
N images or split one image's rays into N contiguous ranges; the only
exchange is the final timing (and, for a split image, a gather of pixel
ranges).  These helpers work with any torch.distributed backend (NCCL on
GPUs, gloo in the CPU tests)."""

import torch


def ray_range(total, rank, world):
    """[start, stop) of the rays rank `rank` of `world` renders."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(total), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(value, device="cpu"):
    """The largest value over all ranks (1 rank: the value itself)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_ranges(local, total, device="cpu"):
    """Concatenate every rank's slice (ray_range order) into the full
    1-D array of `total` entries on every rank."""
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_initialized() else 1
    if world == 1:
        return local
    sizes = [ray_range(total, r, world) for r in range(world)]
    width = max(b - a for a, b in sizes)
    buf = torch.zeros(width, dtype=local.dtype, device=device)
    buf[: local.numel()] = local.to(device)
    parts = [torch.zeros(width, dtype=local.dtype, device=device) for _ in range(world)]
    dist.all_gather(parts, buf)
    return torch.cat([p[: b - a] for p, (a, b) in zip(parts, sizes)])
