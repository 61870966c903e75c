"""Host logic of the multi-GPU path: independent replicas.

Images are independent units of the --find_obj path (findObjectDataset,
libPictStruct/objectdetect_aux.cpp:322-406, loops over images with no
exchange between them; --distribute splits the image range over jobs,
apps/partapp/main.cpp:355-400).  On N GPUs every rank processes its own
contiguous range of images; the only communication is the timing reduction
(max over ranks) and an optional gather of results on rank 0.  No collective
touches the data path.
"""
from __future__ import annotations


def image_range(n_images: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [first, last) image range of `rank`: the first
    n_images % world ranks get one extra image (the --first/--numimgs split
    of a distributed run)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    base, extra = divmod(max(0, n_images), world)
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Max of a per-rank scalar (the timed region's duration) over ranks."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device=None) -> float:
    """Sum of a per-rank count (images processed) over ranks."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def throughput(images_all_ranks: float, ms_max: float) -> float:
    """Whole-job images/s: images of all ranks over the slowest rank's time."""
    if ms_max <= 0:
        raise ValueError("non-positive duration")
    return images_all_ranks / (ms_max / 1e3)


def gather_results(obj, dist=None):
    """Rank 0 receives every rank's picklable result list (None elsewhere)."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return [obj]
    world = dist.get_world_size()
    out = [None] * world if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
