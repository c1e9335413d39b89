"""Independent replicas across processes/GPUs and the merge of their tallies.

The transport path has no exchange step: histories are independent, so N
ranks simulate disjoint history ranges (disjoint Philox counters) and the
only collective is the final sum of the float64 images and of the number of
samples - the merge the reference performs on files after split runs
(opengate/actors/dataitems.py:1238-1247, 249-277: images added, number of
samples summed).
"""

import numpy as np


def history_range(rank, world_size, n_total, first=0):
    """[begin, end) of the histories rank ``rank`` simulates out of ``n_total``."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("invalid rank / world size")
    per = n_total // world_size
    extra = n_total % world_size
    begin = first + rank * per + min(rank, extra)
    end = begin + per + (1 if rank < extra else 0)
    return begin, end


class _DeviceImage:
    """A library-owned FP64 device image as a CUDA array (zero copy)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def merge_tallies_device(engine, which, n_samples, group=None):
    """In-place sum over all ranks of an engine's FP64 device images (NCCL
    all_reduce on the library's own buffers, no host round trip) and of the
    sample count; afterwards every rank's engine.image(...) returns the merged
    image.  ``which``: the GG_IMG_* kinds to merge.  Without torch.distributed
    initialised this is a no-op."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return int(n_samples)
    if dist.get_backend(group) != "nccl":
        raise RuntimeError("merge_tallies_device needs the nccl backend (merge_tallies merges host images)")
    dev = torch.device("cuda", torch.cuda.current_device())
    for w in which:
        ptr, n = engine.image_device(w)
        t = torch.as_tensor(_DeviceImage(ptr, n), device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    cnt = torch.tensor([int(n_samples)], dtype=torch.int64, device=dev)
    dist.all_reduce(cnt, op=dist.ReduceOp.SUM, group=group)
    torch.cuda.synchronize(dev)
    return int(cnt.item())


def merge_tallies(images, n_samples, group=None):
    """Sums float64 images and the sample count over all ranks (all_reduce SUM).

    ``images`` is a list of numpy arrays; returns (list of summed arrays, total
    samples).  Without torch.distributed initialised this is the identity.
    """
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return [np.asarray(im, dtype=np.float64) for im in images], int(n_samples)
    backend = dist.get_backend(group)
    device = "cuda" if backend == "nccl" else "cpu"
    out = []
    for im in images:
        t = torch.from_numpy(np.ascontiguousarray(im, dtype=np.float64)).to(device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out.append(t.cpu().numpy())
    n = torch.tensor([int(n_samples)], dtype=torch.int64, device=device)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    return out, int(n.item())
