"""Ray sharding across ranks.

A ray query depends only on the ray, the two BVHs and the network parameters, so a multi-GPU job
partitions the rays across ranks and runs one independent query per rank: there is no collective
on the data path. The reference renders on one GPU; its wavefront (src/cuda/neural/path/path_module.cu:54-137)
has no cross-ray exchange either, so the shards' results concatenate to the unsharded result.

The only cross-rank step is the reduction of a benchmark's timing (the slowest rank).
"""


def shard_bounds(n, rank, world):
    """[start, end) of rank's contiguous share of n rays; shares differ by at most one ray."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, rem = divmod(int(n), int(world))
    start = rank * base + min(rank, rem)
    return start, start + base + (1 if rank < rem else 0)


def shard(rays, rank, world):
    """The rows of rays (any array with rays along axis 0) that rank answers."""
    s, e = shard_bounds(len(rays), rank, world)
    return rays[s:e]


def max_over_ranks(values, group=None):
    """Element-wise maximum of a list of floats over the ranks of a torch.distributed group.

    Runs on whatever device the backend wants (CPU tensors for gloo, the current CUDA device for
    NCCL); returns the input unchanged when torch.distributed is not initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [float(v) for v in values]
    device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return [float(v) for v in t.cpu()]
