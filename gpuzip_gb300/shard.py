"""Multi-GPU form of the batched and served workloads: replicas that share nothing. Independent
streams are assigned to ranks largest first, each to the rank holding the fewest bytes so far, so
every rank decodes its own share with no exchange during the decode; the job's time is the
slowest rank's (a max over ranks after a barrier)."""
import heapq


def shard_streams(sizes, world_size):
    """Stream indices per rank (ascending within a rank): largest stream first, each to the rank
    with the fewest bytes so far (ties: the lower rank)."""
    if world_size < 1:
        raise ValueError("world_size must be at least 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(world_size)]
    shares = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + sizes[i], r))
    return [sorted(s) for s in shares]


def max_over_ranks(value, device="cpu"):
    """`value` (seconds) maximised over the ranks of the default process group (itself when
    torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
