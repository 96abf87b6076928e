"""Replica execution over ranks (one process per GPU).

The geometry path shards with no data exchange: views and AOIs are independent for the
projection, the fit and the rasterisation, and the fusion is per AOI.  Each rank runs its
own share of AOIs on its own GPU; the only collectives are the timing barrier and the
max-over-ranks of the elapsed time (and sums of the work counters) that a whole-job
throughput needs.  The process group is NCCL on GPUs and gloo on CPU.
"""
import os

import torch
import torch.distributed as dist


def rank_info():
    """(rank, world_size, local_rank) from the torchrun environment (defaults: one process)."""
    return (int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1')),
            int(os.environ.get('LOCAL_RANK', '0')))


def init(backend=None):
    """Join the process group when world_size > 1; returns (rank, world, local_rank)."""
    rank, world, local = rank_info()
    if world > 1 and not dist.is_initialized():
        if backend is None:
            backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if backend == 'nccl':
            dist.init_process_group('nccl', device_id=torch.device(f'cuda:{local}'))
        else:
            dist.init_process_group(backend)
    return rank, world, local


def shard_balanced(costs, world):
    """Indices of items per rank, balancing the summed cost (largest first onto the least
    loaded rank); every item lands on exactly one rank, each list in ascending order."""
    loads = [0.0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (loads[q], q))
        out[r].append(i)
        loads[r] += costs[i]
    return [sorted(o) for o in out]


def _reduce(value, op, device):
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value, device='cpu'):
    return _reduce(value, dist.ReduceOp.MAX, device)


def sum_over_ranks(value, device='cpu'):
    return _reduce(value, dist.ReduceOp.SUM, device)


def barrier():
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def job_throughput(units_this_rank, elapsed_this_rank, device='cpu'):
    """Whole-job rate: the units all ranks processed over the slowest rank's time."""
    return sum_over_ranks(units_this_rank, device) / max_over_ranks(elapsed_this_rank, device)


def finish():
    if dist.is_initialized():
        dist.destroy_process_group()
