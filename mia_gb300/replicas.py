"""Replica runs on several GPUs of one node: one process per GPU, each
working on its own pairs (the pairs are independent, so the data path has
no collective).  Only the timing crosses ranks: a barrier on both sides of
the timed region and the maximum of the ranks' step times, from which the
whole-job rate is the units all ranks processed divided by that time.

The launcher (torchrun) sets RANK / LOCAL_RANK / WORLD_SIZE / MASTER_*;
the process group is NCCL when CUDA is present, gloo otherwise (the CPU
tests run two gloo ranks).
"""
import os


def env():
    """(world_size, rank, local_rank) from the launcher's environment"""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend=None):
    """join the process group when there is more than one rank; returns
    world_size"""
    ws, _, _ = env()
    if ws > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend or ("nccl" if torch.cuda.is_available() else "gloo"))
    return ws


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(value, device=None):
    """the maximum of a float over all ranks (the value itself on one rank)"""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, seconds_per_rank, world_size, device=None):
    """units of all ranks over the slowest rank's time (weak scaling: every
    rank processes units_per_rank)"""
    t = max_over_ranks(seconds_per_rank, device)
    return world_size * units_per_rank / t, t
