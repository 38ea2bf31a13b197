"""One process per GPU: rank discovery, the split of tiles between ranks, and the
job-wide timing reduction.

Every (tile, input vector) solve is independent, so ranks exchange no data on
the solve path: each rank solves its own tiles and only the elapsed time is
combined -- the job takes as long as its slowest rank (max over ranks), and its
rate counts the solves of every rank.  The reference runs one process on one
device (pimtorch/pimfixedpoint/fixedPoint/nn/commonConst.py:273-280 builds a
single CUDA extension); a layer's tiles (the numX axis of ir_drop_gs,
split_arr_matmul.cu:204-220) are the natural unit to spread over several.
"""
import os


def rank_env():
    """(rank, world_size, local_rank) from the launcher's environment (torchrun)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_seed(base, rank):
    """Seed of a rank's own synthetic tiles (weak scaling: every rank a new set)."""
    return base + rank


def split_tiles(total, rank, world):
    """[lo, hi) of the numX range a rank solves when a fixed set of tiles is
    shared (strong scaling): contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside world of %d" % (rank, world))
    base, extra = divmod(total, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest of every rank's value (all ranks get it); ``dist`` is
    torch.distributed after init_process_group, or None for one process."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Units per second of the whole job: every rank's units over the slowest
    rank's time (``ms``, already the max over ranks)."""
    return units_per_rank * world / (ms / 1e3)
