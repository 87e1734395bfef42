"""Particle sharding over ranks, one GPU per rank.

Particles are independent once the patch coefficients exist, so N ranks each hold the whole
dataset (data swarm, patch set-ups) and a contiguous range of the particle swarm, advance it with
no exchange, and assemble results by pid once at the end.  The assembly is the single-collective
analogue of AssembleArray_Allreduce (src/interface/interface_utils.c:188-263): every rank writes
its rows at pid - 1 of a zero array of nglobal rows and one SUM all-reduce combines them; rows of
particles that left the domain stay zero, as lagrbf_output leaves them.

The reference decomposes space instead (DMDA halo + per-stage migration); that is needed only when
the coefficients outgrow one device, which the 280 GB HBM of one GPU does not approach here.
"""
import numpy as np


def shard_range(nglobal, rank, world):
    """[start, end) of rank's particles: contiguous, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    base, extra = divmod(int(nglobal), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(coords, rank, world):
    """Rank's particles and their global 1-based pids (the pidx argument of lagrbf_fill_swarm)."""
    start, end = shard_range(len(coords), rank, world)
    return np.ascontiguousarray(coords[start:end]), np.arange(start + 1, end + 1, dtype=np.int64)


def assemble_by_pid(nglobal, local_values, local_pid, group=None, device="cpu"):
    """Global [nglobal, ncomp] array from every rank's rows (pid 0 = absent row, skipped)."""
    import torch
    import torch.distributed as dist

    local_values = np.asarray(local_values, dtype=np.float64)
    ncomp = local_values.shape[1] if local_values.ndim == 2 else 1
    out = np.zeros((nglobal, ncomp))
    pid = np.asarray(local_pid, dtype=np.int64)
    keep = pid > 0
    if np.any(pid[keep] > nglobal):
        raise ValueError("pid beyond nglobal")
    out[pid[keep] - 1] = local_values.reshape(len(pid), ncomp)[keep]
    t = torch.from_numpy(out).to(device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()
