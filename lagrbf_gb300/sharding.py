"""Particle sharding over ranks, one GPU per rank.

Particles are independent once the patch coefficients exist, so N ranks each hold the whole
dataset (data swarm, patch set-ups) and a contiguous range of the particle swarm, advance it with
no exchange of particle data, and assemble results by pid once at the end.  The assembly is the
single-collective analogue of AssembleArray_Allreduce (src/interface/interface_utils.c:188-263):
every rank writes its rows at pid - 1 of a zero array of nglobal rows and one SUM all-reduce
combines them; rows of particles that left the domain stay zero, as lagrbf_output leaves them.

Two scalars couple the ranks in the reference's algorithm: the CFL step is a global minimum over all
particles (src/advection/advection.c:466) and the Dormand-Prince error a global maximum
(src/advection/dormand_prince.c:93).  step_reducer() turns an all-reduce of the caller's
communication library into the per-step coupling of LagRBFCtx.set_step_reduce (8 bytes each way
per internal step), after which sharded runs take the single-rank steps for any outer interval.

The reference decomposes space instead (DMDA halo + per-stage migration); that is needed only when
the coefficients outgrow one device, which the 280 GB HBM of one GPU does not approach here.  This
module uses numpy only; the communication is the caller's (MPI, torch.distributed, ...).
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


def assemble_by_pid(nglobal, local_values, local_pid, allreduce_sum=None):
    """Global [nglobal, ncomp] array from every rank's rows (pid 0 = absent row, skipped).
    allreduce_sum(array) returns the element-wise sum of array over the ranks (None: one rank)."""
    local_values = np.asarray(local_values, dtype=np.float64)
    ncomp = local_values.shape[1] if local_values.ndim == 2 else 1
    out = np.zeros((nglobal, ncomp))
    pid = np.asarray(local_pid, dtype=np.int64)
    keep = pid > 0
    if np.any(pid[keep] > nglobal):
        raise ValueError("pid beyond nglobal")
    out[pid[keep] - 1] = local_values.reshape(len(pid), ncomp)[keep]
    if allreduce_sum is not None:
        out = np.asarray(allreduce_sum(out), dtype=np.float64).reshape(nglobal, ncomp)
    return out


def step_reducer(allreduce_max):
    """The coupling function of LagRBFCtx.set_step_reduce from allreduce_max(array) -> the
    element-wise maximum of array over the ranks."""
    def fn(vals):
        vals[:] = np.asarray(allreduce_max(np.array(vals, dtype=np.float64)), dtype=np.float64)
    return fn
