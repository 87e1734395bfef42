"""Particle sharding with two CPU ranks (gloo): each rank advances its pid range with the oracle as
the compute engine, results are assembled by pid with one all-reduce, and the assembly equals the
single-rank run bit for bit (particles are independent; dropped particles leave zero rows).

Two cases: outer intervals shorter than the CFL step (lagrbfpy's own loops: every rank takes the
same internal step without coupling), and intervals of several CFL steps with RK4 and
Dormand-Prince, where the ranks agree on the global CFL minimum (src/advection/advection.c:466) and
DOPRI error maximum (dormand_prince.c:93) through the per-step coupling (sharding.step_reducer
over a gloo all-reduce), and every rank sets up every patch (option setup_all_patches): the
reference's lazy set-up follows the particles, so with a subset of them a rank would set up fewer
patches than the single-rank run."""
import os
import socket

import numpy as np
import pytest

from lagrbf_gb300 import sharding
from lagrbf_gb300 import workloads as W

torch = pytest.importorskip("torch")


def _case():
    rng = np.random.default_rng(21)
    xd = W.jittered_lattice(14, 3, rng)
    fd = W.abc_flow(xd)
    xp = W.uniform_points(1203, 3, np.random.default_rng(22))
    xp[:300] = np.clip(xp[:300], 0.0, 0.02) + np.where(xp[:300] > 0.5, 0.96, 0.0)  # near faces: some leave
    opts = dict(dim=3, npartitions=[5] * 3, overlap=W.pu_overlap(5), kernel=2, nfields=3, advection=True,
                advection_scheme=2, advection_cfl=0.3)
    return xd, fd, xp, opts


def _run(xd, fd, xp, pid, opts, interval=4e-3, reduce=None):
    from oracle_lib import Oracle
    o = Oracle(**opts)
    if reduce is not None:
        assert o.set_step_reduce(reduce) == 0
    assert o.fill(False, xp, pidx=pid) == 0
    for k in range(5):  # lagrbfpy's advect_step: data in, interpolate, advect (which clears the data)
        assert o.fill(True, xd, fd) == 0
        assert o.interpolate() == 0
        assert o.advect(k * interval, (k + 1) * interval) == 0
    n = int(pid.max()) if len(pid) else 0
    x, f, p = o.output(n)
    return x, f, p


def _allreduce(op):
    import torch.distributed as dist

    def f(a):
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64))
        dist.all_reduce(t, op=op)
        return t.numpy()
    return f


def _worker(rank, world, port, outdir, scheme, interval, coupled):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    xd, fd, xp, opts = _case()
    opts = dict(opts, advection_scheme=scheme, setup_all_patches=coupled)
    xl, pl = sharding.shard(xp, rank, world)
    red = sharding.step_reducer(_allreduce(dist.ReduceOp.MAX)) if coupled else None
    x, f, p = _run(xd, fd, xl, pl, opts, interval, red)
    # output rows are indexed by pid - 1 over [1, max local pid]; keep this rank's rows
    rows = p[p > 0] - 1
    gx = sharding.assemble_by_pid(len(xp), x[rows], p[p > 0], _allreduce(dist.ReduceOp.SUM))
    gf = sharding.assemble_by_pid(len(xp), f[rows], p[p > 0], _allreduce(dist.ReduceOp.SUM))
    if rank == 0:
        np.savez(os.path.join(outdir, "sharded.npz"), x=gx, f=gf)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shard_ranges_partition_the_swarm():
    for n in (0, 1, 7, 1203):
        for world in (1, 2, 3, 8):
            r = [sharding.shard_range(n, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
            assert max(e - s for s, e in r) - min(e - s for s, e in r) <= 1
    with pytest.raises(ValueError):
        sharding.shard_range(10, 2, 2)


@pytest.mark.parametrize("scheme,interval,coupled", [(2, 4e-3, False), (2, 0.05, True), (3, 0.05, True)])
def test_two_rank_gloo_matches_single_rank(tmp_path, scheme, interval, coupled):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path), scheme, interval, coupled), nprocs=2,
                       join=True, start_method="spawn")
    got = np.load(tmp_path / "sharded.npz")
    xd, fd, xp, opts = _case()
    opts = dict(opts, advection_scheme=scheme, setup_all_patches=coupled)
    x, f, p = _run(xd, fd, xp, np.arange(1, len(xp) + 1, dtype=np.int64), opts, interval)
    assert (p == 0).any() and (p > 0).any()  # some particles left the domain
    assert np.array_equal(got["x"], x) and np.array_equal(got["f"], f)


def test_uncoupled_long_interval_differs():
    """Without the coupling, a rank holding only slower particles takes longer CFL steps than the
    single-rank run: the shards' positions are no longer the single-rank ones."""
    xd, fd, xp, opts = _case()
    opts = dict(opts, setup_all_patches=True)
    pid = np.arange(1, len(xp) + 1, dtype=np.int64)
    x1, _, _ = _run(xd, fd, xp, pid, opts, 0.05)
    xl, pl = sharding.shard(xp, 1, 2)
    x2, _, p2 = _run(xd, fd, xl, pl, opts, 0.05)
    rows = p2[p2 > 0] - 1
    assert not np.array_equal(x2[rows], x1[p2[p2 > 0] - 1])


def test_step_reducer_and_assembly_without_communication():
    vals = np.array([-0.5, 2.0])
    sharding.step_reducer(lambda a: np.maximum(a, [-0.25, 1.0]))(vals)
    assert np.array_equal(vals, [-0.25, 2.0])
    out = sharding.assemble_by_pid(4, np.array([[1.0], [2.0], [3.0]]), np.array([2, 0, 4]))
    assert np.array_equal(out[:, 0], [0.0, 1.0, 0.0, 3.0])
