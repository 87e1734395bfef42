"""Particle sharding with two CPU ranks (gloo): each rank advances its pid range with the oracle as
the compute engine, results are assembled by pid with one all-reduce, and the assembly equals the
single-rank run bit for bit (particles are independent; dropped particles leave zero rows).

The outer interval of each advection call is shorter than the CFL step, as in lagrbfpy's own
loops, so every rank takes the same internal step; a longer interval would couple the ranks
through the global CFL minimum (src/advection/advection.c:466)."""
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


def _run(xd, fd, xp, pid, opts):
    from oracle_lib import Oracle
    o = Oracle(**opts)
    assert o.fill(False, xp, pidx=pid) == 0
    for k in range(5):  # lagrbfpy's advect_step: data in, interpolate, advect (which clears the data)
        assert o.fill(True, xd, fd) == 0
        assert o.interpolate() == 0
        assert o.advect(k * 4e-3, (k + 1) * 4e-3) == 0
    n = int(pid.max()) if len(pid) else 0
    x, f, p = o.output(n)
    return x, f, p


def _worker(rank, world, port, outdir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    xd, fd, xp, opts = _case()
    xl, pl = sharding.shard(xp, rank, world)
    x, f, p = _run(xd, fd, xl, pl, opts)
    # output rows are indexed by pid - 1 over [1, max local pid]; keep this rank's rows
    rows = p[p > 0] - 1
    gx = sharding.assemble_by_pid(len(xp), x[rows], p[p > 0])
    gf = sharding.assemble_by_pid(len(xp), f[rows], p[p > 0])
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


def test_two_rank_gloo_matches_single_rank(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = np.load(tmp_path / "sharded.npz")
    xd, fd, xp, opts = _case()
    x, f, p = _run(xd, fd, xp, np.arange(1, len(xp) + 1, dtype=np.int64), opts)
    assert (p == 0).any() and (p > 0).any()  # some particles left the domain
    assert np.array_equal(got["x"], x) and np.array_equal(got["f"], f)
