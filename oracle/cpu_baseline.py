"""CPU baseline of the reference algorithm on the host cores -- test infrastructure.

Emulates the reference's MPI decomposition: P ranks split the PU node mesh like a DMDA
(PUCreateDMDA, src/partition_of_unity.c:113-150) and each rank owns a local sequential mesh with a
one-cell halo (PUCreateDMDALocal, :152-283), the data points of its local bounding box (the ghost
duplication of SwarmDataAssignMigrateDuplicateGhostPoints, src/swarm/swarm_data.c:90-159) and its
particles.  The support radius and shape parameter keep their global values
(PartitionOfUnityComputeSupport uses the global mesh).  One OpenMP thread per rank runs the
oracle's restatement of the rank's work (all-node PU weights, per-particle block phi, patch dot
products, RK stages) compiled with the reference's optimisation flags.

The sample is bounded: each rank advects `sample` particles placed in a 2x2x2-cell box at the
centre of its owned region, with the rank's full local data and patches.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests"))
import oracle_lib  # noqa: E402


def _lib_fast():
    so = os.path.join(HERE, "_build", "liblagrbf_oracle_fast.so")
    if not os.path.exists(so):
        oracle_lib.build_oracle()
    L = ctypes.CDLL(so)
    L.orc_config_default.argtypes = [ctypes.POINTER(oracle_lib.OrcConfig)]
    L.orc_time_ranks.argtypes = [ctypes.c_int, ctypes.POINTER(oracle_lib.OrcConfig), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                 ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                 ctypes.POINTER(ctypes.c_long)]
    return L


def process_grid(P, dim):
    """Balanced factorisation of P ranks over dim axes (largest factor along x)."""
    f = []
    n = P
    for p in (2, 3, 5, 7):
        while n % p == 0:
            f.append(p)
            n //= p
    if n > 1:
        f.append(n)
    g = [1] * dim
    for p in sorted(f, reverse=True):
        g[int(np.argmin(g))] *= p
    return sorted(g, reverse=True)


def rank_problems(xd, fd, npu, opts, P, sample, seed=0):
    dim = opts["dim"]
    h = 1.0 / (npu - 1)
    radius = opts["overlap"] / float(npu)          # overlap * box / npg^(1/dim) on [0,1]^dim
    grid = process_grid(P, dim)
    rng = np.random.default_rng(seed)
    cfgs, data, parts = [], [], []
    for r in range(P):
        idx = np.unravel_index(r, grid[::-1])[::-1]
        lo_n, hi_n = [], []
        centre = []
        for d in range(dim):
            s = (npu * idx[d]) // grid[d]
            e = (npu * (idx[d] + 1)) // grid[d]
            c0, c1 = s, min(e, npu - 1)               # owned cells
            centre.append(0.5 * (c0 + c1) * h)
            l0, l1 = max(c0 - 1, 0), min(c1 + 1, npu - 1)  # one-cell halo
            lo_n.append(l0)
            hi_n.append(l1)                           # local nodes l0..l1
        O = np.array([lo_n[d] * h for d in range(dim)])
        Lb = np.array([hi_n[d] * h for d in range(dim)])
        nloc = [hi_n[d] - lo_n[d] + 1 for d in range(dim)]
        box = float(np.max(Lb - O))
        overlap_l = radius * (np.prod(nloc) ** (1.0 / dim)) / box
        cfg = oracle_lib.make_config(dim=dim, npartitions=nloc, nfields=opts["nfields"], kernel=opts["kernel"],
                                     overlap=overlap_l, shape_factor=opts["shape_factor"], minCoords=O, maxCoords=Lb,
                                     solve_method=1, advection=True, advection_scheme=opts.get("advection_scheme", 2),
                                     advection_cfl=opts.get("advection_cfl", 0.3))
        m = np.all((xd >= O) & (xd <= Lb), axis=1)
        c = np.array(centre)
        xp = c + rng.uniform(-h, h, (sample, dim))
        cfgs.append(cfg)
        data.append((np.ascontiguousarray(xd[m]), np.ascontiguousarray(fd[m])))
        parts.append(np.ascontiguousarray(xp))
    return cfgs, data, parts


def time_reference(xd, fd, npu, opts, P, sample, nsteps, dt, seed=0):
    """Returns dict(setup_s, step_s, particle_steps, ranks, sample)."""
    L = _lib_fast()
    cfgs, data, parts = rank_problems(xd, fd, npu, opts, P, sample, seed)
    Carr = (oracle_lib.OrcConfig * P)(*cfgs)
    nd = (ctypes.c_int * P)(*[len(d[0]) for d in data])
    npp = (ctypes.c_int * P)(*[len(p) for p in parts])
    xd_p = (ctypes.c_void_p * P)(*[d[0].ctypes.data for d in data])
    fd_p = (ctypes.c_void_p * P)(*[d[1].ctypes.data for d in data])
    xp_p = (ctypes.c_void_p * P)(*[p.ctypes.data for p in parts])
    s_setup, s_step, ps = ctypes.c_double(), ctypes.c_double(), ctypes.c_long()
    rc = L.orc_time_ranks(P, Carr, nd, xd_p, fd_p, npp, xp_p, nsteps, dt, ctypes.byref(s_setup),
                          ctypes.byref(s_step), ctypes.byref(ps))
    if rc:
        raise RuntimeError("oracle baseline failed (%d)" % rc)
    return dict(setup_s=s_setup.value, step_s=s_step.value, particle_steps=ps.value, ranks=P, sample=sample,
                local_data=int(np.mean([len(d[0]) for d in data])))
