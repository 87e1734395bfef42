"""Serving loop on the GPU: a mix of jobs (three datasets, two kept resident by id and reused,
all four RK schemes, FP32 and FP64 evaluation) run concurrently by four workers gives, job by job,
the same particle positions bit for bit as each job run alone; latency statistics are reported."""
import numpy as np
import pytest

from lagrbf_gb300 import workloads as W
from lagrbf_gb300.serving import Server

pytestmark = pytest.mark.gpu


def _datasets():
    rng = np.random.default_rng(5)
    out = []
    for nlat, npu in ((12, 4), (16, 5), (14, 4)):
        xd = W.jittered_lattice(nlat, 3, rng)
        fd = W.abc_flow(xd) if nlat != 16 else W.fourier_field(xd, rng, nmodes=6)
        out.append((xd, fd, npu))
    return out


def _jobs():
    ds = _datasets()
    rng = np.random.default_rng(9)
    jobs = []
    for k in range(10):
        which = k % 3
        xd, fd, npu = ds[which]
        np_ = int(rng.integers(500, 3000))
        xp = 0.1 + 0.8 * rng.uniform(0, 1, (np_, 3))
        job = dict(npartitions=[npu] * 3, particles=xp, dt=2e-3, nsteps=int(rng.integers(2, 5)), scheme=k % 4,
                   fp32=bool(k % 2), dataset_id=(which + 1) if which < 2 else 0)
        first = which == 2 or k < 2
        if first:
            job.update(data_coords=xd, data_values=fd)
        jobs.append(job)
    return jobs


def test_jobs_in_the_mix_match_jobs_alone():
    jobs = _jobs()
    s = Server(hbm_budget_bytes=40e9, nworkers=4)
    ids = [s.submit(**j) for j in jobs]
    mixed = [s.wait(i)[0] for i in ids]
    st = s.stats()
    s.close()
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"] and st["particle_steps"] > 0
    alone = []
    s1 = Server(hbm_budget_bytes=40e9, nworkers=1)
    for j in jobs:
        alone.append(s1.wait(s1.submit(**j))[0])
    assert s1.stats()["datasets_resident"] == 2
    s1.close()
    for a, b in zip(mixed, alone):
        assert np.array_equal(a, b)
        assert np.isfinite(a).all() and (np.abs(a).sum(axis=1) > 0).mean() > 0.9
