"""Serving loop on the GPU: a mix of jobs (three datasets, two kept resident by id and reused,
all four RK schemes, FP32 and FP64 evaluation, two CFL factors) run concurrently by four workers
(owner and sharing contexts, sharing contexts reused between jobs) gives, job by job, the same
particle positions bit for bit as each job run alone; latency statistics are reported."""
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
                   fp32=bool(k % 2), dataset_id=(which + 1) if which < 2 else 0,
                   cfl=0.3 if k % 3 else 0.004)  # 0.004: the CFL step (~1e-3) limits the internal step
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


def test_shared_dataset_gives_the_owners_values():
    """lagrbf_gpu_share_dataset: a context borrowing a resident dataset read-only evaluates a
    particle set exactly as the owner does; sharing needs a ready owner, and the borrowed data
    cannot be refilled."""
    import lagrbf_gb300 as L
    xd, fd, npu = _datasets()[1]
    opts = dict(dim=3, npartitions=[npu] * 3, overlap=W.pu_overlap(npu), shape_factor=1.0, kernel=2, nfields=3,
                eval_precision="fp32", petsc_options={"setup_all_patches": True})
    xp = W.uniform_points(2000, 3, np.random.default_rng(3))
    owner = L.LagRBFCtx(**opts)
    other = L.LagRBFCtx(**opts)
    with pytest.raises(RuntimeError, match="error code 73"):
        other.share_dataset(owner)  # the owner has no data yet
    pid = np.arange(1, len(xp) + 1, dtype=np.int64)
    owner.fill_data(xd, fd)
    owner.fill_points(xp[:10], pidx=pid[:10])
    owner.interpolate_c()
    other.share_dataset(owner)
    with pytest.raises(RuntimeError, match="error code 73"):
        other.fill_data(xd, fd)
    owner.fill_points(xp, pidx=pid)
    owner.interpolate_c()
    other.fill_points(xp, pidx=pid)
    other.interpolate_c()
    a = np.zeros((len(xp), 3)); b = np.zeros((len(xp), 3))
    owner.output(fvals=a)
    other.output(fvals=b)
    assert np.array_equal(a, b) and np.abs(a).max() > 0
    del other
    owner.fill_points(xp[:5], pidx=pid[:5])
    owner.interpolate_c()  # the owner is unaffected by the sharing context's teardown


def test_sharing_while_the_owner_captures_its_step_loop():
    """Contexts share a dataset while the owner's thread keeps advecting its own particles: the
    owner's precision is switched before every interval, which drops its graphs, so each interval
    is captured again as a device-side step loop and sharing often falls inside that capture.
    Sharing must leave the owner's stream alone; every sharer's positions equal those of a sharer
    run before the race, bit for bit, and the owner's run completes."""
    import threading
    import lagrbf_gb300 as L
    xd, fd, npu = _datasets()[0]
    opts = dict(dim=3, npartitions=[npu] * 3, overlap=W.pu_overlap(npu), shape_factor=1.0, kernel=2, nfields=3,
                advection=True, advection_scheme=2, advection_cfl=0.3, dt=2e-3, eval_precision="fp32",
                petsc_options={"setup_all_patches": True})
    rng = np.random.default_rng(21)
    xo = 0.2 + 0.6 * rng.uniform(0, 1, (3000, 3))
    xq = 0.2 + 0.6 * rng.uniform(0, 1, (1500, 3))
    pq = np.arange(1, len(xq) + 1, dtype=np.int64)
    owner = L.LagRBFCtx(**opts)
    owner.fill_data(xd, fd)
    owner.fill_points(xo, pidx=np.arange(1, len(xo) + 1, dtype=np.int64))
    owner.interpolate_c()
    owner.synchronize()

    def sharer_run():
        s = L.LagRBFCtx(**opts)
        s.share_dataset(owner)
        s.fill_points(xq, pidx=pq)
        s.interpolate_c()
        s.advect_resident(0.0, 4e-3)
        x = np.zeros((len(xq), 3))
        s.output(coords=x)
        del s
        return x

    expect = sharer_run()
    errors, results = [], []
    stop = threading.Event()

    def owner_loop():
        try:
            t, k = 0.0, 0
            while not stop.is_set() and k < 400:
                owner.set_precision(k % 2 == 0)
                owner.advect_resident(t, t + 2e-3)
                t += 2e-3
                k += 1
        except Exception as e:  # reported below
            errors.append(e)

    th = threading.Thread(target=owner_loop)
    th.start()
    try:
        for _ in range(30):
            results.append(sharer_run())
    except Exception as e:
        errors.append(e)
    finally:
        stop.set()
        th.join()
    assert not errors, errors
    assert len(results) == 30
    for x in results:
        assert np.array_equal(x, expect)
    assert np.abs(expect).sum() > 0
