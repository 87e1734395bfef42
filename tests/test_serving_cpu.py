"""Serving loop host logic without a GPU: job validation, budget rejection at submission,
unknown dataset ids, a job that cannot get a device reports its error through wait, and
destroying a server with work outstanding."""
import numpy as np
import pytest

from lagrbf_gb300.serving import Server


def _job(rng, **kw):
    xd = rng.uniform(0, 1, (500, 3))
    fd = rng.standard_normal((500, 3))
    xp = rng.uniform(0, 1, (200, 3))
    args = dict(npartitions=[4, 4, 4], particles=xp, dt=1e-3, nsteps=2, data_coords=xd, data_values=fd)
    args.update(kw)
    return args


def test_invalid_jobs_are_rejected():
    rng = np.random.default_rng(0)
    s = Server(hbm_budget_bytes=8e9, nworkers=2)
    with pytest.raises(RuntimeError, match="invalid job"):
        s.submit(**_job(rng, dt=0.0))
    with pytest.raises(RuntimeError, match="invalid job"):
        s.submit(**_job(rng, scheme=7))
    with pytest.raises(RuntimeError, match="unknown dataset id"):
        s.submit(**_job(rng, data_coords=None, data_values=None, dataset_id=42))
    with pytest.raises(RuntimeError, match="needs its data"):
        s.submit(**_job(rng, data_coords=None, data_values=None, dataset_id=0))
    s.close()


def test_budget_rejection():
    rng = np.random.default_rng(1)
    s = Server(hbm_budget_bytes=1e6, nworkers=1)
    with pytest.raises(RuntimeError, match="exceeds the device-memory budget"):
        s.submit(**_job(rng))
    s.close()


def test_job_without_device_fails_through_wait():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rng = np.random.default_rng(2)
    s = Server(hbm_budget_bytes=8e9, nworkers=2)
    ids = [s.submit(**_job(rng, dataset_id=7 if k % 2 else 0)) for k in range(4)]
    for i in ids:
        with pytest.raises(RuntimeError, match="CUDA"):
            s.wait(i)
    st = s.stats()
    assert st["failed"] == 4 and st["completed"] == 0 and st["queued"] == 0
    s.close()


def test_destroy_with_queued_jobs():
    rng = np.random.default_rng(3)
    s = Server(hbm_budget_bytes=8e9, nworkers=1)
    for _ in range(5):
        s.submit(**_job(rng))
    s.close()  # cancels what is queued, joins the worker
