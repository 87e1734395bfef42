"""lagrbf_gpu_bin_points_noalloc (binning with its scratch in a static device array) against the
binning of the context path (lagrbf_fill_swarm + lagrbf_gpu_get_cellids / lagrbf_gpu_get_patch_csr)
on the same points.  Integer results: bit-exact.  The entry point is called several times in a row
so that scratch left by one call cannot leak into the next.  Device buffers for the inputs and
outputs belong to the test (torch); the entry point itself allocates nothing.
"""
import ctypes

import numpy as np
import pytest

import lagrbf_gb300 as L
from lagrbf_gb300 import _lib
from lagrbf_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_CELLS = 1 << 20  # LAGRBF_NOALLOC_MAX_CELLS


def _fn():
    lib = _lib.load_shared_lib()
    f = lib.lagrbf_gpu_bin_points_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double),
                  ctypes.POINTER(ctypes.c_double), ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _bin_noalloc(torch, dim, nodes, x, O=0.0, Lb=1.0):
    """Runs the no-alloc binning on device copies of x; returns host (cellid, cell_start, order)."""
    f = _fn()
    n = len(x)
    ncells = int(np.prod([m - 1 for m in nodes]))
    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    cid = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    start = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
    order = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    nodes_c = (ctypes.c_int32 * 3)(*nodes, *([1] * (3 - len(nodes))))
    O_c = (ctypes.c_double * 3)(*([O] * 3))
    L_c = (ctypes.c_double * 3)(*([Lb] * 3))
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(dim, nodes_c, O_c, L_c, n, xd.data_ptr(), cid.data_ptr(), start.data_ptr(), order.data_ptr(),
           ctypes.c_void_p(stream))
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return cid.cpu().numpy()[:n], start.cpu().numpy(), order.cpu().numpy()[:n]


def _patch_csr_from_cells(dim, nodes, start, order):
    """Patch (node) membership from a cell CSR: adjacent cells in ascending order, each cell's
    points in order -- the layout lagrbf_gpu_get_patch_csr reports."""
    nc = [m - 1 for m in nodes] + [1] * (3 - dim)
    nn = list(nodes) + [1] * (3 - dim)
    pstart, pts = [0], []
    for k in range(nn[2]):
        for j in range(nn[1]):
            for i in range(nn[0]):
                cells = []
                for dk in ((-1, 0) if dim == 3 else (0,)):
                    for dj in (-1, 0):
                        for di in (-1, 0):
                            ci, cj, ck = i + di, j + dj, k + dk
                            if 0 <= ci < nc[0] and 0 <= cj < nc[1] and 0 <= ck < nc[2]:
                                cells.append(ci + cj * nc[0] + ck * nc[0] * nc[1])
                for c in sorted(cells):
                    pts.extend(order[start[c]:start[c + 1]].tolist())
                pstart.append(len(pts))
    return np.array(pstart, dtype=np.int32), np.array(pts, dtype=np.int32)


def _case(dim, npu, nlat, seed):
    rng = np.random.default_rng(seed)
    xd = W.jittered_lattice(nlat, dim, rng)
    # points on the box faces, on interior node planes and at the upper corner
    extra = np.array([[1.0] * dim, [0.0] * dim, [0.5] * dim, [1.0 / (npu - 1)] * dim])
    xd = np.concatenate([xd, extra])
    xp = W.uniform_points(2500, dim, np.random.default_rng(seed + 1))
    opts = dict(dim=dim, npartitions=[npu] * dim, overlap=W.pu_overlap(npu), shape_factor=1.0, kernel=2, nfields=1)
    return xd, xp, opts


@pytest.mark.parametrize("dim,npu,nlat", [(3, 6, 18), (2, 9, 40)])
def test_noalloc_binning_matches_context_path(dim, npu, nlat):
    torch = pytest.importorskip("torch")
    xd, xp, opts = _case(dim, npu, nlat, seed=23 + dim)
    nodes = [npu] * dim
    c = L.LagRBFCtx(**opts)
    c.fill_data(xd, np.zeros((len(xd), 1)))
    c.fill_points(xp)
    ref_cd = c.cellids(True, len(xd))
    ref_cp = c.cellids(False, len(xp))
    ref_ps, ref_pp = c.patch_csr()

    # two calls in a row on different point sets, then the first set again
    for x, ref in ((xd, ref_cd), (xp, ref_cp), (xd, ref_cd)):
        cid, start, order = _bin_noalloc(torch, dim, nodes, x)
        assert np.array_equal(cid, ref)
        counts = np.bincount(ref[ref >= 0], minlength=int(np.prod([m - 1 for m in nodes])))
        assert np.array_equal(start, np.concatenate([[0], np.cumsum(counts)]).astype(np.int32))
        # stable order: point indices grouped by cell, input order within each cell
        keep = np.nonzero(ref >= 0)[0]
        assert np.array_equal(order[: start[-1]], keep[np.argsort(ref[keep], kind="stable")].astype(np.int32))
        if x is xd:
            ps, pp = _patch_csr_from_cells(dim, nodes, start, order)
            assert np.array_equal(ps, ref_ps) and np.array_equal(pp, ref_pp)


def test_noalloc_points_outside_and_crowded_cells():
    """Points outside the box get -1 and no slot; a cell holding more points than the shared-memory
    sort tile is ordered in global memory."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    nodes = [4, 4, 4]
    x = rng.uniform(-0.2, 1.2, size=(6000, 3))
    crowd = rng.uniform(0.0, 0.3, size=(5000, 3))  # all inside cell 0 (h = 1/3)
    x = np.concatenate([x, crowd])
    perm = rng.permutation(len(x))
    x = x[perm]
    for _ in range(2):
        cid, start, order = _bin_noalloc(torch, 3, nodes, x)
        inside = np.all((x >= 0.0) & (x <= 1.0), axis=1)
        t = np.minimum(np.floor(x / (1.0 / 3.0)).astype(np.int64), 2)
        exp = np.where(inside, t[:, 0] + 3 * t[:, 1] + 9 * t[:, 2], -1)
        assert np.array_equal(cid, exp)
        assert start[-1] == inside.sum()
        assert start[1] - start[0] > 4096
        keep = np.nonzero(exp >= 0)[0]
        exp_order = keep[np.argsort(exp[keep], kind="stable")]
        assert np.array_equal(order[: start[-1]], exp_order.astype(np.int32))


def test_noalloc_rejects_meshes_beyond_scratch():
    f = _fn()
    nodes = (ctypes.c_int32 * 3)(1026, 1026, 2)  # 1025*1025 cells > 2^20
    O = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    Lb = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    start = np.zeros(1, dtype=np.int32)  # rejected before any use of the buffer
    rc = f(3, nodes, O, Lb, 0, None, None, start.ctypes.data, None, None)
    assert rc == 63
    assert "static scratch" in _lib.last_error()


def test_noalloc_accepts_the_largest_mesh():
    """Exactly LAGRBF_NOALLOC_MAX_CELLS cells (2D, 1025 x 1025 nodes): accepted, binned like the
    floor((x - O) / h) convention on a few points, corners and the upper face included."""
    torch = pytest.importorskip("torch")
    nodes = (1025, 1025)
    assert (nodes[0] - 1) * (nodes[1] - 1) == MAX_CELLS
    x = np.array([[0.0, 0.0], [1.0, 1.0], [0.5, 0.25], [0.999, 0.001], [0.1234, 0.9876]])
    cid, start, order = _bin_noalloc(torch, 2, nodes, x)
    t = np.minimum(np.floor(x * 1024).astype(np.int64), 1023)
    assert np.array_equal(cid, t[:, 0] + 1024 * t[:, 1])
    assert start[-1] == len(x) and len(start) == MAX_CELLS + 1
    assert np.array_equal(np.sort(order), np.arange(len(x)))


def test_noalloc_records_into_a_stream_capture_and_allocates_nothing():
    """What the entry point is for: after one call (which resolves the scratch address and loads its
    kernels), a call changes neither the device memory in use (cudaMemGetInfo) nor torch's
    allocation, and it can be recorded into the caller's own stream capture (torch.cuda.graph,
    global capture mode: an allocation or synchronisation inside would invalidate the capture);
    replaying the graph gives the eager results."""
    torch = pytest.importorskip("torch")
    dim, npu, nlat = 3, 6, 18
    _, xp, _ = _case(dim, npu, nlat, 31)
    nodes = [npu] * dim
    ref = _bin_noalloc(torch, dim, nodes, xp)  # warm-up, eager
    f = _fn()
    n, ncells = len(xp), (npu - 1) ** dim
    x = torch.from_numpy(np.ascontiguousarray(xp, dtype=np.float64)).cuda()
    cid = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    start = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
    order = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    nodes_c = (ctypes.c_int32 * 3)(*nodes)
    O_c = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    L_c = (ctypes.c_double * 3)(1.0, 1.0, 1.0)

    def call(stream):
        return f(dim, nodes_c, O_c, L_c, n, x.data_ptr(), cid.data_ptr(), start.data_ptr(), order.data_ptr(),
                 ctypes.c_void_p(stream))

    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    assert call(torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0 and torch.cuda.memory_allocated() == alloc0
    for t, r in zip((cid, start, order), ref):
        assert np.array_equal(t.cpu().numpy(), r)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        assert call(torch.cuda.current_stream().cuda_stream) == 0
    for t in (cid, start, order):
        t.fill_(-7)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    for t, r in zip((cid, start, order), ref):
        assert np.array_equal(t.cpu().numpy(), r)
