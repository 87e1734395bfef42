"""Seeded synthetic inputs with the shapes of the benchmark configurations.

No public dataset is involved: the configurations describe jittered lattices of source nodes
carrying analytic velocity fields, and uniformly (or mixture-) distributed particles.

  cellular_2d  : 64x64 jittered lattice on [0,1]^2, u = (sin(pi x) cos(pi y), -cos(pi x) sin(pi y))
  abc_3d       : n^3 jittered lattice on [0,1]^3, ABC flow A=B=C=1 at X = 2 pi x
  fourier_3d   : n^3 jittered lattice, 16 random Fourier modes, amplitudes N(0,1)/|k|^2
  mixture_3d   : isotropic Gaussian clusters plus a uniform background
"""
import numpy as np


def jittered_lattice(n, dim, rng, jitter=0.25):
    h = 1.0 / n
    idx = np.stack(np.meshgrid(*[np.arange(n)] * dim, indexing="ij"), -1).reshape(-1, dim)
    x = (idx + 0.5) * h + rng.uniform(-jitter * h, jitter * h, idx.shape)
    return np.ascontiguousarray(np.clip(x, 0.0, 1.0))


def cellular_flow(x):
    px, py = np.pi * x[:, 0], np.pi * x[:, 1]
    return np.stack([np.sin(px) * np.cos(py), -np.cos(px) * np.sin(py)], 1)


def abc_flow(x, A=1.0, B=1.0, C=1.0):
    X, Y, Z = (2 * np.pi * x[:, d] for d in range(3))
    return np.stack([A * np.sin(Z) + C * np.cos(Y), B * np.sin(X) + A * np.cos(Z), C * np.sin(Y) + B * np.cos(X)], 1)


def fourier_field(x, rng, nmodes=16, kmax=4, ncomp=3):
    out = np.zeros((x.shape[0], ncomp))
    for c in range(ncomp):
        k = rng.integers(-kmax, kmax + 1, (nmodes, x.shape[1]))
        k[np.all(k == 0, 1)] = 1
        a = rng.normal(size=nmodes) / np.sum(k * k, 1)
        ph = rng.uniform(0, 2 * np.pi, nmodes)
        out[:, c] = np.sum(a * np.sin(2 * np.pi * (x @ k.T) + ph), 1)
    return out


def uniform_points(n, dim, rng):
    return np.ascontiguousarray(rng.uniform(0.0, 1.0, (n, dim)))


def mixture_clusters(dim, rng, nclusters=8):
    """Centres U[0.2, 0.8]^dim and widths U[0.02, 0.2] of an isotropic Gaussian mixture."""
    return rng.uniform(0.2, 0.8, (nclusters, dim)), rng.uniform(0.02, 0.2, nclusters)


def mixture_points(n, dim, rng, nclusters=8, background=0.1, clusters=None):
    """n points: a fraction `background` uniform on [0,1]^dim, the rest from the mixture (draws
    outside [0,1]^dim rejected); `clusters` = (centres, widths) reuses a mixture."""
    centres, sig = clusters if clusters is not None else mixture_clusters(dim, rng, nclusters)
    nclusters = len(sig)
    nb = int(n * background)
    out = [rng.uniform(0, 1, (nb, dim))]
    need = n - nb
    while need > 0:
        c = rng.integers(0, nclusters, need)
        p = centres[c] + sig[c, None] * rng.normal(size=(need, dim))
        p = p[np.all((p >= 0) & (p <= 1), 1)]
        out.append(p)
        need -= p.shape[0]
    return np.ascontiguousarray(np.concatenate(out)[:n])


def pu_overlap(n_nodes):
    """overlap giving a support radius of 1.5 node spacings on [0,1]: radius = overlap / n."""
    return 1.5 * n_nodes / (n_nodes - 1)


def config_cellular_2d(np_=10000, seed=1, kernel=6):
    """2D plain method (64x64 lattice, Gaussian eps = 3/h or the reference default kernel)."""
    rng = np.random.default_rng(seed)
    xd = jittered_lattice(64, 2, rng)
    fd = cellular_flow(xd)
    n = 8
    ov = pu_overlap(n)
    epsw = n / ov
    shape = (3 * 64) / epsw if kernel == 6 else 1.0
    xp = uniform_points(np_, 2, np.random.default_rng(seed + 1))
    opts = dict(dim=2, npartitions=[n, n], overlap=ov, shape_factor=shape, kernel=kernel, nfields=2)
    return xd, fd, xp, opts


def config_abc_3d(nlat=128, npu=32, np_=16_777_216, seed=3):
    """3D plain drop-in at scale: nlat^3 jittered lattice, ABC flow, npu^3 PU nodes, Wendland C2."""
    rng = np.random.default_rng(seed)
    xd = jittered_lattice(nlat, 3, rng)
    fd = abc_flow(xd)
    xp = uniform_points(np_, 3, np.random.default_rng(seed + 1))
    opts = dict(dim=3, npartitions=[npu] * 3, overlap=pu_overlap(npu), shape_factor=1.0, kernel=2, nfields=3)
    return xd, fd, xp, opts


def config_uneven_3d(nd=1_000_000, npu=160, np_=8_000_000, seed=5):
    """3D uneven data: 90 % of the points from 8 isotropic Gaussians (widths 0.02-0.2) and 10 %
    uniform, ABC flow, particles from the same mixture; Wendland C2 on a uniform npu^3 PU mesh.
    The PU mesh is fine enough that the densest patch stays a dense system of a few thousand
    points (npu = 160, seed 5: largest patch 1,713 points, 2.3 M non-empty patches)."""
    rng = np.random.default_rng(seed)
    clusters = mixture_clusters(3, rng)
    xd = mixture_points(nd, 3, rng, clusters=clusters)
    fd = abc_flow(xd)
    xp = mixture_points(np_, 3, np.random.default_rng(seed + 1), clusters=clusters)
    opts = dict(dim=3, npartitions=[npu] * 3, overlap=pu_overlap(npu), shape_factor=1.0, kernel=2, nfields=3)
    return xd, fd, xp, opts


def config_precision_3d(nlat=80, npu=32, np_=4_000_000, seed=6):
    """3D precision stress: Gaussian eps_r = 1/h (h = lattice spacing), 16 Fourier modes."""
    rng = np.random.default_rng(seed)
    xd = jittered_lattice(nlat, 3, rng)
    fd = fourier_field(xd, np.random.default_rng(seed + 1))
    ov = pu_overlap(npu)
    epsw = npu / ov
    xp = uniform_points(np_, 3, np.random.default_rng(seed + 2))
    opts = dict(dim=3, npartitions=[npu] * 3, overlap=ov, shape_factor=float(nlat) / epsw, kernel=6, nfields=3)
    return xd, fd, xp, opts


def serving_stream(rng, njobs=60, rate=200.0, ndatasets=6, nd_range=(1e4, 4e5), np_median=1e5,
                   np_range=(1e3, 4e6), reuse=0.3, steps=(1, 50), dt=5e-4):
    """Advection jobs for the serving loop: Poisson arrivals (rate jobs/s), datasets on jittered
    lattices of log-uniform size carrying a 16-mode Fourier field (about 70 points per PU cell),
    particle counts lognormal around np_median, RK order uniform in {1, 2, 4, DP45}, steps uniform.
    A fraction `reuse` of the jobs names one of the datasets already sent; the data go with a
    dataset's first job only.  Yields (arrival time, job keyword arguments)."""
    dsets = []
    for _ in range(ndatasets):
        nd = float(np.exp(rng.uniform(np.log(nd_range[0]), np.log(nd_range[1]))))
        nlat = max(8, int(round(nd ** (1.0 / 3.0))))
        xd = jittered_lattice(nlat, 3, rng)
        fd = fourier_field(xd, rng, nmodes=16)
        npu = max(3, int(round((len(xd) / 70.0) ** (1.0 / 3.0))) + 1)
        dsets.append((xd, fd, npu))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=njobs))
    sent = set()
    out = []
    for k in range(njobs):
        if sent and rng.uniform() < reuse:
            which = int(rng.choice(sorted(sent)))
        else:
            which = int(rng.integers(0, ndatasets))
        xd, fd, npu = dsets[which]
        n = int(np.clip(np.exp(rng.normal(np.log(np_median), 1.0)), np_range[0], np_range[1]))
        job = dict(npartitions=[npu] * 3, particles=rng.uniform(0.0, 1.0, (n, 3)), dt=dt,
                   nsteps=int(rng.integers(steps[0], steps[1] + 1)), scheme=int(rng.integers(0, 4)), fp32=True,
                   dataset_id=which + 1)
        if which not in sent:
            job.update(data_coords=xd, data_values=fd)
            sent.add(which)
        out.append((float(arrivals[k]), job))
    return out
