"""Sample sets and target shapes of the differentiation workload.

Samples: seeded Poisson-disk points in a box by batched dart throwing on a
background grid (cell size r/sqrt(3) holds at most one point).  The reference samples mesh
surfaces with vcglib (projects/poissonDisk), which is not part of this path;
this is a volume sampler of its own.

Target: the signed distance to a union of three randomly placed and rotated
ellipsoids and one torus.  The torus distance is exact; the ellipsoid uses
the usual bound k0 (k0 - 1) / k1 with k0 = |p/r|, k1 = |p/r^2|, which is
exact on the surface and an approximation elsewhere.
"""
import numpy as np

from .rootsets import draw_rootset, mt19937_rand


def poisson_disk(n, lo=-1.0, hi=1.0, seed=0, radius=None, batch=20000, max_batches=400):
    """n Poisson-disk points in [lo, hi]^3: no two closer than `radius`.

    Dart throwing in batches: each batch of uniform candidates is tested
    against the accepted points through a background grid (cell size
    r/sqrt(3), at most one point per cell, 5^3 neighbour cells), and
    candidates of the same batch that conflict with an earlier candidate of
    the batch are dropped (scipy's KD-tree finds those pairs)."""
    from scipy.spatial import cKDTree
    rng = np.random.RandomState(seed)
    L = hi - lo
    if radius is None:
        radius = (L ** 3 / (n * 1.6)) ** (1.0 / 3.0) * 0.78
    cs = radius / np.sqrt(3.0)
    G = int(np.ceil(L / cs))
    grid = -np.ones((G + 4, G + 4, G + 4), dtype=np.int64)  # 2-cell border
    pts = np.empty((n, 3))
    count = 0
    offs = np.array([(a, b, c) for a in range(-2, 3) for b in range(-2, 3) for c in range(-2, 3)])
    r2 = radius * radius
    for _ in range(max_batches):
        cand = lo + L * rng.uniform(size=(batch, 3))
        cell = np.minimum(((cand - lo) / cs).astype(np.int64), G - 1) + 2
        nb = cell[:, None, :] + offs[None, :, :]
        idx = grid[nb[..., 0], nb[..., 1], nb[..., 2]]
        has = idx >= 0
        if count:
            q = pts[np.maximum(idx, 0)]
            d2 = np.sum((q - cand[:, None, :]) ** 2, axis=2)
            ok = ~np.any(has & (d2 < r2), axis=1)
        else:
            ok = np.ones(batch, dtype=bool)
        # a cell already holding a point rejects (it is within r/... of it anyway)
        ok &= grid[cell[:, 0], cell[:, 1], cell[:, 2]] < 0
        sel = np.nonzero(ok)[0]
        if len(sel) > 1:
            pairs = cKDTree(cand[sel]).query_pairs(radius, output_type="ndarray")
            if len(pairs):
                drop = np.zeros(len(sel), dtype=bool)
                drop[np.maximum(pairs[:, 0], pairs[:, 1])] = True
                sel = sel[~drop]
        # two survivors may share a cell only if closer than r/sqrt(3)*sqrt(3) = r: excluded above
        take = sel[:n - count]
        pts[count:count + len(take)] = cand[take]
        grid[cell[take, 0], cell[take, 1], cell[take, 2]] = count + np.arange(len(take))
        count += len(take)
        if count >= n:
            return pts, radius
    raise RuntimeError("Poisson disk sampler reached %d < %d points" % (count, n))


def _rot(u):
    """Rotation matrix from three uniforms (Shoemake's uniform quaternion)."""
    a, b, c = u
    q = np.array([np.sqrt(1 - a) * np.sin(2 * np.pi * b), np.sqrt(1 - a) * np.cos(2 * np.pi * b),
                  np.sqrt(a) * np.sin(2 * np.pi * c), np.sqrt(a) * np.cos(2 * np.pi * c)])
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


class ShapeSDF:
    """Union of 3 ellipsoids and 1 torus, seeded."""

    def __init__(self, seed=0):
        u = mt19937_rand(seed + 1000, 64)
        self.ell = []
        k = 0
        for _ in range(3):
            c = -0.45 + 0.9 * u[k:k + 3]
            r = 0.15 + 0.3 * u[k + 3:k + 6]
            R = _rot(u[k + 6:k + 9])
            self.ell.append((c, r, R))
            k += 9
        self.torus = (-0.3 + 0.6 * u[k:k + 3], 0.3 + 0.2 * u[k + 3], 0.06 + 0.06 * u[k + 4],
                      _rot(u[k + 5:k + 8]))

    def __call__(self, p):
        p = np.asarray(p, dtype=np.float64)
        d = np.full(len(p), np.inf)
        for c, r, R in self.ell:
            q = (p - c) @ R
            k0 = np.linalg.norm(q / r, axis=1)
            k1 = np.linalg.norm(q / (r * r), axis=1)
            d = np.minimum(d, k0 * (k0 - 1.0) / np.maximum(k1, 1e-12))
        c, Rm, rm, R = self.torus
        q = (p - c) @ R
        xy = np.linalg.norm(q[:, :2], axis=1) - Rm
        d = np.minimum(d, np.sqrt(xy * xy + q[:, 2] ** 2) - rm)
        return d


def differentiation_workload(n_samples=200_000, seed=0, max_it=30):
    """64 top / 16 bottom roots in [-1.2,1.2]^4, exponents 1, conformal
    scale; n_samples Poisson-disk samples in [-1,1]^3 with targets from
    ShapeSDF; 30 iterations, escape radius 2."""
    from .rootsets import Grid, conformal_scale
    rs = draw_rootset(seed, 64, 16, -1.2, 1.2)
    rs.scale = conformal_scale(rs, Grid((32, 32, 32), lengths=(2.0, 2.0, 2.0)))
    xyz, _ = poisson_disk(n_samples, seed=seed)
    target = ShapeSDF(seed)(xyz)
    return rs, xyz, target, dict(max_it=max_it, escape=2.0)
