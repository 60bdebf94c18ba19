"""Root sets, grids and the seeded synthetic workloads of the hot path.

A root set is the state of the reference's rational map
R(q) = s * prod_i (q - t_i)^(sigma_t e_i) * [prod_j (q - b_j)^(sigma_b f_j)]^-1
(POLYNOMIAL_4D roots/powers/powerScalar, src/algebra/POLYNOMIAL_4D.h:137-150,
and OPTIMIZE_3D::_expScaling).  Roots are quaternions stored (w, x, y, z).

A grid is a FIELD_3D geometry: resolution, centre, lengths, a rotation
quaternion about the centre and the 4D slice coordinate
(src/geometry/FIELD_3D.h:55-120).

Synthetic inputs are drawn from MT19937 seeded like the reference's
MERSENNETWISTER(seed), each root component as lo + (hi - lo) * rand().
The reference's real root sets (data/*.o3d) are not available, so these
seeded sets stand in for them.
"""
from dataclasses import dataclass, field
from typing import Tuple

import numpy as np


def mt19937_rand(seed: int, n: int) -> np.ndarray:
    """n draws of MERSENNETWISTER(seed).rand() (src/util/MERSENNETWISTER.h:147):
    Matsumoto-Nishimura MT19937 with init_genrand seeding, 32-bit output
    scaled by 1/(2^32 - 1)."""
    mt = [0] * 624
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, 624):
        mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
    out = np.empty(n)
    idx = 624
    for k in range(n):
        if idx >= 624:
            for i in range(624):
                y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        out[k] = y * (1.0 / 4294967295.0)
    return out


@dataclass
class RootSet:
    top_roots: np.ndarray
    top_powers: np.ndarray
    sigma_top: float = 1.0
    bottom_roots: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    bottom_powers: np.ndarray = field(default_factory=lambda: np.zeros(0))
    sigma_bottom: float = 1.0
    scale: float = 1.0

    @property
    def n_top(self):
        return len(self.top_powers)

    @property
    def n_bottom(self):
        return len(self.bottom_powers)


@dataclass
class Grid:
    res: Tuple[int, int, int]
    center: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    lengths: Tuple[float, float, float] = (3.0, 3.0, 3.0)
    rot: Tuple[float, float, float, float] = (1.0, 0.0, 0.0, 0.0)
    slice: float = 0.0

    @property
    def n_voxels(self):
        return int(self.res[0]) * int(self.res[1]) * int(self.res[2])

    @property
    def spacing(self):
        return float(self.lengths[0]) / self.res[0]


def draw_rootset(seed, n_top, n_bottom, lo, hi, exps=(1,), scale=None, scale_range=None):
    """Seeded root set: 4 components per root (top roots, then bottom roots),
    then one exponent draw per root when len(exps) > 1, then the scale draw
    when scale_range is given."""
    n = n_top + n_bottom
    k = 4 * n + (n if len(exps) > 1 else 0) + (1 if scale_range else 0)
    u = mt19937_rand(seed, k)
    roots = lo + (hi - lo) * u[:4 * n].reshape(n, 4)
    pos = 4 * n
    if len(exps) > 1:
        pick = np.minimum((u[pos:pos + n] * len(exps)).astype(int), len(exps) - 1)
        powers = np.array([float(exps[i]) for i in pick])
        pos += n
    else:
        powers = np.full(n, float(exps[0]))
    if scale_range:
        scale = scale_range[0] + (scale_range[1] - scale_range[0]) * u[pos]
    return RootSet(top_roots=roots[:n_top].copy(), top_powers=powers[:n_top].copy(),
                   bottom_roots=roots[n_top:].copy(), bottom_powers=powers[n_top:].copy(),
                   scale=1.0 if scale is None else float(scale))


def cell_centers(grid, res=None):
    """Cell centres (x, y, z) of an unrotated grid of the same extent, at
    resolution `res` (default: the grid's own), as in FIELD_3D::cellCenter."""
    res = grid.res if res is None else res
    axes = []
    for c in range(3):
        d = grid.lengths[c] / res[c]
        axes.append(grid.center[c] - 0.5 * grid.lengths[c] + (np.arange(res[c]) + 0.5) * d)
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([x, y, z], axis=-1).reshape(-1, 3)


def conformal_scale(rs, grid, sample_res=32):
    """exp(-median log|T(q0)/B(q0)|) over a sample_res^3 grid of cell centres.

    The reference picks its scale s from the one-application log map
    (OPTIMIZE_3D::estimateConformalRadius, src/solvers/OPTIMIZE_3D.cpp:4694-4772,
    which sets _expScaling = exp(-threshold) for the threshold that best fits
    a target shape).  Synthetic root sets have no target shape, so the
    threshold here is the median, which puts about half of the sample inside
    after one application.  The quaternion norm is multiplicative, so
    log|T/B| = sigma_t sum e_i log|q-t_i| - sigma_b sum f_j log|q-b_j|.
    """
    p = cell_centers(grid, (sample_res,) * 3)
    q = np.concatenate([p, np.full((len(p), 1), grid.slice)], axis=1)
    acc = np.zeros(len(q))
    for roots, pw, sig, sgn in ((rs.top_roots, rs.top_powers, rs.sigma_top, 1.0),
                                (rs.bottom_roots, rs.bottom_powers, rs.sigma_bottom, -1.0)):
        for r, e in zip(np.asarray(roots).reshape(-1, 4), pw):
            acc += sgn * sig * e * np.log(np.linalg.norm(q - r, axis=1))
    return float(np.exp(-np.median(acc)))


# ---------------------------------------------------------------- workloads
# Plain method: 8 top roots in [-1,1]^4 (seed 0), no bottom roots, unit
# exponents, 20 iterations, escape radius 2, grid [-1.5,1.5]^3 at slice w=0,
# isovalue 0.  With the literal unit scale s = 1 the field is positive
# everywhere (there is no surface); scale="conformal" uses conformal_scale().
def plain_workload(res=64, scale="unit", seed=0):
    rs = draw_rootset(seed, 8, 0, -1.0, 1.0)
    g = Grid((res, res, res))
    if scale == "conformal":
        rs.scale = conformal_scale(rs, g)
    elif scale != "unit":
        rs.scale = float(scale)
    return rs, g, dict(max_it=20, escape=2.0)


# Precision form: 16 top / 8 bottom roots in [-1.2,1.2]^4, exponents in
# {1,2}, a seeded global scale u in [0.5,2], 40 iterations, escape radius 2.
# u multiplies the conformal scale: s = u * conformal_scale (with s = u alone
# every voxel escapes within four iterations and no surface exists).
def _scaled(rs, g):
    rs.scale = rs.scale * conformal_scale(rs, g)
    return rs


def precision_workload(res=256, seed=0):
    rs = draw_rootset(seed, 16, 8, -1.2, 1.2, exps=(1, 2), scale_range=(0.5, 2.0))
    g = Grid((res, res, res))
    return _scaled(rs, g), g, dict(max_it=40, escape=2.0)


# Large grid: 48 top / 24 bottom roots drawn as above, 60 iterations.
def large_workload(res=2200, seed=0):
    rs = draw_rootset(seed, 48, 24, -1.2, 1.2, exps=(1, 2), scale_range=(0.5, 2.0))
    g = Grid((res, res, res))
    return _scaled(rs, g), g, dict(max_it=60, escape=2.0)
