"""Writes tests/golden/fdgrad.npz: OPTIMIZE_3D's central-difference root
gradients (computeLogRationalCenteredGradient, its bottom-root form and
computeCenteredGradient) run by the reference itself (oracle/_ref) on small
seeded cases, with the unmoved map's score.

    QUIJIBO_REF=<QUIJIBO checkout> python tests/golden/gen_fdgrad.py

The distance and curvature fields are polynomials of the cell centres
(`fields`), rebuilt by the tests with the same IEEE operations.  Every
log-rational case has bottom roots: with none, the reference stops on an
Eigen index assertion in this path, so the bottom-free form is checked
against the oracle only.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

# name: (kind, seed, n_top, n_bottom, root range, scale, res, length, slice, max_it)
CASES = {
    "lograt_s03": (0, 5, 3, 2, 1.0, 0.3, 16, 3.0, 0.0, 10),
    "lograt_s1": (0, 5, 3, 2, 1.0, 1.0, 16, 3.0, 0.1, 10),
    "lograt_bottom": (1, 5, 3, 2, 1.0, 1.0, 16, 3.0, 0.1, 10),
    "polynomial": (2, 5, 4, 0, 0.7, 1.0, 16, 2.0, 0.0, 12),
}


def case_inputs(name):
    from quijibo_gb300.rootsets import Grid, draw_rootset
    kind, seed, nt, nb, rr, s, res, length, slc, max_it = CASES[name]
    rs = draw_rootset(seed, nt, nb, -rr, rr, exps=(1,))
    rs.scale = s
    g = Grid((res, res, res), lengths=(length, length, length), slice=slc)
    return kind, rs, g, max_it


def fields(g):
    """Distance to a sphere of radius 0.6 and a curvature-like field, at the
    cell centres of an unrotated grid centred at the origin (x fastest)."""
    n = g.res[0]
    L = g.lengths[0]
    idx = np.indices((n, n, n)).reshape(3, -1)[::-1].T.astype(np.float64)
    c = -L / 2 + (idx + 0.5) * L / n
    x, y, z = c[:, 0], c[:, 1], c[:, 2]
    dist = np.sqrt(x * x + y * y + z * z) - 0.6
    curv = 0.5 + x * x - y * z
    return dist, curv


def main():
    from oracle.oracle import Reference
    ref = Reference("double")
    out = {}
    for name in CASES:
        kind, rs, g, max_it = case_inputs(name)
        dist, curv = fields(g)
        sc, grad = ref.centered_gradient(rs, g, max_it, kind, dist, curv)
        out[name + "_score"] = np.array([sc])
        out[name + "_grad"] = grad
    np.savez(os.path.join(HERE, "fdgrad.npz"), **out)


if __name__ == "__main__":
    main()
