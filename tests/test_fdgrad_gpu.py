"""qjg_centered_gradient on the GPU: OPTIMIZE_3D's central-difference root
gradients, every moved map in one pass, against the reference's outputs
(tests/golden/fdgrad.npz) and the oracle on larger seeded cases: the same
scores and gradients, bit for bit."""
import os
import sys

import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, draw_rootset

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import gen_fdgrad  # noqa: E402


def entries(kind, rs):
    return 4 * {0: rs.n_top + rs.n_bottom, 1: rs.n_bottom, 2: rs.n_top}[kind]


def gpu(ctx, rs, g, max_it, kind, dist, curv):
    h = ctx.upload(rs)
    D = torch.from_numpy(np.ascontiguousarray(dist)).cuda()
    K = torch.from_numpy(np.ascontiguousarray(curv)).cuda()
    try:
        return ctx.centered_gradient(h, g, max_it, kind, D.data_ptr(), entries(kind, rs),
                                     d_curv=K.data_ptr())
    finally:
        ctx.free(h)


@pytest.mark.parametrize("name", sorted(gen_fdgrad.CASES))
def test_matches_reference(ctx, name):
    d = np.load(os.path.join(GOLDEN, "fdgrad.npz"))
    kind, rs, g, max_it = gen_fdgrad.case_inputs(name)
    dist, curv = gen_fdgrad.fields(g)
    sc, grad = gpu(ctx, rs, g, max_it, kind, dist, curv)
    assert sc == d[name + "_score"][0]
    np.testing.assert_array_equal(grad, d[name + "_grad"])


@pytest.mark.parametrize("kind,nt,nb,res,slc", [(0, 6, 3, 40, 0.05), (1, 5, 4, 33, 0.0),
                                                 (0, 4, 0, 24, 0.0), (2, 5, 0, 40, 0.0)])
def test_matches_oracle(ctx, oracle, kind, nt, nb, res, slc):
    rs = draw_rootset(17 + res, nt, nb, -0.9, 0.9, exps=(1,))
    rs.scale = 0.4
    g = Grid((res, res + 3, res - 2), lengths=(2.6, 2.8, 2.4), slice=slc)
    rng = np.random.RandomState(res)
    dist = rng.uniform(-1, 1, g.n_voxels)
    curv = rng.uniform(0, 2, g.n_voxels)
    sc, grad = gpu(ctx, rs, g, 12, kind, dist, curv)
    so, go = oracle.centered_gradient(rs, g, 12, kind, dist, curv)
    assert sc == so
    np.testing.assert_array_equal(grad, go)


def test_rejects_bad_arguments(ctx):
    rs = draw_rootset(1, 2, 1, -1, 1, exps=(1,))
    g = Grid((8, 8, 8))
    h = ctx.upload(rs)
    D = torch.zeros(g.n_voxels, dtype=torch.float64, device="cuda")
    try:
        with pytest.raises(lib.QjgError):
            ctx.centered_gradient(h, g, 5, 7, D.data_ptr(), 12)
        with pytest.raises(lib.QjgError):  # the curvature field is required
            ctx.centered_gradient(h, g, 5, lib.QJG_FD_POLYNOMIAL, D.data_ptr(), 8)
    finally:
        ctx.free(h)
