"""toothOptimizer's BLMVM fits on the GPU (qjg_tanh_fit) against the
reference's own solves (tests/golden/tanh_fit.npz: callConstrainedScaledOnlyTao
then callConstrainedScaledTao with the reference's OPTIMIZE_3D callbacks).
The GPU score and gradients agree with the reference's to ~1e-12, so the
solver takes the same steps: same evaluation count, same solution to 1e-8."""
import os

import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, RootSet

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLD = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                 "tanh_fit.npz")))


def case(tag):
    d = {k[len(tag) + 1:]: v for k, v in GOLD.items() if k.startswith(tag + "_")}
    rs = RootSet(top_roots=d["top_roots"], top_powers=d["top_powers"].copy(),
                 sigma_top=float(d["sigma_top"]), bottom_roots=d["bottom_roots"].reshape(-1, 4),
                 bottom_powers=d["bottom_powers"].copy(), sigma_bottom=float(d["sigma_bottom"]),
                 scale=float(d["scale"]))
    g = Grid(tuple(int(v) for v in d["res"]), tuple(d["center"]), tuple(d["lengths"]),
             slice=float(d["slice"]))
    wg = Grid(tuple(int(v) for v in d["wres"]), tuple(d["wcenter"]), tuple(d["wlengths"]))
    return rs, g, wg, d


def state_of(rs):
    return np.concatenate([rs.bottom_powers, rs.top_powers,
                           [rs.sigma_top, rs.sigma_bottom, rs.scale]])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_scaled_only_then_scaled_fit_match_reference(ctx, tag):
    rs, g, wg, d = case(tag)
    w = torch.from_numpy(d["weights"]).cuda()
    field = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    for mode in (lib.QJG_FIT_SCALED_ONLY, lib.QJG_FIT_SCALED):
        hist = d["hist%d" % mode]
        iters = []
        st = ctx.tanh_fit(mode, rs, g, 1, wg, w.data_ptr(), d_field=field.data_ptr(),
                          monitor=lambda it, f, gn, x: iters.append(f) and False)
        assert st["evaluations"] == len(hist)
        assert st["iterations"] == len(iters)
        np.testing.assert_allclose(state_of(rs), d["out%d" % mode], rtol=1e-8, atol=1e-12)
        # the first evaluation is the start point: its score agrees to the
        # score kernel's own tolerance
        assert st["reason"] in (1, 2, 3, 4, 5)
        assert np.isfinite(st["f"])
        assert abs(st["f"] - hist[-1, 0]) <= 1e-8 * abs(hist[-1, 0]) or \
            np.min(np.abs(hist[:, 0] - st["f"])) <= 1e-8 * abs(st["f"])


def test_fit_field_output_is_the_last_evaluation(ctx):
    rs, g, wg, d = case("a")
    w = torch.from_numpy(d["weights"]).cuda()
    field = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    st = ctx.tanh_fit(lib.QJG_FIT_SCALED_ONLY, rs, g, 1, wg, w.data_ptr(),
                      d_field=field.data_ptr())
    # re-evaluate the score at the solution: equal when the last trial point
    # was accepted (a successful line search ends on it)
    h = ctx.upload(rs)
    f2 = torch.empty_like(field)
    sc, _, _ = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), 3 + rs.n_top + rs.n_bottom,
                                   d_field=f2.data_ptr())
    ctx.free(h)
    assert sc == st["f"]
    assert torch.equal(field, f2)


def test_max_score_is_sum_of_abs_weights(ctx):
    rs, g, wg, d = case("b")
    w = torch.from_numpy(d["weights"]).cuda()
    m = ctx.tanh_max_score(g, wg, w.data_ptr())
    # the weights looked up at the cell centres, summed on the host
    from quijibo_gb300.rootsets import cell_centers
    from oracle.oracle import Oracle, build
    build()
    o = Oracle()
    vals = [o.trilinear(wg, d["weights"], p) for p in cell_centers(g)]
    assert abs(m - np.sum(np.abs(vals))) <= 1e-12 * m


def test_fit_rejects_bad_arguments(ctx):
    rs, g, wg, d = case("a")
    w = torch.from_numpy(d["weights"]).cuda()
    with pytest.raises(lib.QjgError):
        ctx.tanh_fit(7, rs, g, 1, wg, w.data_ptr())
    rs.scale = -1.0
    with pytest.raises(lib.QjgError):
        ctx.tanh_fit(lib.QJG_FIT_SCALED, rs, g, 1, wg, w.data_ptr())
