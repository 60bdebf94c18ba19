"""The optimizer's set-up passes: the inverted distance weight field and the
conformal-radius scan, against the reference's own outputs
(tests/golden/conformal.npz, written by gen_golden.py)."""
import numpy as np
import pytest

from conftest import load_case
from oracle.oracle import conformal_radius, inverted_distance
from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid


def case():
    rs, g, p, d = load_case("conformal")
    dg = Grid(tuple(int(v) for v in d["dres"]), tuple(d["dcenter"]), tuple(d["dlengths"]))
    return rs, g, dg, d


def test_oracle_inverted_distance_matches_reference():
    _, _, dg, d = case()
    dist = d["dist"].reshape(dg.res[::-1])
    np.testing.assert_array_equal(inverted_distance(dist).ravel(), d["inv"])
    np.testing.assert_allclose(inverted_distance(dist, True).ravel(), d["inv_norm"], rtol=1e-13,
                               atol=0)


def test_oracle_conformal_scan_matches_reference(oracle):
    rs, g, dg, d = case()
    score, thr, es = conformal_radius(oracle, rs, g, dg, d["dist"])
    assert es == pytest.approx(float(d["exp_scaling"]), rel=1e-14)
    assert score == pytest.approx(float(d["score"]), rel=1e-11)


@pytest.mark.gpu
def test_gpu_inverted_distance_matches_reference(ctx):
    torch = pytest.importorskip("torch")
    _, _, dg, d = case()
    dist = torch.from_numpy(d["dist"].copy()).cuda()
    out = torch.empty_like(dist)
    for norm, key in ((0, "inv"), (1, "inv_norm")):
        ctx.inverted_distance(dg.res, dist.data_ptr(), norm, out.data_ptr())
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        if norm:
            np.testing.assert_allclose(got, d[key], rtol=1e-13, atol=0)
        else:
            np.testing.assert_array_equal(got, d[key])


@pytest.mark.gpu
def test_gpu_conformal_radius_matches_reference(ctx):
    torch = pytest.importorskip("torch")
    rs, g, dg, d = case()
    h = ctx.upload(rs)
    dist = torch.from_numpy(d["dist"].copy()).cuda()
    # twice on one context, after another field pass: the scan's field must
    # not inherit the work counters of earlier launches
    for _ in range(2):
        score, thr, es = ctx.conformal_radius(h, g, dg, dist.data_ptr())
        assert es == pytest.approx(float(d["exp_scaling"]), rel=1e-14)
        assert score == pytest.approx(float(d["score"]), rel=1e-11)
        f = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
        ctx.field(h, g, ctx.iter_params(3, 2.0), f.data_ptr())
    ctx.free(h)


@pytest.mark.gpu
def test_gpu_inverted_distance_rejects_fields_without_sign_change(ctx):
    torch = pytest.importorskip("torch")
    dist = torch.ones(6 * 5 * 4, dtype=torch.float64, device="cuda")
    out = torch.empty_like(dist)
    with pytest.raises(lib.QjgError, match="sign change"):
        ctx.inverted_distance((6, 5, 4), dist.data_ptr(), 0, out.data_ptr())
