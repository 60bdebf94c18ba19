"""CUDA fitting energies and gradients against the reference and the oracle."""
import numpy as np
import pytest

from conftest import load_case
from quijibo_gb300.rootsets import Grid, cell_centers, conformal_scale, draw_rootset

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _wgrid(d):
    return Grid(tuple(int(v) for v in d["wres"]), tuple(d["wcenter"]), tuple(d["wlengths"]))


def test_tanh_score_and_gradients_match_reference(ctx):
    """Score and the toothOptimizer gradient [log s, bottom exps, top exps,
    sigma_t, sigma_b] against the reference's own OPTIMIZE_3D at maxIterations 1."""
    rs, g, p, d = load_case("tanh_grad")
    wg = _wgrid(d)
    h = ctx.upload(rs)
    w = torch.from_numpy(d["weights"]).cuda()
    f = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    sc, gr, st = ctx.tanh_score_grad(h, g, p["max_it"], wg, w.data_ptr(), len(d["grad"]),
                                     d_field=f.data_ptr())
    ff = f.cpu().numpy().reshape(d["field"].shape)
    assert np.quantile(np.abs(ff - d["field"]) / np.abs(d["field"]), 0.999) <= 1e-12
    assert abs(sc - d["score"]) <= 1e-11 * abs(d["score"])
    np.testing.assert_allclose(gr, d["grad"], rtol=1e-10, atol=1e-11 * np.abs(d["grad"]).max())
    assert st["overflowed"] == 0 and st["bad_terms"] == 0
    ctx.free(h)


@pytest.mark.parametrize("max_it", [1, 3])
def test_tanh_gradients_match_oracle_larger_grid(ctx, oracle, max_it):
    rs = draw_rootset(21, 12, 6, -1.2, 1.2, exps=(1, 2))
    rs.sigma_top, rs.sigma_bottom = 0.97, 1.03
    g = Grid((25, 25, 25))
    rs.scale = conformal_scale(rs, g)
    wg = Grid((20, 20, 20), lengths=(3.1, 3.1, 3.1))
    c = cell_centers(wg)
    wts = np.cos(c[:, 0] + 2 * c[:, 1]) * np.exp(-np.sum(c ** 2, axis=1))
    sc0, gr0, f0 = oracle.tanh_score_grad(rs, g, wg, wts, max_it)
    h = ctx.upload(rs)
    w = torch.from_numpy(wts).cuda()
    sc, gr, st = ctx.tanh_score_grad(h, g, max_it, wg, w.data_ptr(), len(gr0))
    assert abs(sc - sc0) <= 1e-10 * abs(sc0)
    np.testing.assert_allclose(gr, gr0, rtol=1e-9, atol=1e-10 * np.abs(gr0).max())
    ctx.free(h)


def test_tanh_gradient_matches_finite_differences_fp64(ctx):
    """At maxIterations 1 the analytic top-exponent and sigma gradients are
    derivatives of the score (the bottom ones follow the reference's own
    formula); central differences in FP64 pin the top/sigma/log s entries."""
    rs, g, p, d = load_case("tanh_grad")
    wg = _wgrid(d)
    w = torch.from_numpy(d["weights"]).cuda()
    n = len(d["grad"])

    def score(mod):
        h = ctx.upload(mod)
        s, _, _ = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), n)
        ctx.free(h)
        return s

    h = ctx.upload(rs)
    _, gr, _ = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), n)
    ctx.free(h)
    import copy
    eps = 1e-5
    nb, nt = rs.n_bottom, rs.n_top
    checks = {0: "log_s", 1 + nb: "top0", 1 + nb + nt - 1: "toplast", 1 + nb + nt: "sigma_t"}
    for k in checks:
        up, dn = copy.deepcopy(rs), copy.deepcopy(rs)
        if k == 0:
            up.scale, dn.scale = rs.scale * np.exp(eps), rs.scale * np.exp(-eps)
        elif k == 1 + nb + nt:
            up.sigma_top, dn.sigma_top = rs.sigma_top + eps, rs.sigma_top - eps
        else:
            i = k - 1 - nb
            up.top_powers = rs.top_powers.copy(); up.top_powers[i] += eps
            dn.top_powers = rs.top_powers.copy(); dn.top_powers[i] -= eps
        fd = (score(up) - score(dn)) / (2 * eps)
        assert abs(fd - gr[k]) <= 1e-5 * max(abs(gr[k]), 1e-3 * np.abs(gr).max()), (checks[k], fd, gr[k])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_tanh_overflow_pass_matches_reference(ctx, tag):
    """Voxels whose FP64 map overflows: the reference recomputes them in long
    double (field, score and every gradient's overflow pass); here in
    extended range.  (a) the large power scalar and tiny scale a line search
    of toothOptimizer tries, sigma_b = 0, where the reference's bottom
    gradients are not numbers; (b) both polynomials beyond range."""
    rs, g, p, d = load_case("tanh_overflow")
    rs.sigma_top, rs.sigma_bottom, rs.scale = (float(v) for v in d[tag + "_sigmas"])
    wg = _wgrid(d)
    h = ctx.upload(rs)
    w = torch.from_numpy(d["weights"]).cuda()
    f = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    n = 3 + rs.n_top + rs.n_bottom
    sc, gr, st = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), n, d_field=f.data_ptr())
    ctx.free(h)
    assert st["overflowed"] > 0
    ff, rf = f.cpu().numpy().ravel(), d[tag + "_field"].ravel()
    fin = np.isfinite(rf)
    assert np.array_equal(fin, np.isfinite(ff)) and np.array_equal(ff[~fin], rf[~fin])
    # extended range carries ~1e-13 absolute error in log|q| of the
    # recomputed voxels (an exponent of ~1000 in FP64), the rest is FP64-exact
    assert np.max(np.abs(ff[fin] - rf[fin])) <= 1e-11 * max(1.0, np.abs(rf[fin]).max())
    assert abs(sc - d[tag + "_score"]) <= 1e-11 * abs(d[tag + "_score"])
    rg = d[tag + "_grad"]
    assert np.array_equal(np.isnan(gr), np.isnan(rg))
    ok = ~np.isnan(rg)
    np.testing.assert_allclose(gr[ok], rg[ok], rtol=1e-8, atol=1e-12 * max(1e-30, np.abs(rg[ok]).max()))
