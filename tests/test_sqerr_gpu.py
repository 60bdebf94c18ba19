"""Squared-error energy on the distance estimate: forward against the oracle,
adjoint gradient against central finite differences (FP64, step 1e-4)."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, conformal_scale, draw_rootset
from quijibo_gb300.samples import ShapeSDF, poisson_disk

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def small_case(n=3000, nt=8, nb=4, seed=2):
    rs = draw_rootset(seed, nt, nb, -1.2, 1.2, exps=(1, 2))
    rs.scale = conformal_scale(rs, Grid((24, 24, 24), lengths=(2.0, 2.0, 2.0)))
    xyz, _ = poisson_disk(n, seed=seed)
    return rs, xyz, ShapeSDF(seed)(xyz)


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


@pytest.mark.parametrize("max_it", [1, 10])
def test_forward_matches_oracle(ctx, oracle, max_it):
    rs, xyz, t = small_case()
    p = dev(lib.params_of(rs))
    e = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), dev(xyz).data_ptr(),
                   dev(t).data_ptr(), max_it, 2.0)
    eo = oracle.sqerr_energy(rs, xyz, t, max_it, 2.0)
    assert abs(e - eo) <= 1e-9 * abs(eo), (e, eo)
    e32 = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), dev(xyz).data_ptr(),
                     dev(t).data_ptr(), max_it, 2.0, precision=lib.QJG_FP32)
    assert abs(e32 - eo) <= 1e-3 * abs(eo)


def _fd_check(ctx, rs, xyz, t, max_it, params_to_check, h=1e-4, precision=lib.QJG_FP64):
    nt, nb = rs.n_top, rs.n_bottom
    p0 = lib.params_of(rs)
    X, T = dev(xyz), dev(t)
    out = []
    for k in params_to_check:
        its = []
        for sgn in (0, 1, -1):
            p = p0.copy()
            p[k] += sgn * h
            it = torch.empty(len(t), dtype=torch.int32, device="cuda")
            ctx.energy(dev(p).data_ptr(), nt, nb, len(t), X.data_ptr(), T.data_ptr(), max_it, 2.0,
                       d_iters=it.data_ptr())
            its.append(it.cpu().numpy())
        stable = (its[0] == its[1]) & (its[0] == its[2])
        Xs, Ts = dev(xyz[stable]), dev(t[stable])
        ns = int(stable.sum())
        ev = []
        for sgn in (1, -1):
            p = p0.copy()
            p[k] += sgn * h
            ev.append(ctx.energy(dev(p).data_ptr(), nt, nb, ns, Xs.data_ptr(), Ts.data_ptr(), max_it,
                                 2.0))
        fd = (ev[0] - ev[1]) / (2 * h)
        g = torch.empty(len(p0), dtype=torch.float64, device="cuda")
        ctx.energy(dev(p0).data_ptr(), nt, nb, ns, Xs.data_ptr(), Ts.data_ptr(), max_it, 2.0,
                   precision=precision, d_grad=g.data_ptr())
        out.append((k, fd, float(g[k]), ns))
    return out


@pytest.mark.parametrize("max_it", [1, 6])
def test_adjoint_matches_central_differences_fp64(ctx, max_it):
    rs, xyz, t = small_case(n=2000)
    nr = rs.n_top + rs.n_bottom
    ks = [0, 1, 2, 3, 4 * (rs.n_top - 1) + 2, 4 * rs.n_top + 1, 4 * (nr - 1) + 3,
          4 * nr, 4 * nr + rs.n_top - 1, 4 * nr + rs.n_top, 5 * nr]
    for k, fd, g, ns in _fd_check(ctx, rs, xyz, t, max_it, ks):
        assert ns > 1500
        assert abs(g - fd) <= 1e-5 * max(abs(fd), 1e-6), (k, g, fd)


def test_fp32_adjoint_tracks_fp64(ctx):
    rs, xyz, t = small_case(n=2000)
    p = dev(lib.params_of(rs))
    n = len(p)
    g64 = torch.empty(n, dtype=torch.float64, device="cuda")
    g32 = torch.empty(n, dtype=torch.float64, device="cuda")
    X, T = dev(xyz), dev(t)
    ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(), 6, 2.0,
               d_grad=g64.data_ptr())
    ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(), 6, 2.0,
               precision=lib.QJG_FP32, d_grad=g32.data_ptr())
    a, b = g64.cpu().numpy(), g32.cpu().numpy()
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    assert rel < 1e-2, rel


@pytest.mark.parametrize("precision", [lib.QJG_FP32, lib.QJG_FP64])
def test_device_lbfgs_decreases_energy(ctx, precision):
    rs, xyz, t = small_case(n=4000)
    p = dev(lib.params_of(rs))
    p0 = p.clone()
    en, st = ctx.fit_lbfgs(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), dev(xyz).data_ptr(),
                           dev(t).data_ptr(), 10, 2.0, steps=15, precision=precision)
    assert st["steps"] >= 5
    assert np.all(np.diff(en) <= 0)
    assert en[-1] < 0.9 * en[0]
    assert not torch.equal(p, p0)
