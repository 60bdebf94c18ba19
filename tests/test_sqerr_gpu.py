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
    # keep the device tensors alive while their addresses are in use
    p, X, T = dev(lib.params_of(rs)), dev(xyz), dev(t)
    e = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                   max_it, 2.0)
    eo = oracle.sqerr_energy(rs, xyz, t, max_it, 2.0)
    assert abs(e - eo) <= 1e-9 * abs(eo), (e, eo)
    e32 = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                     max_it, 2.0, precision=lib.QJG_FP32)
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
            P = dev(p)
            ctx.energy(P.data_ptr(), nt, nb, len(t), X.data_ptr(), T.data_ptr(), max_it, 2.0,
                       d_iters=it.data_ptr())
            its.append(it.cpu().numpy())
        stable = (its[0] == its[1]) & (its[0] == its[2])
        Xs, Ts = dev(xyz[stable]), dev(t[stable])
        ns = int(stable.sum())
        fds = []
        for hh in (h, h / 2):
            ev = []
            for sgn in (1, -1):
                p = dev(p0.copy())
                p[k] += sgn * hh
                ev.append(ctx.energy(p.data_ptr(), nt, nb, ns, Xs.data_ptr(), Ts.data_ptr(), max_it,
                                     2.0))
            fds.append((ev[0] - ev[1]) / (2 * hh))
        g = torch.empty(len(p0), dtype=torch.float64, device="cuda")
        P0 = dev(p0)
        ctx.energy(P0.data_ptr(), nt, nb, ns, Xs.data_ptr(), Ts.data_ptr(), max_it, 2.0,
                   precision=precision, d_grad=g.data_ptr())
        # fds[0]: step h; Richardson (4 fd(h/2) - fd(h)) / 3 cancels the h^2 term
        out.append((k, fds[0], (4 * fds[1] - fds[0]) / 3, float(g[k]), ns))
    return out


@pytest.mark.parametrize("max_it", [1, 6])
def test_adjoint_matches_central_differences_fp64(ctx, max_it):
    rs, xyz, t = small_case(n=2000)
    nr = rs.n_top + rs.n_bottom
    ks = [0, 1, 2, 3, 4 * (rs.n_top - 1) + 2, 4 * rs.n_top + 1, 4 * (nr - 1) + 3,
          4 * nr, 4 * nr + rs.n_top - 1, 4 * nr + rs.n_top, 5 * nr]
    res = _fd_check(ctx, rs, xyz, t, max_it, ks)
    g = np.array([r[3] for r in res])
    fd = np.array([r[1] for r in res])
    fdr = np.array([r[2] for r in res])
    assert min(r[4] for r in res) > 1500
    # against the extrapolated central difference (truncation O(h^4)): the
    # adjoint is the derivative of the FP64 energy to 1e-5 (vector norm)
    assert np.linalg.norm(g - fdr) <= 1e-5 * np.linalg.norm(fdr), (g, fdr)
    # against the plain central difference with step 1e-4, whose own O(h^2)
    # truncation error grows with the number of iterations
    assert np.linalg.norm(g - fd) <= (1e-5 if max_it == 1 else 1e-4) * np.linalg.norm(fd), (g, fd)


@pytest.fixture(scope="module")
def config4():
    """The differentiation workload at its stated shape: 64 top / 16 bottom
    roots in [-1.2,1.2]^4 (401 parameters), conformal scale, 30 iterations,
    escape radius 2; 20k Poisson-disk samples in [-1,1]^3 with the
    ellipsoid-and-torus targets."""
    from quijibo_gb300.samples import differentiation_workload
    rs, xyz, t, p = differentiation_workload(n_samples=20_000, max_it=30)
    return rs, xyz, t, p


def test_fp32_adjoint_tracks_fp64(ctx, config4):
    """At the workload's shape the FP32 recompute adjoint is within 1e-5
    (vector norm) of the FP64 adjoint."""
    rs, xyz, t, p = config4
    P = dev(lib.params_of(rs))
    n = len(P)
    g64 = torch.empty(n, dtype=torch.float64, device="cuda")
    g32 = torch.empty(n, dtype=torch.float64, device="cuda")
    X, T = dev(xyz), dev(t)
    e64 = ctx.energy(P.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                     p["max_it"], p["escape"], d_grad=g64.data_ptr())
    e32 = ctx.energy(P.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                     p["max_it"], p["escape"], precision=lib.QJG_FP32, d_grad=g32.data_ptr())
    a, b = g64.cpu().numpy(), g32.cpu().numpy()
    assert n == 401 and np.all(np.isfinite(a)) and np.linalg.norm(a) > 0
    assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(a), np.linalg.norm(a - b) / np.linalg.norm(a)
    assert abs(e32 - e64) <= 1e-5 * abs(e64)


def test_adjoint_matches_central_differences_at_workload_shape(ctx, config4):
    """FP64 adjoint against central differences with step 1e-4 (FP64) at
    the workload's shape, on 13 parameters: root coordinates of top and
    bottom roots, top and bottom exponents and log s.  Richardson's
    extrapolation (4 fd(h/2) - fd(h)) / 3 removes the O(h^2) truncation
    term; samples whose iteration count changes under the steps are left
    out of both sides (none at this shape)."""
    rs, xyz, t, p = config4
    nr = rs.n_top + rs.n_bottom
    ks = [0, 1, 2, 3, 4 * 17 + 1, 4 * (rs.n_top - 1) + 2, 4 * rs.n_top + 1, 4 * (nr - 1) + 3,
          4 * nr, 4 * nr + 5, 4 * nr + rs.n_top - 1, 4 * nr + rs.n_top, 5 * nr]
    res = _fd_check(ctx, rs, xyz, t, p["max_it"], ks)
    g = np.array([r[3] for r in res])
    fd = np.array([r[1] for r in res])
    fdr = np.array([r[2] for r in res])
    assert min(r[4] for r in res) >= 0.99 * len(t)
    assert np.linalg.norm(g - fdr) <= 1e-5 * np.linalg.norm(fdr), (g, fdr)
    # every parameter on its own, too
    assert np.all(np.abs(g - fdr) <= 1e-5 * np.abs(fdr)), np.abs(g - fdr) / np.abs(fdr)
    assert np.linalg.norm(g - fd) <= 1e-5 * np.linalg.norm(fd)


@pytest.mark.parametrize("precision", [lib.QJG_FP32, lib.QJG_FP64])
def test_device_lbfgs_decreases_energy(ctx, precision):
    rs, xyz, t = small_case(n=4000)
    p = dev(lib.params_of(rs))
    p0 = p.clone()
    X, T = dev(xyz), dev(t)
    en, st = ctx.fit_lbfgs(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(),
                           T.data_ptr(), 10, 2.0, steps=15, precision=precision)
    assert st["steps"] >= 5
    assert np.all(np.diff(en) <= 0)
    assert en[-1] < 0.9 * en[0]
    assert not torch.equal(p, p0)


@pytest.mark.parametrize("precision", [lib.QJG_FP32, lib.QJG_FP64])
def test_energy_sizes_split_and_repeat(ctx, precision):
    """Empty, single-sample and chunk-boundary sample counts; the energy of
    two disjoint halves adds up to the whole; a repeated call gives the same
    bits (the sums do not depend on which lane took which sample)."""
    rs, xyz, t = small_case(n=4500)
    p = dev(lib.params_of(rs))
    nt, nb = rs.n_top, rs.n_bottom

    def run(lo, hi, grad=True):
        X, T = dev(xyz[lo:hi].reshape(-1, 3)), dev(t[lo:hi])
        g = torch.full((len(p),), 7.0, dtype=torch.float64, device="cuda")
        e = ctx.energy(p.data_ptr(), nt, nb, hi - lo, X.data_ptr(), T.data_ptr(), 6, 2.0,
                       precision=precision, d_grad=g.data_ptr() if grad else 0)
        return e, g.cpu().numpy()

    e0, g0 = run(0, 0)
    assert e0 == 0.0 and not g0.any()
    e1, g1 = run(0, 1)
    assert e1 == run(0, 1, grad=False)[0] and np.all(np.isfinite(g1))
    ea, ga = run(0, 2049)
    eb, gb = run(2049, len(t))
    ew, gw = run(0, len(t))
    assert abs((ea + eb) - ew) <= 1e-12 * abs(ew)
    assert np.linalg.norm((ga + gb) - gw) <= (1e-6 if precision == lib.QJG_FP32 else 1e-12) * np.linalg.norm(gw)
    ew2, gw2 = run(0, len(t))
    assert ew2 == ew and np.array_equal(gw2, gw)
    # the forward alone gives the energy of the gradient call
    assert run(0, len(t), grad=False)[0] == ew


@pytest.mark.parametrize("precision", [lib.QJG_FP32, lib.QJG_FP64])
def test_forward_with_two_samples_per_lane(ctx, precision):
    """The forward kernel with two samples per lane runs the same orbits:
    the same map applications and adjoint steps, the energy and gradient
    within rounding of the one-sample kernel's."""
    rs, xyz, t = small_case(n=3000)
    p = dev(lib.params_of(rs))
    X, T = dev(xyz), dev(t)
    out = []
    try:
        for pairs in (False, True):
            lib.set_energy_pairs(pairs)
            g = torch.empty(len(p), dtype=torch.float64, device="cuda")
            e = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                           10, 2.0, precision=precision, d_grad=g.data_ptr())
            out.append((e, g.cpu().numpy(), ctx.energy_last_work()))
    finally:
        lib.set_energy_pairs(False)
    (e0, g0, w0), (e1, g1, w1) = out
    assert w0 == w1 and w0[0] > 0 and w0[1] > 0
    tol = 1e-5 if precision == lib.QJG_FP32 else 1e-12
    assert abs(e1 - e0) <= tol * abs(e0)
    assert np.linalg.norm(g1 - g0) <= tol * np.linalg.norm(g0)


@pytest.mark.parametrize("nt,nb,exps", [(64, 16, (1,)), (48, 24, (1,)), (8, 4, (1, 2)),
                                         (12, 0, (1, 2))])
def test_adjoint_root_groups_match_one_lane(ctx, nt, nb, exps):
    """The FP32 adjoint with the roots spread over groups of 16 lanes (one
    bottom root per lane up to 16, four above) against
    the one-lane adjoint: within 1e-6 (vector norm; the products and sums run
    in another order), as close to the FP64 adjoint as the one-lane form
    (the 8/4 map with exponents 2 is 3e-4 from FP64 in either FP32 form), the
    same bits on a repeated call, the same orbit steps."""
    rs = draw_rootset(5, nt, nb, -1.2, 1.2, exps=exps)
    rs.scale = conformal_scale(rs, Grid((24, 24, 24), lengths=(2.0, 2.0, 2.0)))
    xyz, _ = poisson_disk(6000, seed=5)
    t = ShapeSDF(5)(xyz)
    p = dev(lib.params_of(rs))
    X, T = dev(xyz), dev(t)

    def run(precision):
        g = torch.empty(len(p), dtype=torch.float64, device="cuda")
        e = ctx.energy(p.data_ptr(), nt, nb, len(t), X.data_ptr(), T.data_ptr(), 12, 2.0,
                       precision=precision, d_grad=g.data_ptr())
        return e, g.cpu().numpy(), ctx.energy_last_work()

    try:
        lib.set_energy_adjoint_roots(False)
        e_one, g_one, w_one = run(lib.QJG_FP32)
        lib.set_energy_adjoint_roots(True)
        e_grp, g_grp, w_grp = run(lib.QJG_FP32)
        e_grp2, g_grp2, _ = run(lib.QJG_FP32)
    finally:
        lib.set_energy_adjoint_roots(True)
    e64, g64, _ = run(lib.QJG_FP64)
    assert w_one == w_grp and w_grp[1] > 0
    assert e_grp == e_one and e_grp2 == e_grp and np.array_equal(g_grp2, g_grp)
    assert np.all(np.isfinite(g_grp)) and np.linalg.norm(g64) > 0
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert rel(g_grp, g_one) <= 1e-6, rel(g_grp, g_one)
    assert rel(g_grp, g64) <= 1.1 * rel(g_one, g64) + 1e-6, (rel(g_grp, g64), rel(g_one, g64))


def test_context_pool_keeps_scratch_until_trim(ctx, config4):
    """The context keeps the scratch its calls free (its memory pool) and
    qjg_trim returns it: a repeated gradient call gives the same bits, and
    trimming frees at least the orbit the forward pass kept (samples x
    iterations x 16 bytes)."""
    rs, xyz, t, p = config4
    P = dev(lib.params_of(rs))
    X, T = dev(xyz), dev(t)
    g = torch.empty(len(P), dtype=torch.float64, device="cuda")

    def run():
        e = ctx.energy(P.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                       p["max_it"], p["escape"], precision=lib.QJG_FP32, d_grad=g.data_ptr())
        return e, g.cpu().numpy()

    e0, g0 = run()
    torch.cuda.synchronize()
    kept = torch.cuda.mem_get_info()[0]
    e1, g1 = run()
    assert e1 == e0 and np.array_equal(g1, g0)
    assert torch.cuda.mem_get_info()[0] >= kept - (2 << 20)  # nothing new mapped
    ctx.trim()
    freed = torch.cuda.mem_get_info()[0] - kept
    assert freed >= 0.9 * len(t) * p["max_it"] * 16, freed
    e2, g2 = run()
    assert e2 == e0 and np.array_equal(g2, g0)


@pytest.mark.parametrize("precision", [lib.QJG_FP32, lib.QJG_FP64])
def test_forward_grid_does_not_change_results(ctx, precision):
    """The forward kernel's grid (the sizing rule on a first call, the earlier
    call's orbit steps on a repeated one, or a fixed block count) decides
    only which lane runs which sample: each sample's value is its own and the
    sums run in sample order, so the energy and the gradient keep their bits
    at every block count."""
    rs, xyz, t = small_case(n=20000)
    p = dev(lib.params_of(rs))
    X, T = dev(xyz), dev(t)

    def run():
        g = torch.empty(len(p), dtype=torch.float64, device="cuda")
        e = ctx.energy(p.data_ptr(), rs.n_top, rs.n_bottom, len(t), X.data_ptr(), T.data_ptr(),
                       20, 2.0, precision=precision, d_grad=g.data_ptr())
        return e, g.cpu().numpy(), ctx.energy_last_work()

    first = run()  # sized by the rule (or by an earlier test's call on as many samples)
    out = [run()]  # sized by the first call's orbit steps
    try:
        for per_sm in (1, 2, 6, 9):
            lib.set_energy_forward_blocks(per_sm)
            out.append(run())
    finally:
        lib.set_energy_forward_blocks(0)
    for e, g, w in out:
        assert e == first[0] and np.array_equal(g, first[1]) and w == first[2]
