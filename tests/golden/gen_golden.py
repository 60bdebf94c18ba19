"""Generate the golden fixtures of the hot path from the reference itself.

The reference QUIJIBO is compiled from its own sources by oracle/Makefile
(`make -C oracle ref`) into oracle/_ref/ in two flavours: Real=double and the
shipped default Real=long double.  This script runs it through
oracle/ref_harness.cpp on small seeded cases and stores inputs and outputs in
tests/golden/*.npz.  The reference sources exist only in the development
container, so the fixtures are committed and the tests read them anywhere.

    python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402
from quijibo_gb300.rootsets import (Grid, RootSet, draw_rootset, plain_workload,  # noqa: E402
                                    precision_workload)

OUT = os.path.dirname(os.path.abspath(__file__))


def rs_dict(prefix, rs, g, params):
    return {prefix + "top_roots": rs.top_roots, prefix + "top_powers": rs.top_powers,
            prefix + "sigma_top": rs.sigma_top, prefix + "bottom_roots": rs.bottom_roots,
            prefix + "bottom_powers": rs.bottom_powers, prefix + "sigma_bottom": rs.sigma_bottom,
            prefix + "scale": rs.scale, prefix + "res": np.array(g.res),
            prefix + "center": np.array(g.center), prefix + "lengths": np.array(g.lengths),
            prefix + "rot": np.array(g.rot), prefix + "slice": g.slice,
            prefix + "max_it": params["max_it"], prefix + "escape": params["escape"]}


def main():
    rd, rl = Reference("double"), Reference("ldouble")
    assert rd.sizeof_real == 8 and rl.sizeof_real == 16

    # MT19937 draws and QUATERNION::pow known answers
    mt = {"mt_seed0": rd.mt_rand(0, 64), "mt_seed12345": rd.mt_rand(12345, 64)}
    rng = np.random.RandomState(7)
    qs = np.concatenate([rng.uniform(-2, 2, (40, 4)),
                         [[1.5, 0, 0, 0], [-1.5, 0, 0, 0], [0.5, 1e-9, 0, 0], [0.0, 0.3, -0.2, 0.1]]])
    es = np.concatenate([rng.choice([1.0, 2.0, 3.0, 0.5, 1.7, 0.25], 40), [2.0, 3.0, 1.0, 2.5]])
    pw = np.array([rd.quat_pow(q, e) for q, e in zip(qs, es)])
    np.savez_compressed(os.path.join(OUT, "algebra.npz"), pow_q=qs, pow_e=es, pow_out=pw, **mt)

    cases = {}
    # plain method, literal unit scale and conformal scale
    for name, scale in (("plain_unit", "unit"), ("plain_conf", "conformal")):
        rs, g, p = plain_workload(32, scale=scale)
        cases[name] = (rs, g, p)
    # precision form roots at 32^3
    cases["prec"] = precision_workload(32)
    # rotated, shifted grid with a non-zero slice and non-integer exponents
    rs = draw_rootset(3, 6, 3, -1.0, 1.0, exps=(1, 2))
    rs.top_powers = rs.top_powers * np.array([1.0, 0.5, 1.0, 1.5, 1.0, 1.0])
    rs.sigma_top, rs.sigma_bottom = 1.1, 0.9
    rot = np.array([0.9, 0.1, -0.2, 0.3])
    rot = rot / np.linalg.norm(rot)
    g = Grid((24, 20, 16), center=(0.1, -0.2, 0.05), lengths=(2.8, 2.6, 2.4), rot=tuple(rot),
             slice=0.15)
    from quijibo_gb300.rootsets import conformal_scale
    rs.scale = conformal_scale(rs, g)
    cases["general"] = (rs, g, dict(max_it=12, escape=2.0))

    for name, (rs, g, p) in cases.items():
        d = rs_dict("", rs, g, p)
        d["field"] = rd.field_escape(rs, g, p["max_it"], p["escape"])
        d["field_ld"] = rl.field_escape(rs, g, p["max_it"], p["escape"])
        np.savez_compressed(os.path.join(OUT, "field_%s.npz" % name), **d)

    # the unmodified OPTIMIZE_3D::computeLogScaledPowerRationalMap (escape 2000)
    rs, g, p = precision_workload(24)
    p = dict(max_it=10, escape=2000.0)
    d = rs_dict("", rs, g, p)
    d["field"] = rd.field_map(rs, g, p["max_it"])
    np.savez_compressed(os.path.join(OUT, "field_map2000.npz"), **d)

    # marching cubes: streaming nonlinear, nonlinear on a stored field, linear
    rs, g, p = plain_workload(32, scale="conformal")
    p = dict(max_it=20, escape=2000.0)
    d = rs_dict("", rs, g, p)
    ms = rd.mesh_stream(rs, g, p["max_it"])
    d["stream_verts"], d["stream_tris"] = ms["verts"], ms["tris"]
    f2000 = rd.field_map(rs, g, p["max_it"])
    d["field2000"] = f2000
    mn = rd.mesh_field_nonlinear(rs, g, f2000, p["max_it"])
    d["nonlin_verts"], d["nonlin_tris"] = mn["verts"], mn["tris"]
    f2 = rd.field_escape(rs, g, 20, 2.0)
    d["field2"] = f2
    ml = rd.mesh_linear(g, f2)
    d["linear_verts"], d["linear_tris"] = ml["verts"], ml["tris"]
    np.savez_compressed(os.path.join(OUT, "mesh_plain.npz"), **d)
    rs, g, wg, w = tanh_case()
    rd2 = Reference("double")
    d = rs_dict("", rs, g, dict(max_it=1, escape=20.0))
    sc, gr, f = rd2.tanh_score_grad(rs, g, wg, w, 1)
    d.update(score=sc, grad=gr, field=f, weights=w, wres=np.array(wg.res),
             wcenter=np.array(wg.center), wlengths=np.array(wg.lengths))
    np.savez_compressed(os.path.join(OUT, "tanh_grad.npz"), **d)

    io_case(rd)
    blmvm_case(rd)
    tanh_fit_case(rd)
    tooth_case(rd)
    tanh_overflow_case(rd)
    conformal_case(rd)
    lagrange_case(rd)
    o3d_case(rd)

    print("stream: %d verts %d tris; nonlinear: %d/%d; linear: %d/%d" % (
        len(ms["verts"]), len(ms["tris"]), len(mn["verts"]), len(mn["tris"]), len(ml["verts"]),
        len(ml["tris"])))


def io_inputs():
    """A small field and mesh with values that exercise the number formats:
    signed zeros, tiny and large magnitudes, values that round at the 16th
    decimal."""
    field = np.array([0.0, -0.0, 1.0, -1.0, 1e-300, -2.5e-17, 3.141592653589793, 1e10,
                      -123456.7890123456, 0.1, 2.0 / 3.0, 7.0]).reshape(2, 2, 3)
    res, center, lengths = (3, 2, 2), (0.25, -0.5, 1.0), (3.0, 2.0, 2.5)
    verts = np.array([[0.0, -0.0, 1.0], [1e-17, -1e-17, 0.5], [0.1, 0.2, 0.3],
                      [-1.2345678901234567, 98765.4321, 1.0 / 3.0], [2.5, -2.5, 1e-5],
                      [0.9999999999999999, -0.30000000000000004, 4.440892098500626e-16]])
    tris = np.array([[0, 1, 2], [2, 3, 4], [4, 5, 0], [1, 3, 5]], dtype=np.int32)
    return field, res, center, lengths, verts, tris


def io_case(rd):
    """FIELD_3D::write, TRIANGLE_MESH::writeOBJ and TRIANGLE_MESH::write output
    bytes of io_inputs()."""
    field, res, center, lengths, verts, tris = io_inputs()
    rd.field_write(os.path.join(OUT, "io_field.field3d"), res, center, lengths, field)
    rd.mesh_write(verts, tris, os.path.join(OUT, "io_mesh.obj"), os.path.join(OUT, "io_mesh.raw"))


def lagrange_case(rd):
    """RATIONAL_4D::evaluateLagrange fields (more top than bottom roots, and
    more bottom than top) and the Lagrange streaming mesher."""
    from quijibo_gb300.rootsets import conformal_scale
    d = {}
    for tag, (nt, nb, seed) in (("a", (6, 3, 31)), ("b", (3, 5, 32))):
        rs = draw_rootset(seed, nt, nb, -1.0, 1.0, exps=(1, 2))
        rs.sigma_top, rs.sigma_bottom = 1.0, 1.0
        g = Grid((24, 22, 20), slice=0.1)
        rs.scale = conformal_scale(rs, g)
        d.update(rs_dict(tag + "_", rs, g, dict(max_it=10, escape=2000.0)))
        d[tag + "_field"] = rd.field_lagrange(rs, g, 10, 2000.0)
        d[tag + "_field2"] = rd.field_lagrange(rs, g, 10, 2.0)
    # the mesher on case a
    rs = draw_rootset(31, 6, 3, -1.0, 1.0, exps=(1, 2))
    g = Grid((24, 22, 20), slice=0.1)
    rs.scale = conformal_scale(rs, g)
    m = rd.mesh_lagrange(rs, g, 10)
    d["a_mesh_verts"], d["a_mesh_tris"] = m["verts"], m["tris"]
    np.savez_compressed(os.path.join(OUT, "lagrange.npz"), **d)
    return len(m["tris"])


def o3d_inputs():
    """A small optimizer state: map, fractal, distance (with a sign change)
    and curvature fields."""
    rs = draw_rootset(41, 4, 2, -1.0, 1.0, exps=(1, 2))
    rs.sigma_top, rs.sigma_bottom, rs.scale = 1.25, 0.75, 0.625
    g = Grid((6, 5, 4), center=(0.1, -0.2, 0.3), lengths=(3.0, 2.5, 2.0))
    dg = Grid((5, 4, 3), center=(0.0, 0.05, -0.05), lengths=(2.5, 2.0, 1.5))
    rng = np.random.RandomState(41)
    fractal = rng.standard_normal(g.n_voxels)
    dist = np.linspace(-1.0, 1.0, dg.n_voxels) + 0.013
    curv = rng.uniform(-2, 2, dg.n_voxels)
    return rs, g, fractal, dg, dist, curv


def o3d_case(rd):
    """OPTIMIZE_3D::write of o3d_inputs()."""
    rs, g, fractal, dg, dist, curv = o3d_inputs()
    rd.o3d_write(os.path.join(OUT, "io_state.o3d"), rs, g, fractal, dg, dist, curv)


def conformal_inputs():
    """Map, fractal grid and a signed distance field (union of two
    ellipsoids, negative inside) on a different grid, for the weight field
    and the conformal-radius scan."""
    from quijibo_gb300.rootsets import cell_centers
    rs = draw_rootset(21, 6, 3, -1.0, 1.0, exps=(1, 2))
    rs.sigma_top, rs.sigma_bottom, rs.scale = 1.1, 0.9, 0.37  # the scan ignores all three
    g = Grid((20, 20, 20), slice=0.05)
    dg = Grid((18, 16, 14), center=(0.05, -0.02, 0.0), lengths=(3.2, 3.0, 2.8))
    c = cell_centers(dg)
    e1 = np.sqrt(((c - [0.3, 0.0, 0.1]) ** 2 / np.array([0.6, 0.45, 0.5]) ** 2).sum(1)) - 1.0
    e2 = np.sqrt(((c - [-0.4, 0.2, -0.1]) ** 2 / np.array([0.35, 0.5, 0.4]) ** 2).sum(1)) - 1.0
    dist = np.minimum(e1 * 0.45, e2 * 0.35)
    return rs, g, dg, dist


def conformal_case(rd):
    """FIELD_3D::invertedDistance[Normalized] and estimateConformalRadius."""
    rs, g, dg, dist = conformal_inputs()
    d = rs_dict("", rs, g, dict(max_it=1, escape=20.0))
    d.update(dres=np.array(dg.res), dcenter=np.array(dg.center), dlengths=np.array(dg.lengths),
             dist=dist, inv=rd.inverted_distance(dg, dist, False),
             inv_norm=rd.inverted_distance(dg, dist, True))
    score, es = rd.conformal_radius(rs, g, dg, dist)
    d.update(score=score, exp_scaling=es)
    np.savez_compressed(os.path.join(OUT, "conformal.npz"), **d)


def blmvm_case(rd):
    """TAO_SOLVER::optimizeBLMVM on the objectives of blmvm_problems.py:
    every evaluated point and value, and the solution."""
    from blmvm_problems import problems
    d = {}
    for name, (fun, x0, lo, hi) in problems().items():
        x, hist = rd.blmvm(lambda v: fun(list(v)), x0, lo, hi)
        d[name + "_x"] = x
        d[name + "_f"] = np.array([h[0] for h in hist])
        d[name + "_pts"] = np.array([h[1] for h in hist])
    np.savez_compressed(os.path.join(OUT, "blmvm.npz"), **d)


def tanh_fit_inputs():
    """Two toothOptimizer fits: (a) the tanh_case map, grid and weights;
    (b) the conformal_case map at 25^3 from its conformal scale, weights the
    normalized inverted distance x 100."""
    import copy
    rs_a, g_a, wg_a, w_a = tanh_case()
    rs_b, _, dg, dist = conformal_inputs()
    rs_b = copy.deepcopy(rs_b)
    rs_b.sigma_top = rs_b.sigma_bottom = 1.0
    return [("a", rs_a, g_a, wg_a, w_a), ("b", rs_b, Grid((25, 25, 25), slice=0.05), dg, dist)]


def tanh_fit_case(rd):
    """callConstrainedScaledOnlyTao then callConstrainedScaledTao from its
    result, as optimizeSpecificResolution runs them
    (toothOptimizer.cpp:410-415)."""
    d = {}
    for tag, rs, g, wg, w in tanh_fit_inputs():
        if tag == "b":
            w = rd.inverted_distance(wg, w, True) * 100.0
            _, rs.scale = rd.conformal_radius(rs, Grid((20, 20, 20), slice=0.05), wg,
                                              tanh_fit_inputs()[1][4])
        d.update(rs_dict(tag + "_", rs, g, dict(max_it=1, escape=20.0)))
        d.update({tag + "_weights": w, tag + "_wres": np.array(wg.res),
                  tag + "_wcenter": np.array(wg.center), tag + "_wlengths": np.array(wg.lengths)})
        for mode in (0, 1):
            out, hist = rd.tanh_fit(mode, rs, g, wg, w, 1)
            d["%s_out%d" % (tag, mode)] = out
            d["%s_hist%d" % (tag, mode)] = hist
            nb, nt = rs.n_bottom, rs.n_top
            rs.bottom_powers, rs.top_powers = out[:nb].copy(), out[nb:nb + nt].copy()
            rs.sigma_top, rs.sigma_bottom, rs.scale = out[-3], out[-2], out[-1]
    np.savez_compressed(os.path.join(OUT, "tanh_fit.npz"), **d)


TOOTH_LEVELS = (12, 16, 20)
# seed, amp, root spread: of 48 such problems these two are the ones whose
# reference run keeps its evaluation counts when the input roots move by
# 1e-12 (the rest amplify such a change to O(1) differences)
TOOTH_CASES = {"a": (9, 0.8, 0.2), "b": (1, 1.0, 0.2)}


def tooth_inputs(seed, spread):
    """A toothOptimizer problem in the unit-cube frame of its input files:
    the signed distance of an ellipsoid (negative inside) on a 14 x 16 x 18
    grid over [0, 1]^3; 5 top roots (the first at the origin, the rest within
    `spread` of the centre) and 3 bottom roots (the first near the origin),
    exponents 1 or 2."""
    from quijibo_gb300.rootsets import cell_centers
    rng = np.random.RandomState(seed)
    nt, nb = 5, 3
    top = np.zeros((nt, 4))
    top[1:, :3] = 0.5 + rng.uniform(-spread, spread, (nt - 1, 3))
    top[1:, 3] = rng.uniform(-0.05, 0.05, nt - 1)
    bot = np.zeros((nb, 4))
    bot[:, :3] = 0.5 + rng.uniform(-1.5 * spread, 1.5 * spread, (nb, 3))
    bot[0, :3] = 0.03
    rs = RootSet(top_roots=top, top_powers=rng.choice([1.0, 2.0], nt), bottom_roots=bot,
                 bottom_powers=rng.choice([1.0, 2.0], nb), sigma_top=1.0, sigma_bottom=1.0,
                 scale=1.0)
    dg = Grid((14, 16, 18), center=(0.5, 0.5, 0.5), lengths=(1.0, 1.0, 1.0))
    c = cell_centers(dg) - 0.5
    r = np.sqrt(((c / np.array([0.3, 0.24, 0.2])) ** 2).sum(1))
    dist = (r - 1.0) * 0.22
    g = Grid((4, 4, 4), center=(0.5, 0.5, 0.5), lengths=(1.0, 1.0, 1.0))
    return rs, g, np.zeros(g.n_voxels), dg, dist, dist.copy()


def tooth_case(rd):
    """toothOptimizer's run (without the sdfGen-dependent reweighted solve)
    on tooth_input_<case>.o3d, written by the reference's OPTIMIZE_3D::write,
    at levels TOOTH_LEVELS with fractal radius 4."""
    d = {"levels": np.array(TOOTH_LEVELS), "radius": 4.0}
    for tag, (seed, amp, spread) in TOOTH_CASES.items():
        rs, g, fractal, dg, dist, curv = tooth_inputs(seed, spread)
        path = os.path.join(OUT, "tooth_input_%s.o3d" % tag)
        rd.o3d_write(path, rs, g, fractal, dg, dist, curv)
        out, ev, roots = rd.tooth_run(path, rs.n_top, rs.n_bottom, TOOTH_LEVELS, 4.0, amp)
        d.update({tag + "_out": out, tag + "_evals": ev, tag + "_roots": roots, tag + "_amp": amp,
                  tag + "_n_top": rs.n_top, tag + "_n_bot": rs.n_bottom})
    np.savez_compressed(os.path.join(OUT, "tooth.npz"), **d)


def tanh_overflow_case(rd):
    """The tanh score and gradients where the FP64 map overflows, so the
    reference recomputes voxels in long double: the tooth_inputs("a") map in
    the fractal frame on a 12^3 grid with (a) the large power scalar and small
    scale a BLMVM line search tries (sigma_t 162.73, sigma_b 0, s e^-35.86),
    (b) both polynomials beyond range (sigma_t = sigma_b = 140, s = 1)."""
    seed, amp, spread = TOOTH_CASES["a"]
    rs, _, _, dg, dist, _ = tooth_inputs(seed, spread)
    w = rd.inverted_distance(dg, dist, True)
    R = 4.0
    tr, br = rs.top_roots.copy(), rs.bottom_roots.copy()
    tr[1:, :3] += -0.5
    br[1:, :3] += -0.5
    rs.top_roots, rs.bottom_roots = tr * R, br * R
    rs.top_powers[1:] *= amp
    rs.bottom_powers[1:] *= amp
    c = (np.array(dg.center) - 0.5) * R
    wg = Grid(dg.res, tuple(c), tuple(np.array(dg.lengths) * R))
    g = Grid((12, 12, 12), tuple(c), wg.lengths)
    d = rs_dict("", rs, g, dict(max_it=1, escape=20.0))
    d.update(weights=w, wres=np.array(wg.res), wcenter=np.array(wg.center),
             wlengths=np.array(wg.lengths))
    for tag, (st, sb, sc) in (("a", (162.72999184, 0.0, np.exp(-35.86015467))),
                              ("b", (140.0, 140.0, 1.0))):
        rs.sigma_top, rs.sigma_bottom, rs.scale = st, sb, sc
        score, grad, field = rd.tanh_score_grad(rs, g, wg, w, 1)
        d.update({tag + "_sigmas": np.array([st, sb, sc]), tag + "_score": score,
                  tag + "_grad": grad, tag + "_field": field})
    np.savez_compressed(os.path.join(OUT, "tanh_overflow.npz"), **d)


def tanh_case():
    """The tanh-weighted score and gradients (maxIterations 1, as toothOptimizer
    runs them) on a 16^3 grid with a weight field on a different grid."""
    from quijibo_gb300.rootsets import cell_centers, conformal_scale
    rs = draw_rootset(11, 8, 4, -1.0, 1.0, exps=(1, 2))
    rs.sigma_top, rs.sigma_bottom = 1.05, 0.95
    g = Grid((16, 16, 16))
    rs.scale = conformal_scale(rs, g)
    wg = Grid((12, 12, 12), center=(0.05, 0.0, -0.05), lengths=(3.2, 3.2, 3.2))
    c = cell_centers(wg)
    w = np.exp(-np.sum(c ** 2, axis=1)) * np.cos(2 * c[:, 0]) + 0.3
    return rs, g, wg, w


if __name__ == "__main__":
    main()
