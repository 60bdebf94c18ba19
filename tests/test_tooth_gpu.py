"""toothOptimizer's run on the GPU (qjg_tooth_optimize) against the
reference's own main loop (tests/golden/tooth.npz: ref_tooth_run, i.e.
OPTIMIZE_3D::read, the frame change, the amplitude, and per level the
conformal scan, the scaled-only, scaled and unweighted solves through
TAO_SOLVER::optimizeBLMVM), plus the reweighting arithmetic."""
import os

import numpy as np
import pytest

from quijibo_gb300 import lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLD = dict(np.load(os.path.join(GOLDEN, "tooth.npz")))


def level_state(path):
    st = lib.o3d_read(path)
    return np.concatenate([st["bottom_powers"], st["top_powers"],
                           [st["sigma_top"], st["sigma_bottom"], st["scale"]]]), st


# The reference's run amplifies rounding: moving its input roots by 1e-12
# (relative) moves its end states by up to 1.7e-6 / 9.5e-5 in the exponents
# and power scalars, 1.2e-3 / 2.1e-2 in the scale, and 8.5e-12 / 1.3e-8 in the
# level's final score (cases a / b), with the same evaluation counts.  The GPU
# score and gradients differ from the reference's by ~1e-12, so the end states
# are compared at ten times those spreads.
RTOL = {"a": (1.7e-5, 1.2e-2, 1e-10), "b": (1e-3, 0.2, 1.3e-7)}


@pytest.mark.parametrize("tag", ["a", "b"])
def test_run_matches_reference(ctx, tag, tmp_path):
    levels = tuple(int(v) for v in GOLD["levels"])
    out = ctx.tooth_optimize(os.path.join(GOLDEN, "tooth_input_%s.o3d" % tag), levels,
                             float(GOLD["radius"]), float(GOLD[tag + "_amp"]),
                             output_prefix=str(tmp_path / "run"))
    ref, ev = GOLD[tag + "_out"], GOLD[tag + "_evals"]
    r_par, r_scale, r_score = RTOL[tag]
    for l, res in enumerate(levels):
        L = out[l]
        assert L["res"] == res and L["reweighted"] == 0
        assert [L["solve"][k]["evaluations"] for k in (0, 1, 3)] == ev[l].tolist()
        state, st = level_state(str(tmp_path / ("run_res_%d.o3d" % res)))
        np.testing.assert_allclose(state[:-1], ref[l][:-2], rtol=r_par, atol=1e-12)
        assert abs(state[-1] - ref[l][-2]) <= r_scale * abs(ref[l][-2])
        assert abs(L["final_score"] - ref[l][-1]) <= r_score * abs(ref[l][-1])
        assert st["fractal"][0] == (res, res, res)
        # OPTIMIZE_3D::write's header: the resolution and box setScoreFields took
        # from the distance field
        assert st["res"] == st["distance"][0] and st["center"] == st["distance"][1]
    # the frame change moves the roots exactly as the reference does
    roots = np.concatenate([st["top_roots"].reshape(-1, 4), st["bottom_roots"].reshape(-1, 4)])
    assert np.array_equal(roots, GOLD[tag + "_roots"])


def test_reweight_matches_restatement(ctx):
    from oracle.oracle import reweight_inside
    rng = np.random.RandomState(5)
    n = 50_000
    md = rng.uniform(-1, 1, n)
    fd = md + rng.uniform(-0.3, 0.3, n)
    w = np.where(md < 0, -1.0, 0.25) * rng.uniform(0.1, 1.0, n)
    d = [torch.from_numpy(a).cuda() for a in (md, fd, w)]
    o = torch.empty_like(d[2])
    poor, well = ctx.reweight_inside(n, d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(),
                                     o.data_ptr())
    ref, rp, rw = reweight_inside(md, fd, w)
    assert abs(poor - rp) <= 1e-12 * abs(rp) and abs(well - rw) <= 1e-12 * abs(rw)
    np.testing.assert_allclose(o.cpu().numpy(), ref, rtol=1e-12, atol=0)


def test_run_with_reweighting_and_checkpoints(ctx, tmp_path):
    """The reweighted solve: the level's mesh goes to the signed-distance
    callback (standing in for the reference's sdfGen), its answer reweights
    the inside; the monitor's state file is written."""
    from oracle.oracle import reweight_inside
    calls = []
    holder = {}

    def sdf(verts, tris, grid):
        calls.append((len(verts), len(tris), tuple(grid.res)))
        st = lib.o3d_read(os.path.join(GOLDEN, "tooth_input_a.o3d"))
        # the target's distance in the fractal frame, shifted: some inside
        # cells become "missed", the rest "covered"
        fd = st["distance"][3].ravel() * 4.0 + 0.15
        holder["fd"] = fd
        return fd
    ck = tmp_path / "output.o3d"
    out = ctx.tooth_optimize(os.path.join(GOLDEN, "tooth_input_a.o3d"), (12,), 4.0,
                             float(GOLD["a_amp"]), output_prefix=str(tmp_path / "rw"),
                             checkpoint_path=str(ck), sdf=sdf)
    L = out[0]
    assert L["reweighted"] == 1 and len(calls) == 1
    assert calls[0][1] == L["mesh_tris"] > 0 and calls[0][2] == (14, 16, 18)
    assert L["solve"][2]["evaluations"] >= 1
    # the region sums agree with the restatement on the same fields
    st = lib.o3d_read(str(tmp_path / "rw_res_12.o3d"))
    md = st["distance"][3].ravel()
    dres = st["distance"][0]
    dd = torch.from_numpy(np.ascontiguousarray(lib.o3d_read(
        os.path.join(GOLDEN, "tooth_input_a.o3d"))["distance"][3].ravel())).cuda()
    w = torch.empty_like(dd)
    ctx.inverted_distance(dres, dd.data_ptr(), True, w.data_ptr())
    _, rp, rw = reweight_inside(md, holder["fd"], w.cpu().numpy())
    assert abs(L["poor_sum"] - rp) <= 1e-12 * abs(rp)
    assert abs(L["well_sum"] - rw) <= 1e-12 * abs(rw)
    assert L["checkpoints"] >= 1 and ck.exists()
    assert lib.o3d_read(str(ck))["fractal"][0] == (12, 12, 12)


def test_run_rejects_bad_configuration(ctx, tmp_path):
    with pytest.raises(lib.QjgError):
        ctx.tooth_optimize(str(tmp_path / "missing.o3d"), (12,))
    with pytest.raises(lib.QjgError):
        ctx.tooth_optimize(os.path.join(GOLDEN, "tooth_input_a.o3d"), (1,))
    with pytest.raises(lib.QjgError):
        ctx.tooth_optimize(os.path.join(GOLDEN, "tooth_input_a.o3d"), (12,), fractal_radius=0.0)
