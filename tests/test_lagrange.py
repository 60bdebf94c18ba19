"""The Lagrange form of the map (RATIONAL_4D::evaluateLagrange: top and
bottom factors interleaved) and the Lagrange streaming mesher, against the
reference's own outputs (tests/golden/lagrange.npz, written by gen_golden.py)."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, RootSet

GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__file__), "golden",
                                    "lagrange.npz")


def case(tag):
    d = np.load(GOLDEN)
    g = lambda k: d[tag + "_" + k]  # noqa: E731
    rs = RootSet(top_roots=g("top_roots"), top_powers=g("top_powers"),
                 sigma_top=float(g("sigma_top")), bottom_roots=g("bottom_roots").reshape(-1, 4),
                 bottom_powers=g("bottom_powers"), sigma_bottom=float(g("sigma_bottom")),
                 scale=float(g("scale")))
    rs.lagrange = True
    grid = Grid(tuple(int(v) for v in g("res")), tuple(g("center")), tuple(g("lengths")),
                tuple(g("rot")), float(g("slice")))
    return rs, grid, d


@pytest.mark.parametrize("tag", ["a", "b"])
@pytest.mark.parametrize("escape,key", [(2000.0, "field"), (2.0, "field2")])
def test_oracle_lagrange_field_matches_reference(oracle, tag, escape, key):
    rs, g, d = case(tag)
    f = oracle.field(rs, g, 10, escape)["field"].ravel()
    np.testing.assert_array_equal(f, d[tag + "_" + key])


def test_oracle_lagrange_mesh_matches_reference(oracle):
    rs, g, d = case("a")
    f = oracle.field(rs, g, 10, 2000.0)["field"]
    m = oracle.mesh(rs, g, f, 1, 10, 2000.0)
    np.testing.assert_array_equal(m["tris"], d["a_mesh_tris"])
    np.testing.assert_array_equal(m["verts"], d["a_mesh_verts"])


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["a", "b"])
@pytest.mark.parametrize("escape,key", [(2000.0, "field"), (2.0, "field2")])
def test_gpu_lagrange_field_matches_reference(ctx, tag, escape, key):
    rs, g, d = case(tag)
    h = ctx.upload(rs)
    it = ctx.iter_params(10, escape, lagrange=True)
    f, _, _ = ctx.field_host(h, g, it)
    ctx.free(h)
    ref = d[tag + "_" + key]
    rel = np.abs(f.ravel() - ref) / np.maximum(np.abs(ref), 1e-300)
    assert np.array_equal(f.ravel() > 0, ref > 0)
    assert np.quantile(rel, 0.999) <= 1e-12 and rel.max() <= 1e-9


@pytest.mark.gpu
def test_gpu_lagrange_mesh_matches_reference(ctx):
    torch = pytest.importorskip("torch")
    rs, g, d = case("a")
    h = ctx.upload(rs)
    it = ctx.iter_params(10, 2000.0, lagrange=True)
    cap = 4 * g.n_voxels
    v = torch.empty(3 * cap, dtype=torch.float64, device="cuda")
    t = torch.empty(3 * cap, dtype=torch.int32, device="cuda")
    _, st = ctx.mesh_stream(h, g, it, d_verts64=v.data_ptr(), vert_cap=cap, d_tris=t.data_ptr(),
                            tri_cap=cap)
    ctx.free(h)
    tris = t[:3 * st["n_tris"]].cpu().numpy().reshape(-1, 3)
    verts = v[:3 * st["n_verts"]].cpu().numpy().reshape(-1, 3)
    np.testing.assert_array_equal(tris, d["a_mesh_tris"])
    np.testing.assert_allclose(verts, d["a_mesh_verts"], rtol=0, atol=1e-12)
    assert st["n_unbracketed"] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["a", "b"])
@pytest.mark.parametrize("escape,key", [(2000.0, "field"), (2.0, "field2")])
@pytest.mark.parametrize("refine_pow", [lib.QJG_REFINE_INT, lib.QJG_REFINE_POW])
def test_gpu_lagrange_precision_form(ctx, tag, escape, key, refine_pow):
    """The precision form in the Lagrange order (FP32 bulk, double-float
    re-run, FP64 band): the reference's sign map, and every voxel within
    1e-6 relative of the FP64 Lagrange field of the same algebra (which is
    the reference's to 1e-9, above)."""
    rs, g, d = case(tag)
    h = ctx.upload(rs)
    f64, _, _ = ctx.field_host(h, g, ctx.iter_params(10, escape, lagrange=True,
                                                     refine_pow=refine_pow))
    f, _, st = ctx.field_host(h, g, ctx.iter_params(10, escape, precision=lib.QJG_FP32_REFINE,
                                                    refine_pow=refine_pow, rel_tol=1e-6,
                                                    lagrange=True))
    band, _, _ = ctx.field_host(h, g, ctx.iter_params(10, escape, precision=lib.QJG_FP32_REFINE,
                                                      refine_pow=refine_pow, lagrange=True))
    ctx.free(h)
    ref = d[tag + "_" + key].reshape(f.shape)
    assert np.array_equal(f > 0, ref > 0)
    assert np.array_equal(band > 0, ref > 0)
    rel = np.abs(f - f64) / np.maximum(np.abs(f64), 1e-300)
    assert rel.max() <= 1e-6, rel.max()
    assert st["refined"] > 0


@pytest.mark.gpu
def test_gpu_lagrange_precision_mesh_matches_reference(ctx):
    """The streaming mesher in the precision form and the Lagrange order:
    the reference's triangles; bisection decisions taken in FP32 or
    double-float only where they equal FP64's, so the vertices are the FP64
    form's."""
    torch = pytest.importorskip("torch")
    rs, g, d = case("a")
    h = ctx.upload(rs)
    it = ctx.iter_params(10, 2000.0, precision=lib.QJG_FP32_REFINE, refine_pow=lib.QJG_REFINE_INT,
                         rel_tol=1e-6, lagrange=True)
    cap = 4 * g.n_voxels
    v = torch.empty(3 * cap, dtype=torch.float64, device="cuda")
    t = torch.empty(3 * cap, dtype=torch.int32, device="cuda")
    _, st = ctx.mesh_stream(h, g, it, d_verts64=v.data_ptr(), vert_cap=cap, d_tris=t.data_ptr(),
                            tri_cap=cap)
    ctx.free(h)
    tris = t[:3 * st["n_tris"]].cpu().numpy().reshape(-1, 3)
    verts = v[:3 * st["n_verts"]].cpu().numpy().reshape(-1, 3)
    np.testing.assert_array_equal(tris, d["a_mesh_tris"])
    np.testing.assert_allclose(verts, d["a_mesh_verts"], rtol=0, atol=1e-12)
    assert st["n_unbracketed"] == 0 and st["map_evals_fp32"] > 0
