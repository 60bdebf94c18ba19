"""CUDA marching cubes against the reference's own meshes and the oracle."""
import numpy as np
import pytest

from conftest import load_case
from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, plain_workload, precision_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class Out:
    """Device output buffers sized for a grid."""

    def __init__(self, n_vox, v_cap=None, t_cap=None):
        self.v_cap = v_cap if v_cap is not None else 3 * n_vox + 16
        self.t_cap = t_cap if t_cap is not None else 5 * n_vox + 16
        self.v64 = torch.empty(3 * self.v_cap, dtype=torch.float64, device="cuda")
        self.v32 = torch.empty(3 * self.v_cap, dtype=torch.float32, device="cuda")
        self.tris = torch.empty(3 * self.t_cap, dtype=torch.int32, device="cuda")

    def kw(self):
        return dict(d_verts64=self.v64.data_ptr(), d_verts32=self.v32.data_ptr(),
                    vert_cap=self.v_cap, d_tris=self.tris.data_ptr(), tri_cap=self.t_cap)

    def result(self, st):
        nv, nt = st["n_verts"], st["n_tris"]
        return (self.v64[:3 * nv].view(-1, 3).cpu().numpy(),
                self.v32[:3 * nv].view(-1, 3).cpu().numpy(),
                self.tris[:3 * nt].view(-1, 3).cpu().numpy())


def field_dev(ctx, h, g, it):
    f = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    ctx.field(h, g, it, f.data_ptr())
    torch.cuda.synchronize()
    return f


def test_linear_matches_reference_exactly(ctx):
    rs, g, p, d = load_case("mesh_plain")
    f = torch.from_numpy(d["field2"].reshape(-1)).cuda()
    out = Out(g.n_voxels)
    _, st = ctx.mesh_field(None, g, None, f.data_ptr(), lib.QJG_EDGE_LINEAR, **out.kw())
    v64, v32, tris = out.result(st)
    np.testing.assert_array_equal(tris, d["linear_tris"])
    np.testing.assert_array_equal(v64, d["linear_verts"])
    np.testing.assert_array_equal(v32, d["linear_verts"].astype(np.float32))


def _bisect_close(v, ref, h):
    """Bisection vertices: identical except where a midpoint value within a
    last-ulp difference of zero takes the other branch (at most h/2 apart)."""
    diff = np.abs(v - ref).max(axis=1)
    assert (diff == 0).mean() > 0.995, (diff > 0).sum()
    assert diff.max() <= 0.5 * h


def test_nonlinear_field_mesher_matches_reference(ctx):
    rs, g, p, d = load_case("mesh_plain")
    h = ctx.upload(rs)
    f = torch.from_numpy(d["field2000"].reshape(-1)).cuda()
    it = ctx.iter_params(p["max_it"], p["escape"])
    out = Out(g.n_voxels)
    _, st = ctx.mesh_field(h, g, it, f.data_ptr(), lib.QJG_EDGE_BISECT, **out.kw())
    v64, _, tris = out.result(st)
    np.testing.assert_array_equal(tris, d["nonlin_tris"])
    _bisect_close(v64, d["nonlin_verts"], g.spacing)
    assert st["n_unbracketed"] == 0 and st["map_evals"] > 2 * st["n_verts"]
    ctx.free(h)


@pytest.mark.parametrize("slab_nz", [0, 1, 5])
def test_streaming_mesher_matches_reference(ctx, slab_nz):
    rs, g, p, d = load_case("mesh_plain")
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"])
    out = Out(g.n_voxels)
    _, st = ctx.mesh_stream(h, g, it, slab_nz=slab_nz, **out.kw())
    v64, _, tris = out.result(st)
    np.testing.assert_array_equal(tris, d["stream_tris"])
    _bisect_close(v64, d["stream_verts"], g.spacing)
    assert st["slabs"] >= 1
    ctx.free(h)


@pytest.mark.parametrize("wl", ["plain", "precision"])
def test_mesh_matches_oracle_64(ctx, oracle, wl):
    if wl == "plain":
        rs, g, p = plain_workload(64, scale="conformal")
    else:
        rs, g, p = precision_workload(64)
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"])
    f = field_dev(ctx, h, g, it)
    fo = oracle.field(rs, g, p["max_it"], p["escape"])["field"]
    assert np.array_equal(f.cpu().numpy().reshape(fo.shape) > 0, fo > 0)
    for mode in (lib.QJG_EDGE_LINEAR, lib.QJG_EDGE_BISECT):
        out = Out(g.n_voxels)
        _, st = ctx.mesh_field(h, g, it, f.data_ptr(), mode, slab_nz=7, **out.kw())
        v64, _, tris = out.result(st)
        o = oracle.mesh(rs, g, fo, mode, p["max_it"], p["escape"])
        np.testing.assert_array_equal(tris, o["tris"])
        if mode == lib.QJG_EDGE_LINEAR:
            np.testing.assert_allclose(v64, o["verts"], rtol=0, atol=1e-12)
        else:
            _bisect_close(v64, o["verts"], g.spacing)
    ctx.free(h)


@pytest.mark.parametrize("res,slab_nz", [((48, 40, 37), 0), ((130, 24, 70), 16)])
def test_dense_random_sign_field_matches_oracle(ctx, oracle, res, slab_nz):
    """A field of random signs: about half of the cubes carry triangles, many
    more per 64-voxel unit than a surface gives, so a slab's cube scan needs
    more block sums than its unit scan (the buffer grows for them); the
    linear mesh equals the oracle's."""
    g = Grid(res)
    f = np.random.RandomState(sum(res)).uniform(-1.0, 1.0, g.n_voxels)
    fd = torch.from_numpy(f).cuda()
    out = Out(g.n_voxels)
    _, st = ctx.mesh_field(None, g, None, fd.data_ptr(), lib.QJG_EDGE_LINEAR, slab_nz=slab_nz,
                           **out.kw())
    v64, _, tris = out.result(st)
    o = oracle.mesh(None, g, f, lib.QJG_EDGE_LINEAR, 1, 2.0)
    assert len(tris) > 2 * g.n_voxels // 3
    np.testing.assert_array_equal(tris, o["tris"])
    np.testing.assert_allclose(v64, o["verts"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("res", [64, 160])
def test_fp32_refine_stream_topology_matches_fp64(ctx, res):
    rs, g, p = precision_workload(res)
    h = ctx.upload(rs)
    res = []
    for prec in (lib.QJG_FP64, lib.QJG_FP32_REFINE):
        it = ctx.iter_params(p["max_it"], p["escape"], precision=prec,
                             refine_pow=lib.QJG_REFINE_INT)
        out = Out(g.n_voxels)
        _, st = ctx.mesh_stream(h, g, it, slab_nz=16, **out.kw())
        res.append((out.result(st), st))
    (a64, _, at), sa = res[0]
    (b64, _, bt), sb = res[1]
    np.testing.assert_array_equal(at, bt)
    assert sb["field"]["refined"] > 0
    # the FP32-first bisection (with its double-float tier for points FP32
    # cannot decide) takes every decision the FP64 one takes, so the vertices
    # are the same doubles
    assert sb["map_evals_fp32"] > sb["map_evals"] and sa["map_evals_fp32"] == 0
    assert sb["map_evals_ff"] > sb["map_evals"] and sa["map_evals_ff"] == 0
    assert sa["n_unbracketed"] == 0 and sb["n_unbracketed"] == 0
    np.testing.assert_array_equal(b64, a64)
    ctx.free(h)


def test_capacity_error_reports_needed_counts(ctx):
    rs, g, p, d = load_case("mesh_plain")
    f = torch.from_numpy(d["field2"].reshape(-1)).cuda()
    out = Out(g.n_voxels, v_cap=10, t_cap=10)
    rc, st = ctx.mesh_field(None, g, None, f.data_ptr(), lib.QJG_EDGE_LINEAR, check=False,
                            **out.kw())
    assert rc == -5
    assert st["n_verts"] == len(d["linear_verts"]) and st["n_tris"] >= len(d["linear_tris"])


def test_degenerate_grids_give_empty_meshes(ctx):
    rs, _, p = plain_workload(8, scale="conformal")
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"])
    for res in [(1, 1, 1), (5, 5, 1), (1, 6, 6), (6, 1, 6)]:
        g = Grid(res)
        out = Out(g.n_voxels)
        _, st = ctx.mesh_stream(h, g, it, **out.kw())
        assert st["n_verts"] == 0 and st["n_tris"] == 0
    ctx.free(h)


def test_phase_timing_of_the_streaming_mesher(ctx):
    rs, g, p = precision_workload(48)
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                         refine_pow=lib.QJG_REFINE_INT)
    out = Out(g.n_voxels)
    _, off = ctx.mesh_stream(h, g, it, slab_nz=16, **out.kw())
    assert off["ms_field"] == 0 and off["ms_classify"] == 0
    ctx.set_timing(True)
    try:
        _, st = ctx.mesh_stream(h, g, it, slab_nz=16, **out.kw())
    finally:
        ctx.set_timing(False)
    assert st["n_tris"] == off["n_tris"] > 0
    for k in ("ms_field", "ms_classify", "ms_vertices", "ms_triangles", "ms_filter"):
        assert st[k] > 0, k
    ctx.free(h)
