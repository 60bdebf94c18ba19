"""The streaming mesher as a fixed launch sequence (qjg_mesh_prepare,
qjg_mesh_stream_async, qjg_mesh_async_result): every count stays on the
device, so the whole mesh can be captured into a CUDA graph.  It gives
qjg_mesh_stream's vertices, triangles and counters bit for bit, run directly
or replayed from a graph, and reports a mesh that outgrows its capacities."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import plain_workload, precision_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

KEYS = ("n_verts", "n_tris", "n_degenerate", "slabs", "map_evals", "map_evals_fp32",
        "map_evals_ff", "n_unbracketed")


class Bufs:
    def __init__(self, vcap, tcap):
        self.vcap, self.tcap = vcap, tcap
        self.v64 = torch.zeros(3 * vcap, dtype=torch.float64, device="cuda")
        self.v32 = torch.zeros(3 * vcap, dtype=torch.float32, device="cuda")
        self.tris = torch.zeros(3 * tcap, dtype=torch.int32, device="cuda")

    def kw(self):
        return dict(d_verts64=self.v64.data_ptr(), d_verts32=self.v32.data_ptr(),
                    vert_cap=self.vcap, d_tris=self.tris.data_ptr(), tri_cap=self.tcap)

    def out(self, st):
        nv, nt = st["n_verts"], st["n_tris"]
        return (self.v64[:3 * nv].cpu().numpy(), self.v32[:3 * nv].cpu().numpy(),
                self.tris[:3 * nt].cpu().numpy())

    def clear(self):
        self.v64.zero_()
        self.v32.zero_()
        self.tris.zero_()


def case(name):
    if name == "plain":
        rs, g, p = plain_workload(40, scale="conformal")
        return rs, g, p, dict(precision=lib.QJG_FP64), 0
    rs, g, p = precision_workload(56)
    if name == "precision":
        return rs, g, p, dict(precision=lib.QJG_FP32_REFINE, refine_pow=lib.QJG_REFINE_INT,
                              rel_tol=1e-6), 0
    if name == "precision_slabs":
        return rs, g, p, dict(precision=lib.QJG_FP32_REFINE, refine_pow=lib.QJG_REFINE_INT), 9
    if name == "fp64_slabs":
        return rs, g, p, dict(precision=lib.QJG_FP64), 13
    if name == "lagrange":
        return rs, g, p, dict(precision=lib.QJG_FP32_REFINE, refine_pow=lib.QJG_REFINE_INT,
                              rel_tol=1e-6, lagrange=True), 17
    raise KeyError(name)


def host_path(ctx, h, g, it, slab_nz, vcap, tcap):
    b = Bufs(vcap, tcap)
    _, st = ctx.mesh_stream(h, g, it, slab_nz=slab_nz, **b.kw())
    return b.out(st), st


def same(a, b, sa, sb):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    for k in KEYS:
        assert sa[k] == sb[k], (k, sa[k], sb[k])
    for k in ("voxels", "voxel_iters", "refined", "nonfinite", "rerun"):
        assert sa["field"][k] == sb["field"][k], k


@pytest.mark.parametrize("name", ["plain", "precision", "precision_slabs", "fp64_slabs",
                                  "lagrange"])
def test_fixed_sequence_equals_stream(ctx, name):
    rs, g, p, kw, slab_nz = case(name)
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"], **kw)
    vcap, tcap = 3 * g.n_voxels // 4 + 64, 3 * g.n_voxels // 2 + 64
    try:
        ref, st_ref = host_path(ctx, h, g, it, slab_nz, vcap, tcap)
        assert st_ref["n_tris"] > 1000
        ctx.mesh_prepare(g, vcap, tcap, slab_nz=slab_nz)
        b = Bufs(vcap, tcap)
        for _ in range(2):  # a second run on the same buffers gives the same mesh
            b.clear()
            ctx.mesh_stream_async(h, g, it, slab_nz=slab_nz, **b.kw())
            torch.cuda.synchronize()
            _, st = ctx.mesh_async_result()
            same(b.out(st), ref, st, st_ref)
    finally:
        ctx.free(h)


def test_graph_replay_equals_stream(ctx):
    rs, g, p, kw, slab_nz = case("precision_slabs")
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"], **kw)
    vcap, tcap = 3 * g.n_voxels // 4 + 64, 3 * g.n_voxels // 2 + 64
    try:
        ref, st_ref = host_path(ctx, h, g, it, slab_nz, vcap, tcap)
        ctx.mesh_prepare(g, vcap, tcap, slab_nz=slab_nz)
        b = Bufs(vcap, tcap)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):  # one run outside the capture: modules loaded
            ctx.mesh_stream_async(h, g, it, slab_nz=slab_nz, stream=s.cuda_stream, **b.kw())
        s.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s, capture_error_mode="thread_local"):
            ctx.mesh_stream_async(h, g, it, slab_nz=slab_nz, stream=s.cuda_stream, **b.kw())
        for _ in range(2):
            b.clear()
            torch.cuda.synchronize()
            graph.replay()
            torch.cuda.synchronize()
            _, st = ctx.mesh_async_result()
            same(b.out(st), ref, st, st_ref)
    finally:
        ctx.free(h)


def test_capacity_and_preparation(ctx):
    rs, g, p, kw, slab_nz = case("precision")
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"], **kw)
    try:
        b = Bufs(64, 128)
        fresh = lib.Context(0)
        hf = fresh.upload(rs)
        with pytest.raises(lib.QjgError):  # not prepared
            fresh.mesh_stream_async(hf, g, it, **b.kw())
        fresh.free(hf)
        fresh.close()
        ctx.mesh_prepare(g, 64, 128)
        ctx.mesh_stream_async(h, g, it, **b.kw())
        torch.cuda.synchronize()
        rc, st = ctx.mesh_async_result(check=False)
        assert rc == lib.QJG_ERR_CAPACITY
        # the host path reports what the mesh needs
        rc, st = ctx.mesh_stream(h, g, it, check=False, **b.kw())
        assert rc == lib.QJG_ERR_CAPACITY and st["n_verts"] > 64
    finally:
        ctx.free(h)
