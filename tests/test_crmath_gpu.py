"""The QJG_LIBM_CR form on the GPU: the correctly rounded transcendentals
give the same bits on the device as in the CPU oracle, and the plain FP64
field, the FP64 refine band and the meshers' FP64 evaluations built on them
equal the oracle restated with the same functions on every voxel and vertex.
What remains between them and the reference's double build is the C
library's own rounding (tests/test_crmath.py)."""
import os

import numpy as np
import pytest

from conftest import load_case
from quijibo_gb300 import lib
from quijibo_gb300.rootsets import precision_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "crmath.npz")
FIELD_CASES = ["plain_unit", "plain_conf", "prec", "general", "map2000"]


def device_eval(name, x):
    X = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    Y = torch.empty_like(X)
    lib.crmath_eval(name, X.data_ptr(), Y.data_ptr(), X.numel())
    torch.cuda.synchronize()
    return Y.cpu().numpy()


@pytest.mark.parametrize("name", lib.CRM_FUNCTIONS)
def test_device_functions_equal_host_functions(oracle, name):
    g = np.load(GOLDEN)
    x = g[name + "_x"]
    np.testing.assert_array_equal(device_eval(name, x), g[name + "_cr"])
    rng = np.random.RandomState(3)
    lo, hi = {"exp": (-40, 40), "log": (-700, 700), "sin": (-2e3, 2e3), "cos": (-2e3, 2e3),
              "acos": (-1, 1)}[name]
    x = rng.uniform(lo, hi, 100_000)
    if name == "log":
        x = np.exp(x)
    np.testing.assert_array_equal(device_eval(name, x), oracle.crm(name, x))


def _oracle_cr(oracle, fn, *a, **kw):
    oracle.set_libm(True)
    try:
        return fn(*a, **kw)
    finally:
        oracle.set_libm(False)


@pytest.mark.parametrize("name", FIELD_CASES)
def test_fp64_cr_field_equals_oracle_on_every_voxel(ctx, oracle, name):
    rs, g, p, d = load_case("field_" + name)
    h = ctx.upload(rs)
    try:
        it = ctx.iter_params(p["max_it"], p["escape"], libm=lib.QJG_LIBM_CR)
        f, _, st = ctx.field_host(h, g, it)
    finally:
        ctx.free(h)
    o = _oracle_cr(oracle, oracle.field, rs, g, p["max_it"], p["escape"], iters=True)
    np.testing.assert_array_equal(f, o["field"])
    assert st["voxel_iters"] == int(o["iters"].sum())
    # and so the reference's bits on most voxels, 1.2e-12 on the rest
    ref = d["field"]
    rel = np.abs(f - ref) / np.maximum(np.abs(ref), 1e-300)
    assert rel.max() <= 1.2e-12 and np.array_equal(f > 0, ref > 0)


def test_precision_form_with_cr_band_is_within_rel_tol(ctx, oracle):
    """FP32 bulk + double-float re-run + an FP64 band in the reference's polar
    pow with correctly rounded functions: the band voxels are the oracle's
    bits, the rest within rel_tol."""
    rs, g, p = precision_workload(48)
    h = ctx.upload(rs)
    try:
        it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                             refine_pow=lib.QJG_REFINE_POW, rel_tol=1e-6, libm=lib.QJG_LIBM_CR)
        f, _, st = ctx.field_host(h, g, it)
    finally:
        ctx.free(h)
    o = _oracle_cr(oracle, oracle.field, rs, g, p["max_it"], p["escape"])["field"]
    rel = np.abs(f - o) / np.maximum(np.abs(o), 1e-300)
    assert st["refined"] > 0 and rel.max() <= 1e-6
    assert np.array_equal(f > 0, o > 0)
    assert np.mean(f == o) >= st["refined"] / f.size


def test_streaming_mesher_cr_equals_oracle(ctx, oracle):
    """The plain FP64 streaming mesher with correctly rounded functions: the
    oracle's triangles and the oracle's bisection vertices, bit for bit."""
    rs, g, p, d = load_case("mesh_plain")
    h = ctx.upload(rs)
    n = g.n_voxels
    v = torch.empty(3 * (3 * n + 16), dtype=torch.float64, device="cuda")
    t = torch.empty(3 * (5 * n + 16), dtype=torch.int32, device="cuda")
    try:
        it = ctx.iter_params(p["max_it"], p["escape"], libm=lib.QJG_LIBM_CR)
        _, st = ctx.mesh_stream(h, g, it, d_verts64=v.data_ptr(), vert_cap=3 * n + 16,
                                d_tris=t.data_ptr(), tri_cap=5 * n + 16)
        f, _, _ = ctx.field_host(h, g, it)
    finally:
        ctx.free(h)
    nv, nt = st["n_verts"], st["n_tris"]
    fo = _oracle_cr(oracle, oracle.field, rs, g, p["max_it"], p["escape"])["field"]
    np.testing.assert_array_equal(f, fo)
    o = _oracle_cr(oracle, oracle.mesh, rs, g, fo, lib.QJG_EDGE_BISECT, p["max_it"], p["escape"])
    np.testing.assert_array_equal(t[:3 * nt].view(-1, 3).cpu().numpy(), o["tris"])
    np.testing.assert_array_equal(v[:3 * nv].view(-1, 3).cpu().numpy(), o["verts"])
    np.testing.assert_array_equal(o["tris"], d["stream_tris"])
