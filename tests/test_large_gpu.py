"""The large-grid workload at its stated size: 48 top / 24 bottom roots drawn
in [-1.2,1.2]^4 with exponents {1,2}, s = u * conformal scale, 60
iterations, escape radius 2, a 2200^3 grid over [-1.5,1.5]^3.

Two full z-slices are computed through qjg_field's slab range, the unit the
2200^3 pass streams, in four forms: the precision form at rel_tol = 1e-6
(FP32 bulk, double-float re-run, FP64 band), the plain FP64 form (the
reference's polar pow per root term), FP64 with integer powers as repeated
products (the precision form's algebra), and FP32 alone.  The slices lie at
z = 1840, where the FP32 orbits overflow or underflow most often (about
4,800 voxels per slice) and the surface crosses the slice."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import large_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RES = 2200
Z0 = 1840
# 128 x 128 cells of slice Z0 that the surface crosses (about half inside)
WINDOW = (240, 368, 320, 448)  # x0, x1, y0, y1


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


@pytest.fixture(scope="module")
def slices(ctx):
    rs, g, p = large_workload(RES)
    h = ctx.upload(rs)
    XY = g.res[0] * g.res[1]
    forms = {
        "refine": dict(precision=lib.QJG_FP32_REFINE, refine_pow=lib.QJG_REFINE_INT, rel_tol=1e-6),
        "fp64": dict(precision=lib.QJG_FP64),
        "fp64_int": dict(precision=lib.QJG_FP64, refine_pow=lib.QJG_REFINE_INT),
        "fp32": dict(precision=lib.QJG_FP32),
    }
    out = {}
    buf = torch.empty(2 * XY, dtype=torch.float64, device="cuda")
    try:
        for k, kw in forms.items():
            it = ctx.iter_params(p["max_it"], p["escape"], **kw)
            ctx.field(h, g, it, buf.data_ptr(), z0=Z0, z1=Z0 + 2)
            st = ctx.stats()
            out[k] = (buf.cpu().numpy().reshape(2, g.res[1], g.res[0]), st)
    finally:
        ctx.free(h)
    return rs, g, p, out


def test_large_precision_form_within_1e6_of_fp64(slices):
    """Identical sign map and at most 1e-6 relative error on every voxel of
    the two slices, against FP64 of the same algebra; against the plain FP64
    form (reference rounding of pow) the sign map is identical too."""
    _, g, _, out = slices
    f, st = out["refine"]
    f64, _ = out["fp64_int"]
    assert np.array_equal(f > 0, f64 > 0), int(((f > 0) != (f64 > 0)).sum())
    assert rel_err(f, f64).max() <= 1e-6
    assert st["voxels"] == 2 * g.res[0] * g.res[1]
    assert st["rerun"] > 0 and st["refined"] > 0
    fp, _ = out["fp64"]
    assert np.array_equal(f > 0, fp > 0)
    assert np.quantile(rel_err(f, fp), 0.999) <= 1e-6


def test_large_fp64_matches_oracle_window(slices, oracle):
    """The plain FP64 form against the oracle (the C restatement pinned
    bit-exact to the reference's double build) on a 128 x 128 window of one
    slice: the same cells of the same 2200^3 grid.  As on the reference
    fixtures, the two differ only inside the libm transcendentals."""
    rs, g, p, out = slices
    x0, x1, y0, y1 = WINDOW
    o = oracle.field_window(rs, g, p["max_it"], p["escape"], x0, x1, y0, y1, Z0, Z0 + 1)[0]
    f = out["fp64"][0][0, y0:y1, x0:x1]
    assert 0.2 < (o > 0).mean() < 0.8  # the surface crosses the window
    rel = rel_err(f, o)
    assert np.quantile(rel, 0.999) <= 1e-12, np.quantile(rel, 0.999)
    assert np.array_equal(f > 0, o > 0)


def test_large_fp32_nonfinite_voxels_are_refined(slices):
    """Voxels whose FP32 orbit overflows (inf or NaN) or underflows (|q|^2
    below 1e-36, a field below -41.4) go to FP64: in the precision form they
    carry the FP64 values."""
    _, _, _, out = slices
    f32, st32 = out["fp32"]
    f, st = out["refine"]
    f64, _ = out["fp64_int"]
    bad = ~np.isfinite(f32) | (f32 <= 0.5 * np.log(1e-36))
    assert bad.sum() > 1000 and st32["nonfinite"] > 1000
    assert st["refined"] >= bad.sum()
    assert np.array_equal(np.isfinite(f[bad]), np.isfinite(f64[bad]))
    ok = np.isfinite(f64[bad])
    assert rel_err(f[bad][ok], f64[bad][ok]).max() <= 1e-12
