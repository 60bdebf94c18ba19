"""Known-answer checks restated from the reference's own test routines, with
no reference output involved: POLYNOMIAL_4D::rationalTest
(src/algebra/POLYNOMIAL_4D.cpp:520-577) checks a rational map against closed
forms: (z^2 - 1) / z^2 = 1 - 1/z^2 and its derivative 2 / z^3.  Here the map
with top roots +1, -1 and bottom roots 0, 0 (exponents 1, s = 1) is run for
one iteration, where log|q_1| = log|1 - q^-2| for every quaternion q (all
factors are polynomials in q, so they commute), and on a plane of complex
points (third and fourth coordinates 0) the distance estimate is
log|R| / |R'/R| with |R'/R| = |2 / (z (z^2 - 1))| (R holomorphic there).
The oracle and (tests marked gpu) every field form are held to them."""
import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, RootSet


def rational_rootset():
    return RootSet(top_roots=np.array([[1.0, 0, 0, 0], [-1.0, 0, 0, 0]]),
                   top_powers=np.array([1.0, 1.0]), sigma_top=1.0,
                   bottom_roots=np.zeros((2, 4)), bottom_powers=np.array([1.0, 1.0]),
                   sigma_bottom=1.0, scale=1.0)


def quat_centres(g):
    """Cell centres of an unrotated grid as quaternions (w, x, y, z) = (x, y, z, slice)."""
    X, Y, Z = g.res
    idx = np.indices((Z, Y, X)).reshape(3, -1)  # z, y, x
    c = [g.center[k] - 0.5 * g.lengths[k] + (idx[2 - k] + 0.5) * g.lengths[k] / g.res[k]
         for k in range(3)]
    return np.stack([c[0], c[1], c[2], np.full(c[0].shape, g.slice)], axis=1)


def one_minus_inv_square_log(q):
    """log|1 - q^-2| with q^-1 = conj(q) / |q|^2 (NumPy float64)."""
    n2 = np.sum(q * q, axis=1)
    inv = q * np.array([1.0, -1, -1, -1]) / n2[:, None]
    w, x, y, z = inv.T
    sq = np.stack([w * w - x * x - y * y - z * z, 2 * w * x, 2 * w * y, 2 * w * z], axis=1)
    r = -sq
    r[:, 0] += 1.0
    return np.log(np.sqrt(np.sum(r * r, axis=1)))


GRID3 = Grid((24, 20, 16), center=(0.1, -0.2, 0.3), lengths=(3.0, 2.5, 2.0), slice=0.35)
PLANE = Grid((40, 36, 1), center=(0.05, 0.02, 0.0), lengths=(3.0, 2.8, 0.1), slice=0.0)


def check_field(f, g, tol):
    """|f - log|1 - q^-2|| <= tol max(|value|, 1) (an absolute floor where
    |R| crosses 1 and the logarithm vanishes)."""
    ref = one_minus_inv_square_log(quat_centres(g))
    err = np.abs(f.reshape(-1) - ref) / np.maximum(np.abs(ref), 1.0)
    assert err.max() <= tol, err.max()


def check_de(f, de, g, tol):
    z = quat_centres(g)
    zc = z[:, 0] + 1j * z[:, 1]
    grad = np.abs(2.0 / (zc * (zc * zc - 1.0)))
    expect = f.reshape(-1) / grad
    err = np.abs(de.reshape(-1) - expect) / np.maximum(np.abs(expect), 1e-2)
    assert err.max() <= tol, err.max()


def test_oracle_rational_known_answer(oracle):
    rs = rational_rootset()
    o = oracle.field(rs, GRID3, 1, 1e30)
    check_field(o["field"], GRID3, 1e-13)
    o = oracle.field(rs, PLANE, 1, 1e30, de=True)
    check_field(o["field"], PLANE, 1e-13)
    check_de(o["field"], o["de"], PLANE, 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,libm", [(lib.QJG_FP64, lib.QJG_LIBM_DEVICE),
                                            (lib.QJG_FP64, lib.QJG_LIBM_CR),
                                            (lib.QJG_FP32_REFINE, lib.QJG_LIBM_DEVICE)])
def test_gpu_rational_known_answer(ctx, precision, libm):
    rs = rational_rootset()
    h = ctx.upload(rs)
    try:
        kw = dict(precision=precision, libm=libm, want_de=True)
        if precision == lib.QJG_FP32_REFINE:
            kw.update(refine_pow=lib.QJG_REFINE_INT, rel_tol=1e-6)
        it = ctx.iter_params(1, 1e30, **kw)
        f, _, _ = ctx.field_host(h, GRID3, it)
        check_field(f, GRID3, 1e-13 if precision == lib.QJG_FP64 else 1e-6)
        f, de, _ = ctx.field_host(h, PLANE, it, de=True)
        check_field(f, PLANE, 1e-13 if precision == lib.QJG_FP64 else 1e-6)
        # the distance estimate is an FP32 output (computed in FP32 on the
        # precision form's FP32 voxels)
        check_de(f, de, PLANE, 1e-6 if precision == lib.QJG_FP64 else 1e-5)
    finally:
        ctx.free(h)
