"""The FP32 energy's fast angle (csrc/energy.cu, atan01_fast and
atan2_pos_fast): the degree-7 polynomial in t^2 fitted for the library and its
octant reduction, restated here in float64 from the FP32 coefficients in the
source, against numpy's arctan2.  Pins the "2.3e-7 relative" the source states
for the polynomial and the reduction to [0, pi] for y >= 0."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "quijibo_gb300", "csrc", "energy.cu")


def _coefficients():
    src = open(SRC).read()
    body = src[src.index("float atan01_fast(float t)"):]
    body = body[:body.index("return p * t;")]
    first = float(re.search(r"float p = (-?[0-9.]+)f;", body).group(1))
    rest = [float(v) for v in re.findall(r"p = fmaf\(p, u, (-?[0-9.]+)f\);", body)]
    return np.float32([first] + rest).astype(np.float64)


def atan01(t):
    u = t * t
    c = _coefficients()
    p = np.full_like(t, c[0])
    for k in c[1:]:
        p = p * u + k
    return p * t


def atan2_pos(y, x):
    ax = np.abs(x)
    mx, mn = np.maximum(ax, y), np.minimum(ax, y)
    safe = mx > 1.17549435e-38
    a = np.where(safe, atan01(np.where(safe, mn / np.where(safe, mx, 1.0), 0.0)), 0.0)
    a = np.where(y > ax, np.pi / 2 - a, a)
    return np.where(x < 0, np.pi - a, a)


def test_polynomial_is_degree_7_in_t_squared():
    assert len(_coefficients()) == 8


def test_polynomial_relative_error():
    t = np.linspace(1e-6, 1.0, 200001)
    rel = np.abs(atan01(t) - np.arctan(t)) / np.arctan(t)
    assert rel.max() <= 2.3e-7, rel.max()


def test_octant_reduction_matches_arctan2():
    rng = np.random.default_rng(0)
    y = np.abs(rng.normal(size=100000)) * 10.0 ** rng.uniform(-3, 3, 100000)
    x = rng.normal(size=100000) * 10.0 ** rng.uniform(-3, 3, 100000)
    # the axes and the diagonals, where the reduction switches branch
    y = np.concatenate([y, [0.0, 0.0, 1.0, 1.0, 1.0, 2.0, 0.0]])
    x = np.concatenate([x, [1.0, -1.0, 0.0, 1.0, -1.0, 2.0, 0.0]])
    ref = np.arctan2(y, x)
    got = atan2_pos(y, x)
    assert np.all((got >= 0) & (got <= np.pi + 1e-12))
    assert np.max(np.abs(got - ref)) <= 2.3e-7 * np.pi
