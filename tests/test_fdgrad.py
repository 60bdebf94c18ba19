"""OPTIMIZE_3D's central-difference root gradients (computeCenteredGradient,
computeLogRationalCenteredGradient, computeLogRationalBottomCenteredGradient)
in the C oracle against the reference's own outputs (tests/golden/fdgrad.npz,
written by tests/golden/gen_fdgrad.py): the same scores and gradients, bit
for bit."""
import os
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import gen_fdgrad  # noqa: E402


@pytest.mark.parametrize("name", sorted(gen_fdgrad.CASES))
def test_oracle_matches_reference(oracle, name):
    d = np.load(os.path.join(GOLDEN, "fdgrad.npz"))
    kind, rs, g, max_it = gen_fdgrad.case_inputs(name)
    dist, curv = gen_fdgrad.fields(g)
    sc, grad = oracle.centered_gradient(rs, g, max_it, kind, dist, curv)
    assert sc == d[name + "_score"][0]
    np.testing.assert_array_equal(grad, d[name + "_grad"])
    assert np.count_nonzero(grad) > 0
