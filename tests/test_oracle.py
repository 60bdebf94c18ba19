"""The CPU oracle against fixtures produced by the reference itself
(tests/golden/gen_golden.py runs the reference compiled from its sources)."""
import numpy as np
import pytest

from conftest import load_case
from quijibo_gb300.rootsets import mt19937_rand

FIELD_CASES = ["plain_unit", "plain_conf", "prec", "general"]


def test_mt19937_matches_reference(oracle):
    d = np.load("tests/golden/algebra.npz")
    for seed, key in ((0, "mt_seed0"), (12345, "mt_seed12345")):
        assert np.array_equal(mt19937_rand(seed, 64), d[key])
        assert np.array_equal(oracle.mt_rand(seed, 64), d[key])


def test_quat_pow_matches_reference(oracle):
    d = np.load("tests/golden/algebra.npz")
    out = np.array([oracle.quat_pow(q, e) for q, e in zip(d["pow_q"], d["pow_e"])])
    assert np.array_equal(out, d["pow_out"])


@pytest.mark.parametrize("name", FIELD_CASES)
def test_field_bit_exact_vs_reference(oracle, name):
    rs, g, p, d = load_case("field_" + name)
    out = oracle.field(rs, g, p["max_it"], p["escape"])["field"]
    # same operation order, no fused multiply-add: identical doubles
    np.testing.assert_array_equal(out, d["field"])


def test_field_escape2000_matches_unmodified_reference_map(oracle):
    rs, g, p, d = load_case("field_map2000")
    out = oracle.field(rs, g, p["max_it"], p["escape"])["field"]
    np.testing.assert_array_equal(out, d["field"])


@pytest.mark.parametrize("name", FIELD_CASES)
def test_long_double_witness(name):
    """The reference's own long-double build agrees with its double build to
    well below 1e-9 on these cases and has the same sign map."""
    _, _, _, d = load_case("field_" + name)
    f, fl = d["field"], d["field_ld"]
    rel = np.abs(f - fl) / np.maximum(np.abs(fl), 1e-300)
    assert rel.max() < 1e-9
    assert np.array_equal(f > 0, fl > 0)


@pytest.mark.parametrize("kind,mode", [("stream", 1), ("nonlin", 1), ("linear", 0)])
def test_mesh_matches_reference(oracle, kind, mode):
    rs, g, p, d = load_case("mesh_plain")
    classify = d["field2"] if kind == "linear" else d["field2000"]
    m = oracle.mesh(rs, g, classify, mode, p["max_it"], p["escape"])
    np.testing.assert_array_equal(m["tris"], d[kind + "_tris"])
    np.testing.assert_array_equal(m["verts"], d[kind + "_verts"])
    assert m["unbracketed"] == 0


def test_mesh_nonempty_fixture():
    _, _, _, d = load_case("mesh_plain")
    assert len(d["stream_tris"]) > 1000


def test_tanh_score_and_gradients_match_reference(oracle):
    from quijibo_gb300.rootsets import Grid
    rs, g, p, d = load_case("tanh_grad")
    wg = Grid(tuple(int(v) for v in d["wres"]), tuple(d["wcenter"]), tuple(d["wlengths"]))
    sc, gr, f = oracle.tanh_score_grad(rs, g, wg, d["weights"], p["max_it"])
    np.testing.assert_array_equal(f, d["field"])
    # the reference sums in a different voxel order: rounding-level differences
    assert abs(sc - d["score"]) <= 1e-13 * abs(d["score"])
    np.testing.assert_allclose(gr, d["grad"], rtol=1e-12, atol=1e-12 * np.abs(d["grad"]).max())
