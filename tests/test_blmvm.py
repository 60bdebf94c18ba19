"""The BLMVM solver (qjg_blmvm) against the reference's own TAO port:
every evaluated point bit-identical to the ones TAO_SOLVER::optimizeBLMVM
evaluated (tests/golden/blmvm.npz, made by gen_golden.py), on smooth, boxed,
non-smooth, non-finite and inconsistent objectives.  Host-only: no GPU."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from blmvm_problems import FLT_MAX, problems, quad  # noqa: E402
from quijibo_gb300 import lib  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "blmvm.npz"))
REASON = {"rosen2_box": 1, "quad12": 1, "kinks5": -2, "pinned3": -6}


def run(fun, x0, lo, hi, **kw):
    pts, fs = [], []

    def rec(x):
        f, g = fun(list(x))
        pts.append(x.copy())
        fs.append(f)
        return f, g
    x, st = lib.blmvm(rec, x0, lo, hi, **kw)
    return x, np.array(pts), np.array(fs), st


@pytest.mark.parametrize("name", sorted(problems()))
def test_iterates_bit_identical_to_reference(name):
    fun, x0, lo, hi = problems()[name]
    x, pts, fs, st = run(fun, x0, lo, hi)
    gp, gf = GOLD[name + "_pts"], GOLD[name + "_f"]
    assert len(fs) == len(gf) == st["evaluations"]
    assert np.array_equal(pts.view(np.uint64), gp.view(np.uint64))
    assert np.array_equal(fs, gf, equal_nan=True)
    assert np.array_equal(x.view(np.uint64), GOLD[name + "_x"].view(np.uint64))
    if name in REASON:
        assert st["reason"] == REASON[name]


def test_live_against_reference_with_transcendental_objective():
    """Where the reference is built: an objective with exp/tanh/cos, both
    solvers driven in this process."""
    from oracle.oracle import REF_SO, Reference
    if not os.path.exists(REF_SO["double"]):
        pytest.skip("reference not built here")
    c = np.linspace(0.2, 1.5, 9)

    def fun(x):
        x = np.asarray(x)
        t = np.tanh(3 * (x - c))
        f = float(-np.sum(t * np.cos(x)) + 0.05 * np.sum(x * x))
        return f, -(3 * (1 - t * t) * np.cos(x) - t * np.sin(x)) + 0.1 * x
    lo, hi = [-FLT_MAX] + [0.0] * 8, [FLT_MAX] * 9
    xr, hist = Reference("double").blmvm(fun, np.linspace(0.1, 2.0, 9), lo, hi)
    x, pts, fs, st = run(fun, np.linspace(0.1, 2.0, 9), lo, hi)
    assert len(hist) == len(fs)
    for (f0, p0), f1, p1 in zip(hist, fs, pts):
        assert f0 == f1 and np.array_equal(p0, p1)
    assert np.array_equal(x, xr)


def test_bounds_hold_and_start_is_projected():
    fun, _, lo, hi = problems()["rosen8_box"]
    x, pts, _, _ = run(fun, [5.0] * 8, lo, hi)
    assert np.all(pts >= lo) and np.all(pts <= hi)
    assert np.array_equal(pts[0], np.full(8, 0.7))
    assert np.all(x <= 0.7)


def test_monitor_ends_the_run():
    fun, x0, lo, hi = problems()["rosen7"]
    seen = []

    def mon(it, f, gnorm, xp):
        seen.append((it, f))
        return it >= 3
    _, _, _, st = run(fun, x0, lo, hi, monitor=mon)
    assert [s[0] for s in seen] == [1, 2, 3]
    assert st["reason"] == 8 and st["iterations"] == 3


def test_settings_limit_iterations():
    fun, x0, lo, hi = problems()["kinks5"]
    _, _, _, st = run(fun, x0, lo, hi, settings=lib.blmvm_settings(max_it=10))
    assert st["reason"] == -2 and st["iterations"] == 11


def test_objective_errors_stop_the_solver():
    calls = []

    def bad(x):
        calls.append(1)
        if len(calls) == 3:
            raise ValueError("objective failed")
        return quad(list(x))
    with pytest.raises(ValueError):
        lib.blmvm(bad, [1.0, 2.0, 3.0], [-FLT_MAX, 0, 0], [FLT_MAX] * 3)
    assert len(calls) == 3


def test_bad_arguments():
    L = lib.load()
    x = np.ones(3)
    lo, hi = np.array([0.0, 2.0, 0.0]), np.array([1.0, 1.0, 1.0])  # lo > hi
    fn = lib.OBJECTIVE_FN(lambda *a: 0)
    dp = lib._dp
    rc = L.qjg_blmvm(3, x.ctypes.data_as(dp), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), fn,
                     None, lib.MONITOR_FN(), None, None, None)
    assert rc == -1
    rc = L.qjg_blmvm(0, x.ctypes.data_as(dp), lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), fn,
                     None, lib.MONITOR_FN(), None, None, None)
    assert rc == -1


def test_defaults_are_the_references():
    st = lib.blmvm_settings()
    assert (st.max_it, st.ls_max_funcs) == (2000, 30)
    assert (st.fatol, st.frtol, st.gatol, st.grtol, st.gttol) == (1e-8, 1e-8, 1e-8, 1e-8, 0.0)
