import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle, build
    build()
    return Oracle()


@pytest.fixture(scope="session")
def ctx():
    from quijibo_gb300 import lib
    c = lib.Context(0)
    yield c
    c.close()


def load_case(name):
    """A golden case: (RootSet, Grid, params, npz dict)."""
    from quijibo_gb300.rootsets import Grid, RootSet
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    rs = RootSet(top_roots=d["top_roots"], top_powers=d["top_powers"],
                 sigma_top=float(d["sigma_top"]), bottom_roots=d["bottom_roots"].reshape(-1, 4),
                 bottom_powers=d["bottom_powers"], sigma_bottom=float(d["sigma_bottom"]),
                 scale=float(d["scale"]))
    g = Grid(tuple(int(v) for v in d["res"]), tuple(d["center"]), tuple(d["lengths"]),
             tuple(d["rot"]), float(d["slice"]))
    return rs, g, dict(max_it=int(d["max_it"]), escape=float(d["escape"])), d
