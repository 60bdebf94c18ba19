"""The C-ABI library builds, loads and exports every entry point that
include/quijibo_gpu.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = "".join(open(os.path.join(ROOT, "include", h)).read()
                   for h in sorted(os.listdir(os.path.join(ROOT, "include"))) if h.endswith(".h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qjg_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def libpath():
    from quijibo_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared()
    assert "qjg_field" in names and "qjg_rootset_upload" in names


def test_library_exports_every_declared_symbol(libpath):
    lib = ctypes.CDLL(libpath)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_header(libpath):
    from quijibo_gb300 import lib
    assert set(declared()) <= set(lib.EXPORTS), set(declared()) - set(lib.EXPORTS)
