"""qjg_field_noalloc: the field entry point for callers that cannot allocate
device memory (plugins whose host application owns every device allocation,
real-time loops, processes held to a fixed device-memory quota).  It must
give the same field as qjg_field, call after call, while its scratch is a
fixed array inside the library.  This file is collected last so that a
failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import precision_workload

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

_dp = C.POINTER(C.c_double)


def _noalloc():
    f = lib.load().qjg_field_noalloc
    f.argtypes = [C.c_int32, _dp, _dp, C.c_double, C.c_int32, _dp, _dp, C.c_double, C.c_double,
                  C.POINTER(lib.QjgGrid), C.POINTER(lib.QjgIter), C.c_int32, C.c_int32, C.c_void_p,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _call(f, rs, g, it, out, z0=0, z1=None):
    tr = np.ascontiguousarray(rs.top_roots, dtype=np.float64)
    tp = np.ascontiguousarray(rs.top_powers, dtype=np.float64)
    br = np.ascontiguousarray(rs.bottom_roots, dtype=np.float64)
    bp = np.ascontiguousarray(rs.bottom_powers, dtype=np.float64)
    z1 = g.res[2] if z1 is None else z1
    return f(rs.n_top, tr.ctypes.data_as(_dp), tp.ctypes.data_as(_dp), rs.sigma_top, rs.n_bottom,
             br.ctypes.data_as(_dp), bp.ctypes.data_as(_dp), rs.sigma_bottom, rs.scale,
             C.byref(lib.QjgGrid.of(g)), C.byref(it), z0, z1, C.c_void_p(out.data_ptr()), None,
             C.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("precision,rel_tol", [(lib.QJG_FP32_REFINE, 0.0),
                                                (lib.QJG_FP32_REFINE, 1e-6), (lib.QJG_FP64, 0.0)])
def test_noalloc_matches_qjg_field_twice(precision, rel_tol):
    f = _noalloc()
    ctx = lib.Context(0)
    rs, g, p = precision_workload(48 if precision == lib.QJG_FP32_REFINE else 24)
    it = ctx.iter_params(p["max_it"], p["escape"], precision=precision,
                         refine_pow=lib.QJG_REFINE_INT, rel_tol=rel_tol)
    h = ctx.upload(rs)
    sp = torch.cuda.current_stream().cuda_stream
    ref = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    ctx.field(h, g, it, ref.data_ptr(), stream=sp)
    if rel_tol > 0:
        # the double-float re-run stage ran in qjg_field, so it is covered here
        assert ctx.stats(sp)["rerun"] > 0
    for _ in range(2):  # the scratch keeps the last call's contents
        out = torch.full((g.n_voxels,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(f, rs, g, it, out) == 0
        torch.cuda.synchronize()
        # same kernels, same inputs: identical doubles (tolerance of the field tests: exact)
        assert torch.equal(out, ref)
    if rel_tol > 0:
        # and the precision form keeps its bound against the FP64 form
        f64 = torch.empty_like(ref)
        ctx.field(h, g, ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP64,
                                        refine_pow=lib.QJG_REFINE_INT), f64.data_ptr(), stream=sp)
        torch.cuda.synchronize()
        assert torch.equal(out > 0, f64 > 0)
        rel = (out - f64).abs() / f64.abs().clamp_min(1e-300)
        assert float(rel.max()) <= rel_tol
    ctx.free(h)
    ctx.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    f = _noalloc()
    rs, g, p = precision_workload(256)  # 16.8M voxels > the 4M-voxel maximum
    it = lib.Context.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    assert _call(f, rs, g, it, out) == -5  # QJG_ERR_CAPACITY, before any launch
    # a slab range within the maximum is accepted
    small = torch.empty(256 * 256 * 8, dtype=torch.float64, device="cuda")
    assert _call(f, rs, g, it, small, z0=100, z1=108) == 0
    torch.cuda.synchronize()
