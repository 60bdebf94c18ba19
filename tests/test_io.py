"""File formats against the bytes the reference's own writers produce
(tests/golden/io_*, made by gen_golden.py through FIELD_3D::write,
TRIANGLE_MESH::writeOBJ, TRIANGLE_MESH::write and OPTIMIZE_3D::write)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from gen_golden import io_inputs  # noqa: E402
from quijibo_gb300 import lib  # noqa: E402

GOLDEN = os.path.join(HERE, "golden")


def golden(name):
    with open(os.path.join(GOLDEN, name), "rb") as f:
        return f.read()


def test_field3d_bytes_match_reference_writer(tmp_path):
    field, res, center, lengths, _, _ = io_inputs()
    out = tmp_path / "f.field3d"
    lib.field3d_write(out, res, center, lengths, field)
    assert out.read_bytes() == golden("io_field.field3d")


def test_field3d_read_round_trip(tmp_path):
    field, res, center, lengths, _, _ = io_inputs()
    r, c, ln, f = lib.field3d_read(os.path.join(GOLDEN, "io_field.field3d"))
    assert r == res
    np.testing.assert_array_equal(c, center)
    np.testing.assert_array_equal(ln, lengths)
    assert np.array_equal(f.view(np.uint64), field.view(np.uint64))  # -0.0 kept


def test_obj_text_matches_reference_writer(tmp_path):
    _, _, _, _, verts, tris = io_inputs()
    out = tmp_path / "m.obj"
    lib.mesh_write_obj(out, verts, tris)
    assert out.read_bytes() == golden("io_mesh.obj")


def test_raw_mesh_matches_reference_writer(tmp_path):
    _, _, _, _, verts, tris = io_inputs()
    out = tmp_path / "m.raw"
    lib.mesh_write_raw(out, verts, tris)
    assert out.read_bytes() == golden("io_mesh.raw")


def test_obj_from_fp32_vertices_prints_their_double_value(tmp_path):
    _, _, _, _, verts, tris = io_inputs()
    v32 = verts.astype(np.float32)
    out = tmp_path / "m32.obj"
    lib.mesh_write_obj(out, v32, tris)
    lines = out.read_text().splitlines()
    assert lines[3] == "v %.16f %.16f %.16f" % tuple(float(x) for x in v32[3])
    assert lines[-1] == "f 2 4 6"


def test_large_obj_is_ordered_across_threads(tmp_path):
    rng = np.random.RandomState(3)
    v = rng.uniform(-1e3, 1e3, (20011, 3))
    t = rng.randint(0, len(v), (30007, 3)).astype(np.int32)
    out = tmp_path / "big.obj"
    lib.mesh_write_obj(out, v, t)
    lines = out.read_text().splitlines()
    assert len(lines) == len(v) + len(t)
    for i in (0, 1, 9999, 20010):
        assert lines[i] == "v %.16f %.16f %.16f" % tuple(v[i])
    for j in (0, 15003, 30006):
        assert lines[len(v) + j] == "f %d %d %d" % tuple(t[j] + 1)


def test_huge_coordinates_are_printed_whole(tmp_path):
    v = np.array([[1e300, -1e300, 0.5]])
    out = tmp_path / "huge.obj"
    lib.mesh_write_obj(out, v, np.zeros((0, 3), dtype=np.int32))
    assert out.read_text() == "v %.16f %.16f %.16f\n" % tuple(v[0])


def test_io_errors_are_reported(tmp_path):
    field, res, center, lengths, _, _ = io_inputs()
    with pytest.raises(lib.QjgError):
        lib.field3d_write(tmp_path / "no" / "such" / "dir.f3d", res, center, lengths, field)
    with pytest.raises(lib.QjgError):
        lib.field3d_read(tmp_path / "missing.field3d")
    small = np.empty(3)
    L = lib.load()
    rc = L.qjg_field3d_read(os.path.join(GOLDEN, "io_field.field3d").encode(),
                            lib.C.c_void_p(small.ctypes.data), 3)
    assert rc == -5  # QJG_ERR_CAPACITY


@pytest.mark.gpu
def test_writers_take_device_buffers(tmp_path):
    torch = pytest.importorskip("torch")
    field, res, center, lengths, verts, tris = io_inputs()
    fd = torch.from_numpy(field.ravel().copy()).cuda()
    vd = torch.from_numpy(verts.ravel().copy()).cuda()
    v32 = torch.from_numpy(verts.astype(np.float32).ravel().copy()).cuda()
    td = torch.from_numpy(tris.ravel().copy()).cuda()
    torch.cuda.synchronize()
    lib.field3d_write(tmp_path / "f", res, center, lengths, fd.data_ptr())
    assert (tmp_path / "f").read_bytes() == golden("io_field.field3d")
    lib.mesh_write_obj(tmp_path / "m.obj", vd.data_ptr(), td.data_ptr(), n_verts=len(verts),
                       n_tris=len(tris), fp32=False)
    assert (tmp_path / "m.obj").read_bytes() == golden("io_mesh.obj")
    lib.mesh_write_raw(tmp_path / "m.raw", vd.data_ptr(), td.data_ptr(), n_verts=len(verts),
                       n_tris=len(tris))
    assert (tmp_path / "m.raw").read_bytes() == golden("io_mesh.raw")
    lib.mesh_write_obj(tmp_path / "m32.obj", v32.data_ptr(), td.data_ptr(), n_verts=len(verts),
                       n_tris=len(tris), fp32=True)
    host32 = tmp_path / "h32.obj"
    lib.mesh_write_obj(host32, verts.astype(np.float32), tris)
    assert (tmp_path / "m32.obj").read_bytes() == host32.read_bytes()
    back = torch.empty_like(fd)
    L = lib.load()
    assert L.qjg_field3d_read(str(tmp_path / "f").encode(), lib.C.c_void_p(back.data_ptr()),
                              back.numel()) == 0
    torch.cuda.synchronize()
    assert torch.equal(back.view(torch.int64), fd.view(torch.int64))


def test_o3d_reader_takes_the_reference_state_file():
    from gen_golden import o3d_inputs
    rs, g, fractal, dg, dist, curv = o3d_inputs()
    st = lib.o3d_read(os.path.join(GOLDEN, "io_state.o3d"))
    np.testing.assert_array_equal(st["top_roots"], rs.top_roots)
    np.testing.assert_array_equal(st["top_powers"], rs.top_powers)
    np.testing.assert_array_equal(st["bottom_roots"], rs.bottom_roots)
    np.testing.assert_array_equal(st["bottom_powers"], rs.bottom_powers)
    assert (st["sigma_top"], st["sigma_bottom"], st["scale"]) == (1.25, 0.75, 0.625)
    assert st["res"] == g.res and st["center"] == g.center and st["lengths"] == g.lengths
    for name, grid, data in (("fractal", g, fractal), ("distance", dg, dist),
                             ("curvature", dg, curv)):
        res, c, ln, f = st[name]
        assert res == grid.res and c == grid.center and ln == grid.lengths
        np.testing.assert_array_equal(f.ravel(), data)


def test_o3d_writer_round_trips(tmp_path):
    from gen_golden import o3d_inputs
    rs, g, fractal, dg, dist, curv = o3d_inputs()
    out = tmp_path / "s.o3d"
    lib.o3d_write(out, rs, g.res, g.center, g.lengths,
                  {"fractal": (g.res, g.center, g.lengths, fractal),
                   "distance": (dg.res, dg.center, dg.lengths, dist),
                   "curvature": (dg.res, dg.center, dg.lengths, curv)})
    st = lib.o3d_read(out)
    np.testing.assert_array_equal(st["top_roots"], rs.top_roots)
    np.testing.assert_array_equal(st["distance"][3].ravel(), dist)
    # the reference's own reader takes it too (where the reference is built)
    from oracle.oracle import REF_SO, Reference
    if not os.path.exists(REF_SO["double"]):
        pytest.skip("reference not built here")
    ref = Reference("double").o3d_read(out)
    np.testing.assert_array_equal(ref["top_roots"], rs.top_roots)
    np.testing.assert_array_equal(ref["bottom_powers"], rs.bottom_powers)
    assert (ref["sigma_top"], ref["sigma_bottom"], ref["scale"]) == (1.25, 0.75, 0.625)
    # (OPTIMIZE_3D::read rebuilds its fractal from the score fields, so only
    # the distance field survives as stored)
    np.testing.assert_array_equal(ref["dist"][:dg.n_voxels], dist)


def test_o3d_reader_rejects_truncated_files(tmp_path):
    data = open(os.path.join(GOLDEN, "io_state.o3d"), "rb").read()
    out = tmp_path / "cut.o3d"
    out.write_bytes(data[:len(data) // 2])
    with pytest.raises(lib.QjgError):
        lib.o3d_read(out)
