"""The drop-in, end to end: the reference's bunnyMarchingCubes3D driver
(projects/bunnyMarchingCubes3D/bunnyMarchingCubes3D.cpp:655-735, unchanged
source) linked against the GPU library through the adapter's --wrap
bindings, run on the committed configuration, against the unmodified
driver's own outputs (tests/golden/gen_dropin.py): the OBJ has the
reference's faces, its vertices within half a voxel (the field and the
bisection run in FP64 where the reference uses glibc's transcendentals), and
the edge-cache file has the reference's bytes.  The same for the
lagrangeBunny3D driver (projects/lagrangeBunny3D/lagrangeBunny3D.cpp, the
Lagrange-order streaming mesher), in the plain FP64 form and the precision
form (QJG_PRECISION=fp32refine).

The edge cache is also checked through the C ABI alone (qjg_mesh_capture,
qjg_mesh_edge_cache_write) on the driver's inputs, which needs no reference
sources.  The driver build needs them: a QUIJIBO checkout named by
QUIJIBO_REF, or the copy `make -C oracle stage` leaves in oracle/_ref."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from quijibo_gb300 import lib
from quijibo_gb300.rootsets import Grid, RootSet

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def fixture():
    return dict(np.load(os.path.join(GOLDEN, "dropin_ref.npz")))


def read_obj(path):
    v, f = [], []
    for line in open(path):
        t = line.split()
        if t and t[0] == "v":
            v.append([float(a) for a in t[1:4]])
        elif t and t[0] == "f":
            f.append([int(a.split("/")[0]) - 1 for a in t[1:4]])
    return np.array(v).reshape(-1, 3), np.array(f, dtype=np.int64).reshape(-1, 3)


def check_mesh(verts, faces, d):
    h = float(d["lengths"]) / int(d["res"])
    assert len(faces) > 1000
    np.testing.assert_array_equal(faces, d["faces"])
    assert verts.shape == d["verts"].shape
    err = np.abs(verts - d["verts"]).max(axis=1)
    assert err.max() <= 0.5 * h, err.max()
    # the bisection stops at the same midpoints almost everywhere
    assert np.mean(err <= 1e-12) >= 0.99


def driver_inputs():
    """What the driver meshes (bunnyMarchingCubes3D.cpp:422-466): the state's
    roots moved by QUATERNION(t_x, t_y, t_z, 0), i.e. (w, x, y, z) += (0, 0,
    0.05, 0) for the root translation (0, 0, 0.05), the field centre moved by
    the translation, the configured resolution, slice 0, escape radius 2000
    (TRIANGLE_MESH.cpp:97)."""
    s = lib.o3d_read(os.path.join(GOLDEN, "dropin_state.o3d"))
    q = np.array([0.0, 0.0, 0.05, 0.0])
    rs = RootSet(top_roots=s["top_roots"] + q, top_powers=s["top_powers"],
                 sigma_top=s["sigma_top"], bottom_roots=s["bottom_roots"] + q,
                 bottom_powers=s["bottom_powers"], sigma_bottom=s["sigma_bottom"],
                 scale=s["scale"])
    c = s["center"]
    res = int(fixture()["res"])
    g = Grid((res,) * 3, center=(c[0], c[1], c[2] + 0.05), lengths=tuple(s["lengths"]))
    return rs, g


def test_edge_cache_through_c_abi(ctx, tmp_path):
    d = fixture()
    rs, g = driver_inputs()
    h = ctx.upload(rs)
    it = ctx.iter_params(int(d["max_it"]), 2000.0)
    cap = 4 * g.res[0] * g.res[1] * 8
    v = torch.empty(3 * cap, dtype=torch.float64, device="cuda")
    t = torch.empty(3 * cap, dtype=torch.int32, device="cuda")
    ctx.mesh_capture(True)
    try:
        for _ in range(2):  # the capture restarts with every call
            _, st = ctx.mesh_stream(h, g, it, d_verts64=v.data_ptr(), vert_cap=cap,
                                    d_tris=t.data_ptr(), tri_cap=cap)
            path = tmp_path / "edges.cache"
            ctx.mesh_edge_cache_write(path)
            assert np.array_equal(np.fromfile(path, dtype=np.uint8), d["cache"])
    finally:
        ctx.mesh_capture(False)
        ctx.free(h)
    edges, cubes = lib.mesh_edge_cache_read(path)
    assert len(edges) == st["n_verts"] and len(cubes) > 0
    n = st["n_verts"]
    check_mesh(v[:3 * n].cpu().numpy().reshape(-1, 3),
               t[:3 * st["n_tris"]].cpu().numpy().reshape(-1, 3).astype(np.int64), d)


def _reference_tree():
    ref = os.environ.get("QUIJIBO_REF", "")
    if ref and os.path.isdir(os.path.join(ref, "src")):
        return ref
    stage = os.path.join(ROOT, "oracle", "_ref", "src_stage")
    return stage if os.path.isdir(os.path.join(stage, "src")) else None


@pytest.mark.skipif(_reference_tree() is None,
                    reason="reference sources absent (QUIJIBO_REF unset, no oracle/_ref/src_stage)")
def test_wrapped_driver_matches_reference_driver(tmp_path):
    from quijibo_gb300 import build
    build.build()
    adir = os.path.join(ROOT, "quijibo_gb300", "adapter")
    subprocess.run(["make", "-s", "-j16", "-C", adir, "bunny", "FLAVOUR=double",
                    "REF=" + _reference_tree()], check=True, timeout=900)
    exe = os.path.join(adir, "_build_double", "bunnyMarchingCubes3D_gpu")
    for name in ("dropin_state.o3d", "dropin.cfg"):
        shutil.copy(os.path.join(GOLDEN, name), tmp_path)
    d = fixture()
    res, it = int(d["res"]), int(d["max_it"])
    env = dict(os.environ)
    env.pop("QJG_PRECISION", None)  # the plain FP64 form
    r = subprocess.run([exe, "dropin.cfg"], cwd=tmp_path, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    verts, faces = read_obj(tmp_path / ("dropin.res.%d.iterations.%d_translationz.obj" % (res, it)))
    check_mesh(verts, faces, d)
    cache = tmp_path / ("dropin.res.%d.iterations.%d.cache" % (res, it))
    assert np.array_equal(np.fromfile(cache, dtype=np.uint8), d["cache"])
    # a second run finds the cache; the mesh is the same
    r = subprocess.run([exe, "dropin.cfg"], cwd=tmp_path, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "does not match" not in r.stdout
    verts2, faces2 = read_obj(tmp_path / ("dropin.res.%d.iterations.%d_translationz.obj" % (res, it)))
    assert np.array_equal(faces2, faces) and np.array_equal(verts2, verts)


@pytest.mark.skipif(_reference_tree() is None,
                    reason="reference sources absent (QUIJIBO_REF unset, no oracle/_ref/src_stage)")
@pytest.mark.parametrize("precision", ["", "fp32refine"])
def test_wrapped_lagrange_driver_matches_reference_driver(tmp_path, precision):
    from quijibo_gb300 import build
    build.build()
    adir = os.path.join(ROOT, "quijibo_gb300", "adapter")
    subprocess.run(["make", "-s", "-j16", "-C", adir, "lagrange", "FLAVOUR=double",
                    "REF=" + _reference_tree()], check=True, timeout=900)
    exe = os.path.join(adir, "_build_double", "lagrangeBunny3D_gpu")
    for name in ("dropin_state.o3d", "dropin_lagrange.cfg"):
        shutil.copy(os.path.join(GOLDEN, name), tmp_path)
    d = dict(np.load(os.path.join(GOLDEN, "dropin_lagrange_ref.npz")))
    res, it = int(d["res"]), int(d["max_it"])
    env = dict(os.environ)
    env.pop("QJG_PRECISION", None)
    if precision:
        env["QJG_PRECISION"] = precision
    r = subprocess.run([exe, "dropin_lagrange.cfg"], cwd=tmp_path, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    verts, faces = read_obj(tmp_path / ("dropin_lagrange.res.%d.iterations.%d_translationz.obj"
                                        % (res, it)))
    check_mesh(verts, faces, d)
