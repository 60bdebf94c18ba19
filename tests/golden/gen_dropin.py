"""Generate the drop-in fixtures: the reference's own bunnyMarchingCubes3D
and lagrangeBunny3D drivers, unmodified
(projects/bunnyMarchingCubes3D/bunnyMarchingCubes3D.cpp,
projects/lagrangeBunny3D/lagrangeBunny3D.cpp, built by `make -C oracle
driver` in the Real=double flavour), run on a small configuration.  Each
driver reads an optimizer state (.o3d), moves the roots and the field centre
by the root translation, meshes the map with the streaming marching-cubes
constructor (bunny: the quotient map, writing its edge cache; lagrange: the
Lagrange order) and writes the OBJ.  tests/test_dropin_gpu.py runs the same
drivers linked against the GPU library through the adapter and compares
their files with these.

    QUIJIBO_REF=<QUIJIBO checkout> make -C oracle ref driver
    python tests/golden/gen_dropin.py

Outputs (committed): dropin_state.o3d (written by the reference's
OPTIMIZE_3D::write), dropin.cfg, dropin_ref.npz (the OBJ's vertices and faces
and the cache file's bytes), dropin_lagrange.cfg, dropin_lagrange_ref.npz
(the Lagrange driver's OBJ).
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402
from quijibo_gb300.rootsets import Grid, precision_workload  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "bunnyMarchingCubes3D_ref")
LAGRANGE_DRIVER = os.path.join(ROOT, "oracle", "_ref", "lagrangeBunny3D_ref")
RES, MAX_IT = 40, 20
CFG = """root translation = (0.0,0.0,0.05)
optimization file = dropin_state.o3d
max iterations = %d
field res = %d
output prefix = ./dropin
""" % (MAX_IT, RES)
# the driver's output names (bunnyMarchingCubes3D.cpp:75-78, 456-466)
OBJ = "dropin.res.%d.iterations.%d_translationz.obj" % (RES, MAX_IT)
CACHE = "dropin.res.%d.iterations.%d.cache" % (RES, MAX_IT)
# lagrangeBunny3D.cpp:124-129 reads the same keys; its OBJ name: :101-104
LAGRANGE_CFG = CFG.replace("./dropin", "./dropin_lagrange")
LAGRANGE_OBJ = "dropin_lagrange.res.%d.iterations.%d_translationz.obj" % (RES, MAX_IT)


def read_obj(path):
    """Vertices (float64) and 0-based faces of an OBJ written by
    TRIANGLE_MESH::writeOBJ."""
    v, f = [], []
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            v.append([float(a) for a in t[1:4]])
        elif t[0] == "f":
            f.append([int(a.split("/")[0]) - 1 for a in t[1:4]])
    return np.array(v, dtype=np.float64).reshape(-1, 3), np.array(f, dtype=np.int64).reshape(-1, 3)


def state():
    """The optimizer state: the precision workload's map (16 top / 8 bottom
    roots, exponents {1, 2}, conformal scale) with a fractal field header over
    [-1.5, 1.5]^3 (the driver meshes that box) and small distance and
    curvature fields."""
    rs, _, _ = precision_workload(32)
    g = Grid((4, 4, 4), center=(0.0, 0.0, 0.0), lengths=(3.0, 3.0, 3.0))
    dg = Grid((4, 4, 4), center=(0.0, 0.0, 0.0), lengths=(3.0, 3.0, 3.0))
    dist = np.linspace(-1.0, 1.0, dg.n_voxels)
    return rs, g, np.zeros(g.n_voxels), dg, dist, np.zeros(dg.n_voxels)


def main():
    if not os.path.exists(DRIVER):
        raise SystemExit("build the reference driver first: make -C oracle ref driver")
    rd = Reference("double")
    o3d = os.path.join(OUT, "dropin_state.o3d")
    rd.o3d_write(o3d, *state())
    with open(os.path.join(OUT, "dropin.cfg"), "w") as f:
        f.write(CFG)
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(o3d, d)
        shutil.copy(os.path.join(OUT, "dropin.cfg"), d)
        subprocess.run([DRIVER, "dropin.cfg"], cwd=d, check=True, stdout=subprocess.DEVNULL)
        verts, faces = read_obj(os.path.join(d, OBJ))
        cache = np.fromfile(os.path.join(d, CACHE), dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, "dropin_ref.npz"), verts=verts, faces=faces, cache=cache,
                        res=RES, max_it=MAX_IT, lengths=3.0)
    print("dropin: %d vertices, %d faces, cache %d bytes" % (len(verts), len(faces), len(cache)))
    with open(os.path.join(OUT, "dropin_lagrange.cfg"), "w") as f:
        f.write(LAGRANGE_CFG)
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(o3d, d)
        shutil.copy(os.path.join(OUT, "dropin_lagrange.cfg"), d)
        subprocess.run([LAGRANGE_DRIVER, "dropin_lagrange.cfg"], cwd=d, check=True,
                       stdout=subprocess.DEVNULL)
        verts, faces = read_obj(os.path.join(d, LAGRANGE_OBJ))
    np.savez_compressed(os.path.join(OUT, "dropin_lagrange_ref.npz"), verts=verts, faces=faces,
                        res=RES, max_it=MAX_IT, lengths=3.0)
    print("dropin lagrange: %d vertices, %d faces" % (len(verts), len(faces)))


if __name__ == "__main__":
    main()
