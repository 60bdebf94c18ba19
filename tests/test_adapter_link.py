"""The reference drivers link against the GPU library through the adapter's
--wrap bindings (needs the reference sources; skipped where they are absent,
as on the GPU machine).  Linking proves every wrapped reference symbol resolves
to the adapter; running the drivers needs their .o3d inputs, which are not
available."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("QUIJIBO_REF", "")


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "src")),
                    reason="reference sources absent (QUIJIBO_REF unset)")
def test_reference_drivers_link_through_adapter():
    from quijibo_gb300 import build
    build.build()
    adir = os.path.join(ROOT, "quijibo_gb300", "adapter")
    subprocess.run(["make", "-s", "-j8", "-C", adir, "all", "REF=" + REF], check=True)
    for exe in ("bunnyMarchingCubes3D_gpu", "toothOptimizer_gpu", "lagrangeBunny3D_gpu"):
        path = os.path.join(adir, "_build", exe)
        assert os.path.exists(path)
        syms = subprocess.run(["nm", path], capture_output=True, text=True, check=True).stdout
        assert "__wrap__ZN11OPTIMIZE_3D32computeLogScaledPowerRationalMap" in syms
    tooth = subprocess.run(["nm", os.path.join(adir, "_build", "toothOptimizer_gpu")],
                           capture_output=True, text=True, check=True).stdout
    assert "__wrap__ZN11OPTIMIZE_3D14computeScoreAPEv" in tooth
    lag = subprocess.run(["nm", os.path.join(adir, "_build", "lagrangeBunny3D_gpu")],
                         capture_output=True, text=True, check=True).stdout
    # the 10-argument (Lagrange) streaming mesher constructor
    assert ("__wrap__ZN13TRIANGLE_MESHC1ERK5TVEC3IeES3_RKS0_IiERK13POLYNOMIAL_4DS9_eieeRK10QUATERNION\n"
            in lag)
