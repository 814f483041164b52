"""The source-level binding (curvib_old_gb300/compat/poisson_gb300.c) on the real
libcvb and a GPU, against the reference's own routines.

tests/compat/glue_real.c builds a UserMG with the reference's MG_Initial steps
and FormMetrics (oracle harness), drives PoissonSetup_GB300 ->
PoissonSolver_MG_GB300 -> UpdatePressure_GB300 -> Projection_GB300 ->
Convection_GB300 through the real library, and compares Ucont, Phi, P, Ucat
and Conv with VolumeFlux_rev / PoissonLHSNew / PoissonRHS / UpdatePressure /
Projection / Contra2Cart / GhostNodeVelocity / Convection of the reference
compiled against the PETSc shim.  The binding and the driver include the
reference's variables.h, so both are compiled from the preprocessed units
oracle/build_ref.sh leaves in oracle/_ref/src/ (made where the reference
checkout is, and carried with the repository); without them the test skips.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
PRE = ROOT / "oracle" / "_ref" / "src"


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_binding_on_the_real_library_matches_reference(tmp_path, precision):
    from curvib_old_gb300 import _lib
    from oracle import oracle as O
    if not (PRE / "glue_real.i").exists() or not (PRE / "poisson_gb300.i").exists() or shutil.which("gcc") is None:
        pytest.skip("preprocessed reference units not present")
    ref = O.build_reference()
    assert ref is not None and ref.exists()
    lib = Path(_lib.lib_path())
    _lib.lib()
    exe = tmp_path / "glue_real"
    subprocess.run(["gcc", "-std=gnu99", "-O1", "-ffp-contract=off", "-g", "-rdynamic", "-w", str(PRE / "poisson_gb300.i"), str(PRE / "glue_real.i"),
                    "-L", str(lib.parent), "-lcvb", f"-Wl,-rpath,{lib.parent}", "-L", str(ref.parent), "-lcvbref",
                    f"-Wl,-rpath,{ref.parent}", "-lm", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), precision], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
