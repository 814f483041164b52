"""The source-level binding curvib_old_gb300/compat/poisson_gb300.c, on the CPU.

It is compiled against the reference's own variables.h (with the oracle's PETSc
API shim standing in for PETSc), so a type or field-name mismatch with CURVIB's
UserCtx fails here.  tests/compat/glue_check.c then drives it on a UserMG that
the reference's MG_Initial steps and FormMetrics built (oracle harness), with a
recording stand-in for libcvb, and checks what reaches the library and what
the binding leaves in the ghosted vectors.  A second test checks that every
libcvb symbol the binding uses is exported by the real library.

Needs the reference checkout (for variables.h); skipped without it.
"""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]
GLUE = ROOT / "curvib_old_gb300" / "compat" / "poisson_gb300.c"
COMPAT_TESTS = ROOT / "tests" / "compat"

pytestmark = pytest.mark.skipif(
    not (O.REF_DIR / "variables.h").exists() or shutil.which("gcc") is None,
    reason="needs the reference checkout (variables.h) and gcc")


def _includes():
    return ["-I", str(ROOT / "oracle" / "petsc_shim" / "include"), "-I", str(O.REF_DIR),
            "-I", str(ROOT / "include"), "-I", str(GLUE.parent), "-I", str(COMPAT_TESTS)]


def _compile_glue(out: Path) -> Path:
    obj = out / "poisson_gb300.o"
    # every call must be declared: an undeclared libcvb or PETSc call would be an
    # implicit declaration with the wrong argument types
    subprocess.run(["gcc", "-std=gnu99", "-O1", "-Wall", "-Werror=implicit-function-declaration",
                    "-Werror=incompatible-pointer-types", "-Werror=int-conversion", "-c", str(GLUE),
                    "-o", str(obj)] + _includes(), check=True)
    return obj


def test_binding_drives_libcvb_from_a_usermg(tmp_path):
    ref = O.build_reference()
    assert ref is not None and ref.exists()
    obj = _compile_glue(tmp_path)
    exe = tmp_path / "glue_check"
    subprocess.run(["gcc", "-std=gnu99", "-O1", "-w", str(obj), str(COMPAT_TESTS / "cvb_record.c"),
                    str(COMPAT_TESTS / "glue_check.c"), "-L", str(ref.parent), "-lcvbref",
                    f"-Wl,-rpath,{ref.parent}", "-lm", "-o", str(exe)] + _includes(), check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout


def test_binding_uses_only_exported_entry_points(tmp_path):
    from curvib_old_gb300 import build, _lib
    build.build()
    obj = _compile_glue(tmp_path)
    nm = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True, check=True).stdout
    used = sorted({ln.split()[-1] for ln in nm.splitlines() if ln.split() and ln.split()[-1].startswith("cvb_")})
    assert "cvb_poisson_solver_mg" in used and "cvb_setup_hierarchy" in used
    L = ctypes.CDLL(str(_lib.lib_path()))
    missing = [n for n in used if not hasattr(L, n)]
    assert not missing, missing
