"""The C-ABI library: it builds, loads and exports every entry point include/cvb.h
declares.  No GPU work here -- creating a context needs a device."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    text = (ROOT / "include" / "cvb.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cvb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_path():
    names = _declared()
    for must in ("cvb_init", "cvb_setup_hierarchy", "cvb_poisson_rhs", "cvb_poisson_solve",
                 "cvb_poisson_solver_mg", "cvb_volume_flux_rev", "cvb_update_pressure", "cvb_projection"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from curvib_old_gb300 import build, _lib
    build.build()
    L = ctypes.CDLL(str(_lib.lib_path()))
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing
    # the Python bindings cover the same surface
    assert set(_declared()) <= set(_lib.EXPORTS)


def test_default_options_without_a_gpu():
    from curvib_old_gb300 import _lib
    o = _lib.default_opts()
    assert o.precision == _lib.MIXED and o.restart == 30
    # zebra line Gauss-Seidel, over-relaxed (SOR range 0 < omega < 2)
    assert o.smoother == _lib.ZEBRA and 1.0 < o.omega < 2.0
    assert (o.pre_sweeps, o.post_sweeps) == (2, 2)
    assert o.rtol == 1e-8 and o.project_rhs == 1


def test_ibm_ray_offsets_match_srand_rand_and_leave_the_callers_sequence():
    """cvb_ibm_ray_offsets draws randomdirection's offsets (ibm.c:101-104) from a
    private generator state: the values equal srand(seed); rand() (the oracle
    calls exactly that), and the caller's rand() sequence goes on undisturbed."""
    import numpy as np
    from curvib_old_gb300 import build, _lib
    from oracle import oracle as O
    build.build()
    L = _lib.lib()
    n = 64
    got = np.zeros(n)
    assert L.cvb_ibm_ray_offsets(n, _lib.ptr(got)) == 0
    want = np.zeros(n)
    O.lib().orc_ibm_ray_offsets(n, want.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(got, want)
    assert (np.abs(got) <= 0.5).all() and len(set(got.tolist())) == n
    libc = ctypes.CDLL(None)
    libc.srand(12345)
    seq = [libc.rand() for _ in range(3)]
    libc.srand(12345)
    first = libc.rand()
    assert L.cvb_ibm_ray_offsets(n, _lib.ptr(got)) == 0
    assert [first, libc.rand(), libc.rand()] == seq
