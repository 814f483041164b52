"""Failure paths, exercised on the host side of the GPU path: every one returns a
status and a message, and leaves the context usable.  None of them faults,
traps or hangs the GPU: the bad inputs are caught before or between kernels.

Cases: a NaN right-hand side (NAN_DETECTED), a zero iteration budget and a
right-hand side outside the operator's range without the range projection
(NOT_CONVERGED), corrupted nvert codes and levels that are not a coarsening
(BAD_INPUT), a device-memory cap below what the set-up needs (OOM, from the
context's own allocation guard standing in for a failing cudaMalloc), and a
solve before any set-up (NOT_SETUP).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0


def _problem(cells=(12, 12, 12), nl=2):
    from curvib_old_gb300 import workload as W
    return W.make_problem(cells, (1.0, 1.0, 1.0), 2.0, True, (False, False, False), [(0.5, 0.5, 0.5, 0.25)],
                          nlevels=nl)


def _rhs(ctx, P):
    from curvib_old_gb300 import workload as W
    uc, _, _ = ctx.volume_flux_rev(P.ucont, 0.0, 1)
    b, _ = ctx.poisson_rhs(uc, DT, ST)
    return W.noisy_rhs(b, P.nvert, P.metrics[-1]["Aj"], DT, seed=3)


@pytest.fixture(scope="module")
def setup():
    from curvib_old_gb300.solver import PoissonContext
    P = _problem()
    ctx = PoissonContext().setup(P)
    b = _rhs(ctx, P)
    yield ctx, P, b
    ctx.close()


def _status(exc):
    from curvib_old_gb300 import _lib
    return _lib.STATUS_NAMES[exc.value.status]


def test_nan_rhs(setup):
    from curvib_old_gb300._lib import CvbError
    ctx, P, b = setup
    bad = b.copy()
    bad[3, 4, 5] = np.nan
    with pytest.raises(CvbError) as e:
        ctx.solve(bad)
    assert _status(e) == "NAN_DETECTED"
    phi, st = ctx.solve(b)  # the context still works
    assert st["status"] == 0


def test_zero_iteration_budget(setup):
    from curvib_old_gb300._lib import CvbError
    ctx, P, b = setup
    with pytest.raises(CvbError) as e:
        ctx.solve(b, max_it=0)
    assert _status(e) == "NOT_CONVERGED"
    _, st = ctx.solve(b, max_it=0, check=False)
    assert st["status"] == 1 and st["iterations"] == 0


def test_incompatible_rhs_needs_the_range_projection(setup):
    from curvib_old_gb300._lib import CvbError
    ctx, P, b = setup
    aj = P.metrics[-1]["Aj"]
    fl = np.zeros(b.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = P.nvert[1:-1, 1:-1, 1:-1] < 0.1
    off = b.copy()
    off[fl] += 1e-2 * np.abs(b).max() * aj[fl]  # a component outside range(A)
    with pytest.raises(CvbError) as e:
        ctx.solve(off, project_rhs=0, max_it=40)
    assert _status(e) == "NOT_CONVERGED"
    phi, st = ctx.solve(off, project_rhs=1, max_it=100)
    assert st["status"] == 0 and st["rhs_projected"] != 0.0


@pytest.mark.parametrize("value", [np.nan, -1.0, np.inf])
def test_corrupted_nvert(value):
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300.solver import PoissonContext
    P = _problem()
    P.nvert[4, 5, 6] = value
    ctx = PoissonContext()
    try:
        with pytest.raises(CvbError) as e:
            ctx.setup(P)
        assert _status(e) == "BAD_INPUT" and "nvert" in str(e.value)
    finally:
        ctx.close()


def test_levels_that_are_not_a_coarsening():
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300.solver import PoissonContext
    P = _problem()
    Q = _problem(cells=(16, 16, 16))
    P.metrics[0] = Q.metrics[0]  # coarse level of another box
    ctx = PoissonContext()
    try:
        with pytest.raises(CvbError) as e:
            ctx.setup(P)
        assert _status(e) == "BAD_INPUT" and "coarsening" in str(e.value)
    finally:
        ctx.close()


def test_device_limit_gives_oom_and_recovers():
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300.solver import PoissonContext
    P = _problem()
    ctx = PoissonContext()
    try:
        ctx.set_device_limit(1 << 20)
        with pytest.raises(CvbError) as e:
            ctx.setup(P)
        assert _status(e) == "OOM"
        ctx.set_device_limit(0)
        ctx.setup(P)
        phi, st = ctx.solve(_rhs(ctx, P))
        assert st["status"] == 0
    finally:
        ctx.close()


def test_solve_before_setup():
    from curvib_old_gb300 import _lib
    from curvib_old_gb300.solver import PoissonContext
    ctx = PoissonContext()
    try:
        o = _lib.default_opts()
        st = _lib.SolveStats()
        rc = _lib.lib().cvb_solve_resident(ctx._ctx, __import__("ctypes").byref(o), __import__("ctypes").byref(st))
        assert _lib.STATUS_NAMES[rc] == "NOT_SETUP"
    finally:
        ctx.close()
