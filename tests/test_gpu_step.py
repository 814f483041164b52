"""The projection step through the reference's entry points.

Bar: cvb_poisson_solver_mg (VolumeFlux_rev, PoissonRHS and the solve in one
call, the right-hand side kept on the device) returns the same corrected
fluxes and the same pressure, bit for bit, as the three calls made one after
another with the right-hand side passing through host memory; UpdatePressure
and Projection on its result match the oracle.
"""
import numpy as np
import pytest

from cases import build
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0


@pytest.mark.parametrize("name", ["box_sphere", "channel_periodic"])
@pytest.mark.parametrize("precision", [0, 1])
def test_solver_mg_equals_its_steps(name, precision):
    import types
    from curvib_old_gb300.solver import PoissonContext
    c = build(name)
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], ucont=c["ucont"], bctype=c["bctype"],
                              semi=c["semi"], per=c["per"])
    ctx = PoissonContext().setup(P)
    try:
        phi1, uc1, st1 = ctx.poisson_solver_mg(P.ucont, DT, ST, immersed=1, precision=precision, rtol=1e-10)
        uc2, _, _ = ctx.volume_flux_rev(P.ucont, 0.0, 1)
        b, _ = ctx.poisson_rhs(uc2, DT, ST)
        phi2, st2 = ctx.solve(b, precision=precision, rtol=1e-10)
        assert np.array_equal(uc1, uc2)
        assert st1["iterations"] == st2["iterations"] and np.array_equal(phi1, phi2)
        L = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
        p0 = np.zeros_like(phi1)
        p_g, phi_g = ctx.update_pressure(p0, phi1)
        uc_g = ctx.projection(phi_g, DT, ST, uc1)
        p_o, phi_o, uc_o = O.update_and_project(L, p0, phi1, uc1, DT, ST)
        assert np.array_equal(p_g, p_o) and np.array_equal(phi_g, phi_o) and np.array_equal(uc_g, uc_o)
    finally:
        ctx.close()
