"""The steps after Projection's flux correction on the GPU (libcvb.so through
its C ABI) against the CPU oracle: Contra2Cart (rhs.c:25) and
GhostNodeVelocity (bcs.c:3645), bit for bit, on the parity scenarios and on
the slip / moving-lid / O-grid variants with blanked cells (nvert > 7); the
one-call projection against the three steps; boundary types that are not
covered refused with nothing written.  A slip face on the low y side gives NaN,
as in the reference (its normal comes from the ring cell's eta, which
FormMetrics leaves zero), so arrays compare with NaN equal to NaN.  Convection (rhs.c:1463), the first
term of the momentum right-hand side, bit for bit on the same boxes.
"""
import types

import numpy as np
import pytest

from cases import POST_U_BC, POST_VARIANTS, SCENARIOS, build, conv_edge_nvert, post_inputs, seeded
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0
# key -> (scenario, bctype or None for the scenario's own, blanked cells, seed)
CASES = {name: (name, None, [], 0) for name in SCENARIOS}
CASES.update(POST_VARIANTS)


def _problem(key):
    scen, bct, blank, seed = CASES[key]
    c = build(scen)
    nv = c["nvert"].copy()
    for (k, j, i) in blank:
        nv[k, j, i] = 8.0
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=nv, ucont=c["ucont"], bctype=bct or c["bctype"],
                              semi=c["semi"], per=c["per"], nl=c["nl"])
    return P, seed


@pytest.fixture(scope="module")
def ctxs():
    from curvib_old_gb300.solver import PoissonContext
    out = {}
    for key in CASES:
        P, seed = _problem(key)
        ctx = PoissonContext().setup(P)
        if key in POST_VARIANTS:
            # the annulus face's cell centres and the rheology plates' velocity
            ctx.set_cell_centres(P.metrics[-1]["Cent"])
            ctx.set_plate_velocity(POST_U_BC)
        out[key] = (ctx, P, O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi), seed)
    yield out
    for c, _, _, _ in out.values():
        c.close()


@pytest.mark.parametrize("key", sorted(CASES))
def test_contra2cart_and_ghost_nodes_bit_exact(ctxs, key):
    ctx, P, L, seed = ctxs[key]
    ucat0, ubcs0 = post_inputs(P.nvert.shape, seed)
    c_g = ctx.contra2cart(P.ucont, ucat0)
    c_o = O.contra2cart(L, P.ucont, ucat0)
    assert np.array_equal(c_g, c_o)
    # the cells Contra2Cart leaves alone keep their input
    untouched = (P.nvert >= 0.1) & (P.nvert <= 7.0)
    untouched[[0, -1], :, :] = untouched[:, [0, -1], :] = untouched[:, :, [0, -1]] = True
    assert untouched.any() and not untouched.all()
    assert np.array_equal(c_g[untouched], ucat0[untouched])
    ub_g, u_g = ctx.ghost_node_velocity(ubcs0, c_o)
    extra = (P.metrics[-1]["Cent"], POST_U_BC) if key in POST_VARIANTS else (None, 0.0)
    rc, ub_o, u_o = O.ghost_node_velocity(L, ubcs0, c_o, *extra)
    assert rc == 0
    assert np.array_equal(ub_g, ub_o, equal_nan=True)
    assert np.array_equal(u_g, u_o, equal_nan=True)


@pytest.mark.parametrize("key", ["box_sphere", "channel_periodic", "triply_periodic", "slip_lid_ogrid",
                                 "periodic_slip_y", "annulus_y", "rheology_plates"])
def test_projection_cart_equals_the_three_steps(ctxs, key):
    ctx, P, L, seed = ctxs[key]
    fine = P.nvert.shape
    _, phi_o, uc_o = O.update_and_project(L, seeded(fine, 400), seeded(fine, 401), P.ucont, DT, ST)
    ucat0, ubcs0 = post_inputs(fine, seed)
    uc_g, ub_g, u_g = ctx.projection_cart(phi_o, DT, ST, P.ucont, ubcs0, ucat0)
    assert np.array_equal(uc_g, uc_o)
    extra = (P.metrics[-1]["Cent"], POST_U_BC) if key in POST_VARIANTS else (None, 0.0)
    rc, ub_o, u_o = O.ghost_node_velocity(L, ubcs0, O.contra2cart(L, uc_o, ucat0), *extra)
    assert rc == 0
    assert np.array_equal(ub_g, ub_o, equal_nan=True)
    assert np.array_equal(u_g, u_o, equal_nan=True)


@pytest.mark.parametrize("bct", [[1, 1, 11, 1, 1, 1]])
def test_uncovered_boundary_types_refused(bct):
    """An annulus face before the cell centres were given is refused, with
    nothing written, and the context stays usable."""
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300.solver import PoissonContext
    c = build("box_sphere")
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], ucont=c["ucont"], bctype=bct,
                              semi=c["semi"], per=c["per"], nl=c["nl"])
    ctx = PoissonContext().setup(P)
    try:
        ucat0, ubcs0 = post_inputs(c["nvert"].shape, 0)
        with pytest.raises(CvbError) as e:
            ctx.ghost_node_velocity(ubcs0, ucat0)
        assert e.value.status == 4  # CVB_BAD_INPUT
        with pytest.raises(CvbError):
            ctx.projection_cart(np.zeros(c["nvert"].shape), DT, ST, c["ucont"], ubcs0, ucat0)
        # the context stays usable: Contra2Cart does not depend on the types
        assert np.array_equal(ctx.contra2cart(c["ucont"], ucat0),
                              O.contra2cart(O.OLevel(c["metrics"][-1], c["nvert"], bct, c["semi"]),
                                            c["ucont"], ucat0))
    finally:
        ctx.close()


@pytest.mark.parametrize("key", sorted(CASES))
def test_divergence_matches_oracle(ctxs, key):
    """Divergence (main.c:469-593): the maximum and its first index, from a host
    Ucont and from the device copy the one-call projection leaves."""
    ctx, P, L, seed = ctxs[key]
    assert ctx.divergence(P.ucont) == O.divergence(L, P.ucont)
    fine = P.nvert.shape
    _, phi_o, uc_o = O.update_and_project(L, seeded(fine, 400), seeded(fine, 401), P.ucont, DT, ST)
    ucat0, ubcs0 = post_inputs(fine, seed)
    ctx.projection_cart(phi_o, DT, ST, P.ucont, ubcs0, ucat0)
    m, at = ctx.divergence()
    assert (m, at) == O.divergence(L, uc_o)


@pytest.mark.parametrize("key", sorted(CASES))
def test_convection_bit_exact(ctxs, key):
    """Convection (rhs.c:1463-1946), QUICK and central, bit for bit against the
    oracle, periodic seams included."""
    ctx, P, L, seed = ctxs[key]
    ucat0, _ = post_inputs(P.nvert.shape, seed)
    for central in (False, True):
        rc, want = O.convection(L, P.ucont, ucat0, int(central))
        assert rc == 0
        got = ctx.convection(P.ucont, ucat0, central)
        assert got.tobytes() == want.tobytes(), central  # signed zeros included
        assert want[1:-1, 1:-1, 1:-1].any()


def test_convection_edges_and_device_inputs():
    """Convection next to the high ends, beside nvert of exactly 0.1 and blanked
    cells (the reference's one-sided forms and its reads past the row ends);
    then on the Ucont and Ucat the one-call projection leaves on the device."""
    from curvib_old_gb300.solver import PoissonContext
    P, seed = _problem("box_sphere")
    P.nvert = conv_edge_nvert(P.nvert)
    L = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
    ctx = PoissonContext().setup(P)
    try:
        ucat0, ubcs0 = post_inputs(P.nvert.shape, seed)
        for central in (0, 1):
            assert np.array_equal(ctx.convection(P.ucont, ucat0, central), O.convection(L, P.ucont, ucat0, central)[1])
        # zero fluxes and velocities of either sign, and values above 2^1000,
        # where the kernel takes the full QUICK expression
        uc_sp, u_sp = P.ucont.copy(), ucat0.copy()
        uc_sp[5, 5, 5] = (0.0, -0.0, 0.0)
        uc_sp[7, 3, 4, 0] = -0.0
        u_sp[4, 5, 6] = (0.0, -0.0, 2.0 ** 1010)
        u_sp[6, 6, 3, 1] = -(2.0 ** 1005)
        u_sp[3, 8, 8] = 0.0
        u_sp[3, 8, 9] = -0.0
        for central in (0, 1):
            want = O.convection(L, uc_sp, u_sp, central)[1]
            assert np.isfinite(want).all()
            assert ctx.convection(uc_sp, u_sp, central).tobytes() == want.tobytes(), central
        fine = P.nvert.shape
        _, phi_o, _ = O.update_and_project(L, seeded(fine, 400), seeded(fine, 401), P.ucont, DT, ST)
        uc, _, u = ctx.projection_cart(phi_o, DT, ST, P.ucont, ubcs0, ucat0)
        assert np.array_equal(ctx.convection(), O.convection(L, uc, u)[1])
    finally:
        ctx.close()


@pytest.mark.parametrize("key", sorted(CASES))
def test_metrics_divergence_matches_oracle(ctxs, key):
    """MetricsDivergence (metrics.c:1551-1625) of the metrics the context holds:
    the maximum and its first index, bit for bit."""
    ctx, P, L, seed = ctxs[key]
    assert ctx.metrics_divergence() == O.metrics_divergence(L)


def test_convection_across_periodic_seams():
    """The periodic channel with blocked cells next to its x and z seams
    (cases.CONV_SEAM): the seam faces take the full QUICK form across the seam
    where both sides are fluid and the one-sided forms beside the blocked cells."""
    from cases import conv_seam_nvert
    from curvib_old_gb300.solver import PoissonContext
    P, seed = _problem("channel_periodic")
    P.nvert = conv_seam_nvert(P.nvert)
    L = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
    ctx = PoissonContext().setup(P)
    try:
        ucat0, _ = post_inputs(P.nvert.shape, seed)
        for central in (0, 1):
            rc, want = O.convection(L, P.ucont, ucat0, central)
            assert rc == 0 and ctx.convection(P.ucont, ucat0, central).tobytes() == want.tobytes(), central
    finally:
        ctx.close()
