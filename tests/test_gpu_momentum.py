"""The momentum right-hand side on the GPU against the CPU oracle, bit for bit.

Viscous (rhs.c:1947), FormFunction1 (rhs.c:2567) and CalcRHS
(implicitsolver.c:6449) through the C ABI on the walled scenarios, QUICK and
central, first step and second-order backward; on box_sphere also with the
cells whose tangential pressure derivative the reference leaves unassigned
(cases.MOM_EDGES: the value of the previous cell in its loop order stands)
and with a convective-outflow face; FormBCS (bcs.c:4436) and the pseudo-time
iteration ImpRK (implicitsolver.c:7094) on the all-wall scenarios.  The oracle
is pinned to the reference's own routines (tests/test_oracle_pin.py).  Results are compared as bytes, so
signed zeros count; the periodic boxes are refused.
"""
import math
import types

import numpy as np
import pytest

from cases import MOM_DT, MOM_REN, SCENARIOS, build, mom_edge_nvert, momentum_inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ctx(c, nvert, bctype):
    from curvib_old_gb300.solver import PoissonContext
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=nvert, ucont=c["ucont"], bctype=bctype, semi=c["semi"])
    return PoissonContext().setup(P)


def _same(a, b):
    return np.ascontiguousarray(a).tobytes() == np.ascontiguousarray(b).tobytes()


CASES = [(n, "plain") for n in sorted(SCENARIOS) if not SCENARIOS[n][1][0] and not any(SCENARIOS[n][1])] + \
        [("box_sphere", "edges"), ("box_sphere", "outflow8")]


@pytest.mark.parametrize("name,variant", CASES)
def test_momentum_rhs_matches_oracle(name, variant):
    c = build(name)
    nvert = mom_edge_nvert(c["nvert"]) if variant == "edges" else c["nvert"]
    bctype = list(c["bctype"][:5]) + [8] if variant == "outflow8" else list(c["bctype"])
    ctx = _ctx(c, nvert, bctype)
    try:
        L = O.OLevel(c["metrics"][-1], nvert, bctype, c["semi"])
        ucat0, p, uo, urm = momentum_inputs(nvert.shape)
        assert _same(ctx.viscous(ucat0, MOM_REN), O.viscous(L, ucat0, MOM_REN))
        ring = np.random.default_rng(3).standard_normal(nvert.shape + (3,))  # rhs's incoming ring stays
        for central in (0, 1):
            f_g, u_g = ctx.form_function1(c["ucont"], ucat0, p, MOM_REN, central, rhs=ring)
            rc, f_o, u_o = O.form_function1(L, c["ucont"], ucat0, p, MOM_REN, central, rhs=ring)
            assert rc == 0 and _same(u_g, u_o) and _same(f_g, f_o), central
        for ti in (1, 5):
            r_g, _ = ctx.calc_rhs(c["ucont"], uo, urm, ucat0, p, MOM_REN, MOM_DT, ti, 0, rhs=ring)
            rc, r_o, _ = O.calc_rhs(L, c["ucont"], uo, urm, ucat0, p, MOM_REN, MOM_DT, ti, 0, rhs=ring)
            assert rc == 0 and _same(r_g, r_o), ti
    finally:
        ctx.close()


@pytest.mark.parametrize("name", ["channel_periodic", "triply_periodic"])
def test_periodic_boxes_viscous_and_refusals(name):
    """On periodic boxes Viscous (which reads the box alone) matches the oracle
    bit for bit; FormFunction1 and CalcRHS, whose periodic seam branches are
    not restated, are refused."""
    from curvib_old_gb300._lib import CVB_BAD_INPUT, CvbError
    c = build(name)
    ctx = _ctx(c, c["nvert"], c["bctype"])
    try:
        L = O.OLevel(c["metrics"][-1], c["nvert"], c["bctype"], c["semi"])
        ucat0, p, _, _ = momentum_inputs(c["nvert"].shape)
        assert _same(ctx.viscous(ucat0, MOM_REN), O.viscous(L, ucat0, MOM_REN))
        with pytest.raises(CvbError) as e:
            ctx.form_function1(c["ucont"], ucat0, p, MOM_REN)
        assert e.value.status == CVB_BAD_INPUT
    finally:
        ctx.close()


WALLED = [n for n in sorted(SCENARIOS) if not any(SCENARIOS[n][1])]


@pytest.mark.parametrize("name", WALLED)
def test_form_bcs_and_imp_rk_match_oracle(name):
    """FormBCS (bcs.c:4436) and the pseudo-time iteration ImpRK
    (implicitsolver.c:7094) on the all-wall scenarios, bit for bit against the
    oracle, which is pinned to the reference's own routines: converged, stopped
    at imp_MAX_IT, and with iterations undone and the step halved (the counts
    checked too); on box_sphere also with cells.MOM_EDGES' nvert."""
    from cases import IMP_ATOL, IMP_RK_RUNS, IMP_RTOL, imp_rk_inputs
    c = build(name)
    for nvert in ([c["nvert"], mom_edge_nvert(c["nvert"])] if name == "box_sphere" else [c["nvert"]]):
        bctype = list(c["bctype"])
        ctx = _ctx(c, nvert, bctype)
        try:
            L = O.OLevel(c["metrics"][-1], nvert, bctype, c["semi"])
            ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(nvert.shape, c["ucont"])
            _, _, u_g, p_g = ctx.form_bcs(c["ucont"], ubcs1, ucat1, p1)
            rc, _, _, u_o, p_o = O.form_bcs(L, c["ucont"], ubcs1, ucat1, p1)
            assert rc == 0 and _same(u_g, u_o) and _same(p_g, p_o)
            rejected = 0
            for ti, cfl, max_it in IMP_RK_RUNS:
                uc_g, u_g, p_g, st_g, _ = ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0,
                                                     cfl, ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it)
                rc, uc_o, u_o, p_o, st_o, _ = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT,
                                                       1.0, cfl, ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it)
                assert rc == 0
                assert (st_g["pseudo_iterations"], st_g["rejected"]) == (st_o.pseudo_iterations, st_o.rejected)
                assert st_g["lambda"] == st_o.lambda_ and st_g["norm_du"] == st_o.norm_du
                assert _same(uc_g, uc_o) and _same(u_g, u_o) and _same(p_g, p_o), (ti, cfl, max_it)
                rejected += st_o.rejected
            assert rejected > 0  # the halving branch ran
        finally:
            ctx.close()


@pytest.mark.parametrize("name", ["box_sphere", "blocked_slab"])
def test_inlet_outlet_match_oracle(name):
    """InflowFlux (bcs.c:99) with the constant and shaped profiles, FormBCS's outlet
    correction with an immersed-boundary flux, and ImpRK on the scenario's grid
    with an inlet on k = 0 and an outlet on the last k face, bit for bit
    against the oracle (pinned to the reference's routines): ucont, ubcs, ucat,
    p, FluxInSum and the iteration counts."""
    from cases import (FLUX_INTP_SUM, IMP_ATOL, IMP_RK_RUNS, IMP_RTOL, INLET_PROFILES, SHAPED_INLETS, TABLE_INLETS,
                       UNIFORM_INLETS, imp_rk_inputs, inlet_plane, inlet_table)
    from curvib_old_gb300._lib import CVB_BAD_INPUT, CvbError
    c = build(name)
    bctype = [1, 1, 1, 1, 5, 4]
    ctx = _ctx(c, c["nvert"], bctype)
    try:
        L = O.OLevel(c["metrics"][-1], c["nvert"], bctype, c["semi"])
        ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(c["nvert"].shape, c["ucont"])
        for prof in INLET_PROFILES:
            uc_g, ub_g, f_g = ctx.inflow_flux(c["ucont"], ubcs1, prof)
            rc, uc_o, ub_o, f_o = O.inflow_flux(L, c["ucont"], ubcs1, prof)
            assert rc == 0 and _same(uc_g, uc_o) and _same(ub_g, ub_o) and f_g == f_o, prof
        plane = inlet_plane(c["nodes"], c["nvert"].shape)
        for prof, cm in SHAPED_INLETS:
            ctx.set_inlet_nodes(plane, cm)
            uc_g, ub_g, f_g = ctx.inflow_flux(c["ucont"], ubcs1, prof)
            rc, uc_o, ub_o, f_o = O.inflow_flux(L, c["ucont"], ubcs1, prof, 0.0, plane, cm)
            assert rc == 0 and _same(uc_g, uc_o) and _same(ub_g, ub_o) and f_g == f_o, prof
        prof, cm = SHAPED_INLETS[1]
        ctx.set_inlet_nodes(plane, cm)
        ti, cfl, max_it = IMP_RK_RUNS[0]
        uc_g, u_g, p_g, st_g, ub_g = ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti,
                                                0, 0, IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM)
        rc, uc_o, u_o, p_o, st_o, ub_o = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl,
                                                  ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM, plane, cm)
        assert rc == 0 and st_g["pseudo_iterations"] == st_o.pseudo_iterations
        assert all(_same(a, b) for a, b in ((uc_g, uc_o), (u_g, u_o), (p_g, p_o), (ub_g, ub_o)))
        for prof, flux_in, t in UNIFORM_INLETS:
            ctx.set_inlet_flux(flux_in, t)
            O.set_inlet_globals(flux_in, t)
            uc_g, ub_g, f_g = ctx.inflow_flux(c["ucont"], ubcs1, prof)
            rc, uc_o, ub_o, f_o = O.inflow_flux(L, c["ucont"], ubcs1, prof)
            assert rc == 0 and _same(uc_g, uc_o) and _same(ub_g, ub_o) and f_g == f_o, prof
        assert ctx.inlet_flux_in() == math.sin(2 * 3.14159 * 37 / 200.)
        uc_g, u_g, p_g, st_g, ub_g = ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti,
                                                0, 0, IMP_ATOL, IMP_RTOL, max_it, 8, FLUX_INTP_SUM)
        rc, uc_o, u_o, p_o, st_o, ub_o = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl,
                                                  ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, 8, FLUX_INTP_SUM)
        assert rc == 0 and st_g["pseudo_iterations"] == st_o.pseudo_iterations
        assert all(_same(a, b) for a, b in ((uc_g, uc_o), (u_g, u_o), (p_g, p_o), (ub_g, ub_o)))
        tbl = inlet_table()
        ctx.set_inlet_table(tbl)
        O.set_inlet_table(tbl)
        try:
            for prof, cm, t in TABLE_INLETS:
                ctx.set_inlet_nodes(plane, cm)
                ctx.set_inlet_flux(0.0, t)
                O.set_inlet_globals(0.0, t)
                uc_g, ub_g, f_g = ctx.inflow_flux(c["ucont"], ubcs1, prof)
                rc, uc_o, ub_o, f_o = O.inflow_flux(L, c["ucont"], ubcs1, prof, 0.0, plane, cm)
                assert rc == 0 and _same(uc_g, uc_o) and _same(ub_g, ub_o) and f_g == f_o, prof
            prof, cm, _ = TABLE_INLETS[0]
            ctx.set_inlet_nodes(plane, cm)
            uc_g, u_g, p_g, st_g, ub_g = ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl,
                                                    ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM)
            rc, uc_o, u_o, p_o, st_o, ub_o = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0,
                                                      cfl, ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM,
                                                      plane, cm)
            assert rc == 0 and st_g["pseudo_iterations"] == st_o.pseudo_iterations
            assert all(_same(a, b) for a, b in ((uc_g, uc_o), (u_g, u_o), (p_g, p_o), (ub_g, ub_o)))
            ctx.set_inlet_flux(0.0, 2000)  # the reference's column -1000: refused
            with pytest.raises(CvbError) as e:
                ctx.inflow_flux(c["ucont"], ubcs1, 0)
            assert e.value.status == CVB_BAD_INPUT
        finally:
            O.set_inlet_table(None)
        uc_i, ub_i, f = ctx.inflow_flux(c["ucont"], ubcs1, 1)
        got = ctx.form_bcs(uc_i, ub_i, ucat1, p1, f, FLUX_INTP_SUM)
        rc, *want = O.form_bcs(L, uc_i, ub_i, ucat1, p1, f, FLUX_INTP_SUM)
        assert rc == 0 and all(_same(a, b) for a, b in zip(got, want))
        for ti, cfl, max_it in IMP_RK_RUNS:
            uc_g, u_g, p_g, st_g, ub_g = ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl,
                                                    ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, 1, FLUX_INTP_SUM)
            rc, uc_o, u_o, p_o, st_o, ub_o = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0,
                                                      cfl, ti, 0, 0, IMP_ATOL, IMP_RTOL, max_it, 1, FLUX_INTP_SUM)
            assert rc == 0
            assert (st_g["pseudo_iterations"], st_g["rejected"]) == (st_o.pseudo_iterations, st_o.rejected)
            assert all(_same(a, b) for a, b in ((uc_g, uc_o), (u_g, u_o), (p_g, p_o), (ub_g, ub_o))), (ti, cfl)
            assert st_g["flux_in_sum"] == O.inflow_flux(L, uc_g, ub_g, 1)[3]
    finally:
        ctx.close()


def test_imp_rk_refuses_other_face_types():
    from curvib_old_gb300._lib import CVB_BAD_INPUT, CvbError
    from cases import imp_rk_inputs
    c = build("box_sphere")
    for bctype, prof in ((list(c["bctype"][:5]) + [8], 1), ([1, 1, 1, 1, 1, 4], 1), ([1, 1, 1, 1, 5, 4], 4)):
        ctx = _ctx(c, c["nvert"], bctype)
        try:
            ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(c["nvert"].shape, c["ucont"])
            calls = [lambda: ctx.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, 1.0, 1, 0,
                                        inletprofile=prof)]
            if prof == 1:
                calls.append(lambda: ctx.form_bcs(c["ucont"], ubcs1, ucat1, p1))
            for call in calls:
                with pytest.raises(CvbError) as e:
                    call()
                assert e.value.status == CVB_BAD_INPUT, bctype
        finally:
            ctx.close()
