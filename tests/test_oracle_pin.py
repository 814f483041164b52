"""The CPU oracle and the workload generator against the reference's own outputs.

The digests in tests/golden/reference_digests.json were produced by the
reference's poisson.c / metrics.c / implicitsolver.c compiled unmodified against
a single-process PETSc API shim (tests/golden/make_golden.py).  Everything here
must agree bit for bit: masks, index maps and FP64 values alike.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from cases import (IBM_CASES, POST_VARIANTS, SCENARIOS, build, conv_edge_nvert, digest, digest_nan, ibm_inputs,
                   post_inputs, seeded)
from curvib_old_gb300 import workload as W
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
REF = json.loads((GOLD / "reference_digests.json").read_text())


def csr_digest(A):
    A = A.tocsr().copy()
    A.sort_indices()
    return {"indptr": digest(A.indptr.astype(np.int64)), "indices": digest(A.indices.astype(np.int64)),
            "data": digest(A.data), "nnz": int(A.nnz)}


def _setup(name):
    z = np.load(GOLD / f"{name}.npz")
    c = build(name, nodes=z["nodes"])
    c["nvert"], c["ucont"] = z["nvert"], z["ucont"]
    return c


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_metrics_generator_matches_reference(name):
    c = _setup(name)
    for l, m in enumerate(c["metrics"]):
        for nm in W.METRIC_NAMES + W.JACOBIAN_NAMES:
            assert digest(m[nm]) == REF["scenarios"][name]["metrics"][l][nm], (l, nm)


def _levels(c):
    nl, semi, bct = c["nl"], c["semi"], c["bctype"]
    Ls = [None] * nl
    Ls[-1] = O.OLevel(c["metrics"][-1], c["nvert"], bct, semi)
    for l in range(nl - 2, -1, -1):
        nvc = O.nvert_restrict(Ls[l + 1], c["metrics"][l]["Aj"].shape, l == 0, semi)
        Ls[l] = O.OLevel(c["metrics"][l], nvc, bct, semi)
    return Ls


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_oracle_matches_reference(name):
    c = _setup(name)
    ref = REF["scenarios"][name]
    dt, st = REF["dt"], REF["st"]
    Ls = _levels(c)
    nl = c["nl"]
    for l in range(nl):
        assert digest(Ls[l].nvert) == ref["nvert"][l], ("nvert", l)
        assert csr_digest(O.lhs_csr(Ls[l])) == ref["lhs"][l], ("lhs", l)
    mns, kske = O.fully_blocked(Ls[0])
    assert mns == ref["multinullspace"]
    if mns:
        mz, my, mx = Ls[0].shape
        assert digest(kske.reshape(my, mx, 2)[1:-1, 1:-1, 0].astype(np.int64)) == ref["kske"]
    uc, f, a = O.volume_flux_rev(Ls[-1], c["ucont"], 0.0, 1)
    assert digest(uc) == ref["volume_flux"]["ucont"]
    assert repr(f) == ref["volume_flux"]["flux"] and repr(a) == ref["volume_flux"]["area"]
    b, s = O.poisson_rhs(Ls[-1], uc, dt, st)
    assert digest(b) == ref["rhs"]["b"] and repr(s) == ref["rhs"]["compat_sum"]
    for l in range(1, nl):
        assert digest(O.restrict(Ls[l], Ls[l - 1], seeded(Ls[l].shape, 100 + l))) == ref["restrict"][l - 1]
        assert digest(O.interpolate(Ls[l - 1], Ls[l], seeded(Ls[l - 1].shape, 200 + l))) == \
            ref["interpolate"][l - 1]
    for l in range(nl):
        y = O.nullspace(Ls[l], seeded(Ls[l].shape, 300 + l), mns if l == 0 else False, kske)
        assert digest(y) == ref["nullspace"][l], ("nullspace", l)
    fine = Ls[-1].shape
    p, phi, u2 = O.update_and_project(Ls[-1], seeded(fine, 400), seeded(fine, 401), uc, dt, st)
    assert digest(p) == ref["update_project"]["p"]
    assert digest(phi) == ref["update_project"]["phi"]
    assert digest(u2) == ref["update_project"]["ucont"]
    _check_post(Ls[-1], c["ucont"], 0, ref["post"])
    m, at = O.divergence(Ls[-1], c["ucont"])
    assert repr(m) == ref["divergence"]["max"] and at == ref["divergence"]["at"]
    m, at = O.metrics_divergence(Ls[-1])
    assert repr(m) == ref["metrics_divergence"]["max"] and at == ref["metrics_divergence"]["at"]
    _check_convection(c, Ls[-1], ref["convection"])
    if "convection_edges" in ref:
        Le = O.OLevel(c["metrics"][-1], conv_edge_nvert(c["nvert"]), c["bctype"], c["semi"])
        _check_convection(c, Le, ref["convection_edges"])
    if "convection_seam" in ref:
        from cases import conv_seam_nvert
        Ls_ = O.OLevel(c["metrics"][-1], conv_seam_nvert(c["nvert"]), c["bctype"], c["semi"])
        _check_convection(c, Ls_, ref["convection_seam"])


def _check_convection(c, L, want):
    """Convection (rhs.c:1463-1946), QUICK and central, periodic faces included."""
    ucat0, _ = post_inputs(L.shape, 0)
    for key, central in (("quick", 0), ("central", 1)):
        rc, conv = O.convection(L, c["ucont"], ucat0, central)
        assert rc == 0 and digest(conv) == want[key], key


def _check_post(L, ucont, seed, want, cent=None, u_bc=0.0):
    ucat0, ubcs0 = post_inputs(L.shape, seed)
    c2c = O.contra2cart(L, ucont, ucat0)
    assert digest_nan(c2c) == want["contra2cart"]
    rc, ub, u = O.ghost_node_velocity(L, ubcs0, c2c, cent, u_bc)
    assert rc == 0
    assert digest_nan(ub) == want["ghost_ubcs"]
    assert digest_nan(u) == want["ghost_ucat"]


@pytest.mark.parametrize("vname", sorted(POST_VARIANTS))
def test_post_projection_variants_match_reference(vname):
    """Contra2Cart and GhostNodeVelocity with slip, moving-lid, O-grid, annulus
    and rheology faces and blanked cells (nvert > 7) against the reference's
    own bcs.c / rhs.c."""
    from cases import POST_U_BC
    scen, bct, blank, seed = POST_VARIANTS[vname]
    c = _setup(scen)
    nv = c["nvert"].copy()
    for (k, j, i) in blank:
        nv[k, j, i] = 8.0
    L = O.OLevel(c["metrics"][-1], nv, bct, c["semi"])
    _check_post(L, c["ucont"], seed, REF["post_variants"][vname], c["metrics"][-1]["Cent"], POST_U_BC)


@pytest.mark.parametrize("name", sorted(IBM_CASES))
def test_ibm_search_matches_reference(name):
    """The immersed-body classification (ibm_search_advanced, ibm.c:4197-4740):
    ray-cast inside test, layer, phase-change fix, per-body codes and clean-up,
    body after body, against the reference's own ibm.c."""
    scen, bodies, frac, seed = IBM_CASES[name]
    c = _setup(scen)
    cent = c["metrics"][-1]["Cent"]
    meshes, nvert_o = ibm_inputs(name, cent.shape[:3])
    nv = np.zeros(cent.shape[:3])
    for b, (xyz, tri, nf) in enumerate(meshes):
        rc, nv = O.ibm_search(cent, xyz, tri, nf, b, len(meshes), nvert_o, nv)
        assert rc == 0
    assert digest(nv) == REF["ibm"][name]
    assert (nv == 3.0 + (len(meshes) - 1) / 1000.0).any()  # the last body has solid cells


def test_ghost_node_velocity_refuses_unrestated_types():
    """An annulus face without the cell centres, and a periodic face whose
    opposite is not, are refused with nothing written."""
    c = _setup("box_sphere")
    ucat0, ubcs0 = post_inputs(c["nvert"].shape, 0)
    for bct in ([1, 1, 11, 1, 1, 1], [1, 7, 1, 1, 1, 1]):
        L = O.OLevel(c["metrics"][-1], c["nvert"], bct, c["semi"])
        rc, ub, u = O.ghost_node_velocity(L, ubcs0, ucat0)
        assert rc == -1 and np.array_equal(u, ucat0) and np.array_equal(ub, ubcs0)


@pytest.mark.parametrize("name", ["box_sphere", "channel_periodic"])
def test_operator_invariants(name):
    """A 1 = 0 on fluid rows (right null vector) and (1/aj)^T A = 0 (left null vector)."""
    c = _setup(name)
    L = _levels(c)[-1]
    A = O.lhs_csr(L)
    nv = L.nvert
    fluid = np.zeros(nv.shape, bool)
    fluid[1:-1, 1:-1, 1:-1] = nv[1:-1, 1:-1, 1:-1] < 0.1
    one = fluid.astype(float).ravel()
    r = (A @ one).reshape(nv.shape)
    scale = np.abs(A.diagonal()).max()
    assert np.abs(r[fluid]).max() < 1e-11 * scale
    w = np.where(fluid, 1.0 / c["metrics"][-1]["Aj"], 0.0).ravel()
    lt = (A.T @ w).reshape(nv.shape)
    assert np.abs(lt[fluid]).max() < 1e-11 * np.abs(w).max() * scale / np.abs(c["metrics"][-1]["Aj"]).min()


@pytest.mark.skipif(not (O.REF_DIR / "poisson.c").exists(), reason="reference checkout not present")
def test_oracle_matches_live_reference_random_grid():
    """A grid not in the fixtures, run through the reference itself."""
    cells, per, nl = (10, 14, 6), (True, False, False), 2
    nodes = W.box_nodes(cells, (2.0, 1.0, 0.5), 1.5, True)
    bct = [7, 7, 1, 1, 1, 1]
    coords = W.level_coordinates(nodes, nl)
    mets = [W.form_metrics(x, per) for x in coords]
    nvf = W.sphere_nvert(mets[-1]["Cent"], [(1.0, 0.4, 0.25, 0.2)])
    R = O.Reference(nodes, nl, bct)
    for l in range(nl):
        for nm in ("IAj", "ICsi", "KZet", "Aj"):
            assert np.array_equal(R.field(l, nm, 3 if nm in W.METRIC_NAMES else 1), mets[l][nm])
    R.set_nvert(nl - 1, nvf)
    R.nvert_restrict()
    Lf = O.OLevel(mets[-1], nvf, bct)
    Lc = O.OLevel(mets[0], O.nvert_restrict(Lf, mets[0]["Aj"].shape, True), bct)
    assert np.array_equal(R.field(0, "Nvert"), Lc.nvert)
    for l, L in ((0, Lc), (1, Lf)):
        d = R.lhs_csr(l) - O.lhs_csr(L)
        d.eliminate_zeros()
        assert d.nnz == 0


def _check_momentum(c, nvert, bctype, want):
    from cases import MOM_DT, MOM_REN, momentum_inputs
    L = O.OLevel(c["metrics"][-1], nvert, bctype, c["semi"])
    ucat0, p, uo, urm = momentum_inputs(nvert.shape)
    assert digest(O.viscous(L, ucat0, MOM_REN)) == want["viscous"]
    if want.get("periodic"):
        # FormFunction1's periodic seam branches are not restated
        rc, _, _ = O.form_function1(L, c["ucont"], ucat0, p, MOM_REN)
        assert rc == -1
        return
    for central in (0, 1):
        rc, f, u = O.form_function1(L, c["ucont"], ucat0, p, MOM_REN, central)
        assert rc == 0 and digest(f) == want[f"ff1_{central}"] and digest(u) == want[f"ff1_ucat_{central}"]
    for ti in (1, 5):
        rc, r, _ = O.calc_rhs(L, c["ucont"], uo, urm, ucat0, p, MOM_REN, MOM_DT, ti, 0)
        assert rc == 0 and digest(r) == want[f"calc_rhs_{ti}"], ti
    if "form_bcs" in want:
        from cases import IMP_ATOL, IMP_RK_RUNS, IMP_RTOL, imp_rk_inputs
        ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(nvert.shape, c["ucont"])
        rc, _, _, u, pp = O.form_bcs(L, c["ucont"], ubcs1, ucat1, p1)
        assert rc == 0 and {"ucat": digest(u), "p": digest(pp)} == want["form_bcs"]
        for ti, cfl, max_it in IMP_RK_RUNS:
            rc, uc, u, pp, _, _ = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti,
                                           0, 0, IMP_ATOL, IMP_RTOL, max_it)
            assert rc == 0
            assert {"ucont": digest(uc), "ucat": digest(u), "p": digest(pp)} == want[f"imp_rk_{ti}_{cfl}_{max_it}"], \
                (ti, cfl, max_it)
    elif all(b == 1 for b in bctype):
        raise AssertionError("all-wall scenario without FormBCS / ImpRK digests")


@pytest.mark.parametrize("name", ["box_sphere", "blocked_slab"])
def test_inlet_outlet_matches_reference(name):
    """InflowFlux (bcs.c:99-400) with the constant and shaped inlet profiles, FormBCS's
    outlet flux correction (bcs.c:4914-4998) with an immersed-boundary flux,
    and ImpRK (implicitsolver.c:7094-7257) on a box with an inlet on k = 0 and
    an outlet on the last k face, bit for bit."""
    from cases import (FLUX_INTP_SUM, IMP_ATOL, IMP_RK_RUNS, IMP_RTOL, INLET_OUTLET_SCENARIOS, INLET_PROFILES, MOM_DT,
                       MOM_REN, SHAPED_INLETS, TABLE_INLETS, UNIFORM_INLETS, imp_rk_inputs, inlet_plane, inlet_table)
    assert name in INLET_OUTLET_SCENARIOS
    c = _setup(name)
    want = REF["scenarios"][name]["inlet_outlet"]
    bct = [1, 1, 1, 1, 5, 4]
    L = O.OLevel(c["metrics"][-1], c["nvert"], bct, c["semi"])
    ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(c["nvert"].shape, c["ucont"])
    for prof in INLET_PROFILES:
        rc, uc, ub, f = O.inflow_flux(L, c["ucont"], ubcs1, prof)
        assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)} == want[f"inflow_{prof}"]
    plane = inlet_plane(c["nodes"], c["nvert"].shape)
    for prof, cm in SHAPED_INLETS:
        rc, uc, ub, f = O.inflow_flux(L, c["ucont"], ubcs1, prof, 0.0, plane, cm)
        assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)} == want[f"inflow_{prof}"]
    prof, cm = SHAPED_INLETS[1]
    ti, cfl, max_it = IMP_RK_RUNS[0]
    rc, uc, u, pp, _, ub = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                    IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM, plane, cm)
    assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)} == \
        want[f"imp_rk_shaped_{prof}"]
    for prof, flux_in, t in UNIFORM_INLETS:
        O.set_inlet_globals(flux_in, t)
        rc, uc, ub, f = O.inflow_flux(L, c["ucont"], ubcs1, prof)
        assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)} == want[f"inflow_{prof}"]
    rc, uc, u, pp, _, ub = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                    IMP_ATOL, IMP_RTOL, max_it, 8, FLUX_INTP_SUM)
    assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)} == \
        want["imp_rk_uniform_8"]
    O.set_inlet_table(inlet_table())
    try:
        for prof, cm, t in TABLE_INLETS:
            O.set_inlet_globals(0.0, t)
            rc, uc, ub, f = O.inflow_flux(L, c["ucont"], ubcs1, prof, 0.0, plane, cm)
            assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)} == \
                want[f"inflow_{prof}"]
        rc, uc, u, pp, _, ub = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0,
                                        0, IMP_ATOL, IMP_RTOL, max_it, 0, FLUX_INTP_SUM, plane, TABLE_INLETS[0][1])
        assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)} == \
            want["imp_rk_table_0"]
        O.set_inlet_globals(0.0, 2000)  # the reference's column -1000: outside the table
        assert O.inflow_flux(L, c["ucont"], ubcs1, 0, 0.0, plane)[0] == -1
    finally:
        O.set_inlet_table(None)
    rc, uc, ub, f = O.inflow_flux(L, c["ucont"], ubcs1, 1)
    rc, uc, ub, u, pp = O.form_bcs(L, uc, ub, ucat1, p1, f, FLUX_INTP_SUM)
    assert rc == 0 and {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)} == \
        want["form_bcs"]
    for ti, cfl, max_it in IMP_RK_RUNS:
        rc, uc, u, pp, _, ub = O.imp_rk(L, c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                        IMP_ATOL, IMP_RTOL, max_it, 1, FLUX_INTP_SUM)
        assert rc == 0
        assert {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)} == \
            want[f"imp_rk_{ti}_{cfl}_{max_it}"], (ti, cfl, max_it)
    # a shaped profile without its nodes, a profile that is not restated, an
    # outlet without the inlet
    assert O.inflow_flux(L, c["ucont"], ubcs1, 4)[0] == -1
    assert O.inflow_flux(L, c["ucont"], ubcs1, 5, 0.0, plane)[0] == -1
    L2 = O.OLevel(c["metrics"][-1], c["nvert"], [1, 1, 1, 1, 1, 4], c["semi"])
    assert O.form_bcs(L2, c["ucont"], ubcs1, ucat1, p1)[0] == -1


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_momentum_rhs_matches_reference(name):
    """Viscous, FormFunction1 and CalcRHS (rhs.c:1947-3351, implicitsolver.c:
    6449-6713) bit for bit; on box_sphere also with cells whose tangential
    pressure derivative the reference leaves unassigned (cases.MOM_EDGES) and
    with a convective-outflow face (bctype[5] 8).  On the all-wall boxes also
    FormBCS (bcs.c:4436-5889) and the pseudo-time iteration ImpRK
    (implicitsolver.c:7094-7257): converged, stopped at imp_MAX_IT, and with
    the step halved."""
    from cases import mom_edge_nvert
    c = _setup(name)
    ref = REF["scenarios"][name]
    _check_momentum(c, c["nvert"], c["bctype"], ref["momentum"])
    if "momentum_edges" in ref:
        _check_momentum(c, mom_edge_nvert(c["nvert"]), c["bctype"], ref["momentum_edges"])
        _check_momentum(c, c["nvert"], list(c["bctype"][:5]) + [8], ref["momentum_outflow8"])
