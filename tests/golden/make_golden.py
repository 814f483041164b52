"""Generate the golden fixtures from the reference's own routines.

Runs CURVIB's poisson.c / metrics.c / implicitsolver.c / rhs.c / bcs.c,
compiled unmodified against the single-process PETSc API shim
(oracle/build_ref.sh), on the small scenarios of tests/cases.py and records
SHA-256 digests of every output, including the immersed-body classification
(ibm_search_advanced, ibm.c) of tests/cases.IBM_CASES, whose meshes are stored
in ibm_meshes.npz, and the checks Divergence (main.c) and MetricsDivergence
(metrics.c), and the convective term Convection (rhs.c).  The post-projection steps (Contra2Cart,
GhostNodeVelocity) also run on the variants of cases.POST_VARIANTS, which put
slip, moving-lid and O-grid faces and blanked cells on the same grids.  The
inputs (node coordinates, nvert, fluxes) are stored beside the digests so the
tests do not depend on the platform's sin/tanh.  Needs the reference checkout,
given as the argument or in CVB_REFERENCE_DIR; the fixtures it writes are
committed and the tests read only those.

usage: python tests/golden/make_golden.py REFERENCE_DIR
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from cases import (FLUX_INTP_SUM, IMP_ATOL, IMP_RK_RUNS, IMP_RTOL, INLET_OUTLET_SCENARIOS, INLET_PROFILES,  # noqa: E402
                   MOM_DT, MOM_REN, SHAPED_INLETS, TABLE_INLETS, UNIFORM_INLETS, inlet_table,
                   conv_seam_nvert, imp_rk_inputs, mom_edge_nvert, momentum_inputs)
from cases import (IBM_CASES, POST_U_BC, POST_VARIANTS, SCENARIOS, build, conv_edge_nvert, digest, digest_nan,  # noqa: E402
                   ibm_inputs, post_inputs, seeded)
from curvib_old_gb300 import workload as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
DT, ST = 1e-3, 1.0


def csr_digest(A):
    A = A.tocsr().copy()
    A.sort_indices()
    return {"indptr": digest(A.indptr.astype(np.int64)), "indices": digest(A.indices.astype(np.int64)),
            "data": digest(A.data), "nnz": int(A.nnz)}


def run(name):
    c = build(name)
    nl = c["nl"]
    R = O.Reference(c["nodes"], nl, c["bctype"], c["semi"])
    rec = {"metrics": [], "nvert": [], "lhs": []}
    for l in range(nl):
        rec["metrics"].append({nm: digest(R.field(l, nm, 3 if nm in W.METRIC_NAMES else 1))
                               for nm in W.METRIC_NAMES + W.JACOBIAN_NAMES})
    R.set_nvert(nl - 1, c["nvert"])
    mns, kske = R.nvert_restrict()
    rec["multinullspace"] = bool(mns)
    mz, my, mx = R.shape(0)
    rec["kske"] = digest(kske.reshape(my, mx, 2)[1:-1, 1:-1, 0].astype(np.int64)) if mns else None
    for l in range(nl):
        rec["nvert"].append(digest(R.field(l, "Nvert")))
        rec["lhs"].append(csr_digest(R.lhs_csr(l)))
    uc, f, a = R.volume_flux(c["ucont"], 0.0, 1)
    rec["volume_flux"] = {"ucont": digest(uc), "flux": repr(f), "area": repr(a)}
    R.set_ucont(uc)
    b, s = R.rhs(DT, ST)
    rec["rhs"] = {"b": digest(b), "compat_sum": repr(s)}
    rec["restrict"], rec["interpolate"], rec["nullspace"] = [], [], []
    for l in range(1, nl):
        rec["restrict"].append(digest(R.restrict(l - 1, seeded(R.shape(l), 100 + l))))
        rec["interpolate"].append(digest(R.interpolate(l, seeded(R.shape(l - 1), 200 + l))))
    for l in range(nl):
        rec["nullspace"].append(digest(R.nullspace(l, seeded(R.shape(l), 300 + l))))
    fine = R.shape(nl - 1)
    p, phi, u2 = R.update_and_project(seeded(fine, 400), seeded(fine, 401), uc, DT, ST)
    rec["update_project"] = {"p": digest(p), "phi": digest(phi), "ucont": digest(u2)}
    rec["post"] = post(R, c["nvert"], c["ucont"], 0)
    R.set_nvert(nl - 1, c["nvert"])
    m, at = R.divergence(c["ucont"])
    rec["divergence"] = {"max": repr(m), "at": at}
    m, at = R.metrics_divergence()
    rec["metrics_divergence"] = {"max": repr(m), "at": at}
    rec["convection"] = convection(R, c["nvert"], c["ucont"], c["bctype"])
    if name == "box_sphere":
        rec["convection_edges"] = convection(R, conv_edge_nvert(c["nvert"]), c["ucont"], c["bctype"])
        R.set_nvert(nl - 1, c["nvert"])
    if name == "channel_periodic":
        rec["convection_seam"] = convection(R, conv_seam_nvert(c["nvert"]), c["ucont"], c["bctype"])
        R.set_nvert(nl - 1, c["nvert"])
    rec["momentum"] = momentum(R, c["nvert"], c["ucont"], c["bctype"])
    if name == "box_sphere":
        rec["momentum_edges"] = momentum(R, mom_edge_nvert(c["nvert"]), c["ucont"], c["bctype"])
        R.set_nvert(nl - 1, c["nvert"])
        bct = list(c["bctype"][:5]) + [8]  # convective outflow on the last k face
        R8 = O.Reference(c["nodes"], nl, bct, c["semi"])
        R8.set_nvert(nl - 1, c["nvert"])
        rec["momentum_outflow8"] = momentum(R8, c["nvert"], c["ucont"], bct)
        R = O.Reference(c["nodes"], nl, c["bctype"], c["semi"])
    if name in INLET_OUTLET_SCENARIOS:
        rec["inlet_outlet"] = inlet_outlet(c)
    np.savez_compressed(OUT / f"{name}.npz", nodes=c["nodes"], nvert=c["nvert"], ucont=c["ucont"])
    return rec


def convection(R, nvert, ucont, bctype):
    """Convection (rhs.c:1463) on the ucat of post_inputs(seed 0), QUICK and
    central (periodic faces included)."""
    R.set_nvert(R.nlevels - 1, nvert)
    ucat0, _ = post_inputs(nvert.shape, 0)
    return {"quick": digest(R.convection(ucont, ucat0, 0)), "central": digest(R.convection(ucont, ucat0, 1))}


def momentum(R, nvert, ucont, bctype):
    """Viscous, FormFunction1 (QUICK and central) and CalcRHS (first step and
    second-order backward) on cases.momentum_inputs; Viscous alone for a box
    with a periodic face."""
    R.set_nvert(R.nlevels - 1, nvert)
    ucat0, p, uo, urm = momentum_inputs(nvert.shape)
    out = {"viscous": digest(R.viscous(ucat0, MOM_REN))}
    if 7 in list(bctype):
        # Viscous reads only the box (its ring holds the periodic images);
        # FormFunction1 and CalcRHS have periodic seam branches not restated
        out["periodic"] = True
        return out
    for central in (0, 1):
        f, u = R.form_function1(ucont, ucat0, p, MOM_REN, central)
        out[f"ff1_{central}"] = digest(f)
        out[f"ff1_ucat_{central}"] = digest(u)
    for ti in (1, 5):
        r, _ = R.calc_rhs(ucont, uo, urm, ucat0, p, MOM_REN, MOM_DT, ti, 0)
        out[f"calc_rhs_{ti}"] = digest(r)
    if all(b == 1 for b in bctype):
        # FormBCS and ImpRK (bcs.c:4436, implicitsolver.c:7094), all-wall boxes
        ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(nvert.shape, ucont)
        _, _, u, pp = R.form_bcs(ucont, ubcs1, ucat1, p1)
        out["form_bcs"] = {"ucat": digest(u), "p": digest(pp)}
        with tempfile.TemporaryDirectory() as d:
            cwd = os.getcwd()
            os.chdir(d)  # ImpRK appends to Converge_dU0 in the working directory
            try:
                for ti, cfl, max_it in IMP_RK_RUNS:
                    uc, u, pp, _ = R.imp_rk(ucont, uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                            IMP_ATOL, IMP_RTOL, max_it)
                    out[f"imp_rk_{ti}_{cfl}_{max_it}"] = {"ucont": digest(uc), "ucat": digest(u), "p": digest(pp)}
            finally:
                os.chdir(cwd)
    return out


def inlet_outlet(c):
    """InflowFlux, FormBCS and ImpRK (bcs.c:99, 4436; implicitsolver.c:7094) on
    the scenario's grid with an inlet on the k = 0 face (bctype[4] 5) and an
    outlet on the last (bctype[5] 4): the constant inlet profiles, FormBCS with
    the inlet's flux and an immersed-boundary flux, and cases.IMP_RK_RUNS with
    profile 1; the shaped profiles (cases.SHAPED_INLETS) and ImpRK's first run
    with the pipe profile 4; the uniform profiles (cases.UNIFORM_INLETS) and
    ImpRK's first run with profile 8; the table profiles (cases.TABLE_INLETS)
    and ImpRK's first run with profile 0."""
    bct = [1, 1, 1, 1, 5, 4]
    nl = c["nl"]
    R = O.Reference(c["nodes"], nl, bct, c["semi"])
    R.set_nvert(nl - 1, c["nvert"])
    ucat1, p1, uo1, urm1, ubcs1 = imp_rk_inputs(c["nvert"].shape, c["ucont"])
    out = {}
    for prof in INLET_PROFILES:
        uc, ub, f = R.inflow_flux(c["ucont"], ubcs1, prof)
        out[f"inflow_{prof}"] = {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)}
    for prof, cm in SHAPED_INLETS:
        uc, ub, f = R.inflow_flux(c["ucont"], ubcs1, prof, 0.0, cm)
        out[f"inflow_{prof}"] = {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)}
    for prof, flux_in, ti in UNIFORM_INLETS:
        R.set_inlet_globals(flux_in, ti)
        uc, ub, f = R.inflow_flux(c["ucont"], ubcs1, prof)
        out[f"inflow_{prof}"] = {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)}
    R.set_inlet_table(inlet_table())
    for prof, cm, ti in TABLE_INLETS:
        R.set_inlet_globals(0.0, ti)
        uc, ub, f = R.inflow_flux(c["ucont"], ubcs1, prof, 0.0, cm)
        out[f"inflow_{prof}"] = {"ucont": digest(uc), "ubcs": digest(ub), "flux_in_sum": repr(f)}
    uc, ub, f = R.inflow_flux(c["ucont"], ubcs1, 1)
    uc, ub, u, pp = R.form_bcs(uc, ub, ucat1, p1, f, FLUX_INTP_SUM)
    out["form_bcs"] = {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)}
    with tempfile.TemporaryDirectory() as d:
        cwd = os.getcwd()
        os.chdir(d)
        try:
            for ti, cfl, max_it in IMP_RK_RUNS:
                uc, u, pp, ub = R.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0,
                                         0, IMP_ATOL, IMP_RTOL, max_it, 1, FLUX_INTP_SUM)
                out[f"imp_rk_{ti}_{cfl}_{max_it}"] = {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u),
                                                      "p": digest(pp)}
            prof, cm = SHAPED_INLETS[1]
            ti, cfl, max_it = IMP_RK_RUNS[0]
            uc, u, pp, ub = R.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                     IMP_ATOL, IMP_RTOL, max_it, prof, FLUX_INTP_SUM, cm)
            out[f"imp_rk_shaped_{prof}"] = {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u),
                                            "p": digest(pp)}
            uc, u, pp, ub = R.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                     IMP_ATOL, IMP_RTOL, max_it, 8, FLUX_INTP_SUM)
            out["imp_rk_uniform_8"] = {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)}
            uc, u, pp, ub = R.imp_rk(c["ucont"], uo1, urm1, ucat1, p1, ubcs1, MOM_REN, MOM_DT, 1.0, cfl, ti, 0, 0,
                                     IMP_ATOL, IMP_RTOL, max_it, 0, FLUX_INTP_SUM, TABLE_INLETS[0][1])
            out["imp_rk_table_0"] = {"ucont": digest(uc), "ubcs": digest(ub), "ucat": digest(u), "p": digest(pp)}
        finally:
            os.chdir(cwd)
    return out


def post(R, nvert, ucont, seed, u_bc=0.0):
    """Contra2Cart, then GhostNodeVelocity on its result.  A slip face on the
    low y side takes its normal from eta of the ring cell, which FormMetrics
    leaves zero: the reference's values there are NaN (0/0)."""
    ucat0, ubcs0 = post_inputs(nvert.shape, seed)
    R.set_nvert(R.nlevels - 1, nvert)
    c2c = R.contra2cart(ucont, ucat0)
    ub, u = R.ghost_node_velocity(ubcs0, c2c, u_bc)
    return {"contra2cart": digest_nan(c2c), "ghost_ubcs": digest_nan(ub), "ghost_ucat": digest_nan(u)}


def run_variant(vname):
    scen, bct, blank, seed = POST_VARIANTS[vname]
    c = build(scen)
    nv = c["nvert"].copy()
    for (k, j, i) in blank:
        nv[k, j, i] = 8.0
    R = O.Reference(c["nodes"], c["nl"], bct, c["semi"])
    return post(R, nv, c["ucont"], seed, POST_U_BC)


def run_ibm(name, meshes_out):
    """ibm_search_advanced for every body of the case, one after another."""
    scen, bodies, frac, seed = IBM_CASES[name]
    c = build(scen, nodes=np.load(OUT / f"{scen}.npz")["nodes"])
    R = O.Reference(c["nodes"], c["nl"], c["bctype"], c["semi"])
    shape = R.shape(c["nl"] - 1)
    meshes, nvert_o = ibm_inputs(name, shape)
    nv = np.zeros(shape)
    for b, (xyz, tri, nf) in enumerate(meshes):
        meshes_out[f"{name}_{b}_xyz"], meshes_out[f"{name}_{b}_tri"], meshes_out[f"{name}_{b}_nf"] = xyz, tri, nf
        nv = R.ibm_search(xyz, tri, nf, b, len(meshes), nvert_o, nv)
    return digest(nv)


def run_restart():
    """Digests of the files the reference's Ucont_P_Binary_Output (main.c:285)
    writes for step 37, block 0, on box_sphere's grid (the fields of
    tests/test_io.py::_restart_fields, seed 21)."""
    import hashlib
    import tempfile
    from test_io import _restart_fields
    c = build("box_sphere")
    R = O.Reference(c["nodes"], c["nl"], c["bctype"], c["semi"])
    nvert, ucont, ucat, p = _restart_fields(c["nvert"].shape, 21)
    with tempfile.TemporaryDirectory() as d:
        R.restart_write(d, 37, 0, nvert, ucont, ucat, p)
        return {f.name: hashlib.sha256(f.read_bytes()).hexdigest()[:32] for f in sorted(Path(d).iterdir())}


def main():
    import os
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CVB_REFERENCE_DIR")
    if not ref or O.build_reference(ref) is None:
        sys.exit("usage: make_golden.py REFERENCE_DIR (or set CVB_REFERENCE_DIR): no reference sources given")
    out = {"dt": DT, "st": ST, "scenarios": {}, "post_variants": {}, "ibm": {}}
    for name in SCENARIOS:
        out["scenarios"][name] = run(name)
        print(name, "ok")
    for vname in POST_VARIANTS:
        out["post_variants"][vname] = run_variant(vname)
        print(vname, "ok")
    meshes = {}
    for name in IBM_CASES:
        out["ibm"][name] = run_ibm(name, meshes)
        print(name, "ok")
    out["restart"] = run_restart()
    print("restart ok")
    np.savez_compressed(OUT / "ibm_meshes.npz", **meshes)
    (OUT / "reference_digests.json").write_text(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
