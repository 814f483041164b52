"""Small deterministic scenarios shared by the parity tests and the fixture script."""
from __future__ import annotations

import hashlib

import numpy as np

from curvib_old_gb300 import workload as W

# name -> (cells, periodic (x,y,z), spheres, levels, semi-coarsening (i,j,k), y-stretch, slab)
SCENARIOS = {
    "box_sphere": ((12, 12, 12), (0, 0, 0), [(0.5, 0.5, 0.5, 0.3)], 3, (0, 0, 0), 2.0, False),
    "channel_periodic": ((16, 8, 8), (1, 0, 1), [(0.4, 0.5, 0.5, 0.25)], 2, (0, 0, 0), 2.5, False),
    "ksemi_sphere": ((12, 12, 12), (0, 0, 0), [(0.45, 0.5, 0.55, 0.3)], 2, (0, 0, 1), 2.0, False),
    "blocked_slab": ((8, 8, 8), (0, 0, 0), [], 2, (0, 0, 0), 1.0, True),
    "triply_periodic": ((8, 8, 8), (1, 1, 1), [], 2, (0, 0, 0), 1.0, False),
}


# Post-projection variants (Contra2Cart, GhostNodeVelocity): a scenario's grid
# with other boundary types -- slip walls (3), a moving lid (bctype[5] 2), an
# O-grid outer face (bctype[3] 12) -- and interior cells blanked (nvert 8 > 7,
# which Contra2Cart treats as fluid).  name -> (scenario, bctype, blanked
# (k, j, i) cells, seed of the ucat / ubcs inputs)
POST_VARIANTS = {
    "slip_lid_ogrid": ("box_sphere", [3, 3, 1, 12, 3, 2], [(2, 3, 4), (2, 3, 5), (9, 8, 2)], 1),
    "walls_slip_y": ("box_sphere", [1, 1, 3, 3, 1, 1], [(5, 5, 5)], 2),
    "periodic_slip_y": ("channel_periodic", [7, 7, 3, 3, 7, 7], [(3, 4, 6)], 3),
    # an annulus face (bctype[2] 11, its ubcs from the cell centres) and the
    # rheology plates (bctype 13, the plate velocity POST_U_BC)
    "annulus_y": ("box_sphere", [1, 1, 11, 1, 1, 1], [(5, 5, 5)], 4),
    "rheology_plates": ("box_sphere", [1, 1, 13, 13, 13, 13], [(6, 4, 5)], 5),
}
POST_U_BC = 0.37


# Immersed-body searches (ibm_search_advanced): name -> (scenario whose grid is
# used, bodies [(centre, radius, subdivisions)], fraction of cells solid in the
# previous step's nvert_o, seed).  Bodies are classified one after another
# (ibi = 0, 1, ...), each on the previous one's nvert.
IBM_CASES = {
    "one_sphere": ("box_sphere", [((0.5, 0.5, 0.5), 0.3, 3)], 0.0, 0),
    "periodic_channel": ("channel_periodic", [((0.4, 0.5, 0.5), 0.25, 2)], 0.0, 1),
    "two_bodies_phase_change": ("ksemi_sphere", [((0.35, 0.45, 0.5), 0.22, 3), ((0.72, 0.55, 0.45), 0.15, 3)],
                                0.03, 2),
}


def ibm_inputs(name, shape):
    """The meshes and nvert_o of an IBM_CASES entry (meshes from the committed
    fixture when present, so that they do not depend on the platform's sqrt)."""
    from pathlib import Path
    scen, bodies, frac, seed = IBM_CASES[name]
    fx = Path(__file__).resolve().parent / "golden" / "ibm_meshes.npz"
    meshes = []
    if fx.exists():
        z = np.load(fx)
        for b in range(len(bodies)):
            meshes.append((z[f"{name}_{b}_xyz"], z[f"{name}_{b}_tri"], z[f"{name}_{b}_nf"]))
    else:
        for (ctr, r, sub) in bodies:
            meshes.append(W.sphere_mesh(ctr, r, sub))
    rng = np.random.default_rng(700 + seed)
    nvert_o = np.where(rng.random(shape) < frac, 3.0, 0.0)
    return meshes, nvert_o


def post_inputs(shape, seed):
    """ucat and ubcs ([mz][my][mx][3]) the post-projection steps start from."""
    sh = tuple(shape) + (3,)
    return seeded(sh, 500 + seed), seeded(sh, 600 + seed)


# Convection's edge cases on box_sphere's nvert, (k, j, i, value), negative
# indices counting from the high end: a body cell two cells from the high i,
# j and k ends (the reference's one-sided forms, which past the i and j ends
# read the next row), neighbours of nvert exactly 0.1 (no form applies: the
# face flux stays 0), and a blanked cell (nvert 8, treated as fluid).
CONV_EDGES = [(5, 5, -3, 3.0), (6, -3, 4, 1.3), (-3, 4, 4, 2.0), (3, 3, 2, 0.1), (8, 2, 9, 0.1),
              (7, 7, 7, 8.0), (2, -2, 6, 1.2)]


# Convection across the periodic seams of channel_periodic, (k, j, i, value):
# blocked cells next to the seam in x (i = mx-3, whose image the seam face at
# i = 0 reads, and i = 1) and in z, so that the seam faces take both the full
# QUICK form across the seam and the one-sided forms.
CONV_SEAM = [(4, 4, -3, 3.0), (3, 2, 1, 2.0), (-3, 5, 6, 3.0), (1, 3, 9, 1.3)]


def conv_seam_nvert(nvert):
    nv = np.array(nvert, dtype=np.float64, copy=True)
    for (k, j, i, v) in CONV_SEAM:
        nv[k, j, i] = v
    return nv


def conv_edge_nvert(nvert):
    nv = np.array(nvert, dtype=np.float64, copy=True)
    for (k, j, i, v) in CONV_EDGES:
        nv[k, j, i] = v
    return nv


def bctype_of(per):
    return [7 if per[0] else 1] * 2 + [7 if per[1] else 1] * 2 + [7 if per[2] else 1] * 2


def build(name, nodes=None):
    """Inputs of one scenario: nodes, bctype, per-level metrics, fine nvert, fluxes."""
    cells, per, spheres, nl, semi, beta, slab = SCENARIOS[name]
    per = tuple(bool(p) for p in per)
    if nodes is None:
        nodes = W.box_nodes(cells, (1.0, 1.0, 1.0), beta, True)
    coords = W.level_coordinates(nodes, nl, semi)
    mets = [W.form_metrics(c, per) for c in coords]
    nvf = W.sphere_nvert(mets[-1]["Cent"], spheres)
    if slab:
        # a solid plate across the whole x-y section: every k-line is blocked
        mz = nvf.shape[0]
        nvf[mz // 2 - 2:mz // 2 + 2, 1:-1, 1:-1] = W.SOLID_CODE
    uc = W.ucont_from_velocity(mets[-1], W.taylor_green, per)
    return dict(nodes=nodes, bctype=bctype_of(per), per=per, nl=nl, semi=semi, metrics=mets,
                nvert=nvf, ucont=uc)


def digest(a) -> str:
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()[:32]


def digest_nan(a) -> str:
    """digest() with every NaN replaced by one quiet NaN: the sign and payload
    of a NaN from 0/0 differ between x86 and Arm."""
    a = np.array(a, dtype=np.float64, copy=True)
    a[np.isnan(a)] = np.nan
    return digest(a)


def seeded(shape, seed):
    return np.random.default_rng(seed).standard_normal(shape)


# The momentum right-hand side (Viscous, FormFunction1, CalcRHS): Reynolds
# number and time step of the fractional-step workload, and edge cases on
# box_sphere's nvert, (k, j, i, value): a fluid cell with blocked cells above
# and below it in j, and one below the top wall with a blocked cell under it,
# where FormFunction1 assigns no tangential pressure derivative and the value
# of the previous assignment in its loop order stands (rhs.c:2803-2849).
MOM_REN, MOM_DT = 300.0, 2e-3
MOM_EDGES = [(5, 3, 4, 3.0), (5, 5, 4, 3.0), (6, -3, 6, 3.0), (8, 4, 7, 1.2), (8, 6, 7, 1.3)]


def mom_edge_nvert(nvert):
    nv = np.array(nvert, dtype=np.float64, copy=True)
    for (k, j, i, v) in MOM_EDGES:
        nv[k, j, i] = v
    return nv


def momentum_inputs(shape):
    """ucat, p, ucont_o and ucont_rm1 ([mz][my][mx](x3)) of the momentum checks."""
    sh3 = tuple(shape) + (3,)
    return seeded(sh3, 810), seeded(shape, 811), seeded(sh3, 812), seeded(sh3, 813)


# The pseudo-time iteration of the momentum equation (ImpRK) on the all-wall
# scenarios: (ti, cfl, imp_MAX_IT) -- converged by the absolute tolerance with
# no step halved, stopped at imp_MAX_IT, and with the step halved and
# iterations undone (cfl 3) -- at imp_atol 1e-7, imp_rtol 1e-4 (main.c's
# defaults).
IMP_RK_RUNS = [(1, 1.0, 50), (5, 0.5, 4), (5, 3.0, 50)]
IMP_ATOL, IMP_RTOL = 1e-7, 1e-4
# The inlet / outlet boxes (bctype[4] 5, bctype[5] 4 on a scenario's grid):
# InflowFlux's constant profiles, and the immersed-boundary flux FormBCS's
# outlet adds to the inlet's.
INLET_OUTLET_SCENARIOS = ("box_sphere", "blocked_slab")
INLET_PROFILES = (1, -1, 11)
FLUX_INTP_SUM = 1e-3
# The shaped profiles (2: a parabola across y in [0, 4.1]; 4: a pipe of
# radius 0.5; 7: a parabola across y in [-0.5, 0.5]; 10: a square duct's
# series solution across x in [0, 1], y in [1, 2]), each with a centre
# (CMx_c, CMy_c, CMz_c) that puts the unit box's inlet across its shape.
SHAPED_INLETS = ((2, (0.0, 0.1, 0.0)), (4, (0.1, 0.45, 0.5)), (7, (0.0, 0.5, 0.0)), (10, (0.25, -0.8, 0.0)))

# The uniform profiles InletInterpolation gives: (profile, Flux_in, ti); 3 and
# 6 take Flux_in, 8 sin(2 (3.14159) ti / 200).
UNIFORM_INLETS = ((3, 0.75, 0), (6, -0.3, 0), (8, 0.0, 37))

# The table profiles (profile, centre, ti): 0 and 5 interpolate InletRead's
# table (uinr [101][1001], inlet_table) at the face cell's radius, column
# ti/2 - (ti/2000) 2000.
TABLE_INLETS = ((0, (0.0, 0.5, 0.5), 37), (5, (0.1, 0.45, 0.5), 1500))


def inlet_table():
    """A seeded stand-in for InletRead's uinr [101][1001]."""
    return seeded((101, 1001), 820)


def inlet_plane(nodes, shape):
    """The k = 0 node plane in the box layout ([my][mx][3]) of a case's nodes
    ([KM][JM][IM][3]) on a box of shape (mz, my, mx)."""
    _, my, mx = shape
    plane = np.zeros((my, mx, 3))
    plane[:nodes.shape[1], :nodes.shape[2]] = nodes[0]
    return plane


def imp_rk_inputs(shape, ucont):
    """ucat, p, ucont_o, ucont_rm1 and ubcs of the ImpRK checks: the previous
    steps' fluxes close to ucont, a small pressure, a small wall velocity."""
    sh3 = tuple(shape) + (3,)
    return (seeded(sh3, 810), 0.01 * seeded(shape, 811), 0.99 * ucont, 0.97 * ucont,
            1e-3 * seeded(sh3, 820))
