"""The immersed-body classification on the GPU (cvb_ibm_search, libcvb.so)
against the CPU oracle, bit for bit: the pinned cases of tests/cases.IBM_CASES
(one body; a periodic channel; two bodies with the previous step's solid cells
left fluid), a larger grid and finer mesh than the oracle's pinning cases, a
moving body fed back through cvb_set_nvert, and refused inputs.
"""
import types

import numpy as np
import pytest

from cases import IBM_CASES, build, ibm_inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ctx(c):
    from curvib_old_gb300.solver import PoissonContext
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=np.zeros(c["metrics"][-1]["Aj"].shape), ucont=c["ucont"],
                              bctype=c["bctype"], semi=c["semi"], per=c["per"], nl=c["nl"])
    return PoissonContext().setup(P)


@pytest.mark.parametrize("name", sorted(IBM_CASES))
def test_ibm_search_matches_oracle(name):
    scen = IBM_CASES[name][0]
    c = build(scen)
    cent = c["metrics"][-1]["Cent"]
    meshes, nvert_o = ibm_inputs(name, cent.shape[:3])
    ctx = _ctx(c)
    try:
        nv_g = nv_o = np.zeros(cent.shape[:3])
        for b, (xyz, tri, nf) in enumerate(meshes):
            nv_g = ctx.ibm_search(cent, xyz, tri, nf, b, len(meshes), nvert_o, nv_g)
            rc, nv_o = O.ibm_search(cent, xyz, tri, nf, b, len(meshes), nvert_o, nv_o)
            assert rc == 0
            assert np.array_equal(nv_g, nv_o), (name, b)
        assert (nv_g >= 3.0).any() and ((nv_g >= 1.0) & (nv_g < 1.5)).any()
    finally:
        ctx.close()


def test_ibm_search_larger_grid_and_moving_body():
    """64x48x56 cells, a 5120-triangle sphere: GPU and oracle agree; moved by a
    cell, the body's new nvert (with the old one as nvert_o) agrees too and sets
    up a solvable hierarchy."""
    from curvib_old_gb300 import workload as W
    P = W.make_problem((64, 48, 56), (1.0, 1.0, 1.0), 2.0, True, (False, False, False), [])
    from curvib_old_gb300.solver import PoissonContext
    ctx = PoissonContext().setup(P)
    try:
        cent = P.metrics[-1]["Cent"]
        zero = np.zeros(cent.shape[:3])
        nv_prev = zero
        for step, ctr in enumerate(((0.45, 0.5, 0.5), (0.47, 0.5, 0.5))):
            xyz, tri, nf = W.sphere_mesh(ctr, 0.23, 4)
            # the second step reuses the centres the first one left on the device
            nv_g = ctx.ibm_search(cent if step == 0 else None, xyz, tri, nf, 0, 1, nv_prev, zero)
            rc, nv_o = O.ibm_search(cent, xyz, tri, nf, 0, 1, nv_prev, zero)
            assert rc == 0 and np.array_equal(nv_g, nv_o), step
            assert (nv_g == 3.0).sum() > 1000
            ctx.set_nvert(nv_g)
            b = ctx.poisson_rhs(P.ucont, 1e-3, 1.0)[0]
            phi, st = ctx.solve(b, rtol=1e-8)
            assert st["status"] == 0
            nv_prev = nv_g
    finally:
        ctx.close()


def test_ibm_search_refuses_bad_bodies():
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300 import workload as W
    c = build("box_sphere")
    cent = c["metrics"][-1]["Cent"]
    ctx = _ctx(c)
    try:
        xyz, tri, nf = W.sphere_mesh((0.5, 0.5, 0.5), 0.3, 1)
        zero = np.zeros(cent.shape[:3])
        bad = tri.copy()
        bad[3, 1] = len(xyz)
        flat = xyz.copy()
        flat[:, 2] = 0.5
        for args in ((cent, xyz, bad, nf, 0, 1), (cent, flat, tri, nf, 0, 1), (cent, xyz, tri, nf, 1, 1)):
            with pytest.raises(CvbError) as e:
                ctx.ibm_search(*args, zero, zero)
            assert e.value.status == 4  # CVB_BAD_INPUT
        # still usable
        assert np.array_equal(ctx.ibm_search(cent, xyz, tri, nf, 0, 1, zero, zero),
                              O.ibm_search(cent, xyz, tri, nf, 0, 1, zero, zero)[1])
    finally:
        ctx.close()
