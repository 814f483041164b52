"""Served solve stream (curvib_old_gb300.serve): continuous batching under an
HBM budget.

Bar: every request is served, converged, and its pressure is bit-identical to
the same solve run alone (a fresh context, a batch of one, the same initial
guess), although in the stream it shared rounds with other solves, may have
reused another problem's context and, for warm-started follow-ups, started
from the previous pressure of its problem.
"""
import pytest

import numpy as np

pytestmark = pytest.mark.gpu


def test_stream_results_equal_alone():
    from curvib_old_gb300 import serve as S
    from curvib_old_gb300.solver import PoissonContext, SolveBatch
    stream = S.make_stream(24, 400.0, seed=7, max_cells=48)
    inputs = S.Inputs(stream)
    # room for a few problems at a time: forces context reuse and eviction
    budget = 3 * S.bytes_estimate(48)
    srv = S.Server(inputs, budget_bytes=budget, keep_results=True)
    try:
        rep = srv.run(stream, time_limit=300.0)
    finally:
        srv.close()
    assert rep["served"] == len(stream)
    assert rep["peak_resident_bytes"] <= budget
    assert rep["warm_followups"] > 0 and rep["contexts_reused"] + rep["evictions"] > 0, rep
    by_id = {r.rid: r for r in stream}
    B = SolveBatch(rtol=1e-8, max_it=200)
    try:
        for rid, warm, prev in srv.trace:
            req = by_id[rid]
            phi, st = srv.results[rid]
            assert st["status"] == 0 and st["rel_residual"] <= 1e-8
            c = PoissonContext().setup(inputs.problem(req.n, inputs.nvert[rid]))
            try:
                if warm:
                    c.set_phi(srv.results[prev][0])
                B.submit(c, b=inputs.rhs[rid], warm_start=warm)
                while B.step():
                    pass
                (t, st1), = B.poll()
                alone = c.get_phi()
            finally:
                c.close()
            assert st1["iterations"] == st["iterations"], (rid, st1, st)
            assert np.array_equal(alone, phi), rid
    finally:
        B.close()


def test_setup_like_equals_own_setup():
    """A problem set up on another context's resident metrics is the same problem."""
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    mets, uc = W.box_geometry((24, 24, 24))
    nv1 = W.sphere_nvert(mets[-1]["Cent"], [(0.5, 0.5, 0.5, 0.2)])
    nv2 = W.sphere_nvert(mets[-1]["Cent"], [(0.4, 0.6, 0.45, 0.15), (0.7, 0.3, 0.6, 0.1)])
    P1 = W.Problem(mets, nv1, uc, [1] * 6)
    P2 = W.Problem(mets, nv2, uc, [1] * 6)
    a = PoissonContext().setup(P1)
    b = PoissonContext().setup_like(a, nv2)
    c = PoissonContext().setup(P2)
    try:
        assert b.geometry_bytes()[1] == a.geometry_bytes()[1] != c.geometry_bytes()[1]
        for l in range(c.nlevels):
            assert np.array_equal(b.weights(l), c.weights(l))
        ub, _, _ = b.volume_flux_rev(uc, 0.0, 1)
        uc2, _, _ = c.volume_flux_rev(uc, 0.0, 1)
        assert np.array_equal(ub, uc2)
        rhs, _ = c.poisson_rhs(uc2, 1e-3, 1.0)
        rhs = W.noisy_rhs(rhs, nv2, mets[-1]["Aj"], 1e-3, seed=5)
        pb, sb = b.solve(rhs, rtol=1e-10)
        pc, sc = c.solve(rhs, rtol=1e-10)
        assert sb["iterations"] == sc["iterations"] and np.array_equal(pb, pc)
        a.close()   # the shared metrics stay with b
        pb2, _ = b.solve(rhs, rtol=1e-10)
        assert np.array_equal(pb2, pb)
    finally:
        for x in (a, b, c):
            x.close()
