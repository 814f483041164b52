"""Batch engine (cvb_batch_*): many solves in grouped launches.

Bars: each solve's result is bit-identical alone (a batch of one) and in the
mix, also when solves join a batch that is already running (continuous
batching); it converges to the requested relative residual (checked against
the reference operator's CSR from the oracle) and agrees with the single-solve
path within 1e-8 relative L2, mean removed.
"""
import types

import numpy as np
import pytest

from cases import SCENARIOS, build
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0
RTOL = 1e-10


def _scenario(name):
    c = build(name)
    return types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], ucont=c["ucont"], bctype=c["bctype"],
                                 semi=c["semi"], per=c["per"])


@pytest.fixture(scope="module")
def items():
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    # the fully blocked slab is left out: its two fluid regions need a right-hand
    # side compatible in each region, which the noisy divergence is not
    probs = [_scenario(n) for n in SCENARIOS if n != "blocked_slab"]
    probs.append(W.make_problem((24, 16, 20), (1.0, 1.0, 1.0), 2.0, True, (False, False, False),
                                [(0.45, 0.5, 0.55, 0.2)]))
    probs.append(W.make_problem((32, 16, 16), (2.0, 1.0, 1.0), 2.5, False, (True, False, False), []))
    out = []
    for q, P in enumerate(probs):
        ctx = PoissonContext().setup(P)
        uc, _, _ = ctx.volume_flux_rev(P.ucont, 0.0, 1)
        b, _ = ctx.poisson_rhs(uc, DT, ST)
        b = W.noisy_rhs(b, P.nvert, P.metrics[-1]["Aj"], DT, seed=100 + q)
        out.append((ctx, P, b))
    yield out
    for ctx, _, _ in out:
        ctx.close()


def _run(items, precision, sel=None, smoother=0):
    from curvib_old_gb300.solver import SolveBatch
    sel = range(len(items)) if sel is None else sel
    extra = {} if smoother == 0 else {"smoother": 1, "omega": 1.0, "pre_sweeps": 1, "post_sweeps": 1}
    B = SolveBatch(precision=precision, rtol=RTOL, max_it=100, **extra)
    try:
        for q in sel:
            items[q][0].set_rhs(items[q][2])
        sts = B.solve([items[q][0] for q in sel])
        phis = [items[q][0].get_phi() for q in sel]
    finally:
        B.close()
    return sts, phis


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("smoother", [0, 1])
def test_alone_equals_in_mix(items, precision, smoother):
    sts_all, phis_all = _run(items, precision, smoother=smoother)
    for q in range(len(items)):
        sts1, phis1 = _run(items, precision, [q], smoother=smoother)
        assert sts1[0]["status"] == 0
        assert sts1[0]["iterations"] == sts_all[q]["iterations"]
        assert np.array_equal(phis1[0], phis_all[q]), q


@pytest.mark.parametrize("precision", [0, 1])
def test_converges_and_matches_single(items, precision):
    sts, phis = _run(items, precision)
    for (ctx, P, b), st, phi in zip(items, sts, phis):
        assert st["status"] == 0 and st["rel_residual"] <= RTOL, st
        L = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
        A = O.lhs_csr(L)
        r = b.ravel() - A @ phi.ravel()
        assert np.linalg.norm(r) <= 1.5 * RTOL * np.linalg.norm(b)
        ref, st1 = ctx.solve(b, precision=precision, rtol=RTOL, max_it=100)
        fl = np.zeros(b.shape, dtype=bool)
        fl[1:-1, 1:-1, 1:-1] = P.nvert[1:-1, 1:-1, 1:-1] < 0.1
        d = (phi[fl] - phi[fl].mean()) - (ref[fl] - ref[fl].mean())
        assert np.linalg.norm(d) <= 1e-8 * np.linalg.norm(ref[fl] - ref[fl].mean())
        assert np.all(phi[~fl] == 0.0)


def test_continuous_batching_joins_running_batch(items):
    """Solves submitted while others are mid-flight give the results they give alone."""
    from curvib_old_gb300.solver import SolveBatch
    alone = [_run(items, 1, [q])[1][0] for q in range(len(items))]
    B = SolveBatch(precision=1, rtol=RTOL, max_it=100)
    try:
        half = len(items) // 2
        tickets = {}
        for q in range(half):
            tickets[B.submit(items[q][0], b=items[q][2])] = q
        for _ in range(3):
            B.step()
        for q in range(half, len(items)):
            tickets[B.submit(items[q][0], b=items[q][2])] = q
        done = {}
        for _ in range(10000):
            left = B.step()
            for t, st in B.poll():
                q = tickets[t]
                assert st["status"] == 0, st
                done[q] = B.read_phi(items[q][0])
            if left == 0 and len(done) == len(items):
                break
        assert len(done) == len(items)
        for q in range(len(items)):
            assert np.array_equal(done[q], alone[q]), q
    finally:
        B.close()


def test_rejects_a_context_twice(items):
    from curvib_old_gb300._lib import CvbError
    from curvib_old_gb300.solver import SolveBatch
    B = SolveBatch(precision=1, rtol=RTOL)
    try:
        B.submit(items[0][0])
        with pytest.raises(CvbError):
            B.submit(items[0][0])
        while B.step():
            pass
        assert len(B.poll()) == 1
    finally:
        B.close()


def test_round_limit_times_out_and_batch_stays_usable(items):
    """A round limit below what the solves need makes cvb_batch_solve return
    CVB_TIMEOUT with the solves still in flight; stepping and polling then carry
    them to the results they give without a limit, and the batch solves again
    once the limit is lifted."""
    from curvib_old_gb300._lib import CVB_TIMEOUT, CvbError
    from curvib_old_gb300.solver import SolveBatch
    sel = [0, 1, 2]
    _, alone = _run(items, 1, sel)
    B = SolveBatch(precision=1, rtol=RTOL, max_it=100)
    try:
        for q in sel:
            items[q][0].set_rhs(items[q][2])
        B.set_round_limit(2)
        with pytest.raises(CvbError) as e:
            B.solve([items[q][0] for q in sel])
        assert e.value.status == CVB_TIMEOUT
        assert B.step() > 0
        done = 0
        for _ in range(10000):
            left = B.step()
            for t, st in B.poll():
                assert st["status"] == 0, st
                done += 1
            if left == 0:
                break
        assert done == len(sel)
        for k, q in enumerate(sel):
            assert np.array_equal(items[q][0].get_phi(), alone[k]), q
        B.set_round_limit(0)
        for q in sel:
            items[q][0].set_rhs(items[q][2])
        sts = B.solve([items[q][0] for q in sel])
        assert all(st["status"] == 0 for st in sts)
        for k, q in enumerate(sel):
            assert np.array_equal(items[q][0].get_phi(), alone[k]), q
    finally:
        B.close()


def test_graph_replay_equals_eager_launches(items):
    """Mixed rounds replay their V-cycles from CUDA graphs while the iterating
    set is unchanged; the results must be the eager launches' bit for bit."""
    from curvib_old_gb300.solver import SolveBatch
    out = {}
    for graphs in (True, False):
        B = SolveBatch(precision=1, rtol=RTOL, max_it=100)
        try:
            B.set_graphs(graphs)
            for ctx, _, b in items:
                ctx.set_rhs(b)
            sts = B.solve([ctx for ctx, _, _ in items])
            out[graphs] = (sts, [ctx.get_phi() for ctx, _, _ in items], B.graph_stats())
        finally:
            B.close()
    (s1, p1, g1), (s0, p0, g0) = out[True], out[False]
    assert g1["replays"] > 0 and g1["captures"] >= 1
    assert g0["replays"] == 0
    for q in range(len(items)):
        assert s1[q]["status"] == 0 and s1[q]["iterations"] == s0[q]["iterations"]
        assert np.array_equal(p1[q], p0[q]), q
