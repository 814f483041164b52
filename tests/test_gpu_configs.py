"""The GPU path against the CPU oracle on the workloads the numbers are quoted on.

- box64_sphere_3lev: the 64^3 distorted box with a sphere of radius 0.15, FP64,
  3 multigrid levels.  Every level's restricted nvert and FullyBlocked result
  bit for bit, every level's 19 stored weights equal to the reference
  operator's CSR (PoissonLHSNew through the oracle) bit for bit, the FP64 apply
  within 1e-12 and the FP32 apply within its storage bound, and the converged
  pressure in both precisions against the oracle's own FGMRES + PCMG solve.
- channel256x128x128_5lev: the periodic channel with 5 levels.  The finest
  level's FP64 and FP32 applies against the oracle's CSR; every level's nvert
  and rows; the pressure, mixed and FP64, against the oracle solve.
- box_classes_batched: one problem of each of the five size classes of the
  batched workload (32^3, 48^3, 64x64x96, 96^3, 128x64x64, each with its
  seeded sphere), solved together in one batch, each against the oracle.
- blocked_slab_two_regions: a solid plate across the whole section splits the
  fluid in two (FullyBlocked sets multinullspace on the coarsest level, whose
  null space then has one constant per region, poisson.c:411-496,
  1578-1660).  The right-hand side is made compatible in each region; the
  pressure, each region's mean removed, against a direct solve of the
  reference operator with both region means pinned.

The pressure bar is the one the port states: within 1e-8 relative L2, mean
removed, of an FP64 solve.  Both sides are converged to rtol 1e-12 first: the
solution error of a solve stopped at rtol r is up to the operator's condition
number times r, and the stretched 256x128x128 channel stopped at 1e-10 is
already 1.6e-8 from its converged pressure (the oracle's own 1e-10 answer on
the 64^3 box is 4e-10 from its 1e-12 one).
"""
import numpy as np
import pytest

from oracle import oracle as O
from parity_util import direct_solution, fluid_mask, mean_removed_error, weights_to_csr

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0
GPU_RTOL, ORACLE_RTOL = 1e-12, 1e-12
PHI_BAR = 1e-8


def _rhs(P, Ls, seed, noise=True):
    from curvib_old_gb300 import workload as W
    uc, _, _ = O.volume_flux_rev(Ls[-1], P.ucont, 0.0, 1)
    b, _ = O.poisson_rhs(Ls[-1], uc, DT, ST)
    if noise:
        return W.noisy_rhs(b, Ls[-1].nvert, P.metrics[-1]["Aj"], DT, seed=seed)
    return W.compatible(b, P.metrics[-1]["Aj"], Ls[-1].nvert)


def _check_levels(ctx, P, Ls, all_rows=True):
    for l in range(len(Ls)):
        nv, mns = ctx.get_nvert(l)
        assert np.array_equal(nv, Ls[l].nvert), ("nvert", l)
        if all_rows or l == len(Ls) - 1:
            d = O.lhs_csr(Ls[l]) - weights_to_csr(ctx.weights(l), ctx.shapes[l], P.bctype)
            d.eliminate_zeros()
            assert d.nnz == 0, ("rows differ", l)
    assert mns == O.fully_blocked(Ls[0])[0]


def _check_applies(ctx, Ls, levels):
    for l in levels:
        A = O.lhs_csr(Ls[l])
        x = np.random.default_rng(70 + l).standard_normal(ctx.shapes[l])
        y_ref = (A @ x.ravel()).reshape(x.shape)
        y = ctx.apply(l, x)
        assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max(), ("FP64 apply", l)
        x32 = x.astype(np.float32)
        y32 = ctx.apply_f32(l, x32).astype(np.float64)
        y_ref32 = (A @ x32.astype(np.float64).ravel()).reshape(x.shape)
        bound = 2e-6 * abs(A).max() * np.abs(x).max() * 4
        assert np.abs(y32 - y_ref32).max() <= bound, ("FP32 apply", l)


def _check_solves(ctx, P, Ls, b, x_ref, regions):
    A = O.lhs_csr(Ls[-1])
    for precision in (0, 1):
        phi, st = ctx.solve(b, precision=precision, rtol=GPU_RTOL, max_it=400)
        assert st["status"] == 0 and st["rel_residual"] <= GPU_RTOL, st
        r = b.ravel() - A @ phi.ravel()
        assert np.linalg.norm(r) <= 2 * GPU_RTOL * np.linalg.norm(b), precision
        err = mean_removed_error(phi, x_ref, regions)
        assert err <= PHI_BAR, (precision, err)
        fl = np.zeros(b.shape, dtype=bool)
        for m in regions:
            fl |= m
        assert np.all(phi[~fl] == 0.0)


@pytest.fixture(scope="module")
def box64():
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    P = W.config0_problem(64, nlevels=3)
    Ls = O.levels_for(P)
    ctx = PoissonContext().setup(P)
    yield ctx, P, Ls
    ctx.close()


def test_box64_sphere_3lev_levels_bit_exact(box64):
    ctx, P, Ls = box64
    assert len(Ls) == 3 and ctx.shapes[0] == (18, 18, 18)
    _check_levels(ctx, P, Ls)


def test_box64_sphere_3lev_applies(box64):
    ctx, P, Ls = box64
    _check_applies(ctx, Ls, range(3))


def test_box64_sphere_3lev_solve_vs_oracle(box64):
    ctx, P, Ls = box64
    b = _rhs(P, Ls, seed=0)
    x_ref, its, rr, _, _ = O.solve_mg(Ls, b, rtol=ORACLE_RTOL, max_it=500)
    assert rr <= ORACLE_RTOL
    _check_solves(ctx, P, Ls, b, x_ref, [fluid_mask(Ls[-1].nvert)])


@pytest.fixture(scope="module")
def channel():
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    P = W.config1_problem()
    Ls = O.levels_for(P)
    ctx = PoissonContext().setup(P)
    yield ctx, P, Ls
    ctx.close()


def test_channel256x128x128_5lev_levels_and_applies(channel):
    ctx, P, Ls = channel
    assert len(Ls) == 5 and ctx.shapes[-1] == (130, 130, 258)
    _check_levels(ctx, P, Ls)
    _check_applies(ctx, Ls, [len(Ls) - 1])


def test_channel256x128x128_5lev_solve_vs_oracle(channel):
    ctx, P, Ls = channel
    b = _rhs(P, Ls, seed=0, noise=False)
    x_ref, its, rr, _, _ = O.solve_mg(Ls, b, rtol=ORACLE_RTOL, max_it=500)
    assert rr <= ORACLE_RTOL
    _check_solves(ctx, P, Ls, b, x_ref, [fluid_mask(Ls[-1].nvert)])


@pytest.mark.parametrize("name,rtol,budget", [("channel", 1e-10, 8), ("box64", 1e-8, 10)])
def test_iteration_counts(request, name, rtol, budget):
    """The measured configurations' FGMRES iteration counts at the bench's
    tolerances (channel 6 at 1e-10, box 8 at 1e-8 on the GB300, in both
    precisions) guard the Krylov loop's numerics: a change that still reaches
    the right answer but erodes the basis (a norm taken from ||w||^2 - ||h||^2,
    say) shows up here as many more iterations."""
    ctx, P, Ls = request.getfixturevalue(name)
    b = _rhs(P, Ls, seed=0, noise=name == "box64")
    for precision in (0, 1):
        _, st = ctx.solve(b, precision=precision, rtol=rtol, max_it=400)
        assert st["status"] == 0 and st["iterations"] <= budget, (name, precision, st)


def test_box_classes_batched_vs_oracle():
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext, SolveBatch
    seen, items = set(), []
    for P, seed in W.config3_problems(64, seed=3):
        cells = tuple(c - 2 for c in P.shape[::-1])
        if cells in seen:
            continue
        seen.add(cells)
        Ls = O.levels_for(P)
        b = _rhs(P, Ls, seed=seed)
        ctx = PoissonContext().setup(P)
        ctx.set_rhs(b)
        items.append((P, Ls, b, ctx))
    assert seen == set(W.CONFIG3_SIZES)
    try:
        for precision in (0, 1):
            B = SolveBatch(precision=precision, rtol=GPU_RTOL, max_it=400)
            try:
                for _, _, b, ctx in items:
                    ctx.set_rhs(b)
                sts = B.solve([it[3] for it in items])
            finally:
                B.close()
            for (P, Ls, b, ctx), st in zip(items, sts):
                assert st["status"] == 0 and st["rel_residual"] <= GPU_RTOL, (P.name, st)
                x_ref, its, rr, _, _ = O.solve_mg(Ls, b, rtol=ORACLE_RTOL, max_it=500)
                err = mean_removed_error(ctx.get_phi(), x_ref, [fluid_mask(Ls[-1].nvert)])
                assert err <= PHI_BAR, (P.name, precision, err)
    finally:
        for it in items:
            it[3].close()


def test_blocked_slab_two_regions():
    import types

    from cases import build
    from curvib_old_gb300.solver import PoissonContext
    c = build("blocked_slab")
    P = types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], ucont=c["ucont"], bctype=c["bctype"],
                              semi=c["semi"])
    Ls = O.levels_for(P)
    mns, _ = O.fully_blocked(Ls[0])
    assert mns, "the slab must block every k-line of the coarsest level"
    fl = fluid_mask(Ls[-1].nvert)
    mz = fl.shape[0]
    k = np.arange(mz)[:, None, None]
    regions = [fl & (k < mz // 2), fl & (k >= mz // 2)]
    assert all(m.any() for m in regions) and not (fl & ~(regions[0] | regions[1])).any()
    uc, _, _ = O.volume_flux_rev(Ls[-1], P.ucont, 0.0, 1)
    b, _ = O.poisson_rhs(Ls[-1], uc, DT, ST)
    b = b + np.where(fl, np.random.default_rng(5).uniform(-1e-2, 1e-2, b.shape) / DT, 0.0)
    aj = P.metrics[-1]["Aj"]
    for m in regions:  # compatible in each region: the sum of b/aj over it is 0
        b[m] -= aj[m] * (b[m] / aj[m]).mean()
    A = O.lhs_csr(Ls[-1])
    x_ref = direct_solution(A, b, regions)
    ctx = PoissonContext().setup(P)
    try:
        assert ctx.get_nvert(0)[1] == mns
        _check_solves(ctx, P, Ls, b, x_ref, regions)
    finally:
        ctx.close()
